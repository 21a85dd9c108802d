"""Hard-binned Hess diagrams: the oracle's restatement of bin_cmd and partial_cmd
(src/StarFormationHistories.jl:544-553, 733-757) and the Julia range elements the edges
are built from (calculate_edges :451-476).

The reference holds no tests of bin_cmd; the oracle is pinned by an independent
implementation (numpy's histogram2d, which bins left-closed on the same edge values except
that it keeps points on the last edge, which StatsBase's closed=:left drops), by the edge
rules, and by mass conservation of partial_cmd's trapezoidal IMF weights."""
import numpy as np
import pytest


def test_julia_range_elements(sfh):
    # range(a, b, length=n) and a:s:b hold the correctly rounded decimals, as Julia's do
    r = sfh.julia_range(17.0, 27.0, 101)
    assert list(r) == [float(f"{17 + k / 10:.1f}") for k in range(101)]
    assert r.step == 0.1
    assert sfh.julia_range(0.0, 1.0, 11)[3] == 0.3  # not 3 * 0.1 = 0.30000000000000004
    c = sfh.julia_colon(-1.0, 0.1, 1.5)
    assert len(c) == 26 and list(c) == [float(f"{-1 + k / 10:.1f}") for k in range(26)]
    assert len(sfh.julia_colon(22.0, 0.1, 27.2)) == 53
    assert len(sfh.julia_colon(0.0, 0.3, 1.0)) == 4  # stop is not reached exactly
    # limits that are no ratio of small integers: exact endpoints, interpolation inside
    a, b = 0.012345678901234, 1.98765432109876
    r = sfh.julia_range(a, b, 7)
    assert r[0] == a and r[-1] == b and np.all(np.diff(r) > 0)
    np.testing.assert_allclose(r, np.linspace(a, b, 7), rtol=1e-15)
    e = sfh.calculate_edges(None, [1.5, -1.0], [25.0, 20.0], (26, 51))
    assert e[0][0] == -1.0 and e[0][-1] == 1.5 and e[1][0] == 20.0 and len(e[1]) == 51
    e = sfh.calculate_edges(None, [-1.0, 1.5], [20.0, 25.0], None, 0.1, 0.1)
    assert len(e[0]) == 25 and len(e[1]) == 50


def _points(rng, n, ex, ey, on_edge=0.3):
    x = rng.uniform(ex[0] - 0.2, ex[-1] + 0.2, n)
    y = rng.uniform(ey[0] - 0.2, ey[-1] + 0.2, n)
    k = rng.random(n) < on_edge  # exactly on an edge value (first and last included)
    x[k] = rng.choice(ex, k.sum())
    k = rng.random(n) < on_edge
    y[k] = rng.choice(ey, k.sum())
    return x, y


def _numpy_left_closed(x, y, w, ex, ey):
    keep = (x != ex[-1]) & (y != ey[-1])
    h, _, _ = np.histogram2d(x[keep], y[keep], bins=(ex, ey),
                             weights=None if w is None else w[keep])
    return h


def test_oracle_bin_cmd_matches_numpy(O, sfh):
    rng = np.random.default_rng(5)
    ex = np.asarray(sfh.julia_colon(-0.5, 0.05, 1.6))
    ey = np.asarray(sfh.julia_colon(17.0, 0.1, 27.0))
    x, y = _points(rng, 20000, ex, ey)
    h = O.bin_cmd(x, y, None, ex, ey)
    assert h.shape == (len(ex) - 1, len(ey) - 1)
    assert np.array_equal(h, _numpy_left_closed(x, y, None, ex, ey))
    w = rng.exponential(size=x.size)
    np.testing.assert_allclose(O.bin_cmd(x, y, w, ex, ey), _numpy_left_closed(x, y, w, ex, ey),
                               rtol=1e-12, atol=1e-12)


def test_oracle_bin_cmd_edge_rules(O, sfh):
    ex = np.asarray(sfh.julia_range(0.0, 1.0, 11))
    ey = np.array([0.0, 1.0])
    x = np.array([0.3, 0.0, 1.0, 0.999999, np.nan, -1e-300, np.inf, 0.7])
    y = np.full(x.size, 0.5)
    h = O.bin_cmd(x, y, None, ex, ey)[:, 0]
    expect = np.zeros(10)
    expect[3] += 1  # 0.3 opens bin 4 (1-based), as StatsBase on the range element 0.3
    expect[0] += 1  # the first edge is inside
    expect[9] += 1  # 0.999999; 1.0 (the last edge) is dropped
    expect[7] += 1  # 0.7 == ex[7]
    assert np.array_equal(h, expect)
    # a point on the last y edge is dropped as well
    assert O.bin_cmd([0.5], [1.0], None, ex, ey).sum() == 0.0


def _iso(n=80):
    from sfhgpu import synthetic as S
    m, mags = S.isochrone(9.5, -1.0, n)
    mags = np.asarray(mags, dtype=np.float64)
    return m, mags[0] - mags[1], mags[1]


def test_partial_cmd_oracle_and_host_points(O, sfh):
    m, c, mg = _iso()
    imf = sfh.Kroupa2001()
    ex = np.asarray(sfh.julia_range(c.min() - 0.1, c.max() + 0.1, 61))
    ey = np.asarray(sfh.julia_range(mg.min() + 25.0 - 0.2, mg.max() + 25.0 + 0.2, 81))
    h_or = O.partial_cmd(m, c, mg, O.kroupa2001(), 25.0, 1e4, imf.mean(), ex, ey)
    x, y, w = sfh.partial_cmd_points(m, c, mg, imf, 25.0, 1e4)
    np.testing.assert_allclose(O.bin_cmd(x, y, w, ex, ey), h_or, rtol=1e-12, atol=1e-12)
    # every point is inside the grid: the template holds the summed trapezoid weights,
    # normalize_value / mean_mass times the IMF integral over the isochrone's mass range
    assert h_or.sum() == pytest.approx(w.sum(), rel=1e-13)
    grid = np.linspace(m.min(), m.max(), 200001)
    integral = sfh.trapz(grid, imf(grid))
    assert w.sum() == pytest.approx(1e4 / imf.mean() * integral, rel=2e-3)


def test_julia_ranges_edge_cases(sfh):
    # a descending colon range and a step that does not land on stop
    d = sfh.julia_colon(1.0, -0.25, 0.0)
    assert list(d) == [1.0, 0.75, 0.5, 0.25, 0.0]
    assert list(sfh.julia_colon(0.0, 0.1, 0.35)) == [0.0, 0.1, 0.2, 0.3]
    assert len(sfh.julia_colon(1.0, 0.1, 0.0)) == 0  # empty, as in Julia
    with pytest.raises(ValueError):
        sfh.julia_colon(0.0, 0.0, 1.0)
    with pytest.raises(ValueError):
        sfh.julia_range(0.0, 1.0, 1)
    with pytest.raises(ValueError):
        sfh.julia_range(0.0, np.inf, 5)
    r = sfh.julia_range(2.0, 2.0, 4)
    assert list(r) == [2.0] * 4
    # the Range's step (Julia's step(r)) is what the smooth binning uses
    from sfhgpu.templates import _range
    f, st, n = _range(sfh.julia_range(17.0, 27.0, 101))
    assert (f, st, n) == (17.0, 0.1, 100)
    assert _range(np.linspace(0.0, 1.0, 11))[1] == pytest.approx(0.1, rel=1e-15)


def test_host_argument_checks(sfh):
    e = (np.linspace(0, 1, 11), np.linspace(0, 1, 6))
    with pytest.raises(ValueError):  # ragged inputs
        sfh.bin_cmd(np.zeros(3), np.zeros(2), edges=e)
    with pytest.raises(ValueError):  # weights of another length
        sfh.bin_cmd(np.zeros(3), np.zeros(3), weights=np.ones(2), edges=e)
    with pytest.raises(ValueError):  # edges not increasing
        sfh.bin_cmd(np.zeros(3), np.zeros(3), edges=(np.array([0.0, 1.0, 0.5]), e[1]))
    with pytest.raises(ValueError):  # edges not finite
        sfh.bin_cmd(np.zeros(3), np.zeros(3), edges=(np.array([0.0, np.nan]), e[1]))
    with pytest.raises(ValueError):  # neither edges, nbins nor widths
        sfh.bin_cmd(np.zeros(3), np.ones(3))
    f = [lambda m: np.zeros_like(m)] * 3
    with pytest.raises(ValueError):  # one callable per filter
        sfh.model_cmd(np.zeros((4, 3)), f[:2], f)
    with pytest.raises(ValueError):
        sfh.model_cmd(np.zeros((4, 3)), f, f, biasfuncs=f[:1])
    with pytest.raises(ValueError):  # (nstars, nfilters)
        sfh.model_cmd(np.zeros(4), f[:1], f[:1])
    with pytest.raises(ValueError):  # at most 8 filters
        sfh.model_cmd(np.zeros((2, 9)), [f[0]] * 9, [f[0]] * 9)
