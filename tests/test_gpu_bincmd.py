"""bin_cmd / partial_cmd on the GPU (histogram.cu) against the oracle
(src/StarFormationHistories.jl:544-553, 733-757).

Bin assignment is index work: with unit weights the device histogram equals the oracle's
bit for bit, including points exactly on interior edges (the bin the edge opens), on the
first edge (kept) and on the last (dropped), for both the shared-memory path (grid of at
most 12,288 bins) and the global-atomic path.  Weighted sums are FP64 with another order of
additions: rtol 1e-12."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _points(rng, n, ex, ey, on_edge=0.3):
    x = rng.uniform(ex[0] - 0.2, ex[-1] + 0.2, n)
    y = rng.uniform(ey[0] - 0.2, ey[-1] + 0.2, n)
    k = rng.random(n) < on_edge
    x[k] = rng.choice(ex, k.sum())
    k = rng.random(n) < on_edge
    y[k] = rng.choice(ey, k.sum())
    return x, y


@pytest.mark.parametrize("grid", [(41, 101), (301, 201)])  # 4,000 bins (shared), 60,000 (global)
def test_bin_cmd_exact_bins(sfh, O, grid):
    rng = np.random.default_rng(grid[0])
    ex = sfh.julia_range(-0.5, 1.5, grid[0] + 1)
    ey = sfh.julia_range(17.0, 27.0, grid[1] + 1)
    x, y = _points(rng, 1_000_000, np.asarray(ex), np.asarray(ey))
    h = sfh.bin_cmd(x, y, edges=(ex, ey))
    ref = O.bin_cmd(x, y, None, ex, ey)
    assert h.weights.shape == grid
    assert np.array_equal(h.weights, ref)
    w = rng.exponential(size=x.size)
    hw = sfh.bin_cmd(x, y, weights=w, edges=(ex, ey))
    np.testing.assert_allclose(hw.weights, O.bin_cmd(x, y, w, ex, ey), rtol=1e-12, atol=1e-12)


def test_bin_cmd_limits_and_widths(sfh, O):
    rng = np.random.default_rng(3)
    x = np.round(rng.normal(0.6, 0.3, 50000), 3)  # catalogue precision: many points on edges
    y = np.round(rng.uniform(20.0, 26.0, 50000), 3)
    h = sfh.bin_cmd(x, y, xwidth=0.05, ywidth=0.1)  # xlim / ylim = extrema
    ex, ey = h.edges
    assert ex[0] == x.min() and ex[-1] == x.max() and ey[0] == y.min() and ey[-1] == y.max()
    assert np.array_equal(h.weights, O.bin_cmd(x, y, None, ex, ey))
    # the points on the upper limits fall on the last edges and are dropped
    assert h.weights.sum() == np.sum((x < x.max()) & (y < y.max()))
    h2 = sfh.bin_cmd(x, y, nbins=(30, 40), xlim=(1.5, -0.5), ylim=(26.0, 19.0))
    assert np.array_equal(h2.weights, O.bin_cmd(x, y, None, h2.edges[0], h2.edges[1]))


def test_bin_cmd_empty_outside_and_errors(sfh):
    e = (np.linspace(0, 1, 11), np.linspace(0, 1, 6))
    assert not sfh.bin_cmd(np.array([]), np.array([]), edges=e).weights.any()
    assert not sfh.bin_cmd(np.array([2.0, np.nan]), np.array([0.5, 0.5]), edges=e).weights.any()
    with pytest.raises(ValueError):
        sfh.bin_cmd(np.zeros(3), np.zeros(2), edges=e)
    with pytest.raises(ValueError):
        sfh.bin_cmd(np.zeros(3), np.zeros(3), edges=(np.array([0.0, 1.0, 0.5]), e[1]))


def test_partial_cmd_matches_oracle(sfh, O):
    from sfhgpu import synthetic as S
    m, mags = S.isochrone(9.5, -1.0, 80)
    mags = np.asarray(mags, dtype=np.float64)
    c, mg = mags[0] - mags[1], mags[1]
    imf = sfh.Kroupa2001()
    ex = sfh.julia_range(c.min() - 0.1, c.max() + 0.1, 61)
    ey = sfh.julia_range(mg.min() + 24.8, mg.max() + 25.2, 81)
    h = sfh.partial_cmd(m, c, mg, imf, dmod=25.0, normalize_value=1e4, edges=(ex, ey))
    ref = O.partial_cmd(m, c, mg, O.kroupa2001(), 25.0, 1e4, imf.mean(), ex, ey)
    np.testing.assert_allclose(h.weights, ref, rtol=1e-12, atol=1e-12 * ref.max())
    assert h.weights.sum() == pytest.approx(ref.sum(), rel=1e-13)
    # reference defaults: limits from the unshifted isochrone (dmod = 0 keeps it inside)
    h0 = sfh.partial_cmd(m, c, mg, imf, nbins=(40, 60))
    r0 = O.partial_cmd(m, c, mg, O.kroupa2001(), 0.0, 1.0, imf.mean(), h0.edges[0], h0.edges[1])
    np.testing.assert_allclose(h0.weights, r0, rtol=1e-12, atol=1e-12 * r0.max())
