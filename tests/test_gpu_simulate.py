"""model_cmd (src/simulate.jl:621-680) on the GPU (simulate.cu).

The reference draws from Julia's RNG, so parity is distributional: the kept fraction
follows the detection probabilities (binomial bounds, also per probability band), the
error draws are standard normal after removing σ and the bias (moments within 5 standard
errors), kept stars keep their input order, the draws are a function of (seed, star,
filter) only, and with unit completeness and zero errors the call is the identity.
The last test is the use the reference names for model_cmd, an independent check of
template fidelity: a catalogue drawn from the IMF along an isochrone, mock-observed and
hard-binned (bin_cmd), against the smooth template of partial_cmd_smooth for the same
population (errors, completeness, IMF and distance)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_model_cmd_identity_and_order(sfh):
    rng = np.random.default_rng(1)
    m = rng.uniform(20, 26, (1000, 3))
    one = [lambda x: np.ones_like(x)] * 3
    zero = [lambda x: np.zeros_like(x)] * 3
    out, idx = sfh.model_cmd(m, zero, one, ret_idxs=True, seed=5)
    assert np.array_equal(out, m) and np.array_equal(idx, np.arange(1000))
    out0 = sfh.model_cmd(np.empty((0, 2)), zero[:2], one[:2])
    assert out0.shape == (0, 2)
    with pytest.raises(ValueError):
        sfh.model_cmd(m, zero[:2], one)


def test_model_cmd_statistics(sfh):
    rng = np.random.default_rng(2)
    n = 2_000_000
    m = rng.uniform(20, 28, (n, 2))
    c_true = rng.random(n)
    comp = [lambda x, c=c_true: np.sqrt(c), lambda x, c=c_true: np.sqrt(c)]  # product = c
    err = [lambda x: 0.01 + 0.02 * (x - 20.0), lambda x: np.full_like(x, 0.05)]
    bias = [lambda x: 0.1 * np.ones_like(x), lambda x: -0.02 * (x - 24.0)]
    out, idx = sfh.model_cmd(m, err, comp, bias, seed=123, ret_idxs=True)
    k = idx.size
    exp_k = c_true.sum()
    assert abs(k - exp_k) <= 5 * np.sqrt(np.sum(c_true * (1 - c_true)))
    assert np.all(np.diff(idx) > 0)
    # kept fraction per probability band
    band = np.minimum((c_true * 10).astype(int), 9)
    kept = np.zeros(n, bool)
    kept[idx] = True
    for b in range(10):
        sel = band == b
        p = c_true[sel].mean()
        assert abs(kept[sel].mean() - p) <= 5 * np.sqrt(p * (1 - p) / sel.sum()) + 1e-12
    # standardised errors
    mk = m[idx]
    sig = np.stack([err[0](mk[:, 0]), err[1](mk[:, 1])], 1)
    b = np.stack([bias[0](mk[:, 0]), bias[1](mk[:, 1])], 1)
    z = (out - mk - b) / sig
    se = 1 / np.sqrt(k)
    for j in range(2):
        assert abs(z[:, j].mean()) <= 5 * se
        assert abs(z[:, j].var() - 1) <= 5 * np.sqrt(2) * se
        assert abs(np.mean(z[:, j] ** 3)) <= 5 * np.sqrt(15) * se   # symmetric
        assert abs(np.mean(z[:, j] ** 4) - 3) <= 5 * np.sqrt(96) * se
    assert abs(np.corrcoef(z[:, 0], z[:, 1])[0, 1]) <= 5 * se  # filters independent
    # the same seed repeats, another seed does not; a subset keeps its stars' draws
    out2, idx2 = sfh.model_cmd(m, err, comp, bias, seed=123, ret_idxs=True)
    assert np.array_equal(out, out2) and np.array_equal(idx, idx2)
    out3 = sfh.model_cmd(m, err, comp, bias, seed=124)
    assert out3.shape != out.shape or not np.array_equal(out3, out)


def test_mock_observed_catalogue_matches_smooth_template(sfh):
    from sfhgpu import synthetic as S
    rng = np.random.default_rng(7)
    m_ini, mags = S.isochrone(9.5, -1.0, 400)
    imf = S.imf()
    dmod = 25.0
    xe = sfh.julia_range(0.0, 1.6, 41)
    ye = sfh.julia_range(24.0, 30.0, 61)
    nv = 4.0e5  # stellar mass of the population
    T = sfh.partial_cmd_smooth(m_ini, list(mags), S.error_funcs(), 2, (0, 1), imf,
                               S.completeness_funcs(), dmod=dmod, normalize_value=nv,
                               edges=(xe, ye)).weights
    # the population: Poisson(nv / mean mass) stars from the IMF (inverse CDF on a fine
    # log grid); stars outside the isochrone's mass range have no magnitudes (dropped)
    grid = np.logspace(np.log10(imf.mmin), np.log10(imf.mmax), 400001)
    cdf = np.concatenate([[0.0], np.cumsum(np.diff(grid) * (imf(grid[1:]) + imf(grid[:-1])) / 2)])
    cdf /= cdf[-1]
    nstar = rng.poisson(nv / imf.mean())
    mass = np.interp(rng.random(nstar), cdf, grid)
    mass = mass[(mass >= m_ini.min()) & (mass <= m_ini.max())]
    cat = np.stack([sfh.interpolate_mini(m_ini, mags[f], mass) + dmod for f in range(3)], 1)
    obs = sfh.model_cmd(cat, S.error_funcs(), S.completeness_funcs(), seed=99)
    H = sfh.bin_cmd(obs[:, 0] - obs[:, 1], obs[:, 2], edges=(xe, ye)).weights
    tot_t, tot_h = T.sum(), H.sum()
    sel = T > 20
    chi2 = np.sum((H[sel] - T[sel]) ** 2 / T[sel]) / sel.sum()
    print("template", tot_t, "mock", tot_h, "bins", sel.sum(), "chi2/bin", chi2)
    assert abs(tot_h / tot_t - 1) <= 0.02 + 5 / np.sqrt(tot_t)
    assert chi2 < 1.5
