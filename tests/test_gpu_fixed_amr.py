"""fixed_amr on the GPU (hierarchical/fixed_amr.jl), mirroring fixed_amr_test.jl:60-110
with our own random numbers: noise-free recovery to rtol 1e-5, the renormalisation
warning, and truncated relative weights."""
import warnings

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(a, b, rtol):  # isapprox on vectors
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


@pytest.fixture(scope="module")
def problem(sfh):
    from sfhgpu import GaussianDispersion, LinearAMR, calculate_coeffs, construct_x0_mdf
    la = np.repeat(np.round(np.arange(8.0, 10.0 + 1e-9, 0.1), 10), 26)
    mh = np.tile(np.round(np.arange(-2.5, 0.0 + 1e-9, 0.1), 10), 21)
    amr, disp = LinearAMR(0.05, -1.0 - 0.05 * 12.0), GaussianDispersion(0.2)
    rng = np.random.default_rng(58392)
    sfrs = rng.random(21)
    x = calculate_coeffs(amr, disp, sfrs, la, mh)
    models = rng.random((100 * 100, la.size)) * 100
    data = models @ x
    rw = calculate_coeffs(amr, disp, np.ones(21), la, mh)
    x0 = construct_x0_mdf(la, 13.7, normalize_value=1.0)
    return la, mh, sfrs, models, data, rw, x0


def test_fixed_amr_recovers_noise_free_sfrs(sfh, problem):
    la, mh, sfrs, models, data, rw, x0 = problem
    res = sfh.fixed_amr(models, data, la, mh, rw, x0=x0)
    assert _close(res.mle.mu, sfrs, 1e-5), np.max(np.abs(res.mle.mu / sfrs - 1))
    assert np.all(np.isfinite(res.map.sigma)) and res.map.mu.size == 21


def test_fixed_amr_matches_full_objective(sfh, O, problem):
    """The reduced matrix gives the full objective: -logL and its gradient w.r.t. the
    per-age coefficients against the oracle on the expanded coefficient vector."""
    la, mh, sfrs, models, data, rw, x0 = problem
    M = sfh.Models(np.asfortranarray(models.astype(np.float32)), storage="f32")
    uniq = list(dict.fromkeys(la.tolist()))
    groups = [np.nonzero(la == u)[0] for u in uniq]
    Mr = M.combine(groups, [rw[g] for g in groups])
    rng = np.random.default_rng(3)
    xs = sfrs * np.exp(0.3 * rng.standard_normal(21))
    G = np.empty(21)
    v = sfh.fg_(True, G, xs, Mr, data, np.empty(M.nbins))
    full = np.concatenate([rw[g] * xs[i] for i, g in enumerate(groups)])
    order = np.concatenate(groups)
    coeffs = np.empty(la.size)
    coeffs[order] = full
    Mst = models.astype(np.float32).astype(np.float64)
    v_ref, G_ref, w_ref = O.fg(coeffs, np.asfortranarray(Mst), data)
    assert abs(v - v_ref) <= 1e-5 * max(1.0, data.sum() / 1e4)
    Gi = np.array([np.sum(G_ref[g] * rw[g]) for g in groups])
    scale = np.array([np.sum(np.abs(Mst[:, g] * rw[g]).T @ np.abs(w_ref)) for g in groups])
    assert np.max(np.abs(G - Gi) / scale) <= 5e-6


def test_fixed_amr_warnings_and_truncation(sfh, problem):
    la, mh, sfrs, models, data, rw, x0 = problem
    with pytest.warns(UserWarning):
        sfh.fixed_amr(models, data, la, mh, 2 * rw, x0=x0)
    keep = sfh.truncate_relweights(0.05, rw, la)
    with pytest.warns(UserWarning):
        r3 = sfh.fixed_amr(models[:, keep], data, la[keep], mh[keep], rw[keep], x0=x0)
    assert not _close(r3.mle.mu, sfrs, 1e-5)
    assert _close(r3.mle.mu, sfrs, 1e-2)
    assert np.median((r3.mle.mu - sfrs) / sfrs) < 1e-3
    with warnings.catch_warnings():
        warnings.simplefilter("error")  # relweightsmin renormalises without a warning
        r4 = sfh.fixed_amr(models, data, la, mh, rw, relweightsmin=0.05, x0=x0)
    assert _close(r3.mle.mu, r4.mle.mu, 1e-6)
