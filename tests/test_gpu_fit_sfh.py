"""Device fit_sfh (hierarchical MAP then MLE, generic_fitting.jl:242-409) against scipy's
BFGS over the FP64 oracle's hierarchical objective (mzr.jl:84-215, amr.jl:78-160 with
the transforms and Jacobian terms of generic_fitting.jl:117-171), FP64 template storage.

Optim's iterates cannot be reproduced (HagerZhang line search), so parity is on the
optimum: transformed variables within rtol 1e-5 and the objective within 1e-9 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(sfh, mzr, disp, nages=8, nmh=5, nbins=6000, n_stars=1e5, seed=3):
    rng = np.random.default_rng(seed)
    la = np.repeat(np.linspace(7.0, 10.0, nages), nmh)
    mh = np.tile(np.linspace(-2.5, 0.0, nmh), nages)
    # templates per unit stellar mass (~1e-5 stars per bin and solar mass), so the stellar
    # masses per age are ~1e6 Msun and the mass-metallicity relation sits inside the grid
    M = 1e-5 * rng.random((nbins, nages * nmh)) * (rng.random((nbins, nages * nmh)) > 0.3)
    R = np.exp(0.5 * rng.standard_normal(nages))
    r = sfh.calculate_coeffs(mzr, disp, R, la, mh)
    s = n_stars / (M @ r).sum()
    R *= s
    r = sfh.calculate_coeffs(mzr, disp, R, la, mh)
    data = rng.poisson(M @ r).astype(float)
    return np.asfortranarray(M), R, la, mh, data


def _scipy_fit(O, kind, mzr, disp, M, data, la, mh, th0, map_):
    """BFGS over the oracle's objective in the transformed variables."""
    from scipy.optimize import minimize
    nages = th0.size - 3
    logtf = [True] * nages + [True, kind == "logamr", True]  # α log; β log only for LogarithmicAMR

    def f(th):
        v = np.where(logtf, np.exp(th), th)
        if kind == "mzr":
            val, G = O.mzr_fg(v, mzr.logMstar0, M, data, la, mh)
        else:
            val, G = O.amr_fg(v, mzr.T_max, M, data, la, mh, kind=0 if kind == "linamr" else 1)
        g = G * np.where(logtf, v, 1.0)
        if map_:
            val = val - np.sum(np.where(logtf, th, 0.0))
            g = g - np.where(logtf, 1.0, 0.0)
        return val, g
    r = minimize(f, th0, jac=True, method="BFGS", options={"gtol": 1e-9, "maxiter": 5000})
    return r.x, f(r.x)[0]


@pytest.mark.parametrize("kind", ["mzr", "linamr"])
def test_fit_sfh_matches_scipy_on_the_oracle(sfh, O, kind):
    if kind == "mzr":
        truth = sfh.PowerLawMZR(0.5, -1.0, 6.0)
        start = sfh.PowerLawMZR(0.4, -0.8, 6.0)
    else:
        truth = sfh.LinearAMR(0.1, -2.0, 13.7)
        start = sfh.LinearAMR(0.08, -1.8, 13.7)
    disp = sfh.GaussianDispersion(0.2)
    M, R, la, mh, data = _problem(sfh, truth, disp)
    H = sfh.Models(M, storage="f64")
    x0 = R * np.exp(0.3 * np.random.default_rng(1).standard_normal(R.size))
    res = sfh.fit_sfh(start, sfh.GaussianDispersion(0.25), H, data, la, mh, x0=x0,
                      g_abstol=1e-8)
    assert res.map.result["converged"] and res.mle.result["converged"], (res.map.result, res.mle.result)
    # the same start the device used (renormalised x0, transformed)
    th0 = sfh.sampling.mzr_theta(sfh.fit_sfh_x0(start, sfh.GaussianDispersion(0.25), H, data,
                                                la, mh, x0),
                                 start, sfh.GaussianDispersion(0.25))
    for map_, got in ((True, res.map), (False, res.mle)):
        th_ref, f_ref = _scipy_fit(O, kind, start, None, M, data, la, mh,
                                   th0 if map_ else res.map.theta, map_)
        np.testing.assert_allclose(got.theta, th_ref, rtol=1e-5, atol=1e-6)
        assert abs(got.result["f"] - f_ref) <= 1e-9 * abs(f_ref)
    # natural-scale results and standard errors assembled as the reference does
    nages = R.size
    np.testing.assert_allclose(res.map.mu[:nages], np.exp(res.map.theta[:nages]), rtol=1e-14)
    assert np.all(res.map.sigma > 0)
    assert abs(res.map.disp_model.sigma - res.map.mu[-1]) == 0
    # recovery of the generating model within a few standard errors
    assert abs(res.mle.mu[nages] - truth.alpha) < 5 * res.mle.sigma[nages] + 0.05


def test_fit_sfh_renormalises_nan_x0(sfh):
    """An MZR far from the stellar mass x0 implies gives NaN coefficients: x0 is replicated
    over the metallicity bins and renormalised (generic_fitting.jl:261-283)."""
    truth = sfh.PowerLawMZR(0.5, -1.0, 6.0)
    disp = sfh.GaussianDispersion(0.2)
    M, R, la, mh, data = _problem(sfh, truth, disp)
    H = sfh.Models(M, storage="f64")
    far = sfh.PowerLawMZR(0.5, 80.0, 6.0)  # μ ~ 80: every Gaussian weight underflows
    x0 = np.ones(R.size)
    with pytest.warns(UserWarning):
        x = sfh.fit_sfh_x0(far, disp, H, data, la, mh, x0)
    full = np.tile(x0, 5)
    expect = x0 * data.sum() / (M @ full).sum()  # renormalize_x0 with the replicated coefficients
    np.testing.assert_allclose(x, expect, rtol=1e-12)


def test_sample_sfh_starts_from_the_map_fit(sfh):
    truth = sfh.PowerLawMZR(0.5, -1.0, 6.0)
    disp = sfh.GaussianDispersion(0.2)
    M, R, la, mh, data = _problem(sfh, truth, disp, n_stars=1e6)
    res = sfh.fit_sfh(sfh.PowerLawMZR(0.45, -0.9, 6.0), sfh.GaussianDispersion(0.25),
                      sfh.Models(M, storage="f64"), data, la, mh, x0=R * 1.2)
    Hb = sfh.Models(M.astype(np.float32), storage="bf16x2")
    out = sfh.sample_sfh(Hb, data, la, mh, nsteps=150, nchains=64, nwarmup=150, nleap=10,
                         step0=1e-2, fit=res)
    pm = out["mean"].mean(0)
    nages = R.size
    # posterior means near the MAP point (a few of its standard errors)
    assert np.all(np.abs(pm[:nages] - res.map.mu[:nages]) < 4 * res.map.sigma[:nages] + 1e-9)
    assert abs(pm[nages] - res.map.mu[nages]) < 4 * res.map.sigma[nages]
    assert np.mean(out["accept"]) > 0.3


def test_sample_sfh_nuts_as_the_reference_runs_it(sfh):
    """sample_sfh with a fit and sampler "nuts" is the reference's run: every chain starts
    at the MLE point with the MAP inverse Hessian as a dense metric and a fixed step of
    0.05 without warmup (generic_fitting.jl:470-490); with step adaptation the same run
    recovers the fit."""
    truth = sfh.PowerLawMZR(0.5, -1.0, 6.0)
    disp = sfh.GaussianDispersion(0.2)
    M, R, la, mh, data = _problem(sfh, truth, disp, n_stars=1e6)
    res = sfh.fit_sfh(sfh.PowerLawMZR(0.45, -0.9, 6.0), sfh.GaussianDispersion(0.25),
                      sfh.Models(M, storage="f64"), data, la, mh, x0=R * 1.2)
    Hb = sfh.Models(M.astype(np.float32), storage="bf16x2")
    fixed = sfh.sample_sfh(Hb, data, la, mh, nsteps=20, nchains=16, nwarmup=0, step0=0.05,
                           fit=res, sampler="nuts")
    assert np.all(fixed["step"] == 0.05)        # no warmup: the reference's fixed step
    # with step adaptation around the same dense metric
    out = sfh.sample_sfh(Hb, data, la, mh, nsteps=200, nchains=64, nwarmup=150, step0=0.05,
                         fit=res, sampler="nuts")
    pm = out["mean"].mean(0)
    nages = R.size
    assert np.all(np.abs(pm[:nages] - res.mle.mu[:nages]) < 4 * res.map.sigma[:nages] + 1e-9)
    assert abs(pm[nages] - res.mle.mu[nages]) < 4 * res.map.sigma[nages]
    assert np.mean(out["accept"]) > 0.6, np.mean(out["accept"])
    assert np.mean(out["divergent"]) < 1.0
