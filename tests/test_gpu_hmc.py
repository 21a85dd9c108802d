"""Batched HMC and the hierarchical (MZR) log density on the GPU.

* The MZR log density and gradient (calculate_coeffs + chain rule of mzr.jl:84-215 and
  the transforms / Jacobian terms of generic_fitting.jl:90-199) against the FP64 oracle
  on the same stored templates.
* hmc_sample's posterior against the Laplace approximation around the maximum
  likelihood point (observed Fisher information), which the posterior approaches for
  large counts; acceptance in range.
* sample_sfh (PowerLawMZR + GaussianDispersion) recovers the generating parameters.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16_hilo(x):
    import torch
    t = torch.tensor(np.asarray(x, dtype=np.float32))
    hi = t.to(torch.bfloat16).to(torch.float32)
    lo = (t - hi).to(torch.bfloat16).to(torch.float32)
    return (hi.double() + lo.double()).numpy()


def _mzr_problem(seed=11, nages=5, nmh=6, nbins=3000, scale=1.0):
    from sfhgpu.sampling import GaussianDispersion, PowerLawMZR, calculate_coeffs
    rng = np.random.default_rng(seed)
    la = np.repeat(np.linspace(10.0, 8.0, nages), nmh)
    mh = np.tile(np.linspace(-2.5, 0.0, nmh), nages)
    M = (rng.random((nbins, nages * nmh)) / 1e2).astype(np.float32)
    R = (rng.random(nages) * 1e4 + 1e3) * scale
    mzr, disp = PowerLawMZR(0.5, -1.0, 6.0), GaussianDispersion(0.2)
    coeffs = calculate_coeffs(mzr, disp, R, la, mh)
    data = rng.poisson(M.astype(np.float64) @ coeffs).astype(np.float64)
    return la, mh, np.asfortranarray(M), R, mzr, disp, data


def test_mzr_logdensity_matches_oracle(sfh, O):
    from sfhgpu.sampling import GaussianDispersion, PowerLawMZR, SFH_HMC_MZR, mzr_theta
    la, mh, M32, R, mzr, disp, data = _mzr_problem()
    H = sfh.Models(M32, storage="bf16x2")
    Ms = np.asfortranarray(_bf16_hilo(M32))
    rng = np.random.default_rng(5)
    thetas, nats = [], []
    for _ in range(6):
        Rb = R * np.exp(0.2 * rng.standard_normal(R.size))
        a = 0.5 * np.exp(0.2 * rng.standard_normal())
        b = -1.0 + 0.1 * rng.standard_normal()
        s = 0.2 * np.exp(0.2 * rng.standard_normal())
        thetas.append(mzr_theta(Rb, PowerLawMZR(a, b, 6.0), GaussianDispersion(s)))
        nats.append(np.concatenate([Rb, [a, b, s]]))
    theta = np.stack(thetas)
    logd, grad = sfh.logdensity_batched(H, data, theta, SFH_HMC_MZR, mzr, disp, la, mh)
    nst = data.sum()
    for k, v in enumerate(nats):
        nlogL, Gv = O.mzr_fg(v, 6.0, Ms, data, la, mh)
        na = R.size
        ref_logd = -nlogL + np.sum(np.log(v[:na])) + np.log(v[na]) + np.log(v[na + 2])
        ref_g = np.concatenate([-Gv[:na] * v[:na] + 1.0, [-Gv[na] * v[na] + 1.0, -Gv[na + 1],
                                                          -Gv[na + 2] * v[na + 2] + 1.0]])
        assert abs(logd[k] - ref_logd) <= 1e-2 * max(1.0, nst / 1e4), (logd[k], ref_logd)
        scale = np.abs(ref_g).max()
        np.testing.assert_allclose(grad[k], ref_g, rtol=2e-3, atol=2e-3 * scale)


def test_direct_logdensity_matches_oracle(sfh, O):
    from sfhgpu.sampling import SFH_HMC_DIRECT
    rng = np.random.default_rng(2)
    M32 = np.asfortranarray((rng.random((5000, 12)) * (rng.random((5000, 12)) > 0.3))
                            .astype(np.float32))
    x = rng.random(12) * 50 + 10
    data = rng.poisson(M32.astype(np.float64) @ x).astype(np.float64)
    H = sfh.Models(M32, storage="bf16x2")
    Ms = np.asfortranarray(_bf16_hilo(M32))
    theta = np.log(x)[None, :] + 0.1 * rng.standard_normal((5, 12))
    logd, grad = sfh.logdensity_batched(H, data, theta, SFH_HMC_DIRECT)
    for k in range(5):
        xs = np.exp(theta[k])
        v, G, _ = O.fg(xs, Ms, data)
        # hmc_sample.jl:34-36: logL + Σθ and -G x + 1
        assert abs(logd[k] - (-v + theta[k].sum())) <= 1e-2 * max(1.0, data.sum() / 1e4)
        ref = -G * xs + 1.0
        np.testing.assert_allclose(grad[k], ref, rtol=2e-3, atol=2e-3 * np.abs(ref).max())


def test_hmc_direct_matches_laplace_posterior(sfh):
    rng = np.random.default_rng(21)
    nbins, nt = 4000, 4
    M32 = np.asfortranarray((rng.random((nbins, nt)) ** 3).astype(np.float32))
    x_true = np.array([2000.0, 1000.0, 3000.0, 500.0]) / 100
    data = rng.poisson(M32.astype(np.float64) @ x_true).astype(np.float64)
    Ms = np.asfortranarray(_bf16_hilo(M32))
    _, mle = sfh.fit_templates_lbfgsb(sfh.Models(Ms, storage="f64"), data, x0=x_true,
                                      factr=10.0, pgtol=1e-10)
    m = Ms @ mle
    Hobs = (Ms * (data / m ** 2)[:, None]).T @ Ms  # observed information at the MLE
    sd_lap = np.sqrt(np.diag(np.linalg.inv(Hobs)))
    H = sfh.Models(M32, storage="bf16x2")
    out = sfh.hmc_sample(H, data, nsteps=400, nchains=64, nwarmup=300, nleap=10, seed=3)
    pm = out["mean"].mean(axis=0)
    pv = out["var"].mean(axis=0) + out["mean"].var(axis=0)
    assert 0.5 < out["accept"].mean() < 0.995, out["accept"].mean()
    assert np.all(np.abs(pm - mle) < 0.25 * sd_lap + 3 * np.sqrt(pv / (64 * 100))), (pm, mle, sd_lap)
    ratio = np.sqrt(pv) / sd_lap
    assert np.all((ratio > 0.8) & (ratio < 1.25)), ratio


def test_hmc_mzr_recovers_parameters(sfh):
    la, mh, M32, R, mzr, disp, data = _mzr_problem(seed=8, nbins=6000, scale=5.0)
    H = sfh.Models(M32, storage="bf16x2")
    from sfhgpu.sampling import GaussianDispersion, PowerLawMZR
    out = sfh.sample_sfh(H, data, la, mh, PowerLawMZR(0.4, -0.8, 6.0), GaussianDispersion(0.3),
                         R * 1.1, nsteps=300, nchains=32, nwarmup=300, nleap=10, seed=9)
    na = R.size
    pm = out["mean"].mean(axis=0)
    psd = np.sqrt(out["var"].mean(axis=0) + out["mean"].var(axis=0))
    truth = np.concatenate([R, [0.5, -1.0, 0.2]])
    assert 0.4 < out["accept"].mean() < 0.995, out["accept"].mean()
    z = np.abs(pm - truth) / psd
    assert np.all(z[na:] < 4.0), (pm[na:], psd[na:])
    assert np.median(z[:na]) < 3.0, z[:na]


def _amr_problem(seed=12, nages=5, nmh=6, nbins=3000, scale=1.0):
    from sfhgpu.sampling import GaussianDispersion, LinearAMR, calculate_coeffs
    rng = np.random.default_rng(seed)
    la = np.repeat(np.linspace(10.0, 8.0, nages), nmh)
    mh = np.tile(np.linspace(-2.5, 0.0, nmh), nages)
    M = (rng.random((nbins, nages * nmh)) / 1e2).astype(np.float32)
    R = (rng.random(nages) * 1e4 + 1e3) * scale
    amr, disp = LinearAMR(0.1, -2.2, 13.7), GaussianDispersion(0.2)
    coeffs = calculate_coeffs(amr, disp, R, la, mh)
    data = rng.poisson(M.astype(np.float64) @ coeffs).astype(np.float64)
    return la, mh, np.asfortranarray(M), R, amr, disp, data


def test_amr_logdensity_matches_oracle(sfh, O):
    from sfhgpu.sampling import SFH_HMC_LINEAR_AMR, GaussianDispersion, LinearAMR, mzr_theta
    la, mh, M32, R, amr, disp, data = _amr_problem()
    H = sfh.Models(M32, storage="bf16x2")
    Ms = np.asfortranarray(_bf16_hilo(M32))
    rng = np.random.default_rng(6)
    thetas, nats = [], []
    for _ in range(6):
        Rb = R * np.exp(0.2 * rng.standard_normal(R.size))
        a = 0.1 * np.exp(0.2 * rng.standard_normal())
        b = -2.2 + 0.1 * rng.standard_normal()
        s = 0.2 * np.exp(0.2 * rng.standard_normal())
        thetas.append(mzr_theta(Rb, LinearAMR(a, b, 13.7), GaussianDispersion(s)))
        nats.append(np.concatenate([Rb, [a, b, s]]))
    theta = np.stack(thetas)
    logd, grad = sfh.logdensity_batched(H, data, theta, SFH_HMC_LINEAR_AMR, amr, disp, la, mh)
    nst = data.sum()
    for k, v in enumerate(nats):
        nlogL, Gv = O.amr_fg(v, 13.7, Ms, data, la, mh)
        na = R.size
        ref_logd = -nlogL + np.sum(np.log(v[:na])) + np.log(v[na]) + np.log(v[na + 2])
        ref_g = np.concatenate([-Gv[:na] * v[:na] + 1.0, [-Gv[na] * v[na] + 1.0, -Gv[na + 1],
                                                          -Gv[na + 2] * v[na + 2] + 1.0]])
        assert abs(logd[k] - ref_logd) <= 1e-2 * max(1.0, nst / 1e4), (logd[k], ref_logd)
        scale = np.abs(ref_g).max()
        np.testing.assert_allclose(grad[k], ref_g, rtol=2e-3, atol=2e-3 * scale)


def test_hmc_amr_recovers_parameters(sfh):
    from sfhgpu.sampling import GaussianDispersion, LinearAMR
    la, mh, M32, R, amr, disp, data = _amr_problem(seed=13, nbins=6000, scale=5.0)
    H = sfh.Models(M32, storage="bf16x2")
    out = sfh.sample_sfh(H, data, la, mh, LinearAMR(0.08, -2.0, 13.7), GaussianDispersion(0.3),
                         R * 1.1, nsteps=300, nchains=32, nwarmup=300, nleap=10, seed=9)
    na = R.size
    pm = out["mean"].mean(axis=0)
    psd = np.sqrt(out["var"].mean(axis=0) + out["mean"].var(axis=0))
    truth = np.concatenate([R, [0.1, -2.2, 0.2]])
    assert 0.4 < out["accept"].mean() < 0.995, out["accept"].mean()
    z = np.abs(pm - truth) / psd
    assert np.all(z[na:] < 4.0), (pm[na:], psd[na:])
    assert np.median(z[:na]) < 3.0, z[:na]


def test_log_amr_logdensity_matches_oracle(sfh, O):
    from sfhgpu.sampling import (SFH_HMC_LOG_AMR, GaussianDispersion, LogarithmicAMR, MH_from_Z,
                                 calculate_coeffs, mzr_theta)
    rng = np.random.default_rng(14)
    nages, nmh, nbins = 5, 6, 3000
    la = np.repeat(np.linspace(10.0, 8.0, nages), nmh)
    mh = np.tile(MH_from_Z(10 ** np.linspace(-4, -2, nmh)), nages)
    M32 = np.asfortranarray((rng.random((nbins, nages * nmh)) / 1e2).astype(np.float32))
    R = rng.random(nages) * 1e4 + 1e3
    amr, disp = LogarithmicAMR(1e-4, 5e-5, 13.7), GaussianDispersion(0.2)
    data = rng.poisson(M32.astype(np.float64) @ calculate_coeffs(amr, disp, R, la, mh)).astype(float)
    H = sfh.Models(M32, storage="bf16x2")
    Ms = np.asfortranarray(_bf16_hilo(M32))
    thetas, nats = [], []
    for _ in range(5):
        Rb = R * np.exp(0.2 * rng.standard_normal(R.size))
        a = 1e-4 * np.exp(0.2 * rng.standard_normal())
        b = 5e-5 * np.exp(0.2 * rng.standard_normal())
        s = 0.2 * np.exp(0.2 * rng.standard_normal())
        thetas.append(mzr_theta(Rb, LogarithmicAMR(a, b, 13.7), GaussianDispersion(s)))
        nats.append(np.concatenate([Rb, [a, b, s]]))
    logd, grad = sfh.logdensity_batched(H, data, np.stack(thetas), SFH_HMC_LOG_AMR, amr, disp,
                                        la, mh)
    na = R.size
    for k, v in enumerate(nats):
        nlogL, Gv = O.amr_fg(v, 13.7, Ms, data, la, mh, kind=1)
        ref_logd = -nlogL + np.sum(np.log(v)) 
        ref_g = np.concatenate([-Gv[:na] * v[:na] + 1.0, -Gv[na:] * v[na:] + 1.0])
        assert abs(logd[k] - ref_logd) <= 1e-2 * max(1.0, data.sum() / 1e4), (logd[k], ref_logd)
        np.testing.assert_allclose(grad[k], ref_g, rtol=2e-3, atol=2e-3 * np.abs(ref_g).max())


def test_nuts_direct_matches_laplace_posterior(sfh):
    """The No-U-Turn sampler on hmc_sample's log density: the same Laplace check as the
    fixed-length sampler, trees that stop by turning (no divergences, depth below the
    limit) and per-chain trees that end at different times."""
    rng = np.random.default_rng(21)
    nbins, nt = 4000, 4
    M32 = np.asfortranarray((rng.random((nbins, nt)) ** 3).astype(np.float32))
    x_true = np.array([2000.0, 1000.0, 3000.0, 500.0]) / 100
    data = rng.poisson(M32.astype(np.float64) @ x_true).astype(np.float64)
    Ms = np.asfortranarray(_bf16_hilo(M32))
    _, mle = sfh.fit_templates_lbfgsb(sfh.Models(Ms, storage="f64"), data, x0=x_true,
                                      factr=10.0, pgtol=1e-10)
    m = Ms @ mle
    Hobs = (Ms * (data / m ** 2)[:, None]).T @ Ms
    sd_lap = np.sqrt(np.diag(np.linalg.inv(Hobs)))
    H = sfh.Models(M32, storage="bf16x2")
    out = sfh.hmc_sample(H, data, nsteps=400, nchains=64, nwarmup=300, seed=5, sampler="nuts",
                         max_depth=10)
    pm = out["mean"].mean(axis=0)
    pv = out["var"].mean(axis=0) + out["mean"].var(axis=0)
    assert 0.6 < out["accept"].mean() < 0.99, out["accept"].mean()
    assert np.all(out["divergent"] == 0)
    assert 0.5 < out["depth"].mean() < 9.0, out["depth"].mean()
    assert np.all(np.abs(pm - mle) < 0.25 * sd_lap + 3 * np.sqrt(pv / (64 * 100))), (pm, mle, sd_lap)
    ratio = np.sqrt(pv) / sd_lap
    assert np.all((ratio > 0.8) & (ratio < 1.25)), ratio


def test_nuts_mzr_recovers_parameters_and_draws_are_kept(sfh):
    la, mh, M32, R, mzr, disp, data = _mzr_problem(seed=8, nbins=6000, scale=5.0)
    H = sfh.Models(M32, storage="bf16x2")
    from sfhgpu.sampling import GaussianDispersion, PowerLawMZR
    out = sfh.sample_sfh(H, data, la, mh, PowerLawMZR(0.4, -0.8, 6.0), GaussianDispersion(0.3),
                         R * 1.1, nsteps=300, nchains=32, nwarmup=300, seed=9, sampler="nuts",
                         keep_draws=True, thin=3)
    na = R.size
    pm = out["mean"].mean(axis=0)
    psd = np.sqrt(out["var"].mean(axis=0) + out["mean"].var(axis=0))
    truth = np.concatenate([R, [0.5, -1.0, 0.2]])
    assert 0.5 < out["accept"].mean() < 0.995, out["accept"].mean()
    z = np.abs(pm - truth) / psd
    assert np.all(z[na:] < 4.0), (pm[na:], psd[na:])
    assert np.median(z[:na]) < 3.0, z[:na]
    dr = out["draws"]
    assert dr.shape == (32, 100, na + 3) and np.all(np.isfinite(dr))
    # the kept draws' means agree with the running means up to the thinning
    assert np.all(np.abs(dr.mean(axis=1).mean(0) - pm) < 0.5 * psd)


def test_nuts_is_reproducible(sfh):
    rng = np.random.default_rng(4)
    M32 = np.asfortranarray((rng.random((2000, 3)) ** 2).astype(np.float32))
    data = rng.poisson(M32.astype(np.float64) @ np.array([30.0, 20.0, 10.0])).astype(float)
    H = sfh.Models(M32, storage="bf16x2")
    a = sfh.hmc_sample(H, data, nsteps=50, nchains=8, nwarmup=50, seed=7, sampler="nuts")
    b = sfh.hmc_sample(H, data, nsteps=50, nchains=8, nwarmup=50, seed=7, sampler="nuts")
    assert np.array_equal(a["mean"], b["mean"]) and np.array_equal(a["depth"], b["depth"])


@pytest.mark.parametrize("sampler", ["hmc", "nuts"])
def test_single_chain_runs_on_the_plain_path(sfh, sampler):
    """One chain evaluates the single-vector fg! (no batch for the tensor cores): its
    posterior agrees with the 16-chain run on the batched path."""
    la, mh, M32, R, mzr, disp, data = _mzr_problem(seed=8, nbins=6000, scale=5.0)
    from sfhgpu.sampling import GaussianDispersion, PowerLawMZR
    res = {}
    for nch, steps in ((1, 1500), (16, 200)):
        H = sfh.Models(M32, storage="bf16x2")
        res[nch] = sfh.sample_sfh(H, data, la, mh, PowerLawMZR(0.4, -0.8, 6.0),
                                  GaussianDispersion(0.3), R * 1.1, nsteps=steps, nchains=nch,
                                  nwarmup=300, nleap=10, seed=9, sampler=sampler)
    one, many = res[1], res[16]
    na = R.size
    pm1 = one["mean"][0]
    pm = many["mean"].mean(axis=0)
    psd = np.sqrt(many["var"].mean(axis=0) + many["mean"].var(axis=0))
    assert 0.4 < one["accept"][0] < 0.999
    # hyperparameters within 4 posterior sd of the many-chain mean
    assert np.all(np.abs(pm1[na:] - pm[na:]) < 4 * psd[na:]), (pm1[na:], pm[na:], psd[na:])


def test_nuts_dense_metric_on_the_laplace_covariance(sfh):
    """A dense metric equal to the Laplace covariance of θ = log x whitens the posterior:
    a fixed step of 0.3 without warmup gives high acceptance, short trees and the Laplace
    moments."""
    rng = np.random.default_rng(21)
    nbins, nt = 4000, 4
    M32 = np.asfortranarray((rng.random((nbins, nt)) ** 3).astype(np.float32))
    x_true = np.array([2000.0, 1000.0, 3000.0, 500.0]) / 100
    data = rng.poisson(M32.astype(np.float64) @ x_true).astype(np.float64)
    Ms = np.asfortranarray(_bf16_hilo(M32))
    _, mle = sfh.fit_templates_lbfgsb(sfh.Models(Ms, storage="f64"), data, x0=x_true,
                                      factr=10.0, pgtol=1e-10)
    m = Ms @ mle
    Hobs = (Ms * (data / m ** 2)[:, None]).T @ Ms
    cov_x = np.linalg.inv(Hobs)
    cov_th = cov_x / np.outer(mle, mle)  # θ = log x
    H = sfh.Models(M32, storage="bf16x2")
    theta0 = np.repeat(np.log(mle)[None, :], 64, axis=0)
    out = sfh.hmc_sample(H, data, nsteps=400, nchains=64, nwarmup=0, step0=0.3, seed=8,
                         sampler="nuts", theta0=theta0, minv_dense=cov_th)
    assert out["accept"].mean() > 0.85, out["accept"].mean()
    assert np.all(out["divergent"] == 0) and out["depth"].mean() < 4.0, out["depth"].mean()
    pm = out["mean"].mean(axis=0)
    pv = out["var"].mean(axis=0) + out["mean"].var(axis=0)
    sd_lap = np.sqrt(np.diag(cov_x))
    assert np.all(np.abs(pm - mle) < 0.25 * sd_lap + 3 * np.sqrt(pv / (64 * 100))), (pm, mle)
    ratio = np.sqrt(pv) / sd_lap
    assert np.all((ratio > 0.8) & (ratio < 1.25)), ratio


def test_laplace_metric_matches_the_exact_covariance(sfh):
    """laplace_metric (central differences of the batched gradient in θ = log x) gives the
    Laplace covariance of the direct model at its MLE, whose exact form is known."""
    rng = np.random.default_rng(22)
    nbins, nt = 4000, 5
    M32 = np.asfortranarray((rng.random((nbins, nt)) ** 3).astype(np.float32))
    x_true = np.array([2000.0, 1000.0, 3000.0, 500.0, 1500.0]) / 100
    data = rng.poisson(M32.astype(np.float64) @ x_true).astype(np.float64)
    Ms = np.asfortranarray(_bf16_hilo(M32))
    _, mle = sfh.fit_templates_lbfgsb(sfh.Models(Ms, storage="f64"), data, x0=x_true,
                                      factr=10.0, pgtol=1e-10)
    m = Ms @ mle
    Hobs = (Ms * (data / m ** 2)[:, None]).T @ Ms
    cov_th = np.linalg.inv(Hobs) / np.outer(mle, mle)
    H = sfh.Models(M32, storage="bf16x2")
    cov = sfh.laplace_metric(H, data, np.log(mle))
    assert np.allclose(cov, cov.T)
    assert np.all(np.linalg.eigvalsh(cov) > 0)
    sd, sd_ref = np.sqrt(np.diag(cov)), np.sqrt(np.diag(cov_th))
    assert np.all(np.abs(sd / sd_ref - 1) < 0.02), sd / sd_ref
    corr = cov / np.outer(sd, sd)
    corr_ref = cov_th / np.outer(sd_ref, sd_ref)
    assert np.max(np.abs(corr - corr_ref)) < 0.02
    with pytest.raises(ValueError):
        sfh.laplace_metric(H, data, np.log(mle), step=0.0)

