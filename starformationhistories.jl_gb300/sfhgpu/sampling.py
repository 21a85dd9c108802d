"""Batched HMC and hierarchical (MZR) log densities over the GPU C ABI.

Mirrors hmc_sample (src/fitting/hmc_sample.jl:105-141) and the PowerLawMZR /
GaussianDispersion sampling of sample_sfh (src/fitting/hierarchical/generic_fitting.jl:
458-527) with all chains advanced together on the tensor cores
(sfh_hmc_sample_dev), plus the batched logdensity_and_gradient
(sfh_logdensity_batched_dev).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import check, load
from .core import Models

SFH_HMC_DIRECT, SFH_HMC_MZR, SFH_HMC_LINEAR_AMR, SFH_HMC_LOG_AMR = 0, 1, 2, 3


def MH_from_Z(Z, solZ=0.01524, Y_p=0.2485, gamma=1.78):
    """MH_from_Z, src/utilities.jl:138-145: [M/H] = log10(Z/X) - log10(Z/X)_sun with the
    PARSEC helium relation Y = Y_p + γ Z (NaN where X <= 0)."""
    Z = np.asarray(Z, dtype=np.float64)
    X = 1.0 - (Y_p + gamma * Z + Z)
    Xs = 1.0 - (Y_p + gamma * solZ + solZ)
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.where(X > 0, np.log10(Z / (X * solZ) * Xs), np.nan)


def dMH_dZ(Z, solZ=0.01524, Y_p=0.2485, gamma=1.78):
    """dMH_dZ, src/utilities.jl:152-155."""
    Z = np.asarray(Z, dtype=np.float64)
    return (Y_p - 1.0) / (np.log(10.0) * Z * (Y_p + Z + gamma * Z - 1.0))


class HMCConfig(C.Structure):
    _fields_ = [("nchains", C.c_int32), ("model", C.c_int32), ("ntraj", C.c_int64),
                ("nwarmup", C.c_int64), ("nleap", C.c_int32), ("thin", C.c_int32),
                ("step0", C.c_double), ("target_accept", C.c_double), ("seed", C.c_uint64),
                ("nages", C.c_int32), ("h_age_index", C.POINTER(C.c_int32)),
                ("h_logAge", C.POINTER(C.c_double)), ("h_MH", C.POINTER(C.c_double)),
                ("logMstar0", C.c_double), ("alpha_free", C.c_int32), ("beta_free", C.c_int32),
                ("sigma_free", C.c_int32), ("alpha", C.c_double), ("beta", C.c_double),
                ("sigma", C.c_double), ("T_max", C.c_double), ("d_minv0", C.c_void_p)]


def _bind():
    L = load()
    if not getattr(L, "_sfh_hmc_bound", False):
        vp, i64 = C.c_void_p, C.c_int64
        L.sfh_hmc_sample_dev.argtypes = [vp, vp, vp, C.POINTER(HMCConfig), vp, vp, vp, vp, vp, vp]
        L.sfh_hmc_sample_dev.restype = C.c_int
        L.sfh_nuts_sample_dev.argtypes = [vp, vp, vp, C.POINTER(HMCConfig), C.c_int, vp, vp, vp,
                                          vp, vp, vp, vp, vp, vp]
        L.sfh_nuts_sample_dev.restype = C.c_int
        L.sfh_logdensity_batched_dev.argtypes = [vp, vp, vp, C.POINTER(HMCConfig), vp, vp, vp]
        L.sfh_logdensity_batched_dev.restype = C.c_int
        from ._lib import FitOptions, FitResult
        L.sfh_fit_sfh_dev.argtypes = [vp, vp, vp, C.POINTER(HMCConfig), vp, C.c_int,
                                      C.POINTER(FitOptions), vp, vp, C.POINTER(FitResult)]
        L.sfh_fit_sfh_dev.restype = C.c_int
        L._sfh_hmc_bound = True
        del i64
    return L


@dataclass
class PowerLawMZR:
    """PowerLawMZR(α, MH0, logMstar0, free), src/fitting/hierarchical/mzr.jl:263-284."""
    alpha: float
    MH0: float
    logMstar0: float = 6.0
    free: tuple = (True, True)

    def __call__(self, Mstar):
        return self.MH0 + self.alpha * (np.log10(Mstar) - self.logMstar0)


@dataclass
class LinearAMR:
    """LinearAMR(α, β, T_max, free), src/fitting/hierarchical/amr.jl:170-213: mean [M/H]
    μ = β + α (T_max - t) at lookback time t = 10^(logAge - 9) Gyr; α >= 0."""
    alpha: float
    beta: float
    T_max: float = 13.7
    free: tuple = (True, True)

    def __post_init__(self):
        if self.alpha < 0:
            raise ValueError("α must be ≥ 0")
        if self.T_max <= 0:
            raise ValueError("T_max must be > 0")

    def __call__(self, logAge):
        return self.beta + self.alpha * (self.T_max - 10.0 ** (np.asarray(logAge) - 9.0))

    @classmethod
    def from_constraints(cls, constraint1, constraint2, T_max=13.7, free=(True, True)):
        """LinearAMR from two ([M/H], lookback time in Gyr) constraints, amr.jl:233-248."""
        (mh1, t1), (mh2, t2) = constraint1, constraint2
        dt, dmh = t2 - t1, mh2 - mh1
        if dt == 0:
            raise ValueError("Constraints are given at identical times.")
        if np.sign(dt) == np.sign(dmh):
            raise ValueError("The constraints indicate metallicity decreasing towards present-day.")
        alpha = dmh / -dt
        beta = min(mh1, mh2) - alpha * (T_max - max(t1, t2))
        return cls(alpha, beta, T_max, free)


@dataclass
class LogarithmicAMR:
    """LogarithmicAMR(α, β, T_max, MH_from_Z, dMH_dZ, free), amr.jl:256-290: metal mass
    fraction Z = β + α (T_max - t) at lookback time t (Gyr) and μ = MH_from_Z(Z) with the
    package's default conversion; α, β >= 0 (transforms (1, 1))."""
    alpha: float
    beta: float
    T_max: float = 13.7
    free: tuple = (True, True)

    def __post_init__(self):
        if self.alpha < 0:
            raise ValueError("α must be ≥ 0")
        if self.beta < 0:
            raise ValueError("β must be ≥ 0")
        if self.T_max <= 0:
            raise ValueError("T_max must be > 0")

    def __call__(self, logAge):
        return MH_from_Z(self.beta + self.alpha * (self.T_max - 10.0 ** (np.asarray(logAge) - 9.0)))


@dataclass
class GaussianDispersion:
    """GaussianDispersion(σ, free), src/fitting/hierarchical/dispersion_models.jl:80-110."""
    sigma: float
    free: tuple = (True,)

    def __call__(self, x, mu):
        return np.exp(-((np.asarray(x) - mu) / self.sigma) ** 2 / 2)


def calculate_coeffs(model, disp: GaussianDispersion, mstars, logAge, MH):
    """calculate_coeffs on the host (a handful of values per age): PowerLawMZR
    (mzr.jl:50-79, μ from the cumulative stellar mass) or LinearAMR (amr.jl:50-72,
    μ from the age)."""
    logAge, MH = np.asarray(logAge, float), np.asarray(MH, float)
    uniq = list(dict.fromkeys(logAge.tolist()))
    mstars = np.asarray(mstars, float)
    if len(mstars) != len(uniq):
        raise ValueError("Length of `mstars` must be the same as `unique(logAge)`.")
    if isinstance(model, (LinearAMR, LogarithmicAMR)):
        mu = [model(la) for la in uniq]
    else:
        order = np.argsort(-np.asarray(uniq), kind="stable")
        cum = np.empty(len(uniq))
        cum[order] = np.cumsum(mstars[order])
        mu = [model(c) for c in cum]
    out = np.empty_like(logAge)
    for i, la in enumerate(uniq):
        idx = np.nonzero(logAge == la)[0]
        w = disp(MH[idx], mu[i])
        out[idx] = w * mstars[i] / w.sum()
    return out


def _config(nchains, model, nsteps=0, nwarmup=0, nleap=10, thin=1, step0=0.01, target=0.8,
            seed=0x5F3759DF, mzr=None, disp=None, logAge=None, MH=None):
    cfg = HMCConfig()
    cfg.nchains, cfg.model = int(nchains), int(model)
    cfg.ntraj, cfg.nwarmup, cfg.nleap, cfg.thin = int(nsteps), int(nwarmup), int(nleap), int(thin)
    cfg.step0, cfg.target_accept, cfg.seed = float(step0), float(target), int(seed)
    keep = []
    if model in (SFH_HMC_MZR, SFH_HMC_LINEAR_AMR, SFH_HMC_LOG_AMR):
        logAge = np.asarray(logAge, float)
        uniq = list(dict.fromkeys(logAge.tolist()))
        age_index = np.ascontiguousarray([uniq.index(a) for a in logAge], dtype=np.int32)
        ua = np.ascontiguousarray(uniq, dtype=np.float64)
        mh = np.ascontiguousarray(MH, dtype=np.float64)
        keep += [age_index, ua, mh]
        cfg.nages = len(uniq)
        cfg.h_age_index = age_index.ctypes.data_as(C.POINTER(C.c_int32))
        cfg.h_logAge = ua.ctypes.data_as(C.POINTER(C.c_double))
        cfg.h_MH = mh.ctypes.data_as(C.POINTER(C.c_double))
        cfg.logMstar0 = float(getattr(mzr, "logMstar0", 0.0))
        cfg.T_max = float(getattr(mzr, "T_max", 0.0))
        cfg.alpha_free, cfg.beta_free = int(bool(mzr.free[0])), int(bool(mzr.free[1]))
        cfg.sigma_free = int(bool(disp.free[0]))
        beta = mzr.beta if isinstance(mzr, (LinearAMR, LogarithmicAMR)) else mzr.MH0
        cfg.alpha, cfg.beta, cfg.sigma = float(mzr.alpha), float(beta), float(disp.sigma)
    return cfg, keep


def mzr_theta(mstars, mzr, disp: GaussianDispersion):
    """Transformed variables [log R_j..., log α, β, log σ] (free ones only), the order
    used by logdensity_and_gradient (generic_fitting.jl:117-136); PowerLawMZR and
    LinearAMR share the transforms (α > 0 log-transformed, β untransformed);
    LogarithmicAMR log-transforms β as well (amr.jl:290)."""
    th = list(np.log(np.asarray(mstars, float)))
    if mzr.free[0]:
        th.append(np.log(mzr.alpha))
    if mzr.free[1]:
        if isinstance(mzr, LogarithmicAMR):  # β > 0: log-transformed (amr.jl:290)
            th.append(np.log(mzr.beta))
        else:
            th.append(mzr.beta if isinstance(mzr, LinearAMR) else mzr.MH0)
    if disp.free[0]:
        th.append(np.log(disp.sigma))
    return np.asarray(th)


def logdensity_batched(models: Models, data, theta, model=SFH_HMC_DIRECT, mzr=None, disp=None,
                       logAge=None, MH=None):
    """log p and ∇ log p for B parameter vectors (rows of theta) in one batched call."""
    import torch
    L = _bind()
    dev = torch.device("cuda", models.ctx.device)
    th = torch.as_tensor(np.asarray(theta, float), device=dev).contiguous()
    n = torch.as_tensor(np.asarray(data, float).reshape(-1), device=dev).contiguous()
    B = th.shape[0]
    cfg, keep = _config(B, model, mzr=mzr, disp=disp, logAge=logAge, MH=MH)
    logd = torch.empty(B, dtype=torch.float64, device=dev)
    grad = torch.empty_like(th)
    torch.cuda.synchronize(dev)
    check(L.sfh_logdensity_batched_dev(models.ctx.handle, models.handle, n.data_ptr(),
                                       C.byref(cfg), th.data_ptr(), logd.data_ptr(),
                                       grad.data_ptr()), models.ctx.handle, "logdensity_batched")
    del keep
    return logd.cpu().numpy(), grad.cpu().numpy()


def model_kind(mzr):
    """The sampler's model code for a metallicity model (None: the direct coefficients)."""
    if mzr is None:
        return SFH_HMC_DIRECT
    return (SFH_HMC_LINEAR_AMR if isinstance(mzr, LinearAMR) else
            SFH_HMC_LOG_AMR if isinstance(mzr, LogarithmicAMR) else SFH_HMC_MZR)


def laplace_metric(models: Models, data, theta, mzr=None, disp=None, logAge=None, MH=None,
                   step=1e-2, floor=1e-10):
    """Dense inverse metric for the No-U-Turn sampler from the curvature of log p at theta
    (the Laplace covariance), in the sampler's transformed space: H = -d²log p / dθ² by
    central differences of the batched gradient (2D rows in one evaluation, step `step`
    per coordinate), symmetrised.  Eigenvalues enter by magnitude and no smaller than
    floor x the largest, so the result is positive definite away from the mode as well.
    No reference counterpart: the reference's sample_sfh takes the BFGS inverse Hessian."""
    th = np.asarray(theta, float).reshape(-1)
    D = th.size
    h = np.broadcast_to(np.asarray(step, float), (D,)).copy()
    if np.any(~(h > 0)):
        raise ValueError("step must be positive")
    rows = np.repeat(th[None, :], 2 * D, axis=0)
    k = np.arange(D)
    rows[k, k] += h
    rows[D + k, k] -= h
    _, g = logdensity_batched(models, data, rows, model=model_kind(mzr), mzr=mzr, disp=disp,
                              logAge=logAge, MH=MH)
    H = -(g[:D] - g[D:]) / (2.0 * h[:, None])
    H = 0.5 * (H + H.T)
    w, V = np.linalg.eigh(H)
    w = np.abs(w)
    w = np.maximum(w, floor * max(float(w.max()), 1e-300))
    return (V / w) @ V.T


def _run_hmc(models, data, theta0, cfg, keep, keep_draws, sampler="hmc", max_depth=10,
             minv_dense=None):
    import torch
    L = _bind()
    dev = torch.device("cuda", models.ctx.device)
    th0 = torch.as_tensor(np.asarray(theta0, float), device=dev).contiguous()
    n = torch.as_tensor(np.asarray(data, float).reshape(-1), device=dev).contiguous()
    B, D = th0.shape
    mean = torch.empty((B, D), dtype=torch.float64, device=dev)
    var = torch.empty_like(mean)
    acc = torch.empty(B, dtype=torch.float64, device=dev)
    step = torch.empty(B, dtype=torch.float64, device=dev)
    ndraw = (cfg.ntraj + cfg.thin - 1) // cfg.thin
    draws = torch.empty((B, ndraw, D), dtype=torch.float32, device=dev) if keep_draws else None
    torch.cuda.synchronize(dev)
    if sampler == "nuts":
        depth = torch.empty(B, dtype=torch.float64, device=dev)
        ndiv = torch.empty(B, dtype=torch.int64, device=dev)
        md = None
        if minv_dense is not None:
            md = torch.as_tensor(np.ascontiguousarray(minv_dense, dtype=np.float64), device=dev)
            torch.cuda.synchronize(dev)
        check(L.sfh_nuts_sample_dev(models.ctx.handle, models.handle, n.data_ptr(), C.byref(cfg),
                                    int(max_depth), md.data_ptr() if md is not None else None,
                                    th0.data_ptr(), mean.data_ptr(),
                                    var.data_ptr(), acc.data_ptr(), step.data_ptr(),
                                    depth.data_ptr(), ndiv.data_ptr(),
                                    draws.data_ptr() if keep_draws else None),
              models.ctx.handle, "nuts")
    else:
        if sampler != "hmc":
            raise ValueError("sampler is 'hmc' or 'nuts'")
        check(L.sfh_hmc_sample_dev(models.ctx.handle, models.handle, n.data_ptr(), C.byref(cfg),
                                   th0.data_ptr(), mean.data_ptr(), var.data_ptr(),
                                   acc.data_ptr(), step.data_ptr(),
                                   draws.data_ptr() if keep_draws else None),
              models.ctx.handle, "hmc")
    del keep
    out = {"mean": mean.cpu().numpy(), "var": var.cpu().numpy(), "accept": acc.cpu().numpy(),
           "step": step.cpu().numpy()}
    if sampler == "nuts":
        out["depth"] = depth.cpu().numpy()
        out["divergent"] = ndiv.cpu().numpy()
    if keep_draws:
        out["draws"] = draws.cpu().numpy()
    return out


def hmc_sample(models: Models, data, nsteps, nchains=1, nwarmup=200, nleap=10, step0=0.01,
               target_accept=0.8, seed=20261203, theta0=None, keep_draws=False, thin=1,
               sampler="hmc", max_depth=10, minv_dense=None):
    """hmc_sample(models, data, nsteps, nchains), hmc_sample.jl:105-141: posterior of the
    log coefficients, all chains in lock step.  Returns a dict with per-chain posterior
    mean / variance of the coefficients (natural scale), acceptance and step size, and
    optionally the draws (nchains x ceil(nsteps/thin) x ntemplates).  sampler "hmc":
    fixed-length trajectories of nleap steps; "nuts": DynamicHMC's No-U-Turn sampler
    (sfh_nuts_sample_dev, trees up to max_depth doublings; adds "depth" and "divergent");
    minv_dense (D x D) is a dense inverse metric for "nuts" (DynamicHMC's
    GaussianKineticEnergy(M⁻¹)), kept through warmup."""
    if theta0 is None:
        from .fitting import renormalize_x0
        x0 = renormalize_x0(np.asarray(data, float).reshape(-1), models, np.ones(models.nt))
        rng = np.random.default_rng(seed)
        theta0 = np.log(x0)[None, :] + 0.1 * rng.standard_normal((nchains, models.nt))
    cfg, keep = _config(nchains, SFH_HMC_DIRECT, nsteps, nwarmup, nleap, thin, step0,
                        target_accept, seed)
    return _run_hmc(models, data, theta0, cfg, keep, keep_draws, sampler, max_depth, minv_dense)


def sample_sfh(models: Models, data, logAge, MH, mzr=None, disp: GaussianDispersion = None,
               mstars0=None, nsteps=1000, nchains=1, nwarmup=200, nleap=10, step0=0.01,
               target_accept=0.8, seed=20261203, keep_draws=False, thin=1, jitter=0.05,
               fit=None, sampler="hmc", max_depth=10, minv_dense=None):
    """Posterior sampling of (R_j, α, β, σ) under a PowerLawMZR, LinearAMR or
    LogarithmicAMR metallicity model with GaussianDispersion (sample_sfh,
    generic_fitting.jl:458-527), all chains in lock step.  Means are reported on the
    natural scale in the order [R_j..., α, β, σ] (free parameters only).

    With fit (the CompositeBFGSResult of fit_sfh) and sampler "nuts", the run is the
    reference's: every chain starts at the MLE point and the MAP inverse Hessian is the
    dense metric (:470-490; the reference also keeps its step ϵ = 0.05 with no warmup, i.e.
    step0=0.05, nwarmup=0).  With fit and sampler "hmc", the chains start around the MAP
    point (spread by `jitter` standard deviations of its inverse Hessian) with the diagonal
    of that inverse Hessian as the starting metric.  mzr, disp and mstars0 then come from
    the fit.  sampler "nuts" adds "depth" and "divergent" to the result; minv_dense (D x D)
    replaces the MAP inverse Hessian as its dense metric."""
    rng = np.random.default_rng(seed)
    minv0 = None
    if fit is not None and sampler == "nuts":
        # the reference's sample_sfh: NUTS from the MLE point with the MAP inverse Hessian as
        # a dense metric (generic_fitting.jl:470-490)
        mzr, disp = fit.mle.MH_model, fit.mle.disp_model
        th = np.asarray(fit.mle.theta, float)
        theta0 = np.repeat(th[None, :], nchains, axis=0)
        if minv_dense is None:
            minv_dense = np.asarray(fit.map.invH, float)
    elif fit is not None:
        mzr, disp = fit.map.MH_model, fit.map.disp_model
        th = np.asarray(fit.map.theta, float)
        sd = np.sqrt(np.clip(np.diag(fit.map.invH), 1e-300, None))
        theta0 = th[None, :] + jitter * sd[None, :] * rng.standard_normal((nchains, th.size))
        minv0 = np.ascontiguousarray(np.diag(fit.map.invH), dtype=np.float64)
    else:
        th = mzr_theta(mstars0, mzr, disp)
        theta0 = th[None, :] + jitter * rng.standard_normal((nchains, th.size))
    kind = model_kind(mzr)
    cfg, keep = _config(nchains, kind, nsteps, nwarmup, nleap, thin, step0,
                        target_accept, seed, mzr=mzr, disp=disp, logAge=logAge, MH=MH)
    if minv0 is not None:
        import torch
        d_minv0 = torch.as_tensor(minv0, device=torch.device("cuda", models.ctx.device))
        cfg.d_minv0 = d_minv0.data_ptr()
        keep.append(d_minv0)
    return _run_hmc(models, data, theta0, cfg, keep, keep_draws, sampler, max_depth, minv_dense)


# ---------------------------------------------------------------- fit_sfh (device BFGS)

@dataclass
class BFGSResult:
    """BFGSResult (generic_fitting.jl): natural-scale values `mu` and standard errors
    `sigma` of every variable [R_j..., metallicity-model parameters..., dispersion
    parameters...] (fixed ones included, σ = 0), the inverse Hessian `invH` and the
    transformed optimum `theta` over the free variables, the optimiser outcome `result`,
    and the models with the fitted parameters."""
    mu: np.ndarray
    sigma: np.ndarray
    invH: np.ndarray
    theta: np.ndarray
    result: dict
    MH_model: object
    disp_model: object


@dataclass
class CompositeBFGSResult:
    """The MAP and MLE results of fit_sfh (generic_fitting.jl:318-409)."""
    map: BFGSResult
    mle: BFGSResult


def _model_params(mzr):
    """(fittable parameters, transforms) of a metallicity model: PowerLawMZR (α, MH0),
    transforms (1, 0) (mzr.jl:283-284); LinearAMR (α, β), (1, 0) (amr.jl:212-213);
    LogarithmicAMR (α, β), (1, 1) (amr.jl:289-290)."""
    if isinstance(mzr, LogarithmicAMR):
        return (mzr.alpha, mzr.beta), (1, 1)
    if isinstance(mzr, LinearAMR):
        return (mzr.alpha, mzr.beta), (1, 0)
    return (mzr.alpha, mzr.MH0), (1, 0)


def _update_model(mzr, vals):
    import dataclasses
    if isinstance(mzr, (LinearAMR, LogarithmicAMR)):
        return dataclasses.replace(mzr, alpha=float(vals[0]), beta=float(vals[1]))
    return dataclasses.replace(mzr, alpha=float(vals[0]), MH0=float(vals[1]))


def fit_sfh_x0(MH_model0, disp_model0, models, data, logAge, metallicities, x0):
    """The renormalisation of x0 in fit_sfh (generic_fitting.jl:261-283): x0 scaled so the
    composite holds the data's total; when calculate_coeffs gives NaN (an MZR far from the
    stellar mass x0 implies), x0 replicated over the metallicity bins first, then up to
    five rounds of renormalisation while the coefficients stay finite."""
    import warnings
    from .fitting import renormalize_x0
    full = calculate_coeffs(MH_model0, disp_model0, x0, logAge, metallicities)
    if np.any(np.isnan(full)):
        if not isinstance(MH_model0, (LinearAMR, LogarithmicAMR)):
            warnings.warn("Initial `x0` provided to `fit_sfh` produced NaN coefficients. "
                          "Attempting to renormalize `x0` by replicating across metallicity bins.")
        n_mh = len(dict.fromkeys(np.asarray(metallicities, float).tolist()))
        full = np.tile(np.asarray(x0, float), n_mh)  # Julia's repeat(x0, n)
        x0 = renormalize_x0(data, models, x0, full)
        for i in range(1, 6):
            full = calculate_coeffs(MH_model0, disp_model0, x0, logAge, metallicities)
            if np.any(np.isnan(full)):
                warnings.warn(f"Renormalization of x0 failed to produce valid coefficients "
                              f"after {i} iterations. Returning last valid x0.")
                break
            x0 = renormalize_x0(data, models, x0, full)
    else:
        x0 = renormalize_x0(data, models, x0, full)
    return np.asarray(x0, float)


def fit_sfh(MH_model0, disp_model0, models: Models, data, logAge, metallicities, x0=None,
            g_abstol=1e-8, f_reltol=0.0, x_abstol=0.0, max_iter=1000, max_evals=0,
            graph_slots=8):
    """fit_sfh(MH_model0, disp_model0, models, data, logAge, metallicities; x0),
    src/fitting/hierarchical/generic_fitting.jl:242-409: the MAP and then the MLE of the
    hierarchical model by BFGS, both run on the device (sfh_fit_sfh_dev: the coefficient
    map, fg! and the chain rule in every evaluation, the BFGS loop replayed from CUDA
    graphs).  Returns a CompositeBFGSResult; μ and σ follow the reference's assembly
    (:358-401), including its indexing of the μ vector when some parameters are fixed."""
    import torch
    from ._lib import FitOptions, FitResult
    L = _bind()
    M = models
    logAge = np.asarray(logAge, float)
    metallicities = np.asarray(metallicities, float)
    data = np.asarray(data, float).reshape(-1)
    uniq = list(dict.fromkeys(logAge.tolist()))
    if x0 is None:
        from .fitting import construct_x0_mdf
        x0 = construct_x0_mdf(logAge, 13.7, normalize_value=1e6)
    x0 = np.asarray(x0, float)
    if x0.size != len(uniq):
        raise ValueError("length(x0) != length(unique(logAge))")
    if M.nbins != data.size:
        raise ValueError("size(models, 1) == length(data)")
    if not (M.nt == logAge.size == metallicities.size):
        raise ValueError("size(models, 2) == length(logAge) == length(metallicities)")
    x0 = fit_sfh_x0(MH_model0, disp_model0, M, data, logAge, metallicities, x0)
    theta0 = mzr_theta(x0, MH_model0, disp_model0)
    kind = (SFH_HMC_LINEAR_AMR if isinstance(MH_model0, LinearAMR) else
            SFH_HMC_LOG_AMR if isinstance(MH_model0, LogarithmicAMR) else SFH_HMC_MZR)
    cfg, keep = _config(1, kind, mzr=MH_model0, disp=disp_model0, logAge=logAge,
                        MH=metallicities)
    dev = torch.device("cuda", M.ctx.device)
    d_n = torch.as_tensor(data, device=dev)
    D = theta0.size
    opt = FitOptions()
    opt.transform, opt.max_iter, opt.max_evals, opt.graph_slots = 0, int(max_iter), int(max_evals), int(graph_slots)
    opt.g_abstol, opt.f_reltol, opt.x_abstol, opt.eps = float(g_abstol), float(f_reltol), float(x_abstol), 0.0

    def run(th0, is_map):
        d_th0 = torch.as_tensor(np.asarray(th0, float), device=dev)
        d_out = torch.empty(D, dtype=torch.float64, device=dev)
        d_H = torch.empty((D, D), dtype=torch.float64, device=dev)
        res = FitResult()
        torch.cuda.synchronize(dev)
        check(L.sfh_fit_sfh_dev(M.ctx.handle, M.handle, d_n.data_ptr(), C.byref(cfg),
                                d_th0.data_ptr(), 1 if is_map else 0, C.byref(opt),
                                d_out.data_ptr(), d_H.data_ptr(), C.byref(res)),
              M.ctx.handle, "fit_sfh")
        H = d_H.cpu().numpy()
        info = {"f": res.f, "g_norm": res.g_norm, "iterations": int(res.iterations),
                "evaluations": int(res.evaluations), "status": int(res.status),
                "converged": int(res.status) in (0, 1, 2), "graph": bool(res.graph)}
        return d_out.cpu().numpy(), 0.5 * (H + H.T), info

    th_map, H_map, info_map = run(theta0, True)
    th_mle, H_mle, info_mle = run(th_map, False)
    del keep

    par = _model_params(MH_model0)[0] + (disp_model0.sigma,)
    tf = _model_params(MH_model0)[1] + (1,)
    free = tuple(bool(f) for f in MH_model0.free) + tuple(bool(f) for f in disp_model0.free)
    nb = len(uniq)
    ntot = nb + len(par)
    mu_map, mu_mle = np.empty(ntot), np.empty(ntot)
    s_map, s_mle = np.empty(ntot), np.empty(ntot)
    st_map = np.sqrt(np.clip(np.diag(H_map), 0, None))
    st_mle = np.sqrt(np.clip(np.diag(H_mle), 0, None))
    for i in range(nb):
        mu_map[i], mu_mle[i] = np.exp(th_map[i]), np.exp(th_mle[i])
        s_map[i], s_mle[i] = mu_map[i] * st_map[i], mu_mle[i] * st_mle[i]
    free_count = 0
    for i in range(nb, ntot):
        k = i - nb
        if free[k]:
            j = i - free_count  # as the reference indexes μ_map with j (:377-393)
            if tf[k] == 1:
                mu_map[i], mu_mle[i] = np.exp(th_map[j]), np.exp(th_mle[j])
                s_map[i], s_mle[i] = mu_map[j] * st_map[j], mu_map[j] * st_mle[j]
            elif tf[k] == 0:
                mu_map[i], mu_mle[i] = th_map[j], th_mle[j]
                s_map[i], s_mle[i] = st_map[j], st_mle[j]
            else:
                mu_map[i], mu_mle[i] = -np.exp(th_map[j]), -np.exp(th_mle[j])
                s_map[i], s_mle[i] = -mu_map[j] * st_map[j], -mu_map[j] * st_mle[j]
        else:
            mu_map[i] = mu_mle[i] = par[k]
            s_map[i] = s_mle[i] = 0.0
            free_count += 1
    import dataclasses
    nmh = len(_model_params(MH_model0)[0])

    def res_of(mu, sig, H, th, info):
        return BFGSResult(mu, sig, H, th, info, _update_model(MH_model0, mu[nb:nb + nmh]),
                          dataclasses.replace(disp_model0, sigma=float(mu[nb + nmh])))
    return CompositeBFGSResult(res_of(mu_map, s_map, H_map, th_map, info_map),
                               res_of(mu_mle, s_mle, H_mle, th_mle, info_mle))
