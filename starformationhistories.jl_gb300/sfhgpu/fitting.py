"""Reference-named objective and fit drivers over the GPU C ABI.

Mirrors src/fitting/fitting_base.jl, src/fitting/solvers.jl and
src/fitting/utilities.jl of StarFormationHistories.jl v1.3.1.  Julia's `!`
suffix becomes a trailing underscore (`composite_` is `composite!`,
`fg_` is `fg!`).  Element type T follows the arrays passed (float32 or
float64), including eps(T) in the clamps.
"""
from __future__ import annotations

import ctypes as C
from collections import namedtuple

import numpy as np

from ._lib import SFH_F32, SFH_F64, FitOptions, FitResult, check, load
from .core import Models, as_models, default_context

_dp = None


def _T(*arrays):
    """promote_type of the floating arrays' element types (integers promote to the float)."""
    ts = [np.asarray(a).dtype for a in arrays if a is not None]
    fl = [t for t in ts if np.issubdtype(t, np.floating)]
    if not fl:
        return np.dtype(np.float64)
    return np.result_type(*fl)


def _code(T):
    return SFH_F32 if np.dtype(T) == np.float32 else SFH_F64


def _arr(a, T):
    return np.ascontiguousarray(np.asarray(a).reshape(-1, order="F"), dtype=T)


def _argcheck(cond, msg):
    if not cond:
        raise ValueError(msg)  # the reference throws ArgumentError from @argcheck


def stack_models(models):
    """stack_models(models), src/fitting/utilities.jl:12-13: one column per template,
    each the column-major `vec` of its Hess matrix."""
    return np.asfortranarray(np.stack([np.asarray(m).reshape(-1, order="F") for m in models],
                                      axis=1))


def composite_(composite, coeffs, models):
    """composite!(composite, coeffs, models) flat form, fitting_base.jl:55-65."""
    M = as_models(models)
    _argcheck(np.size(composite) == M.nbins, "axes(composite,1) == axes(models,1)")
    _argcheck(np.size(coeffs) == M.nt, "axes(coeffs,1) == axes(models,2)")
    T = np.asarray(composite).dtype
    code = _code(T)
    r = _arr(coeffs, T)
    out = np.empty(M.nbins, dtype=T)
    ctx = M.ctx
    check(load().sfh_composite(ctx.handle, M.handle, code, r.ctypes.data, out.ctypes.data),
          ctx.handle, "composite!")
    composite[...] = out.reshape(np.shape(composite), order="F")
    return None


def loglikelihood(*args):
    """loglikelihood(composite, data), fitting_base.jl:84-96, or
    loglikelihood(coeffs, models, data), fitting_base.jl:107-125."""
    if len(args) == 3:
        coeffs, models, data = args
        M = as_models(models)
        T = _T(coeffs, data) if M.storage != SFH_F32 else np.result_type(_T(coeffs, data),
                                                                            np.float32)
        c = np.empty(M.nbins, dtype=T)
        composite_(c, coeffs, M)
        return loglikelihood(c, data)
    composite, data = args
    _argcheck(np.shape(composite) == np.shape(data), "axes(composite) == axes(data)")
    T = _T(composite, data)
    c, n = _arr(composite, T), _arr(data, T)
    out = C.c_double()
    ctx = default_context()
    check(load().sfh_loglikelihood(ctx.handle, _code(T), c.ctypes.data, n.ctypes.data, c.size,
                                   C.byref(out)), ctx.handle, "loglikelihood")
    return T.type(out.value)


def grad_loglikelihood_(G, composite, models, data):
    """∇loglikelihood!(G, composite, models, data) flat form, fitting_base.jl:265-285.
    Overwrites composite with 1 - data/max(composite, eps)."""
    M = as_models(models)
    _argcheck(np.size(G) == M.nt, "axes(G,1) == axes(models,2)")
    _argcheck(np.size(composite) == M.nbins == np.size(data),
              "axes(models,1) == axes(data,1) == axes(composite,1)")
    T = np.asarray(composite).dtype
    c, n = _arr(composite, T), _arr(data, T)
    g = np.empty(M.nt, dtype=T)
    ctx = M.ctx
    check(load().sfh_grad_loglikelihood(ctx.handle, M.handle, _code(T), c.ctypes.data,
                                        n.ctypes.data, g.ctypes.data), ctx.handle,
          "∇loglikelihood!")
    composite[...] = c.reshape(np.shape(composite), order="F")
    G[...] = g.astype(np.asarray(G).dtype)
    return G


def grad_loglikelihood(*args):
    """∇loglikelihood forms, fitting_base.jl:144-211: (model, composite, data) for one
    template, (models, composite, data), or (coeffs, models, data)."""
    a0, a1, a2 = args
    if isinstance(a1, Models) or (np.ndim(a1) == 2 and np.ndim(a0) == 1
                                  and np.shape(a1)[1] == np.size(a0)):
        coeffs, models, data = a0, a1, a2
        M = as_models(models)
        T = _T(coeffs, data)
        c = np.empty(M.nbins, dtype=T)
        composite_(c, coeffs, M)
        G = np.empty(M.nt, dtype=T)
        grad_loglikelihood_(G, c, M, data)
        return G
    if np.ndim(a0) == 2 and np.ndim(a1) == 1 and np.shape(a0)[0] == np.size(a1):
        models, composite, data = a0, a1, a2
        M = as_models(models)
        T = _T(composite, data)
        c = _arr(composite, T).copy()
        G = np.empty(M.nt, dtype=T)
        grad_loglikelihood_(G, c, M, data)
        return G
    model, composite, data = a0, a1, a2
    _argcheck(np.shape(model) == np.shape(composite) == np.shape(data),
              "axes(model) == axes(composite) == axes(data)")
    T = _T(model, composite, data)
    M = Models(_arr(model, T).reshape(-1, 1), storage="f32" if T == np.float32 else "f64")
    c = _arr(composite, T).copy()
    G = np.empty(1, dtype=T)
    grad_loglikelihood_(G, c, M, _arr(data, T))
    return T.type(G[0])


_F64 = np.dtype(np.float64)


def _addr(a):
    """Data address of an ndarray (the buffer protocol for writable arrays, a fraction of
    the cost of `.ctypes.data`)."""
    try:
        return C.addressof(C.c_char.from_buffer(a))
    except (TypeError, ValueError, BufferError):
        return a.ctypes.data


def _flat64(a, n, writable=False):
    """True when `a` is a float64 ndarray of n elements laid out flat (column-major)."""
    return (type(a) is np.ndarray and a.dtype == _F64 and a.size == n and a.flags.f_contiguous
            and (not writable or a.flags.writeable))


def fg_(F, G, coeffs, models, data, composite):
    """fg!(F, G, coeffs, models, data, composite), src/fitting/solvers.jl:20-38.
    Returns -logL when F is not None; fills G with -∇logL when G is not None."""
    M = models if isinstance(models, Models) else as_models(models)
    if (_flat64(coeffs, M.nt) and _flat64(data, M.nbins) and _flat64(composite, M.nbins, True)
            and (G is None or _flat64(G, M.nt, True))):
        # Float64 arrays already in the flat layout: straight to the C call
        out = C.c_double()
        ctx = M.ctx
        check(load().sfh_fg(ctx.handle, M.handle, SFH_F64, _addr(coeffs), _addr(data),
                            _addr(composite), _addr(G) if G is not None else None,
                            C.byref(out) if F is not None else None), ctx.handle, "fg!")
        return _F64.type(out.value) if F is not None else None
    _argcheck(np.size(coeffs) == M.nt, "axes(coeffs,1) == axes(models,2)")
    _argcheck(M.nbins == np.size(data) == np.size(composite),
              "axes(models,1) == axes(data,1) == axes(composite,1)")
    T = _T(coeffs, data, composite)
    r, n = _arr(coeffs, T), _arr(data, T)
    # results land in the caller's arrays directly when their memory is the flat layout
    # (a contiguous vector, or a Fortran-ordered Hess matrix); otherwise via a temporary
    c = _flat_out(composite, T, M.nbins)
    g = _flat_out(G, T, M.nt) if G is not None else None
    out = C.c_double()
    ctx = M.ctx
    check(load().sfh_fg(ctx.handle, M.handle, _code(T), r.ctypes.data, n.ctypes.data,
                        c.ctypes.data, g.ctypes.data if g is not None else None,
                        C.byref(out) if F is not None else None), ctx.handle, "fg!")
    if c is not composite:
        composite[...] = c.reshape(np.shape(composite), order="F")
    if G is not None and g is not G:
        G[...] = g
    if F is not None:
        return T.type(out.value)
    return None


def _flat_out(a, T, n):
    """`a` itself when it is a writable ndarray of dtype T whose memory is the n-element
    flat (column-major) layout; else a new buffer."""
    if (isinstance(a, np.ndarray) and a.dtype == T and a.size == n and a.flags.writeable and
            (a.flags.f_contiguous or a.ndim == 1 and a.flags.c_contiguous)):
        return a
    return np.empty(n, dtype=T)


# ---------------------------------------------------------------- initial guesses

def construct_x0(logAge, T_max, normalize_value=1.0):
    """construct_x0, src/fitting/utilities.jl:31-47."""
    logAge = np.asarray(logAge)
    _argcheck(np.log10(T_max) + 9 > logAge.max(), "log10(T_max) + 9 > maximum(logAge)")
    min_la = logAge.min()
    max_la = np.log10(T_max) + 9
    uniq = np.concatenate([np.sort(np.unique(logAge)), [max_la]])
    sfr = normalize_value / (10.0 ** max_la - 10.0 ** min_la)
    num = np.array([np.count_nonzero(logAge == la) for la in uniq])
    dt = np.array([10.0 ** uniq[i + 1] - 10.0 ** uniq[i] for i in range(len(uniq) - 1)])
    out = np.empty_like(logAge, dtype=logAge.dtype if np.issubdtype(logAge.dtype, np.floating)
                        else np.float64)
    for i, la in enumerate(logAge):
        idx = int(np.nonzero(uniq == la)[0][0])
        out[i] = sfr * dt[idx] / num[idx]
    return out


def renormalize_x0(data, models, x0, full_coeffs=None):
    """renormalize_x0, src/fitting/utilities.jl:104-115: x0 scaled by Σn / Σm."""
    M = as_models(models)
    full = x0 if full_coeffs is None else full_coeffs
    T = _T(data, full)
    c = np.empty(M.nbins, dtype=T)
    composite_(c, full, M)
    s = c.sum()
    if s == 0:
        return np.array(x0, copy=True)
    return np.asarray(x0) * (np.sum(data) / s)


# ---------------------------------------------------------------- fit drivers

def fit_templates_lbfgsb(models, data, x0=None, factr=1e-12, pgtol=1e-5, maxiter=15000):
    """fit_templates_lbfgsb, src/fitting/solvers.jl:70-90: box-constrained L-BFGS-B on
    fg! (LBFGSB.jl wraps the same Fortran L-BFGS-B that scipy ships).
    Returns (-logL, coeffs)."""
    from scipy.optimize import fmin_l_bfgs_b
    M = as_models(models)
    data = np.asarray(data, dtype=np.float64).reshape(-1, order="F")
    x0 = np.ones(M.nt) if x0 is None else np.asarray(x0, dtype=np.float64)
    x0 = renormalize_x0(data, M, x0)
    comp = np.empty(M.nbins)
    G = np.empty(M.nt)

    def f(x):
        v = fg_(True, G, x, M, data, comp)
        return float(v), G.copy()

    x, fval, _info = fmin_l_bfgs_b(f, x0, bounds=[(0.0, None)] * M.nt, factr=factr,
                                   pgtol=pgtol, maxiter=maxiter, m=10)
    return fval, x


FIT_LOG_MAP, FIT_LOG_MLE, FIT_SQRT = 0, 1, 2
FIT_STATUS = ("converged (g)", "converged (f)", "converged (x)", "maximum iterations",
              "line search made no progress", "non-finite objective", "maximum evaluations")
BFGSResult = namedtuple("BFGSResult", ["x", "fun", "hess_inv", "nit", "nfev", "status",
                                       "message", "success", "g_norm", "graph"])


def fit_bfgs_device(models, data, theta0, transform, g_abstol=1e-8, f_reltol=0.0,
                    x_abstol=0.0, maxiter=1000, max_evals=0, want_invH=True, graph_slots=0):
    """BFGS over fg! run on the GPU (sfh_fit_bfgs): the minimisation Optim.BFGS performs in
    fit_templates / fit_templates_fast (src/fitting/solvers.jl:172-275) for the transform
    FIT_LOG_MAP (r = exp θ, Jacobian term -Σθ), FIT_LOG_MLE (r = exp θ) or FIT_SQRT
    (r = θ²).  Returns a BFGSResult (x = θ at the minimum, hess_inv = the BFGS inverse
    Hessian in θ when want_invH)."""
    M = as_models(models)
    d = np.ascontiguousarray(np.asarray(data, dtype=np.float64).reshape(-1, order="F"))
    th = np.ascontiguousarray(theta0, dtype=np.float64)
    _argcheck(d.size == M.nbins, "length(data) == size(models, 1)")
    _argcheck(th.size == M.nt, "length(x0) == size(models, 2)")
    opt = FitOptions(int(transform), int(maxiter), int(max_evals), int(graph_slots),
                     float(g_abstol), float(f_reltol), float(x_abstol), 0.0)
    res = FitResult()
    out = np.empty(M.nt)
    invH = np.empty((M.nt, M.nt)) if want_invH else None
    ctx = M.ctx
    check(load().sfh_fit_bfgs(ctx.handle, M.handle, d.ctypes.data, th.ctypes.data, C.byref(opt),
                              out.ctypes.data, invH.ctypes.data if want_invH else None,
                              C.byref(res)), ctx.handle, "fit_bfgs")
    return BFGSResult(out, res.f, invH, int(res.iterations), int(res.evaluations),
                      int(res.status), FIT_STATUS[res.status], res.status <= 2, res.g_norm,
                      bool(res.graph))


def fit_templates_fast(models, data, x0=None, g_abstol=1e-8, maxiter=1000, method="device"):
    """fit_templates_fast, src/fitting/solvers.jl:238-275: BFGS in sqrt space
    (coeffs = θ²), on the GPU (method "device") or by scipy's BFGS over fg! ("scipy").
    Returns (coeffs, result)."""
    M = as_models(models)
    data = np.asarray(data, dtype=np.float64).reshape(-1, order="F")
    x0 = np.ones(M.nt) if x0 is None else np.asarray(x0, dtype=np.float64)
    x0 = np.sqrt(renormalize_x0(data, M, x0))
    if method == "device":
        r = fit_bfgs_device(M, data, x0, FIT_SQRT, g_abstol=g_abstol, maxiter=maxiter,
                            want_invH=False)
        return r.x ** 2, r
    _argcheck(method == "scipy", "method is 'device' or 'scipy'")
    from scipy.optimize import minimize
    comp = np.empty(M.nbins)
    G = np.empty(M.nt)

    def f(s):
        v = fg_(True, G, s * s, M, data, comp)
        return float(v), G * 2.0 * s

    res = minimize(f, x0, jac=True, method="BFGS",
                   options={"gtol": g_abstol, "maxiter": maxiter})
    return res.x ** 2, res


LogTransformFTResult = namedtuple("LogTransformFTResult", ["mu", "sigma", "invH", "result"])
FitTemplatesResult = namedtuple("FitTemplatesResult", ["map", "mle"])


def fit_templates(models, data, x0=None, gtol=1e-8, maxiter=1000, method="device"):
    """fit_templates, src/fitting/solvers.jl:172-221: MAP (log transform with the
    Jacobian term -Σθ) then MLE from the MAP point, both by BFGS (on the GPU with method
    "device", scipy's BFGS over fg! with "scipy"); μ, σ from the BFGS inverse Hessian in
    log space."""
    M = as_models(models)
    data = np.asarray(data, dtype=np.float64).reshape(-1, order="F")
    x0 = np.ones(M.nt) if x0 is None else np.asarray(x0, dtype=np.float64)
    x0 = np.log(renormalize_x0(data, M, x0))
    if method == "device":
        r_map = fit_bfgs_device(M, data, x0, FIT_LOG_MAP, g_abstol=gtol, maxiter=maxiter)
        r_mle = fit_bfgs_device(M, data, r_map.x, FIT_LOG_MLE, g_abstol=gtol, maxiter=maxiter)

        def pack_dev(r):
            mu = np.exp(r.x)
            return LogTransformFTResult(mu, np.sqrt(np.abs(np.diag(r.hess_inv))) * mu,
                                        r.hess_inv, r)
        return FitTemplatesResult(pack_dev(r_map), pack_dev(r_mle))
    _argcheck(method == "scipy", "method is 'device' or 'scipy'")
    from scipy.optimize import minimize
    comp = np.empty(M.nbins)
    G = np.empty(M.nt)

    def fg_map(logx):
        x = np.exp(logx)
        v = fg_(True, G, x, M, data, comp) - logx.sum()
        return float(v), G * x - 1.0

    def fg_mle(logx):
        x = np.exp(logx)
        v = fg_(True, G, x, M, data, comp)
        return float(v), G * x

    opts = {"gtol": gtol, "maxiter": maxiter}
    r_map = minimize(fg_map, x0, jac=True, method="BFGS", options=opts)
    r_mle = minimize(fg_mle, r_map.x, jac=True, method="BFGS", options=opts)

    def pack(r):
        mu = np.exp(r.x)
        invH = np.asarray(r.hess_inv)
        return LogTransformFTResult(mu, np.sqrt(np.abs(np.diag(invH))) * mu, invH, r)

    return FitTemplatesResult(pack(r_map), pack(r_mle))


def construct_x0_mdf(logAge, T_max, normalize_value=1.0):
    """construct_x0_mdf(logAge, T_max), hierarchical/construct_x0_mdf.jl:58-71: stellar mass
    per unique log age for a constant star formation rate since T_max (Gyr)."""
    logAge = np.asarray(logAge, dtype=np.float64)
    _argcheck(np.log10(T_max) + 9 > logAge.max(), "log10(T_max) + 9 > maximum(logAge)")
    max_la = np.log10(T_max) + 9
    sfr = normalize_value / (10.0 ** max_la - 10.0 ** logAge.min())
    uniq = list(dict.fromkeys(logAge.tolist()))
    srt = sorted(uniq) + [max_la]
    dt = np.diff(10.0 ** np.asarray(srt))
    return np.array([sfr * dt[srt.index(la)] for la in uniq])


def truncate_relweights(relweightsmin, relweights, logAge):
    """truncate_relweights, hierarchical/fixed_amr.jl:225-243: indices of the templates whose
    relative weight is at least relweightsmin times the largest of their log age."""
    relweights, logAge = np.asarray(relweights), np.asarray(logAge)
    _argcheck(relweights.size == logAge.size, "length(relweights) == length(logAge)")
    if relweightsmin == 0:
        return np.arange(relweights.size)
    keep = []
    for la in dict.fromkeys(logAge.tolist()):
        good = np.nonzero(logAge == la)[0]
        keep.append(good[relweights[good] >= relweightsmin * relweights[good].max()])
    return np.concatenate(keep)


def fixed_amr(models, data, logAge, metallicities, relweights, relweightsmin=0.0, x0=None,
              gtol=1e-8, maxiter=10000):
    """fixed_amr, hierarchical/fixed_amr.jl:41-188: fit one stellar-mass coefficient per
    unique log age under fixed relative weights (an externally imposed age-metallicity
    relation).  The expansion coeffs[idxs] = relweights[idxs] * x[i] is linear, so the
    templates of each age are combined once on the device into one column and the MAP /
    MLE fits (log transform, BFGS) run on the reduced (nbins, n_ages) matrix.  Returns
    (map, mle) with μ per unique age and σ = sqrt(diag(invH)) in log space
    (fixed_amr.jl:185-186)."""
    import warnings

    from scipy.optimize import minimize
    M = models if isinstance(models, Models) else Models(
        np.asfortranarray(np.asarray(models, dtype=np.float32)), storage="f32")
    data = np.asarray(data, dtype=np.float64).reshape(-1, order="F")
    logAge = np.asarray(logAge, dtype=np.float64)
    metallicities = np.asarray(metallicities, dtype=np.float64)
    relweights = np.array(relweights, dtype=np.float64)
    uniq = list(dict.fromkeys(logAge.tolist()))
    if x0 is None:
        x0 = construct_x0_mdf(logAge, 13.7)
    x0 = np.asarray(x0, dtype=np.float64)
    _argcheck(x0.size == len(uniq), "length(x0) == length(unique(logAge))")
    _argcheck(M.nbins == data.size, "size(models, 1) == length(data)")
    _argcheck(M.nt == logAge.size == metallicities.size == relweights.size,
              "size(models, 2) == length(logAge) == length(metallicities) == length(relweights)")
    _argcheck(np.all(relweights >= 0), "all relative weights must be ≥ 0")
    _argcheck(relweightsmin >= 0, "relweightsmin >= 0")
    keep = truncate_relweights(relweightsmin, relweights, logAge)
    groups, weights = [], []
    for la in uniq:
        good = keep[logAge[keep] == la]
        s = relweights[good].sum()
        if not np.isclose(s, 1.0) and relweightsmin == 0:
            warnings.warn(f"The relative weights for logAge={la} provided to fixed_amr do not "
                          "sum to 1 and will be renormalized.", stacklevel=2)
        groups.append(good)
        weights.append(relweights[good] / s)
    Mr = M.combine(groups, weights, storage="f32")
    x0 = np.log(renormalize_x0(data, Mr, x0))
    comp = np.empty(Mr.nbins)
    G = np.empty(Mr.nt)

    def fg_map(logx):  # fixed_amr.jl:102-125
        x = np.exp(logx)
        v = fg_(True, G, x, Mr, data, comp) - logx.sum()
        return float(v), G * x - 1.0

    def fg_mle(logx):  # fixed_amr.jl:127-149
        x = np.exp(logx)
        v = fg_(True, G, x, Mr, data, comp)
        return float(v), G * x

    opts = {"gtol": gtol, "maxiter": maxiter}
    r_map = minimize(fg_map, x0, jac=True, method="BFGS", options=opts)
    r_mle = minimize(fg_mle, r_map.x, jac=True, method="BFGS", options=opts)

    def pack(r):
        invH = np.asarray(r.hess_inv)
        return LogTransformFTResult(np.exp(r.x), np.sqrt(np.abs(np.diag(invH))), invH, r)

    return FitTemplatesResult(pack(r_map), pack(r_mle))


def fg_batched(models, R, data, want_logl=True, want_grad=True, eps=None):
    """B fg! evaluations in one call on the tensor cores (sfh_fg_batched_dev).

    models: a Models handle stored as "bf16x2"; R: (B, nt) coefficient vectors (torch CUDA
    float64 tensor or numpy); data: (nbins,) observed counts.  Returns (negLogL, G): -logL
    per vector (float64, or None) and -∇logL per vector (B x nt float32, or None), as
    torch CUDA tensors.  Accuracy: with want_logl the composite is exact on the stored FP32
    templates (digit planes, |ΔlogL| <= 1e-6 per 1e4 stars against FP64); the gradient
    accumulates BF16 hi/lo products in FP32 (about 1e-5 of sum_i |M_ij w_i|)."""
    import torch
    M = models if isinstance(models, Models) else Models(np.asarray(models), storage="bf16x2")
    dev = torch.device("cuda", M.ctx.device)
    Rt = torch.as_tensor(R, dtype=torch.float64, device=dev).contiguous()
    nt_t = torch.as_tensor(data, dtype=torch.float64, device=dev).reshape(-1).contiguous()
    B, nt = Rt.shape
    _argcheck(nt == M.nt, "size(R, 2) == size(models, 2)")
    _argcheck(nt_t.numel() == M.nbins, "length(data) == size(models, 1)")
    negL = torch.empty(B, dtype=torch.float64, device=dev) if want_logl else None
    G = torch.empty((B, nt), dtype=torch.float32, device=dev) if want_grad else None
    torch.cuda.current_stream(dev).synchronize()
    e = float(np.finfo(np.float64).eps) if eps is None else float(eps)
    check(load().sfh_fg_batched_dev(M.ctx.handle, M.handle, Rt.data_ptr(), B, nt_t.data_ptr(),
                                    negL.data_ptr() if want_logl else None,
                                    G.data_ptr() if want_grad else None, e),
          M.ctx.handle, "fg_batched")
    return negL, G


class GalaxyDesc(C.Structure):
    """sfh_galaxy: where one galaxy's templates, bins and coefficients sit in the packed
    arrays of a ragged batch."""
    _fields_ = [("model_offset", C.c_int64), ("nbins", C.c_int64), ("ntempl", C.c_int64),
                ("bin_offset", C.c_int64), ("templ_offset", C.c_int64)]


class Galaxies:
    """A ragged batch of independent galaxies (sfh_galaxies handle): galaxy g's
    (nbins_g x ntempl_g) column-major FP32 templates live in one packed CUDA tensor.
    Coefficients / gradients are packed galaxy after galaxy, as are data / composites."""

    def __init__(self, models_packed, nbins, ntempl, model_offsets=None, ctx=None):
        self.ctx = ctx or default_context()
        nbins = np.asarray(nbins, dtype=np.int64)
        ntempl = np.asarray(ntempl, dtype=np.int64)
        _argcheck(nbins.shape == ntempl.shape and nbins.ndim == 1, "one nbins and ntempl per galaxy")
        n = nbins.size
        if model_offsets is None:
            model_offsets = np.concatenate([[0], np.cumsum(nbins * ntempl)[:-1]])
        self.bin_offsets = np.concatenate([[0], np.cumsum(nbins)]).astype(np.int64)
        self.templ_offsets = np.concatenate([[0], np.cumsum(ntempl)]).astype(np.int64)
        desc = (GalaxyDesc * n)()
        for g in range(n):
            desc[g] = GalaxyDesc(int(model_offsets[g]), int(nbins[g]), int(ntempl[g]),
                                 int(self.bin_offsets[g]), int(self.templ_offsets[g]))
        self.models = models_packed  # referenced by the handle: keep alive
        self.nbins, self.ntempl = nbins, ntempl
        h = C.c_void_p()
        check(load().sfh_galaxies_create(self.ctx.handle, models_packed.data_ptr(),
                                         int(models_packed.numel()), desc, n, C.byref(h)),
              self.ctx.handle, "galaxies_create")
        self.handle = h.value

    @property
    def ngal(self):
        return self.nbins.size

    def free(self):
        if getattr(self, "handle", None):
            load().sfh_galaxies_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


def fg_ragged(galaxies: Galaxies, coeffs, data, want_logl=True, want_grad=True, eps=None):
    """fg! (solvers.jl:20-38) for every galaxy of a ragged batch in one device call.
    coeffs / data: packed CUDA float64 tensors (or numpy).  Returns (negLogL per galaxy or
    None, packed G or None, packed composite) as CUDA tensors."""
    import torch
    ctx = galaxies.ctx
    dev = torch.device("cuda", ctx.device)
    r = torch.as_tensor(coeffs, dtype=torch.float64, device=dev).contiguous()
    n = torch.as_tensor(data, dtype=torch.float64, device=dev).contiguous()
    _argcheck(r.numel() == galaxies.templ_offsets[-1], "coefficients do not match the galaxies")
    _argcheck(n.numel() == galaxies.bin_offsets[-1], "data do not match the galaxies")
    comp = torch.empty_like(n)
    G = torch.empty_like(r) if want_grad else None
    negL = torch.empty(galaxies.ngal, dtype=torch.float64, device=dev) if want_logl else None
    eps = float(np.finfo(np.float64).eps) if eps is None else float(eps)
    torch.cuda.current_stream(dev).synchronize()
    check(load().sfh_fg_ragged_dev(ctx.handle, galaxies.handle, r.data_ptr(), n.data_ptr(),
                                   comp.data_ptr(), G.data_ptr() if G is not None else None,
                                   negL.data_ptr() if negL is not None else None, eps),
          ctx.handle, "fg_ragged")
    ctx.synchronize()
    return negL, G, comp
