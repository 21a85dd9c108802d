"""ctypes view of the FP64 CPU oracle (``oracle/sfh_oracle.c``).

TEST INFRASTRUCTURE ONLY: ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use this module as
the checker.  The product (``starformationhistories.jl_gb300``) never imports it.

Each wrapper mirrors the reference function named in its docstring
(StarFormationHistories.jl v1.3.1, file:line).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libsfh_oracle.so")
_lock = threading.Lock()
_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64 = C.c_int64


class ErrModel(C.Structure):
    """exp_photerr(m, a, b, c, d) = a^(b(m-c)) + d capped at ``cap`` (src/utilities.jl:218)."""
    _fields_ = [("a", C.c_double), ("b", C.c_double), ("c", C.c_double), ("d", C.c_double),
                ("cap", C.c_double)]


class ComplModel(C.Structure):
    """Martin2016_complete(m, A, m50, rho) (src/utilities.jl:205)."""
    _fields_ = [("A", C.c_double), ("m50", C.c_double), ("rho", C.c_double)]


class IMF(C.Structure):
    """Continuous broken power law; Kroupa2001(0.08, 100) = breaks (0.5,), alpha (1.3, 2.3)."""
    _fields_ = [("nseg", C.c_int), ("mmin", C.c_double), ("mmax", C.c_double),
                ("breaks", C.c_double * 3), ("alpha", C.c_double * 4)]


def kroupa2001(mmin=0.08, mmax=100.0) -> IMF:
    imf = IMF()
    imf.nseg = 2
    imf.mmin, imf.mmax = mmin, mmax
    imf.breaks[0] = 0.5
    imf.alpha[0], imf.alpha[1] = 1.3, 2.3
    return imf


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -O3 -fopenmp)."""
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "sfh_oracle.c"))):
        subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB_PATH)
            L.sfho_composite.argtypes = [_dp, _i64, _i64, _dp, _dp]
            L.sfho_loglikelihood.argtypes = [_dp, _dp, _i64, C.c_double]
            L.sfho_loglikelihood.restype = C.c_double
            L.sfho_grad_single.argtypes = [_dp, _dp, _dp, _i64, C.c_double]
            L.sfho_grad_single.restype = C.c_double
            L.sfho_grad_inplace.argtypes = [_dp, _dp, _dp, _dp, _i64, _i64, C.c_double]
            L.sfho_fg.argtypes = [C.c_int, C.c_void_p, _dp, _dp, _dp, _dp, _i64, _i64, C.c_double]
            L.sfho_fg.restype = C.c_double
            L.sfho_fg_batched.argtypes = [_dp, _i64, _dp, _dp, _i64, _i64, C.c_double, _dp,
                                          C.c_void_p, C.c_int]
            L.sfho_mini_spacing.argtypes = [_dp, _dp, _dp, _i64, C.c_double, _dp, _i64]
            L.sfho_mini_spacing.restype = _i64
            L.sfho_interpolate_mini.argtypes = [_dp, _dp, _i64, _dp, _i64, _dp]
            L.sfho_midpoints.argtypes = [_dp, _i64, _dp]
            L.sfho_histogram_pix.argtypes = [C.c_double] * 3
            L.sfho_histogram_pix.restype = C.c_double
            L.sfho_gaussian_int_general.argtypes = [C.c_double] * 8
            L.sfho_gaussian_int_general.restype = C.c_double
            L.sfho_gaussian_psf_covariant.argtypes = [C.c_double] * 11
            L.sfho_gaussian_psf_covariant.restype = C.c_double
            L.sfho_addstar_asym.argtypes = [_dp, _i64, _i64] + [C.c_double] * 6 + [_i64, _i64]
            L.sfho_addstar_cov.argtypes = [_dp, _i64, _i64] + [C.c_double] * 11
            L.sfho_bin_cmd_smooth.argtypes = [_dp, _dp, _dp, _dp, _dp, _i64, C.c_int, C.c_double,
                                              C.c_double, _i64, C.c_double, C.c_double, _i64, _dp]
            L.sfho_imf_pdf.argtypes = [C.POINTER(IMF), C.c_double]
            L.sfho_imf_pdf.restype = C.c_double
            L.sfho_imf_mean.argtypes = [C.POINTER(IMF)]
            L.sfho_imf_mean.restype = C.c_double
            L.sfho_calculate_weights.argtypes = [_dp, _dp, _i64, C.POINTER(IMF), C.c_double,
                                                 C.c_double, _dp, _dp]
            L.sfho_partial_cmd_smooth.argtypes = [
                _dp, _dp, _i64, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(ErrModel),
                C.POINTER(ComplModel), C.c_void_p, C.POINTER(IMF), C.c_double, C.c_double,
                C.c_double, C.c_double, C.c_double, _i64, C.c_double, C.c_double, _i64, _dp]
            L.sfho_partial_cmd_smooth.restype = _i64
            L.sfho_bin_cmd.argtypes = [_dp, _dp, C.c_void_p, _i64, _dp, _i64, _dp, _i64, _dp]
            L.sfho_partial_cmd.argtypes = [_dp, _dp, _dp, _i64, C.POINTER(IMF), C.c_double,
                                           C.c_double, C.c_double, _dp, _i64, _dp, _i64, _dp]
            L.sfho_partial_cmd.restype = C.c_int
            L.sfho_mag2flux.argtypes = [C.c_double]
            L.sfho_mag2flux.restype = C.c_double
            L.sfho_flux2mag.argtypes = [C.c_double]
            L.sfho_flux2mag.restype = C.c_double
            L.sfho_trapz.argtypes = [_dp, _dp, _i64]
            L.sfho_trapz.restype = C.c_double
            L.sfho_binary_hess.argtypes = [
                _dp, _dp, _i64, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(ErrModel),
                C.POINTER(ComplModel), C.c_void_p, C.POINTER(IMF), C.c_double, C.c_double,
                C.c_double, C.c_double, _i64, C.c_double, C.c_double, _i64, _dp]
            L.sfho_binary_hess.restype = C.c_int
            L.sfho_partial_cmd_smooth_binary.argtypes = [
                _dp, _dp, _i64, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(ErrModel),
                C.POINTER(ComplModel), C.c_void_p, C.POINTER(IMF), C.c_double, C.c_double,
                C.c_double, C.c_double, C.c_double, C.c_double, _i64, C.c_double, C.c_double,
                _i64, _dp]
            L.sfho_partial_cmd_smooth_binary.restype = C.c_int
            L.sfho_powerlaw_mzr.argtypes = [C.c_double] * 4
            L.sfho_powerlaw_mzr.restype = C.c_double
            L.sfho_gauss_disp.argtypes = [C.c_double] * 3
            L.sfho_gauss_disp.restype = C.c_double
            L.sfho_mzr_calculate_coeffs.argtypes = [C.c_double] * 4 + [_dp, _i64, _dp, _dp, _i64,
                                                                       _dp]
            L.sfho_mzr_calculate_coeffs.restype = C.c_int
            L.sfho_mzr_fg.argtypes = [_dp, _i64, C.c_double, C.c_int, C.c_int, C.c_int, _dp, _dp,
                                      _i64, _i64, _dp, _dp, C.c_double, C.c_void_p]
            L.sfho_mzr_fg.restype = C.c_double
            L.sfho_mlp_param_count.argtypes = [C.c_int] * 4
            L.sfho_mlp_param_count.restype = _i64
            L.sfho_mlp_forward.argtypes = [C.c_int] * 4 + [_dp, _dp, _i64, C.c_int, _dp]
            L.sfho_mlp_loss_grad.argtypes = [C.c_int] * 4 + [_dp, _dp, _dp, _i64, C.c_int, _dp]
            L.sfho_mlp_loss_grad.restype = C.c_double
            L.sfho_poisson_deviance.argtypes = [_dp, _dp, _i64]
            L.sfho_poisson_deviance.restype = C.c_double
            L.sfho_linear_amr.argtypes = [C.c_double] * 4
            L.sfho_linear_amr.restype = C.c_double
            L.sfho_mh_from_z.argtypes = [C.c_double]
            L.sfho_mh_from_z.restype = C.c_double
            L.sfho_dmh_dz.argtypes = [C.c_double]
            L.sfho_dmh_dz.restype = C.c_double
            L.sfho_amr_fg.argtypes = [C.c_int, _dp, _i64, C.c_double, C.c_int, C.c_int, C.c_int,
                                      _dp, _dp, _i64, _i64, _dp, _dp, C.c_double, C.c_void_p]
            L.sfho_amr_fg.restype = C.c_double
            L.sfho_set_threads.argtypes = [C.c_int]
            L.sfho_get_max_threads.restype = C.c_int
            _lib = L
    return _lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def eps_of(dtype) -> float:
    """eps(T) of the promoted element type (fitting_base.jl:89)."""
    return float(np.finfo(np.dtype(dtype)).eps)


def set_threads(n: int) -> None:
    lib().sfho_set_threads(int(n))


def max_threads() -> int:
    return int(lib().sfho_get_max_threads())


# ---------------- fitting_base.jl / solvers.jl ----------------

def composite(M, r):
    """composite!(composite, coeffs, models) flat form, fitting_base.jl:55-65."""
    M = np.asfortranarray(M, dtype=np.float64)
    nb, nt = M.shape
    out = np.empty(nb)
    lib().sfho_composite(M.ravel(order="F"), nb, nt, _f64(r), out)
    return out


def loglikelihood(c, n, eps=eps_of(np.float64)):
    """loglikelihood(composite, data), fitting_base.jl:84-96."""
    c, n = _f64(c).ravel(order="F"), _f64(n).ravel(order="F")
    return lib().sfho_loglikelihood(c, n, c.size, eps)


def grad_single(model, c, n, eps=eps_of(np.float64)):
    """∇loglikelihood(model, composite, data), fitting_base.jl:144-160."""
    return lib().sfho_grad_single(_f64(model).ravel(order="F"), _f64(c).ravel(order="F"),
                                  _f64(n).ravel(order="F"), int(np.size(c)), eps)


def grad_inplace(c, M, n, eps=eps_of(np.float64)):
    """∇loglikelihood!(G, composite, models, data), fitting_base.jl:265-285.
    Returns (G, overwritten composite)."""
    M = np.asfortranarray(M, dtype=np.float64)
    nb, nt = M.shape
    c = _f64(c).copy()
    G = np.empty(nt)
    lib().sfho_grad_inplace(G, c, M.ravel(order="F"), _f64(n), nb, nt, eps)
    return G, c


def fg(r, M, n, want_f=True, want_g=True, eps=eps_of(np.float64)):
    """fg!(F, G, coeffs, models, data, composite), solvers.jl:20-38.
    Returns (-logL or None, G or None, composite after the call)."""
    M = np.asfortranarray(M, dtype=np.float64)
    nb, nt = M.shape
    c = np.empty(nb)
    G = np.empty(nt) if want_g else None
    Gp = G.ctypes.data if want_g else None
    v = lib().sfho_fg(1 if want_f else 0, Gp, _f64(r), M.ravel(order="F"), _f64(n), c, nb, nt,
                      eps)
    return (v if want_f else None), G, c


def fg_batched(R, M, n, nthreads=1, want_g=True, eps=eps_of(np.float64)):
    """B independent fg! calls (R is B x nt); returns (negLogL[B], G[B, nt])."""
    M = np.asfortranarray(M, dtype=np.float64)
    nb, nt = M.shape
    R = np.ascontiguousarray(R, dtype=np.float64)
    B = R.shape[0]
    out = np.empty(B)
    G = np.empty((B, nt)) if want_g else None
    lib().sfho_fg_batched(R.ravel(), B, M.ravel(order="F"), _f64(n), nb, nt, eps, out,
                          G.ctypes.data if want_g else None, int(nthreads))
    return out, G


# ---------------- templates ----------------

def mini_spacing(m_ini, colors, mags, dmag):
    """mini_spacing(m_ini, colors, mags, Δmag, true), StarFormationHistories.jl:110-148."""
    m_ini, colors, mags = _f64(m_ini), _f64(colors), _f64(mags)
    cap = 4096
    while True:
        out = np.empty(cap)
        k = lib().sfho_mini_spacing(m_ini, colors, mags, m_ini.size, float(dmag), out, cap)
        if k >= 0:
            new = out[:k].copy()
            return new, np.diff(new)
        cap = -k


def interpolate_mini(m_ini, mags, new_mini):
    """interpolate_mini, StarFormationHistories.jl:77-81."""
    new_mini = _f64(new_mini)
    out = np.empty(new_mini.size)
    lib().sfho_interpolate_mini(_f64(m_ini), _f64(mags), np.size(m_ini), new_mini,
                                new_mini.size, out)
    return out


def midpoints(v):
    """midpoints(v), StarFormationHistories.jl:417-436."""
    v = _f64(v)
    out = np.empty(max(v.size - 1, 0))
    lib().sfho_midpoints(v, v.size, out)
    return out


def histogram_pix(d, first, step):
    """histogram_pix(d, edges::AbstractRange), StarFormationHistories.jl:502."""
    return lib().sfho_histogram_pix(float(d), float(first), float(step))


def gaussian_int_general(dx, dy, hx, hy, sx, sy, A, B=0.0):
    return lib().sfho_gaussian_int_general(dx, dy, hx, hy, sx, sy, A, B)


def gaussian_psf_covariant(x, y, hx, hy, x0, y0, sx, sy, cov, A, B=0.0):
    return lib().sfho_gaussian_psf_covariant(x, y, hx, hy, x0, y0, sx, sy, cov, A, B)


def addstar_asym(img, x0, y0, sx, sy, A, B=0.0, cutout=None):
    """addstar!(image, GaussianPSFAsymmetric(...), cutout), StarFormationHistories.jl:348-364.
    img is (nx, ny) Fortran-ordered float64, updated in place."""
    nx, ny = img.shape
    if cutout is None:
        cutout = (int(np.ceil(sx * 10)), int(np.ceil(sy * 10)))
    flat = np.ascontiguousarray(img.T).ravel()  # column-major flatten
    lib().sfho_addstar_asym(flat, nx, ny, x0, y0, sx, sy, A, B, int(cutout[0]), int(cutout[1]))
    img[...] = flat.reshape(ny, nx).T


def addstar_cov(img, edges, x0, y0, sx, sy, cov, A, cutout=None):
    """addstar!(hist, GaussianPSFCovariant(...), cutout), StarFormationHistories.jl:366-408."""
    nx, ny = img.shape
    (xf, xs), (yf, ys) = edges
    if cutout is None:
        cutout = (15 * sx, 10 * sy)
    flat = np.ascontiguousarray(img.T).ravel()
    lib().sfho_addstar_cov(flat, nx, ny, xf, xs, yf, ys, x0, y0, sx, sy, cov, A,
                           float(cutout[0]), float(cutout[1]))
    img[...] = flat.reshape(ny, nx).T


def bin_cmd_smooth(x, y, sx, sy, w, cov_mult, xedges, yedges):
    """bin_cmd_smooth, StarFormationHistories.jl:574-621.
    xedges/yedges = (first, step, nbins).  Returns (nx, ny) float64."""
    xf, xs, nx = xedges
    yf, ys, ny = yedges
    out = np.empty(nx * ny)
    x = _f64(x)
    lib().sfho_bin_cmd_smooth(x, _f64(y), _f64(sx), _f64(sy), _f64(w), x.size, int(cov_mult),
                              xf, xs, nx, yf, ys, ny, out)
    return out.reshape(ny, nx).T


def imf_pdf(imf, m):
    return lib().sfho_imf_pdf(C.byref(imf), float(m))


def imf_mean(imf):
    return lib().sfho_imf_mean(C.byref(imf))


def calculate_weights(mini, completeness, imf, normalize_value, mean_mass, spacing=None):
    """calculate_weights, StarFormationHistories.jl:765-776."""
    mini = _f64(mini)
    if spacing is None:
        spacing = np.diff(mini)
    out = np.empty(mini.size - 1)
    lib().sfho_calculate_weights(mini, _f64(completeness), mini.size, C.byref(imf),
                                 float(normalize_value), float(mean_mass), _f64(spacing), out)
    return out


def partial_cmd_smooth(m_ini, mags, err_models, compl_models, y_index, color_indices, imf,
                       dmod, normalize_value, mean_mass, xedges, yedges, bias=None):
    """partial_cmd_smooth (single stars), StarFormationHistories.jl:829-888.
    mags: (nf, n); y_index / color_indices are 0-based.  Returns (nx, ny) float64."""
    mags = np.ascontiguousarray(mags, dtype=np.float64)
    nf, n = mags.shape
    E = (ErrModel * nf)(*err_models)
    Cm = (ComplModel * nf)(*compl_models)
    b = None
    if bias is not None:
        barr = _f64(bias)
        b = barr.ctypes.data
    xf, xs, nx = xedges
    yf, ys, ny = yedges
    out = np.empty(nx * ny)
    k = lib().sfho_partial_cmd_smooth(_f64(m_ini), mags.ravel(), n, nf, int(y_index),
                                      int(color_indices[0]), int(color_indices[1]), E, Cm, b,
                                      C.byref(imf), float(dmod), float(normalize_value),
                                      float(mean_mass), xf, xs, nx, yf, ys, ny, out)
    if k < 0:
        raise ValueError("partial_cmd_smooth: invalid arguments")
    return out.reshape(ny, nx).T


# ---------------- binary-star templates ----------------

def bin_cmd(x, y, w, xedges, yedges):
    """bin_cmd, StarFormationHistories.jl:544-553, on explicit edge vectors.  Returns the
    (nx, ny) float64 weights."""
    x, y, ex, ey = _f64(x), _f64(y), _f64(xedges), _f64(yedges)
    warr = None if w is None else _f64(w)
    nx, ny = ex.size - 1, ey.size - 1
    out = np.empty(nx * ny)
    lib().sfho_bin_cmd(x, y, None if warr is None else warr.ctypes.data, x.size, ex, nx, ey, ny,
                       out)
    return out.reshape(ny, nx).T


def partial_cmd(m_ini, colors, mags, imf, dmod, normalize_value, mean_mass, xedges, yedges):
    """partial_cmd (error-free template), StarFormationHistories.jl:733-757."""
    ex, ey = _f64(xedges), _f64(yedges)
    nx, ny = ex.size - 1, ey.size - 1
    out = np.empty(nx * ny)
    m_ini, colors, mags = _f64(m_ini), _f64(colors), _f64(mags)
    if lib().sfho_partial_cmd(m_ini, colors, mags, m_ini.size, C.byref(imf), float(dmod),
                              float(normalize_value), float(mean_mass), ex, nx, ey, ny, out) < 0:
        raise ValueError("partial_cmd: invalid arguments")
    return out.reshape(ny, nx).T


def mag2flux(m):
    """mag2flux(m) with zero point 0, src/utilities.jl:57."""
    return lib().sfho_mag2flux(float(m))


def flux2mag(f):
    """flux2mag(f) with zero point 0, src/utilities.jl:67."""
    return lib().sfho_flux2mag(float(f))


def trapz(x, y):
    """Trapz.jl trapz(x, y)."""
    x, y = _f64(x), _f64(y)
    return lib().sfho_trapz(x, y, x.size)


def binary_hess(m_ini, mags, err_models, compl_models, y_index, color_indices, imf,
                normalize_value, mean_mass, xedges, yedges, bias=None):
    """binary_hess(RandomBinaryPairs, ...), StarFormationHistories.jl:627-706 (magnitudes
    already shifted by the distance modulus).  Returns (nx, ny) float64."""
    mags = np.ascontiguousarray(mags, dtype=np.float64)
    nf, n = mags.shape
    E = (ErrModel * nf)(*err_models)
    Cm = (ComplModel * nf)(*compl_models)
    b = None
    if bias is not None:
        barr = _f64(bias)
        b = barr.ctypes.data
    xf, xs, nx = xedges
    yf, ys, ny = yedges
    out = np.empty(nx * ny)
    k = lib().sfho_binary_hess(_f64(m_ini), mags.ravel(), n, nf, int(y_index),
                               int(color_indices[0]), int(color_indices[1]), E, Cm, b,
                               C.byref(imf), float(normalize_value), float(mean_mass), xf, xs, nx,
                               yf, ys, ny, out)
    if k < 0:
        raise ValueError("binary_hess: invalid arguments" if k == -1 else
                         "binary_hess: y_index must be one of color_indices")
    return out.reshape(ny, nx).T


def partial_cmd_smooth_binary(m_ini, mags, err_models, compl_models, y_index, color_indices,
                              imf, dmod, normalize_value, mean_mass, binary_fraction, xedges,
                              yedges, bias=None):
    """partial_cmd_smooth with binary_model = RandomBinaryPairs(binary_fraction),
    StarFormationHistories.jl:829-910.  Returns (nx, ny) float64."""
    mags = np.ascontiguousarray(mags, dtype=np.float64)
    nf, n = mags.shape
    E = (ErrModel * nf)(*err_models)
    Cm = (ComplModel * nf)(*compl_models)
    b = None
    if bias is not None:
        barr = _f64(bias)
        b = barr.ctypes.data
    xf, xs, nx = xedges
    yf, ys, ny = yedges
    out = np.empty(nx * ny)
    k = lib().sfho_partial_cmd_smooth_binary(_f64(m_ini), mags.ravel(), n, nf, int(y_index),
                                             int(color_indices[0]), int(color_indices[1]), E, Cm,
                                             b, C.byref(imf), float(dmod), float(normalize_value),
                                             float(mean_mass), float(binary_fraction), xf, xs,
                                             nx, yf, ys, ny, out)
    if k < 0:
        raise ValueError("partial_cmd_smooth_binary: invalid arguments")
    return out.reshape(ny, nx).T


# ---------------- hierarchical MZR ----------------

def mzr_calculate_coeffs(alpha, MH0, logMstar0, sigma, mstars, logAge, MH):
    """calculate_coeffs(PowerLawMZR, GaussianDispersion, ...), mzr.jl:50-79."""
    logAge, MH = _f64(logAge), _f64(MH)
    out = np.empty(logAge.size)
    mstars = _f64(mstars)
    rc = lib().sfho_mzr_calculate_coeffs(alpha, MH0, logMstar0, sigma, mstars, mstars.size,
                                         logAge, MH, logAge.size, out)
    if rc != 0:
        raise ValueError("length(mstars) must equal length(unique(logAge))")
    return out


def mzr_fg(variables, logMstar0, M, n, logAge, MH, free=(True, True, True), want_g=True,
           eps=eps_of(np.float64)):
    """fg!(F, G, PowerLawMZR, GaussianDispersion, variables, ...), mzr.jl:84-215."""
    variables = _f64(variables)
    nages = variables.size - 3
    M = np.asfortranarray(M, dtype=np.float64)
    nb, nt = M.shape
    G = np.empty(variables.size) if want_g else None
    v = lib().sfho_mzr_fg(variables, nages, float(logMstar0), int(free[0]), int(free[1]),
                          int(free[2]), M.ravel(order="F"), _f64(n), nb, nt, _f64(logAge),
                          _f64(MH), eps, G.ctypes.data if want_g else None)
    return v, G


def linear_amr(alpha, beta, T_max, logAge):
    """LinearAMR(α, β, T_max)(logAge), amr.jl:205."""
    return lib().sfho_linear_amr(float(alpha), float(beta), float(T_max), float(logAge))


def mh_from_z(Z):
    """MH_from_Z(Z) with the package defaults, src/utilities.jl:138-145."""
    return lib().sfho_mh_from_z(float(Z))


def dmh_dz(Z):
    """dMH_dZ(Z), src/utilities.jl:152-155."""
    return lib().sfho_dmh_dz(float(Z))


def amr_fg(variables, T_max, M, n, logAge, MH, free=(True, True, True), want_g=True,
           eps=eps_of(np.float64), kind=0):
    """fg!(F, G, AMR, GaussianDispersion, variables, ...), amr.jl:78-160; kind 0 LinearAMR,
    kind 1 LogarithmicAMR (MH_from_Z)."""
    variables = _f64(variables)
    nages = variables.size - 3
    M = np.asfortranarray(M, dtype=np.float64)
    nb, nt = M.shape
    G = np.empty(variables.size) if want_g else None
    v = lib().sfho_amr_fg(int(kind), variables, nages, float(T_max), int(free[0]), int(free[1]),
                          int(free[2]), M.ravel(order="F"), _f64(n), nb, nt, _f64(logAge),
                          _f64(MH), eps, G.ctypes.data if want_g else None)
    return v, G


# ---------------- learned template emulator (no reference counterpart) ----------------

def mlp_param_count(shape):
    return int(lib().sfho_mlp_param_count(*shape))


def mlp_forward(shape, params, X, bf16=True):
    """FP64 MLP forward (GELU hidden layers); bf16 rounds every matmul operand."""
    X = _f64(X)
    B = X.shape[0]
    Y = np.empty((B, shape[3]))
    lib().sfho_mlp_forward(*shape, _f64(params), X.ravel(), B, int(bf16), Y.ravel())
    return Y


def mlp_loss_grad(shape, params, X, T, bf16=True):
    """(MSE loss, gradient w.r.t. the flat parameter block) in FP64."""
    X, T = _f64(X), _f64(T)
    g = np.empty(mlp_param_count(shape))
    loss = lib().sfho_mlp_loss_grad(*shape, _f64(params), X.ravel(), T.ravel(), X.shape[0],
                                    int(bf16), g)
    return loss, g


def poisson_deviance(exact, emul):
    """Poisson deviance per star of emul against exact."""
    e, t = _f64(emul).ravel(), _f64(exact).ravel()
    return lib().sfho_poisson_deviance(t, e, t.size)


# ---------------- many templates at once (a process pool over the single-thread oracle) ----

def _pcs_job(args):
    (m_ini, mags, err, compl, y_index, color_indices, dmod, normalize_value, ex, ey) = args
    imf = kroupa2001()
    return partial_cmd_smooth(m_ini, mags, [ErrModel(*e) for e in err],
                              [ComplModel(*c) for c in compl], y_index, color_indices, imf, dmod,
                              normalize_value, imf_mean(imf), ex, ey)


def partial_cmd_smooth_many(jobs, processes=None):
    """partial_cmd_smooth (StarFormationHistories.jl:829-888) for many isochrones with a
    Kroupa2001(0.08, 100) IMF, in a pool of processes started with ``spawn`` (safe after the
    caller has used a GPU).  ``jobs``: tuples (m_ini, mags, err (a, b, c, d, cap) tuples,
    completeness (A, m50, rho) tuples, y_index, color_indices, dmod, normalize_value,
    (x first, step, n), (y first, step, n)).  Returns the (nx, ny) arrays in job order."""
    import multiprocessing as mp
    jobs = list(jobs)
    processes = processes or min(len(jobs), os.cpu_count() or 1)
    if processes <= 1:
        return [_pcs_job(j) for j in jobs]
    with mp.get_context("spawn").Pool(processes) as pool:
        return pool.map(_pcs_job, jobs, chunksize=1)
