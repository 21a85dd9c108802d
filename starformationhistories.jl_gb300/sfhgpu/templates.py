"""Template (Hess diagram) construction over the GPU C ABI.

Mirrors src/StarFormationHistories.jl of StarFormationHistories.jl v1.3.1:
isochrone preprocessing (mini_spacing :110-148, interpolate_mini :77-92,
calculate_weights :765-776, midpoints :417-436, calculate_edges :451-476) runs on
the host with arbitrary Python callables exactly like the reference's Julia
callables; the stamp loop of bin_cmd_smooth (:574-621) runs on the GPU.
`partial_cmd_smooth_batch` runs the whole of partial_cmd_smooth on the GPU for
closed-form error/completeness/IMF models (many templates per call).
"""
from __future__ import annotations

import ctypes as C
import math
from collections import namedtuple
from fractions import Fraction

import numpy as np

from ._lib import ComplModel, ErrModel, IMFParams, check, load
from .core import default_context

Histogram = namedtuple("Histogram", ["edges", "weights"])


# ---------------------------------------------------------------- callables (src/utilities.jl)

def Martin2016_complete(m, A, m50, rho):
    """Martin2016_complete, src/utilities.jl:205."""
    return A / (1.0 + np.exp((np.asarray(m) - m50) / rho))


def exp_photerr(m, a, b, c, d):
    """exp_photerr, src/utilities.jl:218."""
    return a ** (b * (np.asarray(m) - c)) + d


class BrokenPowerLawIMF:
    """Continuous broken power-law IMF normalised on [mmin, mmax]; Kroupa2001 stand-in
    (InitialMassFunctions.jl is a test dependency of the reference, not vendored)."""

    def __init__(self, mmin, mmax, breaks, alphas):
        self.mmin, self.mmax = float(mmin), float(mmax)
        self.breaks = list(breaks)
        self.alphas = list(alphas)
        lo = [self.mmin] + self.breaks
        hi = self.breaks + [self.mmax]
        self.seg = []
        s = 1.0
        for k, a in enumerate(self.alphas):
            if k > 0:
                s *= lo[k] ** (a - self.alphas[k - 1])
            self.seg.append((lo[k], hi[k], s, a))

        def integ(p):
            tot = 0.0
            for lo_, hi_, s_, a_ in self.seg:
                q = -a_ + p + 1.0
                tot += s_ * (np.log(hi_ / lo_) if abs(q) < 1e-14 else (hi_ ** q - lo_ ** q) / q)
            return tot

        self._norm = integ(0)
        self._mean = integ(1) / self._norm

    def pdf(self, m):
        m = np.asarray(m, dtype=np.float64)
        out = np.zeros_like(m)
        for k, (lo, hi, s, a) in enumerate(self.seg):
            last = (k == len(self.seg) - 1)
            sel = (m >= lo) & ((m <= hi) if last else (m < hi))
            out[sel] = s * m[sel] ** (-a) / self._norm
        return out

    __call__ = pdf

    def mean(self):
        return self._mean

    def params(self) -> IMFParams:
        p = IMFParams()
        p.nseg = len(self.alphas)
        p.mmin, p.mmax = self.mmin, self.mmax
        for i, b in enumerate(self.breaks):
            p.breaks[i] = b
        for i, a in enumerate(self.alphas):
            p.alpha[i] = a
        return p


def Kroupa2001(mmin=0.08, mmax=100.0):
    """Kroupa (2001) IMF on [mmin, mmax] for mmin >= 0.08: slopes 1.3 below 0.5 Msun, 2.3 above."""
    return BrokenPowerLawIMF(mmin, mmax, [0.5], [1.3, 2.3])


# ---------------------------------------------------------------- isochrone utilities

def mini_spacing(m_ini, colors, mags, dmag, ret_spacing=False):
    """mini_spacing, src/StarFormationHistories.jl:110-148."""
    m_ini, colors, mags = (np.asarray(a, dtype=np.float64) for a in (m_ini, colors, mags))
    if not (m_ini.shape == colors.shape == mags.shape):
        raise ValueError("axes(m_ini) == axes(mags) == axes(colors)")
    first = m_ini[0]
    idx = np.argsort(m_ini, kind="stable")
    m, mg, co = m_ini[idx], mags[idx], colors[idx]
    d = np.hypot(np.diff(co), np.diff(mg))
    out = [np.array([first])]
    for i in range(len(m) - 1):
        if d[i] > dmag:
            n = int(np.ceil(d[i] / dmag))
            step = (m[i + 1] - m[i]) / n
            out.append(m[i] + step * np.arange(1, n + 1, dtype=np.float64))
        else:
            out.append(np.array([m[i + 1]]))
    allv = np.concatenate(out)
    _, first_idx = np.unique(allv, return_index=True)
    new = allv[np.sort(first_idx)]
    return (new, np.diff(new)) if ret_spacing else new


def _dedup_knots(k):
    k = k.copy()
    last = k[0]
    for i in range(1, len(k)):
        if k[i] == last:
            k[i] = np.nextafter(k[i - 1], np.inf)
        else:
            last = k[i]
    return k


def interpolate_mini(m_ini, mags, new_mini):
    """interpolate_mini, src/StarFormationHistories.jl:77-81 (sort_ingested,
    src/simulate.jl:54-63, then linear interpolation on the knots)."""
    m_ini = np.asarray(m_ini, dtype=np.float64)
    mags = np.asarray(mags, dtype=np.float64)
    idx = np.argsort(m_ini, kind="stable")
    k = _dedup_knots(m_ini[idx])
    v = mags[idx]
    x = np.asarray(new_mini, dtype=np.float64)
    j = np.clip(np.searchsorted(k, x, side="right") - 1, 0, len(k) - 2)
    t = (x - k[j]) / (k[j + 1] - k[j])
    out = v[j] * (1.0 - t) + v[j + 1] * t
    out = np.where(x <= k[0], v[0], out)
    return np.where(x >= k[-1], v[-1], out)


def midpoints(v):
    """midpoints(v), src/StarFormationHistories.jl:417-436 (element form)."""
    v = np.asarray(v, dtype=np.float64)
    return v[:-1] + np.diff(v) / 2.0


def calculate_weights(mini, completeness, imf, normalize_value, mean_mass, spacing=None):
    """calculate_weights, src/StarFormationHistories.jl:765-776."""
    mini = np.asarray(mini, dtype=np.float64)
    sp = np.diff(mini) if spacing is None else np.asarray(spacing)
    p = np.asarray(imf(mini), dtype=np.float64)
    w = sp * (p[:-1] + p[1:]) / 2.0
    return w * np.asarray(completeness)[:-1] * normalize_value / mean_mass


def histogram_pix(d, edges):
    """histogram_pix(d, edges::AbstractRange), src/StarFormationHistories.jl:502."""
    f, s, _ = _range(edges)
    return (np.asarray(d) - f) / s + 1.0


def histogram_data(x, edges):
    """histogram_data(x, edges::AbstractRange), src/StarFormationHistories.jl:518."""
    f, s, _ = _range(edges)
    return (np.asarray(x) - 1.0) * s + f


class Range(np.ndarray):
    """Edge vector built like a Julia float range: the element values of
    range(start, stop, length=n) or start:step:stop, with `step` the value Julia's
    step(r) returns.  Slices and arithmetic give plain arrays."""

    def __new__(cls, values, step):
        obj = np.asarray(values, dtype=np.float64).view(cls)
        obj.step = float(step)
        return obj

    def __array_finalize__(self, obj):
        self.step = None


_MAXINT_F32 = 16777216      # maxintfloat(Float32)
_MAXINT_F64 = 9007199254740992


def _rat(x):
    """Base.rat (twiceprecision.jl): the continued-fraction convergent a/b of x with
    Float64(a) / Float64(b) == x, or the last one with |a|, |b| <= 2^24."""
    y = x
    a = d = 1
    b = c = 0
    while abs(y) <= _MAXINT_F32:
        f = math.trunc(y)
        y -= f
        a, c = f * a + c, a
        b, d = f * b + d, b
        if max(abs(a), abs(b)) > _MAXINT_F32:
            return c, d
        if float(a) / float(b) == x:
            break
        y = math.inf if y == 0 else 1.0 / y
    return a, b


def _tdiv(p, q):
    """Julia div on integers (truncates toward zero)."""
    r = abs(p) // abs(q)
    return r if (p >= 0) == (q >= 0) else -r


def julia_range(start, stop, length):
    """The elements of Julia's range(start, stop; length) for Float64 (base/twiceprecision.jl,
    range_start_stop_length): when start and stop are ratios of small integers the elements
    are the correctly rounded values of the exact rational interpolation (so
    range(17.0, 27.0, length=101) holds 17.3, not 17 + 3 * 0.1), otherwise of the exact
    interpolation of the two doubles.  Julia evaluates these in twice precision; the two
    agree except when an exact value lies within ~1e-32 relative of a rounding boundary."""
    start, stop, n = float(start), float(stop), int(length)
    if n < 2:
        raise ValueError("an edge range needs length >= 2")
    if not (math.isfinite(start) and math.isfinite(stop)):
        raise ValueError("range endpoints must be finite")
    if start == stop:
        return Range(np.full(n, start), 0.0)
    lo, hi = Fraction(start), Fraction(stop)
    sn, sd = _rat(start)
    en, ed = _rat(stop)
    if sd != 0 and ed != 0:
        den = math.lcm(abs(sd), abs(ed))
        if den != 0 and abs(den * start) <= _MAXINT_F64 and abs(den * stop) <= _MAXINT_F64:
            sn, en = round(den * start), round(den * stop)
            if sn / den == start and en / den == stop:
                lo, hi = Fraction(sn, den), Fraction(en, den)
    vals = [float(lo + (hi - lo) * i / (n - 1)) for i in range(n)]
    vals[0], vals[-1] = start, stop
    return Range(vals, float((hi - lo) / (n - 1)))


def julia_colon(start, step, stop):
    """The elements of Julia's start:step:stop for Float64 (base/twiceprecision.jl, the
    IEEEFloat colon method): exact rational arithmetic when start, step and stop are ratios
    of small integers (so -1.0:0.1:1.5 holds 0.3 exactly), else start + k * step taken
    literally, with the length rounded as Julia rounds it."""
    start, step, stop = float(start), float(step), float(stop)
    if step == 0:
        raise ValueError("range step cannot be zero")
    pn, pd = _rat(step)
    if pd != 0 and pn / pd == step:
        sn, sd = _rat(start)
        en, ed = _rat(stop)
        if sd != 0 and ed != 0 and sn / sd == start and en / ed == stop:
            den = math.lcm(abs(sd), abs(pd))
            if (den != 0 and abs(start * den) <= _MAXINT_F64 and abs(step * den) <= _MAXINT_F64
                    and den % abs(sd) == 0 and den % abs(pd) == 0):
                sn, pn = round(start * den), round(step * den)
                ln = max(0, _tdiv(den * en - ed * sn + pn * ed, pn * ed))

                def between(a, x, b):
                    return a <= x <= b or b <= x <= a
                if (between(start, start + (ln - 1) * step, stop + step / 2) and
                        not between(start, start + ln * step, stop)):
                    vals = [float(Fraction(sn + k * pn, den)) for k in range(ln)]
                    return Range(vals, float(Fraction(pn, den)))
    lf = (stop - start) / step
    if lf < 0:
        ln = 0
    elif lf == 0:
        ln = 1
    else:
        ln = round(lf) + 1
        stop2 = start + (ln - 1) * step
        ln -= int(start < stop < stop2) + int(start > stop > stop2)
    s0, st = Fraction(start), Fraction(step)
    return Range([float(s0 + k * st) for k in range(ln)], step)


def _range(e):
    """(first, step, number of bins) of an evenly spaced edge vector; `step` as Julia's
    step(r) when e is a Range."""
    jstep = getattr(e, "step", None)
    e = np.asarray(e, dtype=np.float64)
    if e.ndim != 1 or e.size < 2:
        raise ValueError("edges must be evenly spaced vectors of length >= 2")
    step = (e[-1] - e[0]) / (e.size - 1)
    if not np.allclose(np.diff(e), step, rtol=1e-9, atol=0.0):
        raise ValueError("edges must be AbstractRange-like (evenly spaced)")
    if jstep is not None and jstep != 0.0:
        step = jstep
    return float(e[0]), float(step), int(e.size - 1)


def _edge_values(e):
    """The element values of an increasing edge vector (hard binning compares against them)."""
    v = np.ascontiguousarray(e, dtype=np.float64)
    if v.ndim != 1 or v.size < 2:
        raise ValueError("edges must be vectors of length >= 2")
    if not (np.all(np.isfinite(v)) and np.all(np.diff(v) > 0)):
        raise ValueError("edges must be finite and increasing")
    return v


def calculate_edges(edges=None, xlim=None, ylim=None, nbins=None, xwidth=None, ywidth=None):
    """calculate_edges, src/StarFormationHistories.jl:451-476: `edges` as given, else
    Julia ranges range(lim[1], lim[2], length=nbins) (julia_range) over the sorted limits."""
    if edges is not None:
        return tuple(e if isinstance(e, Range) else np.asarray(e, dtype=np.float64)
                     for e in edges)
    xlim, ylim = sorted(xlim), sorted(ylim)
    if nbins is None:
        if xwidth is None or ywidth is None:
            raise ValueError("If edges and nbins are not provided, xwidth and ywidth must be.")
        nbins = (int(round((xlim[1] - xlim[0]) / xwidth)), int(round((ylim[1] - ylim[0]) / ywidth)))
    return (julia_range(xlim[0], xlim[1], nbins[0]), julia_range(ylim[0], ylim[1], nbins[1]))


# ---------------------------------------------------------------- GPU template builders

def bin_cmd_smooth(colors, mags, color_err, mag_err, cov_mult=0, weights=None, edges=None,
                   xlim=None, ylim=None, nbins=None, xwidth=None, ywidth=None, ctx=None):
    """bin_cmd_smooth, src/StarFormationHistories.jl:574-621, stamps on the GPU.
    Returns Histogram(edges, weights) with weights (nx, ny) float64."""
    if cov_mult not in (-1, 0, 1):
        raise ValueError("cov_mult in (-1, 0, 1)")
    x, y, sx, sy = (np.ascontiguousarray(a, dtype=np.float64) for a in
                    (colors, mags, color_err, mag_err))
    w = np.ones_like(x) if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    if not (x.shape == y.shape == sx.shape == sy.shape == w.shape):
        raise ValueError("axes(colors) == axes(mags) == axes(color_err) == axes(mag_err) == axes(weights)")
    if edges is None:
        xlim = (x.min(), x.max()) if xlim is None else xlim
        ylim = (y.min(), y.max()) if ylim is None else ylim
    e = calculate_edges(edges, xlim, ylim, nbins, xwidth, ywidth)
    (xf, xs, nx), (yf, ys, ny) = _range(e[0]), _range(e[1])
    ctx = ctx or default_context()
    out = np.empty(nx * ny)
    check(load().sfh_bin_cmd_smooth(ctx.handle, x.ctypes.data, y.ctypes.data, sx.ctypes.data,
                                    sy.ctypes.data, w.ctypes.data, x.size, int(cov_mult), xf, xs,
                                    nx, yf, ys, ny, out.ctypes.data), ctx.handle, "bin_cmd_smooth")
    return Histogram(e, out.reshape(ny, nx).T)


def bin_cmd(colors, mags, weights=None, edges=None, xlim=None, ylim=None, nbins=None,
            xwidth=None, ywidth=None, ctx=None):
    """bin_cmd, src/StarFormationHistories.jl:544-553: the hard-binned Hess diagram
    fit(Histogram, (colors, mags), Weights(weights), edges; closed=:left) on the GPU.  Bin
    (i, j) holds xedges[i] <= color < xedges[i+1] and yedges[j] <= mag < yedges[j+1] against
    the edge values themselves; points on the last edge are dropped.  xlim / ylim default to
    the extrema of colors / mags.  Returns Histogram(edges, weights (nx, ny) float64)."""
    x = np.ascontiguousarray(colors, dtype=np.float64)
    y = np.ascontiguousarray(mags, dtype=np.float64)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    if not (x.ndim == y.ndim == 1 and x.shape == y.shape and (w is None or w.shape == x.shape)):
        raise ValueError("length(colors) == length(mags) == length(weights)")
    if edges is None:
        xlim = (x.min(), x.max()) if xlim is None else xlim
        ylim = (y.min(), y.max()) if ylim is None else ylim
    e = calculate_edges(edges, xlim, ylim, nbins, xwidth, ywidth)
    ex, ey = _edge_values(e[0]), _edge_values(e[1])
    nx, ny = ex.size - 1, ey.size - 1
    ctx = ctx or default_context()
    out = np.empty(nx * ny)
    check(load().sfh_bin_cmd(ctx.handle, x.ctypes.data, y.ctypes.data,
                             None if w is None else w.ctypes.data, x.size, ex.ctypes.data, nx,
                             ey.ctypes.data, ny, out.ctypes.data), ctx.handle, "bin_cmd")
    return Histogram(e, out.reshape(ny, nx).T)


def partial_cmd_points(m_ini, colors, mags, imf, dmod=0.0, normalize_value=1.0,
                       mean_mass=None):
    """The weighted points partial_cmd bins (src/StarFormationHistories.jl:733-757): the
    isochrone resampled by mini_spacing (Δmag 0.01), interpolated, magnitudes shifted by dmod,
    trapezoidal IMF weights times normalize_value / mean_mass, the last point dropped."""
    if mean_mass is None:
        mean_mass = imf.mean()
    new_mini, spacing = mini_spacing(m_ini, colors, mags, 0.01, True)
    c = interpolate_mini(m_ini, colors, new_mini)
    m = interpolate_mini(m_ini, mags, new_mini) + dmod
    p = np.asarray(imf(new_mini), dtype=np.float64)
    w = spacing * (p[:-1] + p[1:]) / 2.0
    w = w * (normalize_value / mean_mass)
    return c[:-1], m[:-1], w


def partial_cmd(m_ini, colors, mags, imf, dmod=0.0, normalize_value=1.0, mean_mass=None,
                edges=None, xlim=None, ylim=None, nbins=None, xwidth=None, ywidth=None, ctx=None):
    """partial_cmd, src/StarFormationHistories.jl:733-757: the error-free Hess diagram of an
    isochrone (no photometric smoothing), binned on the GPU.  As in the reference, xlim and
    ylim default to the extrema of the given colors and (unshifted) mags."""
    colors = np.asarray(colors, dtype=np.float64)
    mags = np.asarray(mags, dtype=np.float64)
    if edges is None:
        xlim = (colors.min(), colors.max()) if xlim is None else xlim
        ylim = (mags.min(), mags.max()) if ylim is None else ylim
    x, y, w = partial_cmd_points(m_ini, colors, mags, imf, dmod, normalize_value, mean_mass)
    return bin_cmd(x, y, weights=w, edges=edges, xlim=xlim, ylim=ylim, nbins=nbins,
                   xwidth=xwidth, ywidth=ywidth, ctx=ctx)


def model_cmd(mags, errfuncs, completefuncs, biasfuncs=None, seed=0, ret_idxs=False,
              ctx=None):
    """model_cmd, src/simulate.jl:621-680: mock observation of a catalogue of stellar
    magnitudes.  mags is (nstars, nfilters) (a star's magnitudes in a row, as the
    reference's vector of per-star vectors); errfuncs / completefuncs / biasfuncs are
    per-filter callables on arrays, evaluated here at the input magnitudes as the reference
    evaluates them.  A star is kept when a uniform draw is <= the product of its
    completeness values; kept stars get Gaussian errors and the bias.  The draws (GPU,
    Philox keyed by `seed`) follow the reference's distributions, not its RNG stream.
    Returns the kept magnitudes (input order) and, with ret_idxs, their 0-based indices."""
    m = np.ascontiguousarray(mags, dtype=np.float64)
    if m.ndim != 2:
        raise ValueError("mags must be (nstars, nfilters)")
    n, nf = m.shape
    if not (nf == len(errfuncs) == len(completefuncs)):
        raise ValueError("length(first(mags)) == length(errfuncs) == length(completefuncs)")
    if biasfuncs is not None and len(biasfuncs) != nf:
        raise ValueError("length(biasfuncs) == length(first(mags))")
    if nf > 8:
        raise ValueError("at most 8 filters")
    sigma = np.ascontiguousarray(np.stack(
        [np.broadcast_to(np.asarray(errfuncs[j](m[:, j]), dtype=np.float64), (n,))
         for j in range(nf)], axis=1)) if n else np.empty((0, nf))
    compl = np.ones(n)
    for j in range(nf):
        compl *= np.asarray(completefuncs[j](m[:, j]), dtype=np.float64)
    bias = None
    if biasfuncs is not None and n:
        bias = np.ascontiguousarray(np.stack(
            [np.broadcast_to(np.asarray(biasfuncs[j](m[:, j]), dtype=np.float64), (n,))
             for j in range(nf)], axis=1))
    out = np.empty((n, nf))
    idx = np.empty(n, dtype=np.int64)
    nout = C.c_int64()
    ctx = ctx or default_context()
    check(load().sfh_model_cmd(ctx.handle, m.ctypes.data, sigma.ctypes.data,
                               None if bias is None else bias.ctypes.data, compl.ctypes.data, n,
                               nf, int(seed) & 0xFFFFFFFFFFFFFFFF, out.ctypes.data,
                               idx.ctypes.data, C.byref(nout)), ctx.handle, "model_cmd")
    k = nout.value
    return (out[:k], idx[:k]) if ret_idxs else out[:k]


def partial_cmd_smooth_stars(m_ini, mags, mag_err_funcs, y_index, color_indices, imf,
                             completeness_funcs=None, bias_funcs=None, dmod=0.0,
                             normalize_value=1.0, mean_mass=None, edges=None, xlim=None,
                             ylim=None, nbins=None, xwidth=None, ywidth=None):
    """The star list partial_cmd_smooth hands to bin_cmd_smooth
    (src/StarFormationHistories.jl:829-888): (colors, mags, color_err, mag_err, weights,
    cov_mult, edges) after mini_spacing, interpolation, the callables, the weights, the
    bias and midpoints.  y_index / color_indices are 0-based; callables act on arrays."""
    if len(color_indices) != 2:
        raise ValueError("length(color_indices) == 2")
    nf = len(mags)
    completeness_funcs = completeness_funcs or [lambda m: np.ones_like(m)] * nf
    bias_funcs = bias_funcs or [lambda m: np.zeros_like(m)] * nf
    if not (nf == len(mag_err_funcs) == len(completeness_funcs) == len(bias_funcs)):
        raise ValueError("length(mags) == length(mag_err_funcs) == length(completeness_funcs) == length(bias_funcs)")
    if mean_mass is None:
        mean_mass = imf.mean()
    e = calculate_edges(edges, xlim, ylim, nbins, xwidth, ywidth)
    (xf, xs, nx), (yf, ys, ny) = _range(e[0]), _range(e[1])
    c1, c2 = color_indices
    mags = [np.asarray(m, dtype=np.float64) for m in mags]
    colors = mags[c1] - mags[c2]
    dmag = min(abs(xs), abs(ys))
    new_mini, spacing = mini_spacing(m_ini, colors, mags[y_index], dmag, True)
    iso = [interpolate_mini(m_ini, m, new_mini) + dmod for m in mags]
    err = [np.asarray(mag_err_funcs[i](iso[i]), dtype=np.float64) for i in range(nf)]
    if y_index in (c1, c2):
        xc = c1 if c2 == y_index else c2
        color_err = err[xc]
        compl = completeness_funcs[c1](iso[c1]) * completeness_funcs[c2](iso[c2])
        cov_mult = -1 if y_index == c1 else 1
    else:
        color_err = np.sqrt(err[c1] ** 2 + err[c2] ** 2)
        compl = (completeness_funcs[c1](iso[c1]) * completeness_funcs[c2](iso[c2]) *
                 completeness_funcs[y_index](iso[y_index]))
        cov_mult = 0
    w = calculate_weights(new_mini, compl, imf, normalize_value, mean_mass, spacing)
    biased = [iso[i] + bias_funcs[i](iso[i]) for i in range(nf)]
    col = biased[c1] - biased[c2]
    return (midpoints(col), midpoints(biased[y_index]), midpoints(color_err),
            midpoints(err[y_index]), w, cov_mult, e)


def partial_cmd_smooth(m_ini, mags, mag_err_funcs, y_index, color_indices, imf,
                       completeness_funcs=None, bias_funcs=None, dmod=0.0, normalize_value=1.0,
                       mean_mass=None, edges=None, xlim=None, ylim=None, nbins=None, xwidth=None,
                       ywidth=None, ctx=None):
    """partial_cmd_smooth (single stars), src/StarFormationHistories.jl:829-888.
    y_index / color_indices are 0-based.  Callables act on numpy arrays."""
    x, y, sx, sy, w, cov_mult, e = partial_cmd_smooth_stars(
        m_ini, mags, mag_err_funcs, y_index, color_indices, imf, completeness_funcs, bias_funcs,
        dmod, normalize_value, mean_mass, edges, xlim, ylim, nbins, xwidth, ywidth)
    return bin_cmd_smooth(x, y, sx, sy, cov_mult, weights=w, edges=e, ctx=ctx)


def stamp_bin_updates(x, y, sx, sy, cov_mult, edges):
    """Bins each star's stamp adds to: the window of GaussianPSFAsymmetric
    (size (ceil 10σx, ceil 10σy) in pixels, offsets max(1, size ÷ 2),
    StarFormationHistories.jl:247, 348-364) or GaussianPSFCovariant (half widths
    max(1, round(15σx/Δx/2)), max(1, round(10σy/Δy/2)), :293, 366-408) around the
    ties-to-even rounded centre, clipped to the grid; stars whose clipped window is not
    longer than one bin on both axes add nothing.  The unit of the template build's work."""
    (xf, xs, nx), (yf, ys, ny) = _range(edges[0]), _range(edges[1])
    x, y, sx, sy = (np.asarray(a, dtype=np.float64) for a in (x, y, sx, sy))
    xc = np.rint((x - xf) / xs + 1.0)
    yc = np.rint((y - yf) / ys + 1.0)
    if cov_mult == 0:
        xoff = np.maximum(1, np.floor(np.ceil(10.0 * sx / xs) / 2))
        yoff = np.maximum(1, np.floor(np.ceil(10.0 * sy / ys) / 2))
    else:
        xoff = np.maximum(1, np.rint(15.0 * sx / xs / 2.0))
        yoff = np.maximum(1, np.rint(10.0 * sy / ys / 2.0))
    lx = np.minimum(nx, xc + xoff) - np.maximum(1, xc - xoff) + 1
    ly = np.minimum(ny, yc + yoff) - np.maximum(1, yc - yoff) + 1
    return np.where((lx > 1) & (ly > 1), lx * ly, 0).astype(np.int64)


def err_model(a, b, c, d, cap=np.inf) -> ErrModel:
    """Closed-form exp_photerr(m, a, b, c, d) capped at cap."""
    return ErrModel(a, b, c, d, cap)


def compl_model(A, m50, rho) -> ComplModel:
    """Closed-form Martin2016_complete(m, A, m50, rho)."""
    return ComplModel(A, m50, rho)


def partial_cmd_smooth_batch(m_ini, mags, iso_off, iso_len, y_index, color_indices, err_models,
                             compl_models, imf, dmod, normalize_value, edges, mean_mass=None,
                             bias=None, out=None, ctx=None):
    """Many partial_cmd_smooth calls in one device call (sfh_partial_cmd_smooth_batch_dev).

    m_ini, mags: torch CUDA float64 tensors; mags is (nf, total) with the isochrones of
    all templates concatenated; iso_off / iso_len (numpy int64 / int32) locate template
    t.  dmod and normalize_value are scalars or per-template arrays.  Returns (or fills)
    a CUDA float32 tensor of shape (ntempl, nx*ny): template t's column-major Hess
    diagram is row t (i.e. the (nbins, ntempl) column-major template matrix)."""
    import torch
    ctx = ctx or default_context()
    nf, total = mags.shape
    iso_off = np.ascontiguousarray(iso_off, dtype=np.int64)
    iso_len = np.ascontiguousarray(iso_len, dtype=np.int32)
    nt = iso_off.size
    dm = np.ascontiguousarray(np.broadcast_to(np.asarray(dmod, dtype=np.float64), (nt,)))
    nm = np.ascontiguousarray(np.broadcast_to(np.asarray(normalize_value, dtype=np.float64), (nt,)))
    (xf, xs, nx), (yf, ys, ny) = _range(edges[0]), _range(edges[1])
    if out is None:
        out = torch.empty((nt, nx * ny), dtype=torch.float32, device=m_ini.device)
    E = (ErrModel * nf)(*err_models)
    Cm = (ComplModel * nf)(*compl_models)
    b = None
    if bias is not None:
        barr = np.ascontiguousarray(bias, dtype=np.float64)
        b = barr.ctypes.data
    ip = imf.params()
    mm = imf.mean() if mean_mass is None else float(mean_mass)
    m_ini = m_ini.contiguous()
    mags = mags.contiguous()
    # Inputs were produced on torch's stream; the library runs on the context stream.
    torch.cuda.current_stream(m_ini.device).synchronize()
    check(load().sfh_partial_cmd_smooth_batch_dev(
        ctx.handle, m_ini.data_ptr(), mags.data_ptr(), int(total), iso_off.ctypes.data,
        iso_len.ctypes.data, nt, nf, int(y_index), int(color_indices[0]), int(color_indices[1]),
        E, Cm, b, C.byref(ip), mm, dm.ctypes.data, nm.ctypes.data, xf, xs, nx, yf, ys, ny,
        out.data_ptr()), ctx.handle, "partial_cmd_smooth_batch")
    return out


# ---------------------------------------------------------------- binary models (src/simulate.jl)

class NoBinaries:
    """NoBinaries(), src/simulate.jl:153-157: no binary systems."""

    def binary_system_fraction(self):
        return 0.0

    def binary_number_fraction(self):
        return 0.0

    def binary_mass_fraction(self, imf=None):
        return 0.0


class RandomBinaryPairs:
    """RandomBinaryPairs(fraction), src/simulate.jl:159-190: a fraction of stellar systems
    are pairs of stars drawn from the single-star IMF."""

    def __init__(self, fraction):
        if not (0.0 <= fraction <= 1.0):
            raise ValueError("0 <= fraction <= 1")
        self.fraction = fraction

    def binary_system_fraction(self):
        return self.fraction

    def binary_number_fraction(self):
        b = self.fraction  # 2b / (1 + b), simulate.jl:143
        return 2 * b / (1 + b)

    def binary_mass_fraction(self, imf=None):
        return self.binary_number_fraction()  # simulate.jl:190


def trapz(x, y):
    """Trapz.jl trapz(x, y): the trapezoidal rule."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    return float(np.sum(np.diff(x) * (y[1:] + y[:-1]) / 2.0))


def binary_points(m_ini, mags, y_index, color_indices, dmod, edges, ds=4):
    """The isochrone points partial_cmd_smooth hands to binary_hess
    (src/StarFormationHistories.jl:848-855, 895-897): mini_spacing on the bin step,
    interpolation of every filter plus the distance modulus, every ds-th point; and the
    resampled masses (for the mixing fraction).  Returns (m_ds, mags_ds (nf, n_ds), new_mini)."""
    (xf, xs, nx), (yf, ys, ny) = _range(edges[0]), _range(edges[1])
    c1, c2 = color_indices
    mags = [np.asarray(m, dtype=np.float64) for m in mags]
    colors = mags[c1] - mags[c2]
    new_mini = mini_spacing(m_ini, colors, mags[y_index], min(abs(xs), abs(ys)), False)
    iso = np.stack([interpolate_mini(m_ini, m, new_mini) + dmod for m in mags])
    return new_mini[::ds], np.ascontiguousarray(iso[:, ::ds]), new_mini


def binary_hess_batch(m_ini, mags, iso_off, iso_len, y_index, color_indices, err_models,
                      compl_models, imf, normalize_value, edges, mean_mass=None, bias=None,
                      out=None, ctx=None):
    """binary_hess(RandomBinaryPairs, ...) for many templates (sfh_binary_hess_batch_dev,
    src/StarFormationHistories.jl:627-706).  m_ini, mags: torch CUDA float64 tensors of the
    (downsampled, distance-shifted) isochrone points, mags (nf, total); iso_off / iso_len
    locate template t.  Returns (or fills) a CUDA float32 tensor (ntempl, nx*ny)."""
    import torch
    ctx = ctx or default_context()
    nf, total = mags.shape
    iso_off = np.ascontiguousarray(iso_off, dtype=np.int64)
    iso_len = np.ascontiguousarray(iso_len, dtype=np.int32)
    nt = iso_off.size
    nm = np.ascontiguousarray(np.broadcast_to(np.asarray(normalize_value, dtype=np.float64), (nt,)))
    (xf, xs, nx), (yf, ys, ny) = _range(edges[0]), _range(edges[1])
    if out is None:
        out = torch.empty((nt, nx * ny), dtype=torch.float32, device=m_ini.device)
    E = (ErrModel * nf)(*err_models)
    Cm = (ComplModel * nf)(*compl_models)
    b = None
    if bias is not None:
        barr = np.ascontiguousarray(bias, dtype=np.float64)
        b = barr.ctypes.data
    ip = imf.params()
    mm = imf.mean() if mean_mass is None else float(mean_mass)
    m_ini = m_ini.contiguous()
    mags = mags.contiguous()
    torch.cuda.current_stream(m_ini.device).synchronize()
    check(load().sfh_binary_hess_batch_dev(
        ctx.handle, m_ini.data_ptr(), mags.data_ptr(), int(total), iso_off.ctypes.data,
        iso_len.ctypes.data, nt, nf, int(y_index), int(color_indices[0]), int(color_indices[1]),
        E, Cm, b, C.byref(ip), mm, nm.ctypes.data, xf, xs, nx, yf, ys, ny, out.data_ptr()),
        ctx.handle, "binary_hess_batch")
    return out


def partial_cmd_smooth_binary_batch(m_ini, mags, iso_off, iso_len, y_index, color_indices,
                                    err_models, compl_models, imf, dmod, normalize_value, edges,
                                    binary_model, mean_mass=None, bias=None, out=None, ctx=None):
    """partial_cmd_smooth with a binary model for many templates
    (src/StarFormationHistories.jl:829-910): the single-star batch on the GPU, then for a
    binary fraction > 0 the binary templates of every fourth resampled isochrone point
    (resampling on the host, pairs and smoothing on the GPU) mixed by the binary mass
    fraction times trapz(new_mini, imf(new_mini)).  Arguments as partial_cmd_smooth_batch."""
    import torch
    ctx = ctx or default_context()
    out = partial_cmd_smooth_batch(m_ini, mags, iso_off, iso_len, y_index, color_indices,
                                   err_models, compl_models, imf, dmod, normalize_value, edges,
                                   mean_mass=mean_mass, bias=bias, out=out, ctx=ctx)
    frac = binary_model.binary_system_fraction()
    if frac == 0:
        return out
    nf = mags.shape[0]
    iso_off = np.asarray(iso_off, dtype=np.int64)
    iso_len = np.asarray(iso_len, dtype=np.int32)
    nt = iso_off.size
    dm = np.broadcast_to(np.asarray(dmod, dtype=np.float64), (nt,))
    hm, hg = m_ini.detach().cpu().numpy(), mags.detach().cpu().numpy()
    md, gd, bmf = [], [], np.empty(nt)
    bnf = binary_model.binary_mass_fraction(imf)
    for t in range(nt):
        o, n = int(iso_off[t]), int(iso_len[t])
        m_ds, g_ds, new_mini = binary_points(hm[o:o + n], [hg[f, o:o + n] for f in range(nf)],
                                             y_index, color_indices, dm[t], edges)
        md.append(m_ds)
        gd.append(g_ds)
        bmf[t] = bnf * trapz(new_mini, imf.pdf(new_mini))
    lens = np.array([m.size for m in md], dtype=np.int32)
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)
    d_m = torch.tensor(np.concatenate(md), device=m_ini.device)
    d_g = torch.tensor(np.ascontiguousarray(np.concatenate(gd, axis=1)), device=m_ini.device)
    binary = binary_hess_batch(d_m, d_g, offs, lens, y_index, color_indices, err_models,
                               compl_models, imf, normalize_value, edges, mean_mass=mean_mass,
                               bias=bias, ctx=ctx)
    bm = np.ascontiguousarray(bmf)
    check(load().sfh_mix_binary_templates_dev(ctx.handle, out.data_ptr(), binary.data_ptr(),
                                              bm.ctypes.data, nt, out.shape[1], out.data_ptr()),
          ctx.handle, "mix_binary_templates")
    return out


class HessGrid(C.Structure):
    """sfh_hess_grid: one template's Hess grid and output offset in a ragged batch."""
    _fields_ = [("x_first", C.c_double), ("x_step", C.c_double), ("nx", C.c_int64),
                ("y_first", C.c_double), ("y_step", C.c_double), ("ny", C.c_int64),
                ("out_offset", C.c_int64)]


def partial_cmd_smooth_ragged(m_ini, mags, iso_off, iso_len, y_index, color_indices, err_models,
                              compl_models, imf, dmod, normalize_value, edges, mean_mass=None,
                              bias=None, out=None, ctx=None):
    """Many partial_cmd_smooth calls with their own Hess grids (ragged galaxies) in one
    device call (sfh_partial_cmd_smooth_ragged_dev).  edges: one (xedges, yedges) pair per
    template.  Returns (packed CUDA float32 tensor, offsets): template t's column-major
    (nx_t, ny_t) histogram is out[offsets[t]:offsets[t+1]]."""
    import torch
    ctx = ctx or default_context()
    nf, total = mags.shape
    iso_off = np.ascontiguousarray(iso_off, dtype=np.int64)
    iso_len = np.ascontiguousarray(iso_len, dtype=np.int32)
    nt = iso_off.size
    if len(edges) != nt:
        raise ValueError("one (xedges, yedges) pair per template is required")
    dm = np.ascontiguousarray(np.broadcast_to(np.asarray(dmod, dtype=np.float64), (nt,)))
    nm = np.ascontiguousarray(np.broadcast_to(np.asarray(normalize_value, dtype=np.float64), (nt,)))
    grids = (HessGrid * nt)()
    offsets = np.zeros(nt + 1, dtype=np.int64)
    for t, (xe, ye) in enumerate(edges):
        (xf, xs, nx), (yf, ys, ny) = _range(xe), _range(ye)
        grids[t] = HessGrid(xf, xs, nx, yf, ys, ny, int(offsets[t]))
        offsets[t + 1] = offsets[t] + nx * ny
    if out is None:
        out = torch.empty(int(offsets[-1]), dtype=torch.float32, device=m_ini.device)
    elif out.numel() < offsets[-1]:
        raise ValueError("out is smaller than the packed histograms")
    E = (ErrModel * nf)(*err_models)
    Cm = (ComplModel * nf)(*compl_models)
    b = None
    if bias is not None:
        barr = np.ascontiguousarray(bias, dtype=np.float64)
        b = barr.ctypes.data
    ip = imf.params()
    mm = imf.mean() if mean_mass is None else float(mean_mass)
    m_ini = m_ini.contiguous()
    mags = mags.contiguous()
    torch.cuda.current_stream(m_ini.device).synchronize()
    check(load().sfh_partial_cmd_smooth_ragged_dev(
        ctx.handle, m_ini.data_ptr(), mags.data_ptr(), int(total), iso_off.ctypes.data,
        iso_len.ctypes.data, nt, nf, int(y_index), int(color_indices[0]), int(color_indices[1]),
        E, Cm, b, C.byref(ip), mm, dm.ctypes.data, nm.ctypes.data, grids, int(out.numel()),
        out.data_ptr()), ctx.handle, "partial_cmd_smooth_ragged")
    return out, offsets
