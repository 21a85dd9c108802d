// templates.cu -- template (Hess diagram) construction on sm_103a.
//
// k_stamps replaces bin_cmd_smooth (src/StarFormationHistories.jl:574-621) and
// the two addstar! methods (:345-408) with their kernels
// GaussianPSFAsymmetric / gaussian_int_general (:191-265) and
// GaussianPSFCovariant / gaussian_psf_covariant (:272-340).  One CTA owns a
// band of TY Hess rows of one template in shared memory (FP32); its warps pull
// stars from a shared counter, skip stars whose window misses the band, and
// scatter the bin-integrated Gaussian into the band with shared-memory atomics.
// The band is flushed to HBM with coalesced stores.  Window sizes, ties-to-even
// centroid rounding and the "both clipped lengths > 1" skip follow the
// reference exactly.  erf differences are formed from erfc of |t| so that bins
// in the tails keep relative accuracy in FP32.
//
// k_iso_stars replaces the single-star part of partial_cmd_smooth (:829-888):
// mini_spacing resampling (:110-148, block-wide prefix scan over segments),
// interpolate_mini (:77-81), exp_photerr / Martin2016 callables
// (src/utilities.jl:205,218), calculate_weights (:765-776), bias and midpoints
// (:417-436), emitting one star record per midpoint.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "sfh_internal.cuh"

namespace {

constexpr int kStampThreads = 256;
constexpr int kWarps = kStampThreads / 32;
constexpr size_t kBandBudget = 110 * 1024;

struct Grid2 {
    double xf, xs, yf, ys;
    int nx, ny;
};

// Signed erfc table entry: |value| = erfc(|t|), sign bit = sign of t.
__device__ __forceinline__ float erfc_signed(float t) { return copysignf(erfcf(fabsf(t)), t); }

// erf(tb) - erf(ta) for ta <= tb from signed erfc entries, without cancellation
// when both edges sit in the same tail.
__device__ __forceinline__ float erf_diff(float ea, float eb) {
    const float a = fabsf(ea), b = fabsf(eb);
    if (!signbit(ea)) return a - b;  // 0 <= ta <= tb
    if (signbit(eb)) return b - a;   // ta <= tb < 0
    return (2.0f - a) - b;           // ta < 0 <= tb
}

// Gauss-Legendre 3-point nodes/weights, src/StarFormationHistories.jl:303-304.
__constant__ float c_glx[3] = {-0.7745966692414834f, 0.0f, 0.7745966692414834f};
__constant__ float c_glw[3] = {0.5555555555555556f, 0.8888888888888888f, 0.5555555555555556f};

// exp(-z^2) with the rounding error of z*z folded back in (z*z = p + e exactly).
__device__ __forceinline__ float exp_negsq(float z) {
    const float p = z * z;
    const float e = fmaf(z, z, -p);
    return expf(-p) * (1.0f - e);
}

// erf(ta + h) - erf(ta) = (2/√π) ∫ exp(-t²) dt over one bin, by 3-point Gauss-Legendre.
// Relative error < 3e-7 whenever h * max(1, |t|) <= 0.3 (checked against 50-digit erfc).
__device__ __forceinline__ float gl3_bin(float ta, float h) {
    const float hh = 0.5f * h, tm = ta + hh, d = 0.7745966692414834f * hh;
    return 1.1283791670955126f * hh *
           (0.5555555555555556f * (exp_negsq(tm - d) + exp_negsq(tm + d)) +
            0.8888888888888888f * exp_negsq(tm));
}

// Integral of the unit Gaussian kernel over one bin, erf(ta + h) - erf(ta): quadrature
// for bins narrow against the local scale (no cancellation), erfc differences otherwise.
__device__ __forceinline__ float gauss_bin(float ta, float h) {
    if (h * fmaxf(1.0f, fabsf(ta + 0.5f * h)) <= 0.3f) return gl3_bin(ta, h);
    return erf_diff(erfc_signed(ta), erfc_signed(ta + h));
}

__device__ __forceinline__ int64_t clamp_cut(double v) { return (int64_t)fmin(v, 4.0e9); }

// ---------------------------------------------------------------- asymmetric star
__device__ void star_asym(float *band, float *bx_buf, float *by_buf, const Grid2 &g, int ty0,
                          int tyn, double x, double y, double sx, double sy, double A, int lane) {
    const double x0 = (x - g.xf) / g.xs + 1.0;  // histogram_pix, :502
    const double y0 = (y - g.yf) / g.ys + 1.0;
    const double ssx = sx / g.xs, ssy = sy / g.ys;
    if (!(ssx >= 0.0 && ssy >= 0.0) || !(fabs(x0) < 4.0e15 && fabs(y0) < 4.0e15)) return;
    // size(GaussianPSFAsymmetric) = (ceil(Int, 10σx), ceil(Int, 10σy)), :247
    const int64_t cx = clamp_cut(ceil(ssx * 10.0)), cy = clamp_cut(ceil(ssy * 10.0));
    const int64_t xc = __double2ll_rn(x0), yc = __double2ll_rn(y0);  // round(Int, ·): ties to even
    const int64_t xoff = max((int64_t)1, cx / 2), yoff = max((int64_t)1, cy / 2);
    const int64_t xlo = max((int64_t)1, xc - xoff), xhi = min((int64_t)g.nx, xc + xoff);
    const int64_t ylo = max((int64_t)1, yc - yoff), yhi = min((int64_t)g.ny, yc + yoff);
    if (!(xhi - xlo + 1 > 1 && yhi - ylo + 1 > 1)) return;  // :359
    const int64_t jlo = max(ylo, (int64_t)ty0 + 1), jhi = min(yhi, (int64_t)(ty0 + tyn));
    if (jlo > jhi) return;
    const int lx = (int)(xhi - xlo + 1), ly = (int)(jhi - jlo + 1);
    // Bin i spans pixel coordinates [i, i+1]: evaluate at i + 1/2 with half width 1/2.
    const float invx = (float)(0.7071067811865476 / ssx);
    const float invy = (float)(0.7071067811865476 / ssy);
    const float dx0 = (float)((double)xlo - x0);
    const float dy0 = (float)((double)jlo - y0);
    for (int m = lane; m < lx; m += 32) bx_buf[m] = gauss_bin((dx0 + (float)m) * invx, invx);
    const float a4 = (float)(A * 0.25);
    for (int m = lane; m < ly; m += 32) by_buf[m] = a4 * gauss_bin((dy0 + (float)m) * invy, invy);
    __syncwarp();
    const int total = lx * ly;
    const float inv_lx = 1.0f / (float)lx;
    float *base = band + (int64_t)(jlo - 1 - ty0) * g.nx + (xlo - 1);
    for (int p = lane; p < total; p += 32) {
        const int jj = (int)(((float)p + 0.5f) * inv_lx);
        const int ii = p - jj * lx;
        atomicAdd(base + (int64_t)jj * g.nx + ii, bx_buf[ii] * by_buf[jj]);
    }
    __syncwarp();
}

// ---------------------------------------------------------------- covariant star
__device__ void star_cov(float *band, float *rowbuf, const Grid2 &g, int ty0, int tyn, double x,
                         double y, double sx, double sy, double A, float cov, int lane) {
    if (!(sx >= 0.0 && sy >= 0.0)) return;
    const double xpix = (x - g.xf) / g.xs + 1.0, ypix = (y - g.yf) / g.ys + 1.0;
    if (!(fabs(xpix) < 4.0e15 && fabs(ypix) < 4.0e15)) return;
    const int64_t xp = __double2ll_rn(xpix), yp = __double2ll_rn(ypix);
    // size(GaussianPSFCovariant) = (15σx, 10σy), :293; half widths, :383-384
    const int64_t xoff = max((int64_t)1, (int64_t)__double2ll_rn(fmin(15.0 * sx / g.xs / 2.0, 4.0e9)));
    const int64_t yoff = max((int64_t)1, (int64_t)__double2ll_rn(fmin(10.0 * sy / g.ys / 2.0, 4.0e9)));
    const int64_t xlo = max((int64_t)1, xp - xoff), xhi = min((int64_t)g.nx, xp + xoff);
    const int64_t ylo = max((int64_t)1, yp - yoff), yhi = min((int64_t)g.ny, yp + yoff);
    const int64_t lx = xhi - xlo + 1, lyw = yhi - ylo + 1;
    if (!(lx > 1 && lyw > 1)) return;  // :401
    const int64_t jlo = max(ylo, (int64_t)ty0 + 1), jhi = min(yhi, (int64_t)(ty0 + tyn));
    if (jlo > jhi) return;
    // Bin centres: range(histogram_data(first + 1/2), histogram_data(last + 1/2); length), :390-393
    const double xr0 = ((double)xlo - 0.5) * g.xs + g.xf, xr1 = ((double)xhi - 0.5) * g.xs + g.xf;
    const double yr0 = ((double)ylo - 0.5) * g.ys + g.yf, yr1 = ((double)yhi - 0.5) * g.ys + g.yf;
    const double xrs = (xr1 - xr0) / (double)(lx - 1), yrs = (yr1 - yr0) / (double)(lyw - 1);
    const double hx = xrs / 2.0, hy = yrs / 2.0;
    const double inv_sx = 0.7071067811865476 / sx;  // 1 / (√2 σx)
    // t of the lower x edge of bin e, before the covariance shift: (xr_e - hx - x0)/(√2σx)
    const float bx = (float)((xr0 - hx - x) * inv_sx);
    const float sxr = (float)(xrs * inv_sx);
    const float dyb = (float)(yr0 - y);   // row-0 centre minus y0
    const float yrsf = (float)yrs, hyf = (float)hy;
    const float inv_sy = (float)(1.0 / sy);
    const float invsxf = (float)inv_sx;
    // prefac = A / 2 / sqrt(2π) / σy (:320) times the scaled GL weights w_k * hy (:325)
    const float pref = (float)(A / 2.0 / 2.5066282746310002 / sy * hy);
    const int nrows = (int)(jhi - jlo + 1);
    const int row_off = (int)(jlo - ylo);  // first band row's index inside the full window
    float *band_row0 = band + (int64_t)(jlo - 1 - ty0) * g.nx + (xlo - 1);
    if (sxr <= 0.05f) {
        // Narrow bins in t: per-row GL weights c_k and shifts s_k in shared memory, then
        // every (row, bin) integrates its three sheared x-intervals by quadrature.
        for (int row = lane; row < nrows; row += 32) {
            const float dyc = dyb + (float)(row_off + row) * yrsf;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float dy = dyc + c_glx[k] * hyf;
                rowbuf[6 * row + k] = pref * c_glw[k] * exp_negsq(0.7071067811865476f * dy * inv_sy);
                rowbuf[6 * row + 3 + k] = cov * dy * invsxf;
            }
        }
        __syncwarp();
        const int total = nrows * (int)lx;
        const float inv_lx = 1.0f / (float)lx;
        for (int p = lane; p < total; p += 32) {
            const int row = (int)(((float)p + 0.5f) * inv_lx);
            const int e = p - row * (int)lx;
            const float tb0 = bx + (float)e * sxr;
            float v = 0.f;
#pragma unroll
            for (int k = 0; k < 3; ++k)
                v = fmaf(rowbuf[6 * row + k], gl3_bin(tb0 + rowbuf[6 * row + 3 + k], sxr), v);
            atomicAdd(band_row0 + (int64_t)row * g.nx + e, v);
        }
        __syncwarp();
        return;
    }
    // Wide bins: erfc at the shared bin edges, neighbours exchanged by shuffles.
    const int E = (int)lx + 1;  // edges per row
    const int W = E <= 32 ? E : 32;
    const int rows_per = 32 / W;
    const int nb = W - 1;  // bins per segment pass
    const int seg = lane / W, pos = lane - (lane / W) * W;
    for (int rb = 0; rb < nrows; rb += rows_per) {
        const int row = rb + seg;
        const bool vrow = (seg < rows_per) && (row < nrows);
        float ck[3] = {0.f, 0.f, 0.f}, sk[3] = {0.f, 0.f, 0.f};
        if (vrow) {
            const float dyc = dyb + (float)(row_off + row) * yrsf;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float dy = dyc + c_glx[k] * hyf;
                ck[k] = pref * c_glw[k] * exp_negsq(0.7071067811865476f * dy * inv_sy);
                sk[k] = cov * dy * invsxf;
            }
        }
        for (int e0 = 0; e0 < (int)lx; e0 += nb) {
            const int e = e0 + pos;
            const bool ve = vrow && (e <= (int)lx);
            float ev[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) ev[k] = ve ? erfc_signed(bx + (float)e * sxr + sk[k]) : 0.f;
            float nx_[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) nx_[k] = __shfl_down_sync(0xffffffffu, ev[k], 1);
            if (ve && pos < W - 1 && e < (int)lx) {
                float v = 0.f;
#pragma unroll
                for (int k = 0; k < 3; ++k) v = fmaf(ck[k], erf_diff(ev[k], nx_[k]), v);
                atomicAdd(band_row0 + (int64_t)row * g.nx + e, v);
            }
        }
    }
}

// ---------------------------------------------------------------- k_stamps
__global__ void __launch_bounds__(kStampThreads)
k_stamps(const double *__restrict__ xs, const double *__restrict__ ys,
         const double *__restrict__ sxs, const double *__restrict__ sys,
         const double *__restrict__ ws, const int64_t *__restrict__ start,
         const int32_t *__restrict__ count, const int32_t *__restrict__ covs, Grid2 g, int TY,
         float *__restrict__ out) {
    extern __shared__ float smem[];
    const int t = blockIdx.y;
    const int ty0 = blockIdx.x * TY;
    const int tyn = min(TY, g.ny - ty0);
    float *band = smem;
    const int bandn = tyn * g.nx;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *wb = smem + (size_t)TY * g.nx + (size_t)warp * (g.nx + 6 * TY);
    __shared__ int s_next;
    for (int k = threadIdx.x; k < bandn; k += blockDim.x) band[k] = 0.f;
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();
    const int64_t s0 = start[t];
    const int n = count[t];
    const int cov = covs[t];
    for (;;) {
        int q = 0;
        if (lane == 0) q = atomicAdd(&s_next, 1);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= n) break;
        const int64_t s = s0 + q;
        if (cov == 0)
            star_asym(band, wb, wb + g.nx, g, ty0, tyn, xs[s], ys[s], sxs[s], sys[s], ws[s], lane);
        else
            star_cov(band, wb, g, ty0, tyn, xs[s], ys[s], sxs[s], sys[s], ws[s], (float)cov, lane);
    }
    __syncthreads();
    float *dst = out + (int64_t)t * ((int64_t)g.nx * g.ny) + (int64_t)ty0 * g.nx;
    for (int k = threadIdx.x; k < bandn; k += blockDim.x) dst[k] = band[k];
}

// One band of one template per CTA from a flattened tile list: templates with their own
// Hess grids (ragged galaxies).  Same star loop and band flush as k_stamps.
struct StampTile {
    int32_t t, ty0, ty;  // template, first row, band height of this template
};

__global__ void __launch_bounds__(kStampThreads)
k_stamps_ragged(const double *__restrict__ xs, const double *__restrict__ ys,
                const double *__restrict__ sxs, const double *__restrict__ sys,
                const double *__restrict__ ws, const int64_t *__restrict__ start,
                const int32_t *__restrict__ count, const int32_t *__restrict__ covs,
                const StampTile *__restrict__ tiles, const Grid2 *__restrict__ grids,
                const int64_t *__restrict__ out_off, float *__restrict__ out) {
    extern __shared__ float smem[];
    const StampTile tile = tiles[blockIdx.x];
    const int t = tile.t;
    const Grid2 g = grids[t];
    const int TY = tile.ty, ty0 = tile.ty0;
    const int tyn = min(TY, g.ny - ty0);
    float *band = smem;
    const int bandn = tyn * g.nx;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *wb = smem + (size_t)TY * g.nx + (size_t)warp * (g.nx + 6 * TY);
    __shared__ int s_next;
    for (int k = threadIdx.x; k < bandn; k += blockDim.x) band[k] = 0.f;
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();
    const int64_t s0 = start[t];
    const int n = count[t];
    const int cov = covs[t];
    for (;;) {
        int q = 0;
        if (lane == 0) q = atomicAdd(&s_next, 1);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= n) break;
        const int64_t s = s0 + q;
        if (cov == 0)
            star_asym(band, wb, wb + g.nx, g, ty0, tyn, xs[s], ys[s], sxs[s], sys[s], ws[s], lane);
        else
            star_cov(band, wb, g, ty0, tyn, xs[s], ys[s], sxs[s], sys[s], ws[s], (float)cov, lane);
    }
    __syncthreads();
    float *dst = out + out_off[t] + (int64_t)ty0 * g.nx;
    for (int k = threadIdx.x; k < bandn; k += blockDim.x) dst[k] = band[k];
}

__global__ void k_offsets_to_counts(const int64_t *__restrict__ off, int64_t n,
                                    int32_t *__restrict__ cnt) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) cnt[t] = (int32_t)(off[t + 1] - off[t]);
}

// ---------------------------------------------------------------- k_iso_stars (partial_cmd_smooth)
constexpr int kIsoThreads = 256;
constexpr int kIsoMaxPts = 4096;  // isochrone points per template held in shared memory

struct IsoParams {
    int nf, y_index, c1, c2, covariant;
    double dmag;
    // exp_photerr per filter: σ = min(exp2(b (m - c) log2 a) + d, cap)
    double eb_log2a[8], ec[8], ed[8], ecap[8];
    // Martin2016 per filter
    double cA[8], cm50[8], crho_inv[8];
    double bias[8];
    // IMF: segment k covers [lo_k, hi_k) with density scale_k m^-alpha_k / norm
    int nseg;
    double imf_lo[4], imf_hi[4], imf_scale[4], imf_alpha[4];
    double imf_inv_norm, inv_mean_mass;
    int64_t total;  // stride between filters in the mags array
};

struct IsoPoint {
    double mass, xcol, ymag, cerr, yerr, compl_;
};

__device__ __forceinline__ double imf_pdf(const IsoParams &P, double m) {
    if (!(m >= P.imf_lo[0] && m <= P.imf_hi[P.nseg - 1])) return 0.0;
    int k = 0;
    while (k < P.nseg - 1 && m >= P.imf_hi[k]) ++k;
    return P.imf_scale[k] * P.imf_inv_norm *
           (double)exp2f((float)(-P.imf_alpha[k] * log2(m)));
}

__device__ __forceinline__ double err_eval(const IsoParams &P, int f, double m) {
    const double s = (double)exp2f((float)(P.eb_log2a[f] * (m - P.ec[f]))) + P.ed[f];
    return s < P.ecap[f] ? s : P.ecap[f];
}

__device__ __forceinline__ double compl_eval(const IsoParams &P, int f, double m) {
    return P.cA[f] / (1.0 + (double)__expf((float)((m - P.cm50[f]) * P.crho_inv[f])));
}

// Resampled point q of the isochrone (mini_spacing + interpolate_mini + callables).
__device__ IsoPoint iso_point(const IsoParams &P, const double *m, const double *mags, int n,
                              const int *pos, const int *cnt, double dmod, int q) {
    int k = 0;
    double mass, frac;
    if (q == 0) {
        mass = m[0];
        frac = 0.0;
    } else {
        // largest k in [0, n-2] with pos[k] <= q
        int lo = 0, hi = n - 2;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (pos[mid] <= q) lo = mid; else hi = mid - 1;
        }
        k = lo;
        const int j = q - pos[k] + 1;
        const int c = cnt[k];
        if (c == 1) {
            mass = m[k + 1];
            frac = 1.0;
        } else {
            mass = m[k] + (m[k + 1] - m[k]) / (double)c * (double)j;
            frac = (mass - m[k]) / (m[k + 1] - m[k]);
        }
    }
    const int kk = (q == 0) ? 0 : k;
    double mag[8];
    int fl[3] = {P.c1, P.c2, P.y_index};
#pragma unroll
    for (int u = 0; u < 3; ++u) {
        const int f = fl[u];
        const double *v = mags + (int64_t)f * P.total;
        const double a = v[kk];
        const double b = (kk + 1 < n) ? v[kk + 1] : a;
        mag[u] = ((q == 0) ? a : a * (1.0 - frac) + b * frac) + dmod;
    }
    IsoPoint p;
    p.mass = mass;
    const double e1 = err_eval(P, P.c1, mag[0]), e2 = err_eval(P, P.c2, mag[1]);
    const double ey = err_eval(P, P.y_index, mag[2]);
    double comp = compl_eval(P, P.c1, mag[0]) * compl_eval(P, P.c2, mag[1]);
    if (P.covariant) {
        p.cerr = (P.y_index == P.c1) ? e2 : e1;  // error of the non-y filter, :862
    } else {
        p.cerr = sqrt(e1 * e1 + e2 * e2);        // :871-872
        comp *= compl_eval(P, P.y_index, mag[2]);
    }
    p.yerr = ey;
    p.compl_ = comp;
    p.xcol = (mag[0] + P.bias[P.c1]) - (mag[1] + P.bias[P.c2]);
    p.ymag = mag[2] + P.bias[P.y_index];
    return p;
}

// Segment insertion counts (:128-137) and their exclusive scan, in shared memory.
// Returns N = 1 + sum(cnt) (number of resampled points); sets *bad when masses
// are not strictly increasing.
__device__ int iso_scan(const IsoParams &P, double dmag, const double *m, const double *mg, int n,
                        int *s_cnt, int *s_pos, int *s_warp, int *bad) {
    const int nseg = n - 1;
    for (int k = threadIdx.x; k < nseg; k += blockDim.x) {
        const double *vc1 = mg + (int64_t)P.c1 * P.total, *vc2 = mg + (int64_t)P.c2 * P.total;
        const double *vy = mg + (int64_t)P.y_index * P.total;
        const double dc = (vc1[k + 1] - vc2[k + 1]) - (vc1[k] - vc2[k]);
        const double dy = vy[k + 1] - vy[k];
        const double d = hypot(dc, dy);
        int c = 1;
        if (d > dmag) {
            const double r = ceil(d / dmag);
            c = r < 1.0e7 ? (int)r : 10000000;
        }
        if (!(m[k + 1] > m[k])) atomicExch(bad, 2);
        s_cnt[k] = c;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int carry = 1;
    for (int base = 0; base < nseg; base += blockDim.x) {
        const int k = base + threadIdx.x;
        const int v = (k < nseg) ? s_cnt[k] : 0;
        int incl = v;
#pragma unroll
        for (int o2 = 1; o2 < 32; o2 <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o2);
            if (lane >= o2) incl += y;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        int wpre = 0, tot = 0;
        for (int w = 0; w < kIsoThreads / 32; ++w) {
            if (w < warp) wpre += s_warp[w];
            tot += s_warp[w];
        }
        if (k < nseg) s_pos[k] = carry + wpre + incl - v;
        carry += tot;
        __syncthreads();
    }
    return carry;
}

__global__ void __launch_bounds__(kIsoThreads)
k_iso_count(const double *__restrict__ m_ini, const double *__restrict__ mags,
            const int64_t *__restrict__ iso_off, const int32_t *__restrict__ iso_len, IsoParams P,
            const double *__restrict__ dmag_t, int64_t *__restrict__ nstars_out,
            int *__restrict__ err_flag) {
    __shared__ int s_cnt[kIsoMaxPts];
    __shared__ int s_pos[kIsoMaxPts];
    __shared__ int s_warp[kIsoThreads / 32];
    const int t = blockIdx.x;
    const int n = iso_len[t];
    const double dmag = dmag_t ? dmag_t[t] : P.dmag;
    const int npts = iso_scan(P, dmag, m_ini + iso_off[t], mags + iso_off[t], n, s_cnt, s_pos,
                              s_warp, err_flag);
    if (threadIdx.x == 0) nstars_out[t] = npts - 1;
}

__global__ void __launch_bounds__(kIsoThreads)
k_iso_stars(const double *__restrict__ m_ini, const double *__restrict__ mags,
            const int64_t *__restrict__ iso_off, const int32_t *__restrict__ iso_len,
            const double *__restrict__ dmods, const double *__restrict__ norms, IsoParams P,
            const double *__restrict__ dmag_t, const int64_t *__restrict__ star_off,
            double *__restrict__ sx_,
            double *__restrict__ sy_, double *__restrict__ ssx, double *__restrict__ ssy,
            double *__restrict__ sw, int32_t *__restrict__ count, int *__restrict__ err_flag) {
    __shared__ int s_cnt[kIsoMaxPts];
    __shared__ int s_pos[kIsoMaxPts];
    __shared__ int s_warp[kIsoThreads / 32];
    const int t = blockIdx.x;
    const int n = iso_len[t];
    const double *m = m_ini + iso_off[t];
    const double *mg = mags + iso_off[t];
    const int npts = iso_scan(P, dmag_t ? dmag_t[t] : P.dmag, m, mg, n, s_cnt, s_pos, s_warp,
                              err_flag);
    const int nstars = npts - 1;
    if (nstars != (int)(star_off[t + 1] - star_off[t])) {  // counts come from k_iso_count
        if (threadIdx.x == 0) { count[t] = 0; atomicExch(err_flag, 1); }
        return;
    }
    if (threadIdx.x == 0) count[t] = nstars;
    const double dmod = dmods[t];
    const double wscale = norms[t] * P.inv_mean_mass;
    const int64_t so = star_off[t];
    // One thread per star: endpoints q and q+1, midpoints and weight, :765-776, :884-888.
    for (int q = threadIdx.x; q < nstars; q += blockDim.x) {
        const IsoPoint a = iso_point(P, m, mg, n, s_pos, s_cnt, dmod, q);
        const IsoPoint b = iso_point(P, m, mg, n, s_pos, s_cnt, dmod, q + 1);
        const double w = (b.mass - a.mass) * (imf_pdf(P, a.mass) + imf_pdf(P, b.mass)) / 2.0 *
                         a.compl_ * wscale;
        sx_[so + q] = a.xcol + (b.xcol - a.xcol) / 2.0;
        sy_[so + q] = a.ymag + (b.ymag - a.ymag) / 2.0;
        ssx[so + q] = a.cerr + (b.cerr - a.cerr) / 2.0;
        ssy[so + q] = a.yerr + (b.yerr - a.yerr) / 2.0;
        sw[so + q] = w;
    }
}

// Shared memory of one k_stamps CTA: the FP32 band (TY x nx) plus per-warp buffers
// (nx + 6 TY floats: the x/y factor tables of the separable kernel, or the per-row
// Gauss-Legendre weights and shifts of the covariant kernel).
size_t stamp_smem(int64_t nx, int64_t TY) {
    return ((size_t)TY * nx + (size_t)kWarps * (nx + 6 * TY)) * sizeof(float);
}

// Band height: as many rows as fit in ~110 KB (two CTAs per SM), balanced over tiles.
int band_rows(int64_t nx, int64_t ny) {
    int64_t tymax = 0;
    while (tymax < ny && stamp_smem(nx, tymax + 1) <= kBandBudget) ++tymax;
    if (tymax < 1) return 0;
    const int64_t ntiles = (ny + tymax - 1) / tymax;
    return (int)((ny + ntiles - 1) / ntiles);
}

}  // namespace

int sfh_launch_stamps(sfh_ctx *ctx, const double *d_x, const double *d_y, const double *d_sx,
                      const double *d_sy, const double *d_w, const int64_t *d_start,
                      const int32_t *d_count, const int32_t *d_cov, int64_t ntempl, double xf,
                      double xs, int64_t nx, double yf, double ys, int64_t ny, float *d_out) {
    if (nx < 1 || ny < 1 || nx > (1 << 20) || ny > (1 << 20) || ntempl < 1 || ntempl > 65535)
        return sfh_set_error(ctx, SFH_ERR_ARG, "stamp grid or template count out of range");
    int TY = band_rows(nx, ny);
    if (TY < 1)
        return sfh_set_error(ctx, SFH_ERR_UNSUPPORTED, "Hess grid too wide for a shared-memory band");
    {
        // few templates: shorter bands, so that the grid holds about four CTAs per SM
        // (each band scans its template's stars and skips those that miss it, so the
        // extra bands cost little next to an idle SM)
        const int64_t want = 4 * (int64_t)ctx->sm_count;
        const int64_t have = ntempl * ((ny + TY - 1) / TY);
        if (have < want) {
            const int64_t tiles = std::min<int64_t>((want + ntempl - 1) / ntempl,
                                                    std::max<int64_t>(1, ny / 8));
            TY = (int)std::min<int64_t>(TY, (ny + tiles - 1) / tiles);
        }
    }
    Grid2 g{xf, xs, yf, ys, (int)nx, (int)ny};
    const int ntiles = (int)((ny + TY - 1) / TY);
    const size_t smem = stamp_smem(nx, TY);
    static thread_local bool attr_set = false;
    if (!attr_set) {
        SFH_CK(ctx, cudaFuncSetAttribute(k_stamps, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024));
        attr_set = true;
    }
    dim3 grid(ntiles, (unsigned)ntempl);
    k_stamps<<<grid, kStampThreads, smem, ctx->stream>>>(d_x, d_y, d_sx, d_sy, d_w, d_start,
                                                         d_count, d_cov, g, TY, d_out);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

extern "C" int sfh_bin_cmd_smooth_batch_dev(sfh_ctx *ctx, const double *d_x, const double *d_y,
                                            const double *d_sx, const double *d_sy,
                                            const double *d_w, const int64_t *d_offsets,
                                            const int32_t *h_cov, int64_t ntempl, double xf,
                                            double xs, int64_t nx, double yf, double ys,
                                            int64_t ny, float *d_models) {
    if (!ctx || !d_x || !d_y || !d_sx || !d_sy || !d_w || !d_offsets || !h_cov || !d_models ||
        ntempl < 1)
        return SFH_ERR_ARG;
    for (int64_t t = 0; t < ntempl; ++t)
        if (h_cov[t] < -1 || h_cov[t] > 1) return sfh_set_error(ctx, SFH_ERR_ARG, "cov_mult must be -1, 0 or 1");
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const size_t o_cnt = 0, o_cov = sfh_align256(ntempl * 4);
    int rc = sfh_scratch_reserve(ctx, o_cov + sfh_align256(ntempl * 4));
    if (rc) return rc;
    int32_t *d_cnt = (int32_t *)((char *)ctx->scratch + o_cnt);
    int32_t *d_cov = (int32_t *)((char *)ctx->scratch + o_cov);
    SFH_CK(ctx, cudaMemcpyAsync(d_cov, h_cov, ntempl * 4, cudaMemcpyHostToDevice, ctx->stream));
    k_offsets_to_counts<<<(int)((ntempl + 255) / 256), 256, 0, ctx->stream>>>(d_offsets, ntempl,
                                                                                d_cnt);
    SFH_LAUNCHED(ctx);
    return sfh_launch_stamps(ctx, d_x, d_y, d_sx, d_sy, d_w, d_offsets, d_cnt, d_cov, ntempl, xf,
                             xs, nx, yf, ys, ny, d_models);
}

extern "C" int sfh_bin_cmd_smooth(sfh_ctx *ctx, const double *x, const double *y,
                                  const double *sx, const double *sy, const double *w,
                                  int64_t npts, int cov_mult, double xf, double xs, int64_t nx,
                                  double yf, double ys, int64_t ny, double *hist_out) {
    if (!ctx || !hist_out || npts < 0 || nx < 1 || ny < 1) return SFH_ERR_ARG;
    if (npts > 0 && (!x || !y || !sx || !sy || !w)) return SFH_ERR_ARG;
    if (cov_mult < -1 || cov_mult > 1)  // @argcheck cov_mult in (-1, 0, 1), :578
        return sfh_set_error(ctx, SFH_ERR_ARG, "cov_mult must be -1, 0 or 1");
    for (int64_t i = 0; i < npts; ++i)
        if (sx[i] < 0.0 || sy[i] < 0.0)
            return sfh_set_error(ctx, SFH_ERR_ARG, "photometric errors must be non-negative");
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const int64_t nbins = nx * ny;
    const size_t a5 = sfh_align256((size_t)(npts > 0 ? npts : 1) * 8);
    const size_t o_out = 5 * a5, o_meta = o_out + sfh_align256(nbins * 4);
    int rc = sfh_stage_reserve(ctx, o_meta + 256);
    if (rc) return rc;
    char *b = (char *)ctx->stage;
    const double *src[5] = {x, y, sx, sy, w};
    for (int k = 0; k < 5 && npts > 0; ++k)
        SFH_CK(ctx, cudaMemcpyAsync(b + k * a5, src[k], npts * 8, cudaMemcpyHostToDevice, ctx->stream));
    struct { int64_t start; int32_t count; int32_t cov; } meta{0, (int32_t)npts, cov_mult};
    SFH_CK(ctx, cudaMemcpyAsync(b + o_meta, &meta, sizeof(meta), cudaMemcpyHostToDevice, ctx->stream));
    float *d_out = (float *)(b + o_out);
    rc = sfh_launch_stamps(ctx, (const double *)b, (const double *)(b + a5),
                           (const double *)(b + 2 * a5), (const double *)(b + 3 * a5),
                           (const double *)(b + 4 * a5), (const int64_t *)(b + o_meta),
                           (const int32_t *)(b + o_meta + 8), (const int32_t *)(b + o_meta + 12),
                           1, xf, xs, nx, yf, ys, ny, d_out);
    if (rc) return rc;
    std::vector<float> tmp((size_t)nbins);
    SFH_CK(ctx, cudaMemcpyAsync(tmp.data(), d_out, nbins * 4, cudaMemcpyDeviceToHost, ctx->stream));
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    for (int64_t i = 0; i < nbins; ++i) hist_out[i] = tmp[(size_t)i];
    return SFH_OK;
}

namespace {
// Validates the filter indices, IMF and callables of partial_cmd_smooth and fills the
// device-side parameter block (everything but the grid-dependent Δmag).
int make_iso_params(sfh_ctx *ctx, int nf, int y_index, int c1, int c2, const sfh_err_model *err,
                    const sfh_compl_model *compl_, const double *bias, const sfh_imf *imf,
                    double mean_mass, int64_t total, IsoParams &P) {
    if (nf < 2 || nf > 8 || y_index < 0 || y_index >= nf || c1 < 0 || c1 >= nf || c2 < 0 ||
        c2 >= nf || c1 == c2)
        return sfh_set_error(ctx, SFH_ERR_ARG, "invalid filter indices");
    if (imf->nseg < 1 || imf->nseg > 4 || !(imf->mmin > 0) || !(imf->mmax > imf->mmin) ||
        !(mean_mass > 0))
        return sfh_set_error(ctx, SFH_ERR_ARG, "invalid IMF");
    P = IsoParams{};
    P.nf = nf;
    P.y_index = y_index;
    P.c1 = c1;
    P.c2 = c2;
    P.covariant = (y_index == c1 || y_index == c2) ? 1 : 0;
    P.total = total;
    for (int f = 0; f < nf; ++f) {
        if (!(err[f].a > 0) || !(compl_[f].rho != 0))
            return sfh_set_error(ctx, SFH_ERR_ARG, "invalid error or completeness model");
        P.eb_log2a[f] = err[f].b * std::log2(err[f].a);
        P.ec[f] = err[f].c;
        P.ed[f] = err[f].d;
        P.ecap[f] = err[f].cap;
        P.cA[f] = compl_[f].A;
        P.cm50[f] = compl_[f].m50;
        P.crho_inv[f] = 1.0 / compl_[f].rho;
        P.bias[f] = bias ? bias[f] : 0.0;
    }
    // IMF segments: continuity at the breaks, normalised on [mmin, mmax].
    P.nseg = imf->nseg;
    double s = 1.0, norm = 0.0;
    for (int k = 0; k < imf->nseg; ++k) {
        const double lo = (k == 0) ? imf->mmin : imf->breaks[k - 1];
        const double hi = (k == imf->nseg - 1) ? imf->mmax : imf->breaks[k];
        if (k > 0) s *= std::pow(lo, imf->alpha[k] - imf->alpha[k - 1]);
        P.imf_lo[k] = lo;
        P.imf_hi[k] = hi;
        P.imf_scale[k] = s;
        P.imf_alpha[k] = imf->alpha[k];
        const double p = 1.0 - imf->alpha[k];
        norm += s * (std::fabs(p) < 1e-14 ? std::log(hi / lo) : (std::pow(hi, p) - std::pow(lo, p)) / p);
    }
    P.imf_inv_norm = 1.0 / norm;
    P.inv_mean_mass = 1.0 / mean_mass;
    return SFH_OK;
}

// Isochrone lengths and offsets inside the concatenated point arrays.
int check_isochrones(sfh_ctx *ctx, const int64_t *h_iso_off, const int32_t *h_iso_len,
                     int64_t ntempl, int64_t total) {
    for (int64_t t = 0; t < ntempl; ++t) {
        const int32_t n = h_iso_len[t];
        if (n < 2 || n > kIsoMaxPts)
            return sfh_set_error(ctx, SFH_ERR_ARG, "isochrone length must be in [2, 4096]");
        if (h_iso_off[t] < 0 || h_iso_off[t] + n > total)
            return sfh_set_error(ctx, SFH_ERR_ARG, "isochrone offsets out of range");
    }
    return SFH_OK;
}
}  // namespace

namespace {
// Host-side description of per-template Hess grids (ragged galaxies).
struct RaggedSpec {
    std::vector<Grid2> grids;
    std::vector<int64_t> out_off;
    std::vector<double> dmag;
    std::vector<StampTile> tiles;
    size_t smem = 0;
};

// The two device passes of partial_cmd_smooth for a batch of isochrones (resampled star
// counts, then star records), followed by the stamps on one shared grid (rg == nullptr)
// or on each template's own grid.
int partial_run(sfh_ctx *ctx, const double *d_m_ini, const double *d_mags,
                const int64_t *h_iso_off, const int32_t *h_iso_len, int64_t ntempl,
                const IsoParams &P, int y_index, int c1, const double *h_dmod,
                const double *h_norm, const RaggedSpec *rg, double xf, double xs, int64_t nx,
                double yf, double ys, int64_t ny, float *d_models) {
    cudaStream_t st = ctx->stream;
    // Pass 1: resampled star count per template (one read-back), exact offsets.
    const size_t o_off = 0, o_len = sfh_align256(ntempl * 8), o_dm = o_len + sfh_align256(ntempl * 4);
    const size_t o_nm = o_dm + sfh_align256(ntempl * 8), o_err = o_nm + sfh_align256(ntempl * 8);
    const size_t o_cnt64 = o_err + 256, o_soff = o_cnt64 + sfh_align256(ntempl * 8);
    const size_t o_cnt = o_soff + sfh_align256((ntempl + 1) * 8), o_cov = o_cnt + sfh_align256(ntempl * 4);
    const size_t o_dmag = o_cov + sfh_align256(ntempl * 4);
    const size_t o_stars = o_dmag + sfh_align256(ntempl * 8);
    const double *d_dmag = nullptr;  // per-template Δmag (ragged grids), set once uploaded
    int rc = sfh_scratch_reserve(ctx, o_stars);
    if (rc) return rc;
    char *b = (char *)ctx->scratch;
    SFH_CK(ctx, cudaMemcpyAsync(b + o_off, h_iso_off, ntempl * 8, cudaMemcpyHostToDevice, st));
    SFH_CK(ctx, cudaMemcpyAsync(b + o_len, h_iso_len, ntempl * 4, cudaMemcpyHostToDevice, st));
    SFH_CK(ctx, cudaMemsetAsync(b + o_err, 0, 4, st));
    if (rg) {
        SFH_CK(ctx, cudaMemcpyAsync(b + o_dmag, rg->dmag.data(), ntempl * 8, cudaMemcpyHostToDevice, st));
        d_dmag = (const double *)(b + o_dmag);
    }
    k_iso_count<<<(unsigned)ntempl, kIsoThreads, 0, st>>>(
        d_m_ini, d_mags, (const int64_t *)(b + o_off), (const int32_t *)(b + o_len), P, d_dmag,
        (int64_t *)(b + o_cnt64), (int *)(b + o_err));
    SFH_LAUNCHED(ctx);
    std::vector<int64_t> nst((size_t)ntempl);
    int flag = 0;
    SFH_CK(ctx, cudaMemcpyAsync(nst.data(), b + o_cnt64, ntempl * 8, cudaMemcpyDeviceToHost, st));
    SFH_CK(ctx, cudaMemcpyAsync(&flag, b + o_err, 4, cudaMemcpyDeviceToHost, st));
    SFH_CK(ctx, cudaStreamSynchronize(st));
    if (flag == 2) return sfh_set_error(ctx, SFH_ERR_ARG, "isochrone masses must be strictly increasing");
    std::vector<int64_t> soff((size_t)ntempl + 1, 0);
    for (int64_t t = 0; t < ntempl; ++t) soff[(size_t)t + 1] = soff[(size_t)t] + nst[(size_t)t];
    const int64_t nstar_total = soff[(size_t)ntempl] > 0 ? soff[(size_t)ntempl] : 1;
    // Pass 2: star records, then the stamps.
    const size_t a8 = sfh_align256((size_t)nstar_total * 8);
    const size_t o_grid = o_stars + 5 * a8;
    const size_t o_oof = o_grid + (rg ? sfh_align256(ntempl * sizeof(Grid2)) : 0);
    const size_t o_tiles = o_oof + (rg ? sfh_align256(ntempl * 8) : 0);
    const size_t o_end = o_tiles + (rg ? sfh_align256(rg->tiles.size() * sizeof(StampTile)) : 0);
    rc = sfh_scratch_reserve(ctx, o_end);
    if (rc) return rc;
    b = (char *)ctx->scratch;  // may have moved
    std::vector<int32_t> cov((size_t)ntempl, P.covariant ? (y_index == c1 ? -1 : 1) : 0);
    SFH_CK(ctx, cudaMemcpyAsync(b + o_off, h_iso_off, ntempl * 8, cudaMemcpyHostToDevice, st));
    SFH_CK(ctx, cudaMemcpyAsync(b + o_len, h_iso_len, ntempl * 4, cudaMemcpyHostToDevice, st));
    SFH_CK(ctx, cudaMemcpyAsync(b + o_dm, h_dmod, ntempl * 8, cudaMemcpyHostToDevice, st));
    SFH_CK(ctx, cudaMemcpyAsync(b + o_nm, h_norm, ntempl * 8, cudaMemcpyHostToDevice, st));
    SFH_CK(ctx, cudaMemcpyAsync(b + o_soff, soff.data(), (ntempl + 1) * 8, cudaMemcpyHostToDevice, st));
    SFH_CK(ctx, cudaMemcpyAsync(b + o_cov, cov.data(), ntempl * 4, cudaMemcpyHostToDevice, st));
    SFH_CK(ctx, cudaMemsetAsync(b + o_err, 0, 4, st));
    if (rg) {
        SFH_CK(ctx, cudaMemcpyAsync(b + o_dmag, rg->dmag.data(), ntempl * 8, cudaMemcpyHostToDevice, st));
        d_dmag = (const double *)(b + o_dmag);
        SFH_CK(ctx, cudaMemcpyAsync(b + o_grid, rg->grids.data(), ntempl * sizeof(Grid2),
                                    cudaMemcpyHostToDevice, st));
        SFH_CK(ctx, cudaMemcpyAsync(b + o_oof, rg->out_off.data(), ntempl * 8, cudaMemcpyHostToDevice, st));
        SFH_CK(ctx, cudaMemcpyAsync(b + o_tiles, rg->tiles.data(), rg->tiles.size() * sizeof(StampTile),
                                    cudaMemcpyHostToDevice, st));
    }
    double *sxp = (double *)(b + o_stars), *syp = (double *)(b + o_stars + a8);
    double *ssxp = (double *)(b + o_stars + 2 * a8), *ssyp = (double *)(b + o_stars + 3 * a8);
    double *swp = (double *)(b + o_stars + 4 * a8);
    k_iso_stars<<<(unsigned)ntempl, kIsoThreads, 0, st>>>(
        d_m_ini, d_mags, (const int64_t *)(b + o_off), (const int32_t *)(b + o_len),
        (const double *)(b + o_dm), (const double *)(b + o_nm), P, d_dmag,
        (const int64_t *)(b + o_soff), sxp, syp, ssxp, ssyp, swp, (int32_t *)(b + o_cnt),
        (int *)(b + o_err));
    SFH_LAUNCHED(ctx);
    if (rg) {
        static thread_local bool attr_set = false;
        if (!attr_set) {
            SFH_CK(ctx, cudaFuncSetAttribute(k_stamps_ragged,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
            attr_set = true;
        }
        k_stamps_ragged<<<(unsigned)rg->tiles.size(), kStampThreads, rg->smem, st>>>(
            sxp, syp, ssxp, ssyp, swp, (const int64_t *)(b + o_soff), (const int32_t *)(b + o_cnt),
            (const int32_t *)(b + o_cov), (const StampTile *)(b + o_tiles),
            (const Grid2 *)(b + o_grid), (const int64_t *)(b + o_oof), d_models);
        SFH_LAUNCHED(ctx);
    } else {
        rc = sfh_launch_stamps(ctx, sxp, syp, ssxp, ssyp, swp, (const int64_t *)(b + o_soff),
                               (const int32_t *)(b + o_cnt), (const int32_t *)(b + o_cov), ntempl,
                               xf, xs, nx, yf, ys, ny, d_models);
        if (rc) return rc;
    }
    SFH_CK(ctx, cudaMemcpyAsync(&flag, b + o_err, 4, cudaMemcpyDeviceToHost, st));
    SFH_CK(ctx, cudaStreamSynchronize(st));
    if (flag) return sfh_set_error(ctx, SFH_ERR_CUDA, "resampled star count changed between passes");
    return SFH_OK;
}
}  // namespace

extern "C" int sfh_partial_cmd_smooth_batch_dev(
    sfh_ctx *ctx, const double *d_m_ini, const double *d_mags, int64_t total,
    const int64_t *h_iso_off, const int32_t *h_iso_len, int64_t ntempl, int nf, int y_index,
    int c1, int c2, const sfh_err_model *err, const sfh_compl_model *compl_, const double *bias,
    const sfh_imf *imf, double mean_mass, const double *h_dmod, const double *h_norm, double xf,
    double xs, int64_t nx, double yf, double ys, int64_t ny, float *d_models) {
    if (!ctx || !d_m_ini || !d_mags || !h_iso_off || !h_iso_len || !err || !compl_ || !imf ||
        !h_dmod || !h_norm || !d_models || ntempl < 1 || ntempl > 65535)
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    IsoParams P;
    int rc0 = make_iso_params(ctx, nf, y_index, c1, c2, err, compl_, bias, imf, mean_mass, total, P);
    if (rc0) return rc0;
    P.dmag = std::fmin(std::fabs(xs), std::fabs(ys));  // :851
    if ((rc0 = check_isochrones(ctx, h_iso_off, h_iso_len, ntempl, total))) return rc0;
    return partial_run(ctx, d_m_ini, d_mags, h_iso_off, h_iso_len, ntempl, P, y_index, c1, h_dmod,
                       h_norm, nullptr, xf, xs, nx, yf, ys, ny, d_models);
}

extern "C" int sfh_partial_cmd_smooth_ragged_dev(
    sfh_ctx *ctx, const double *d_m_ini, const double *d_mags, int64_t total,
    const int64_t *h_iso_off, const int32_t *h_iso_len, int64_t ntempl, int nf, int y_index,
    int c1, int c2, const sfh_err_model *err, const sfh_compl_model *compl_, const double *bias,
    const sfh_imf *imf, double mean_mass, const double *h_dmod, const double *h_norm,
    const sfh_hess_grid *h_grids, int64_t models_len, float *d_models) {
    if (!ctx || !d_m_ini || !d_mags || !h_iso_off || !h_iso_len || !err || !compl_ || !imf ||
        !h_dmod || !h_norm || !h_grids || !d_models || ntempl < 1 || ntempl > (1 << 24) ||
        models_len < 1)
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    IsoParams P;
    int rc0 = make_iso_params(ctx, nf, y_index, c1, c2, err, compl_, bias, imf, mean_mass, total, P);
    if (rc0) return rc0;
    if ((rc0 = check_isochrones(ctx, h_iso_off, h_iso_len, ntempl, total))) return rc0;
    RaggedSpec rg;
    rg.grids.resize((size_t)ntempl);
    rg.out_off.resize((size_t)ntempl);
    rg.dmag.resize((size_t)ntempl);
    for (int64_t t = 0; t < ntempl; ++t) {
        const sfh_hess_grid &h = h_grids[t];
        if (h.nx < 1 || h.ny < 1 || h.nx > (1 << 20) || h.ny > (1 << 20) || !(h.x_step != 0) ||
            !(h.y_step != 0))
            return sfh_set_error(ctx, SFH_ERR_ARG, "Hess grid out of range");
        if (h.out_offset < 0 || h.out_offset + h.nx * h.ny > models_len)
            return sfh_set_error(ctx, SFH_ERR_ARG, "template output outside d_models");
        const int TY = band_rows(h.nx, h.ny);
        if (TY < 1)
            return sfh_set_error(ctx, SFH_ERR_UNSUPPORTED, "Hess grid too wide for a shared-memory band");
        rg.grids[(size_t)t] = Grid2{h.x_first, h.x_step, h.y_first, h.y_step, (int)h.nx, (int)h.ny};
        rg.out_off[(size_t)t] = h.out_offset;
        rg.dmag[(size_t)t] = std::fmin(std::fabs(h.x_step), std::fabs(h.y_step));  // :851
        rg.smem = std::max(rg.smem, stamp_smem(h.nx, TY));
        for (int64_t y0 = 0; y0 < h.ny; y0 += TY)
            rg.tiles.push_back(StampTile{(int32_t)t, (int32_t)y0, (int32_t)TY});
    }
    if (rg.tiles.size() > 0x7fffffffu)
        return sfh_set_error(ctx, SFH_ERR_UNSUPPORTED, "too many stamp tiles");
    P.dmag = rg.dmag[0];
    return partial_run(ctx, d_m_ini, d_mags, h_iso_off, h_iso_len, ntempl, P, y_index, c1, h_dmod,
                       h_norm, &rg, 0.0, 0.0, 0, 0.0, 0.0, 0, d_models);
}

// ---------------------------------------------------------------- binary_hess (RandomBinaryPairs)
// src/StarFormationHistories.jl:627-706 for a batch of templates: every pair (i, j > i) of
// interval left points of a template's (downsampled) isochrone is a binary system whose
// magnitudes add in flux (:656), weighted ΔMp ΔMs (imf_i + imf_i+1)(imf_j + imf_j+1) prefac
// (:660-662) times the colour filters' completeness (:666-668), shifted by the bias
// (:677-678) and binned in a left-closed histogram (:680, FP64 atomics); the nonzero bins
// become points at the bin centres with errors at the centres (:684-697) and are smoothed by
// the bin_cmd_smooth stamps (:702).  One thread per pair.
namespace {

constexpr int kPairThreads = 256;

// prefac[t] = norm[t] / mean_mass / 4 / trapz(m, imf(m)) (:642-643); one block per template,
// fixed-order block sum.
__global__ void __launch_bounds__(kPairThreads)
k_bin_prefac(IsoParams P, const double *__restrict__ m, const int64_t *__restrict__ off,
             const int32_t *__restrict__ len, const double *__restrict__ norm,
             double *__restrict__ prefac) {
    __shared__ double s_red[kPairThreads / 32];
    const int t = blockIdx.x, n = len[t];
    const double *mt = m + off[t];
    double acc = 0.0;
    for (int i = threadIdx.x; i + 1 < n; i += blockDim.x)
        acc += (mt[i + 1] - mt[i]) * (imf_pdf(P, mt[i]) + imf_pdf(P, mt[i + 1])) / 2.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < kPairThreads / 32; ++w) tot += s_red[w];
        prefac[t] = norm[t] * P.inv_mean_mass / 4.0 / tot;
    }
}

// fluxes of the two colour filters and the magnitude filter (:644), and IMF values.
__global__ void k_bin_flux(IsoParams P, const double *__restrict__ m, const double *__restrict__ mags,
                           int64_t total, double *__restrict__ fl, double *__restrict__ imfv) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int fs[3] = {P.c1, P.c2, P.y_index};
#pragma unroll
    for (int q = 0; q < 3; ++q) fl[q * total + i] = exp10(-0.4 * mags[(int64_t)fs[q] * total + i]);
    imfv[i] = imf_pdf(P, m[i]);
}

// left-closed histogram bin of v (edges first + k step, step > 0), -1 outside
__device__ __forceinline__ int hist_bin(double v, double first, double step, int n) {
    if (!(v >= first)) return -1;
    int k = (int)floor((v - first) / step);
    if (k > 0 && v < first + (double)k * step) --k;
    if (v >= first + (double)(k + 1) * step) ++k;
    return (k >= 0 && k < n) ? k : -1;
}

// Grid: x -> j blocks, y -> i, z -> template (chunk-relative).  hist is [chunk][nx*ny].
__global__ void __launch_bounds__(kPairThreads)
k_bin_pairs(IsoParams P, const double *__restrict__ m, const double *__restrict__ fl,
            const double *__restrict__ imfv, int64_t total, const int64_t *__restrict__ off,
            const int32_t *__restrict__ len, const double *__restrict__ prefac, Grid2 g,
            int t0, double *__restrict__ hist) {
    const int t = t0 + blockIdx.z, n = len[t], ns = n - 1;
    const int i = blockIdx.y, j = i + 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ns || j >= ns) return;
    const int64_t o = off[t];
    const double *mt = m + o, *iv = imfv + o;
    const double *f1 = fl + o, *f2 = fl + total + o, *fy = fl + 2 * total + o;
    // flux2mag(f) = -5 log10(f) / 2 (:656)
    const double bm1 = -2.5 * log10(f1[i] + f1[j]);
    const double bm2 = -2.5 * log10(f2[i] + f2[j]);
    const double bmy = -2.5 * log10(fy[i] + fy[j]);
    double w = (mt[i + 1] - mt[i]) * (mt[j + 1] - mt[j]) * (iv[i] + iv[i + 1]) * (iv[j] + iv[j + 1]) *
               prefac[t];
    w *= compl_eval(P, P.c1, bm1) * compl_eval(P, P.c2, bm2);
    const double col = (bm1 + P.bias[P.c1]) - (bm2 + P.bias[P.c2]);
    const double ym = bmy + P.bias[P.y_index];
    const int ix = hist_bin(col, g.xf, g.xs, g.nx), iy = hist_bin(ym, g.yf, g.ys, g.ny);
    if (ix >= 0 && iy >= 0)
        atomicAdd(hist + (int64_t)blockIdx.z * g.nx * g.ny + ix + (int64_t)g.nx * iy, w);
}

// nonzero bins of each template (one block per template of the chunk)
__global__ void __launch_bounds__(kPairThreads)
k_bin_count(const double *__restrict__ hist, int64_t nbins, int32_t *__restrict__ cnt) {
    __shared__ int s_red[kPairThreads / 32];
    const double *h = hist + (int64_t)blockIdx.x * nbins;
    int c = 0;
    for (int64_t k = threadIdx.x; k < nbins; k += blockDim.x) c += h[k] != 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int tot = 0;
        for (int w = 0; w < kPairThreads / 32; ++w) tot += s_red[w];
        cnt[blockIdx.x] = tot;
    }
}

// points of the nonzero bins in bin order (x fastest), at start[t]: thread q takes a
// contiguous range of bins; a block scan of the range counts gives its first point.
__global__ void __launch_bounds__(kPairThreads)
k_bin_points(IsoParams P, const double *__restrict__ hist, Grid2 g, const int64_t *__restrict__ start,
             double *__restrict__ px, double *__restrict__ py, double *__restrict__ psx,
             double *__restrict__ psy, double *__restrict__ pw) {
    __shared__ int s_scan[kPairThreads];
    const int64_t nbins = (int64_t)g.nx * g.ny;
    const double *h = hist + (int64_t)blockIdx.x * nbins;
    const int64_t per = (nbins + kPairThreads - 1) / kPairThreads;
    const int64_t k0 = (int64_t)threadIdx.x * per, k1 = k0 + per < nbins ? k0 + per : nbins;
    int c = 0;
    for (int64_t k = k0; k < k1; ++k) c += h[k] != 0.0;
    s_scan[threadIdx.x] = c;
    __syncthreads();
    for (int o = 1; o < kPairThreads; o <<= 1) {  // inclusive scan (Hillis-Steele)
        const int v = threadIdx.x >= o ? s_scan[threadIdx.x - o] : 0;
        __syncthreads();
        s_scan[threadIdx.x] += v;
        __syncthreads();
    }
    int64_t q = start[blockIdx.x] + s_scan[threadIdx.x] - c;
    const int xc = (P.c1 != P.y_index) ? P.c1 : P.c2;
    for (int64_t k = k0; k < k1; ++k) {
        if (h[k] == 0.0) continue;
        const int ix = (int)(k % g.nx), iy = (int)(k / g.nx);
        // edges[k] + step / 2 (:688-689) with the edge correctly rounded by one fma and no
        // further contraction: the centre is a rounding tie of the stamp's pixel
        // (x - first) / step + 1 = k + 1.5, so its exact double decides the stamp's pixel
        const double cx = __dadd_rn(__fma_rn((double)ix, g.xs, g.xf), g.xs / 2.0);
        const double cy = __dadd_rn(__fma_rn((double)iy, g.ys, g.yf), g.ys / 2.0);
        const double xmag = (P.y_index == P.c1) ? cy - cx : cy + cx;  // :692-695
        px[q] = cx;
        py[q] = cy;
        psx[q] = err_eval(P, xc, xmag);
        psy[q] = err_eval(P, P.y_index, cy);
        pw[q] = h[k];
        ++q;
    }
}

__global__ void k_mix_binary(const float *__restrict__ single, const float *__restrict__ binary,
                             const double *__restrict__ bmf, int64_t nbins, int64_t n,
                             float *__restrict__ out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double b = bmf[k / nbins];
    out[k] = (float)((double)single[k] * (1.0 - b) + b * (double)binary[k]);
}

}  // namespace

extern "C" int sfh_binary_hess_batch_dev(sfh_ctx *ctx, const double *d_m_ini, const double *d_mags,
                                         int64_t total_points, const int64_t *h_off,
                                         const int32_t *h_len, int64_t ntempl, int nf,
                                         int y_index, int c1, int c2, const sfh_err_model *err,
                                         const sfh_compl_model *compl_, const double *bias,
                                         const sfh_imf *imf, double mean_mass,
                                         const double *h_norm, double x_first, double x_step,
                                         int64_t nx, double y_first, double y_step, int64_t ny,
                                         float *d_models) {
    if (!ctx || !d_m_ini || !d_mags || !h_off || !h_len || !err || !compl_ || !imf || !h_norm ||
        !d_models || ntempl < 1 || ntempl > 65535 || total_points < 1 || nx < 1 || ny < 1)
        return SFH_ERR_ARG;
    if (!(x_step > 0) || !(y_step > 0))
        return sfh_set_error(ctx, SFH_ERR_ARG, "binary_hess: bin edges must increase");
    if (!(y_index == c1 || y_index == c2))  // :700
        return sfh_set_error(ctx, SFH_ERR_UNSUPPORTED,
                             "binary_hess for y_index not in color_indices is not implemented");
    IsoParams P;
    int rc = make_iso_params(ctx, nf, y_index, c1, c2, err, compl_, bias, imf, mean_mass,
                             total_points, P);
    if (rc) return rc;
    int nmax = 0;
    for (int64_t t = 0; t < ntempl; ++t) {
        if (h_len[t] < 3 || h_len[t] > 65536 || h_off[t] < 0 || h_off[t] + h_len[t] > total_points)
            return sfh_set_error(ctx, SFH_ERR_ARG, "binary_hess: isochrone lengths in [3, 65536]");
        nmax = h_len[t] > nmax ? h_len[t] : nmax;
    }
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int64_t nbins = nx * ny;
    // per-call buffers (template builds are not latency critical)
    const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(ntempl, (256ll << 20) / (nbins * 8)));
    double *fl = nullptr, *imfv = nullptr, *prefac = nullptr, *hist = nullptr, *d_norm = nullptr;
    int64_t *d_off = nullptr, *d_start = nullptr;
    int32_t *d_len = nullptr, *d_cnt = nullptr, *d_cov = nullptr;
    double *pts = nullptr;
    auto cleanup = [&]() {
        cudaStreamSynchronize(st);
        for (void *p : {(void *)fl, (void *)imfv, (void *)prefac, (void *)hist, (void *)d_norm,
                        (void *)d_off, (void *)d_start, (void *)d_len, (void *)d_cnt, (void *)d_cov,
                        (void *)pts})
            if (p) cudaFree(p);
    };
    cudaError_t e = cudaSuccess;
    if ((e = cudaMalloc(&fl, 3 * total_points * 8)) || (e = cudaMalloc(&imfv, total_points * 8)) ||
        (e = cudaMalloc(&prefac, ntempl * 8)) || (e = cudaMalloc(&hist, chunk * nbins * 8)) ||
        (e = cudaMalloc(&d_norm, ntempl * 8)) || (e = cudaMalloc(&d_off, ntempl * 8)) ||
        (e = cudaMalloc(&d_start, chunk * 8)) || (e = cudaMalloc(&d_len, ntempl * 4)) ||
        (e = cudaMalloc(&d_cnt, chunk * 4)) || (e = cudaMalloc(&d_cov, chunk * 4))) {
        cleanup();
        return sfh_cuda_error(ctx, e, "binary_hess buffers");
    }
    cudaMemcpyAsync(d_norm, h_norm, ntempl * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_off, h_off, ntempl * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_len, h_len, ntempl * 4, cudaMemcpyHostToDevice, st);
    std::vector<int32_t> hcov((size_t)chunk, y_index == c1 ? -1 : 1);  // :698
    cudaMemcpyAsync(d_cov, hcov.data(), chunk * 4, cudaMemcpyHostToDevice, st);
    k_bin_flux<<<(unsigned)((total_points + 255) / 256), 256, 0, st>>>(P, d_m_ini, d_mags, total_points,
                                                                    fl, imfv);
    k_bin_prefac<<<(unsigned)ntempl, kPairThreads, 0, st>>>(P, d_m_ini, d_off, d_len, d_norm, prefac);
    ctx->launches += 2;
    Grid2 g{x_first, x_step, y_first, y_step, (int)nx, (int)ny};
    std::vector<int32_t> hcnt((size_t)chunk);
    std::vector<int64_t> hstart((size_t)chunk);
    size_t pts_cap = 0;
    for (int64_t t0 = 0; t0 < ntempl && rc == SFH_OK; t0 += chunk) {
        const int64_t nc = std::min(chunk, ntempl - t0);
        if ((e = cudaMemsetAsync(hist, 0, nc * nbins * 8, st))) { rc = sfh_cuda_error(ctx, e, "memset"); break; }
        dim3 grid((unsigned)((nmax + kPairThreads - 1) / kPairThreads), (unsigned)(nmax - 1), (unsigned)nc);
        k_bin_pairs<<<grid, kPairThreads, 0, st>>>(P, d_m_ini, fl, imfv, total_points, d_off, d_len,
                                                    prefac, g, (int)t0, hist);
        k_bin_count<<<(unsigned)nc, kPairThreads, 0, st>>>(hist, nbins, d_cnt);
        ctx->launches += 2;
        if ((e = cudaMemcpyAsync(hcnt.data(), d_cnt, nc * 4, cudaMemcpyDeviceToHost, st)) ||
            (e = cudaStreamSynchronize(st))) { rc = sfh_cuda_error(ctx, e, "binary_hess counts"); break; }
        int64_t tot = 0;
        for (int64_t q = 0; q < nc; ++q) { hstart[(size_t)q] = tot; tot += hcnt[(size_t)q]; }
        const size_t need = (size_t)std::max<int64_t>(tot, 1) * 5 * 8;
        if (need > pts_cap) {
            if (pts) cudaFree(pts);
            pts = nullptr;
            if ((e = cudaMalloc(&pts, need))) { rc = sfh_cuda_error(ctx, e, "binary_hess points"); break; }
            pts_cap = need;
        }
        const int64_t np = std::max<int64_t>(tot, 1);
        double *px = pts, *py = pts + np, *psx = pts + 2 * np, *psy = pts + 3 * np, *pw = pts + 4 * np;
        cudaMemcpyAsync(d_start, hstart.data(), nc * 8, cudaMemcpyHostToDevice, st);
        k_bin_points<<<(unsigned)nc, kPairThreads, 0, st>>>(P, hist, g, d_start, px, py, psx, psy, pw);
        ctx->launches++;
        rc = sfh_launch_stamps(ctx, px, py, psx, psy, pw, d_start, d_cnt, d_cov, nc, x_first, x_step,
                               nx, y_first, y_step, ny, d_models + t0 * nbins);
        if (rc == SFH_OK && (e = cudaStreamSynchronize(st))) rc = sfh_cuda_error(ctx, e, "binary_hess");
    }
    cleanup();
    return rc;
}

extern "C" int sfh_mix_binary_templates_dev(sfh_ctx *ctx, const float *d_single,
                                            const float *d_binary, const double *h_bmf,
                                            int64_t ntempl, int64_t nbins, float *d_out) {
    if (!ctx || !d_single || !d_binary || !h_bmf || !d_out || ntempl < 1 || nbins < 1)
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    double *d_bmf = nullptr;
    SFH_CK(ctx, cudaMalloc(&d_bmf, ntempl * 8));
    cudaMemcpyAsync(d_bmf, h_bmf, ntempl * 8, cudaMemcpyHostToDevice, ctx->stream);
    const int64_t n = ntempl * nbins;
    k_mix_binary<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(d_single, d_binary, d_bmf,
                                                                       nbins, n, d_out);
    ctx->launches++;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d_bmf);
    return e == cudaSuccess ? SFH_OK : sfh_cuda_error(ctx, e, "mix binary templates");
}
