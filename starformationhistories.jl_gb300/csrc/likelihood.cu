// likelihood.cu -- single-vector Poisson objective on sm_103a.
//
// Replaces, for one coefficient vector r:
//   composite!(composite, coeffs, models)        src/fitting/fitting_base.jl:55-65
//   loglikelihood(composite, data)               src/fitting/fitting_base.jl:84-96
//   ∇loglikelihood!(G, composite, models, data)  src/fitting/fitting_base.jl:265-285
//   fg!(F, G, coeffs, models, data, composite)   src/fitting/solvers.jl:20-38
//
// Both matrix passes are HBM-bound streams over the (nbins, nt) column-major
// template matrix M.  Four kernels:
//   k_gemv_n  : m_i partials over template splits (grid = row blocks x splits)
//   k_finalize: sums the partials, FP64 Poisson terms with a deterministic
//               block/last-block reduction, w_i = 1 - n_i/max(m_i, eps)
//   k_gemv_t  : G_j partials over row chunks, w staged in shared memory
//   k_reduce_g: fixed-order sum of the G partials
// FP32 storage multiplies by r = r_hi + r_lo (two FP32 products) and accumulates the
// products error-free against a power-of-two anchor per bin (sfh_anc_acc), so the
// composite carries ~1e-12 relative error against FP64 arithmetic on the same stored
// templates.
// k_gemv_t walks template columns in the reverse of k_gemv_n's launch order so
// the tail of M that k_gemv_n streamed last is still resident in L2.
#include <cuda_runtime.h>
#include <float.h>

#include "sfh_internal.cuh"

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float x) {
    const float s = __fadd_rn(hi, x);
    const float bp = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    hi = s;
    lo = __fadd_rn(lo, err);
}

// 16-byte streaming load issued in program order with its neighbours (volatile keeps a
// batch of these in flight together instead of interleaving them with the FMAs).
__device__ __forceinline__ float4 ld_stream4(const float *p) {
    float4 v;
    asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p));
    return v;
}

// ---------------------------------------------------------------- k_gemv_n (FP32 storage)
// Groups of 8 template rows are summed error-free against a power-of-two anchor taken
// from the group's own bound sum |M_ij| |r_j| (sfh_anc_acc: no row statistics needed, so
// this kernel also serves callers without a models handle); the groups fold into a
// compensated FP32 pair.
template <bool VEC>
__global__ void __launch_bounds__(kThreads)
k_gemv_n_f32(const float *__restrict__ M, int64_t nbins, int64_t nt,
             const double *__restrict__ r, int kchunk, double *__restrict__ part) {
    extern __shared__ float s_r[];
    float *rhi = s_r, *rlo = s_r + kchunk;
    const int split = blockIdx.y;
    const int64_t j0 = (int64_t)split * kchunk;
    const int kn = (int)min((int64_t)kchunk, nt - j0);
    for (int t = threadIdx.x; t < kn; t += blockDim.x) {
        const double v = r[j0 + t];
        const float h = __double2float_rn(v);
        rhi[t] = h;
        rlo[t] = __double2float_rn(v - (double)h);
    }
    __syncthreads();
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    if (i >= nbins) return;
    const int nr = VEC ? 4 : (int)min((int64_t)4, nbins - i);
    float ah[4] = {0.f, 0.f, 0.f, 0.f}, al[4] = {0.f, 0.f, 0.f, 0.f};
    const float *colp = M + j0 * nbins + i;
    for (int k = 0; k < kn; k += 8) {
        const int kk = min(8, kn - k);
        float m[8][4];
        if (VEC) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (u < kk) v = __ldg(reinterpret_cast<const float4 *>(colp + (int64_t)(k + u) * nbins));
                m[u][0] = v.x;
                m[u][1] = v.y;
                m[u][2] = v.z;
                m[u][3] = v.w;
            }
        } else {
#pragma unroll
            for (int u = 0; u < 8; ++u)
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    m[u][q] = (u < kk && q < nr) ? __ldg(colp + (int64_t)(k + u) * nbins + q) : 0.f;
        }
        float hv[8], lv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            hv[u] = u < kk ? rhi[k + u] : 0.f;
            lv[u] = u < kk ? rlo[k + u] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float b = 0.f;
#pragma unroll
            for (int u = 0; u < 8; ++u) b = fmaf(fabsf(m[u][q]), fabsf(hv[u]), b);
            const float sg = sfh_anchor(b * 1.0009765625f);
            float a = sg, lo = 0.f;
#pragma unroll
            for (int u = 0; u < 8; ++u) sfh_anc_acc(a, lo, m[u][q], hv[u], lv[u]);
            two_sum_acc(ah[q], al[q], __fsub_rn(a, sg));
            al[q] = __fadd_rn(al[q], lo);
        }
    }
    double *dst = part + (int64_t)split * nbins + i;
    for (int q = 0; q < nr; ++q) dst[q] = (double)ah[q] + (double)al[q];
}

// ---------------------------------------------------------------- k_gemv_n (FP64 storage)
__global__ void __launch_bounds__(kThreads)
k_gemv_n_f64(const double *__restrict__ M, int64_t nbins, int64_t nt,
             const double *__restrict__ r, int kchunk, double *__restrict__ part) {
    const int split = blockIdx.y;
    const int64_t j0 = (int64_t)split * kchunk;
    const int kn = (int)min((int64_t)kchunk, nt - j0);
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 2;
    if (i >= nbins) return;
    const bool two = (i + 1 < nbins);
    const bool vec = two && ((nbins & 1) == 0);
    double a0 = 0.0, a1 = 0.0;
    const double *colp = M + j0 * nbins + i;
    for (int k = 0; k < kn; ++k) {
        const double rk = __ldg(r + j0 + k);
        const double *c = colp + (int64_t)k * nbins;
        if (vec) {
            const double2 v = __ldg(reinterpret_cast<const double2 *>(c));
            a0 = fma(v.x, rk, a0);
            a1 = fma(v.y, rk, a1);
        } else {
            a0 = fma(__ldg(c), rk, a0);
            if (two) a1 = fma(__ldg(c + 1), rk, a1);
        }
    }
    double *dst = part + (int64_t)split * nbins + i;
    dst[0] = a0;
    if (two) dst[1] = a1;
}

// ---------------------------------------------------------------- k_finalize
struct FinArgs {
    const double *part;   // ksplit x nbins partials, or NULL (composite is the input)
    int ksplit;
    int64_t nbins;
    const double *data;
    double eps;
    double *composite;    // in (when part == NULL) / out
    float2 *w32;          // w as FP32 hi/lo (FP32 storage) or NULL
    double *w64;          // w as FP64 (FP64 storage) or NULL
    int want_logl;
    int want_w;           // compute w and overwrite composite with it
    int write_m;          // write m into composite (when !want_w)
    double *logl_part;    // gridDim.x
    unsigned int *counter;
    double *negLogL;      // receives -logL (or +logL when logl_sign = -1)
    double logl_sign;
};

__global__ void __launch_bounds__(kThreads) k_finalize(FinArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double term = 0.0;
    if (i < a.nbins) {
        double m;
        if (a.part) {
            m = 0.0;
            for (int s = 0; s < a.ksplit; ++s) m += a.part[(int64_t)s * a.nbins + i];
        } else {
            m = a.composite[i];
        }
        const double ci = m > a.eps ? m : a.eps;
        if (a.want_logl || a.want_w) {
            const double ni = a.data[i];
            if (a.want_logl) term = (ni > 0.0) ? (ni - ci - ni * log(ni / ci)) : -ci;
            if (a.want_w) {
                const double w = 1.0 - ni / ci;
                a.composite[i] = w;
                if (a.w32) {
                    const float h = __double2float_rn(w);
                    a.w32[i] = make_float2(h, __double2float_rn(w - (double)h));
                }
                if (a.w64) a.w64[i] = w;
            } else if (a.write_m) {
                a.composite[i] = m;
            }
        } else if (a.write_m) {
            a.composite[i] = m;
        }
    }
    if (!a.want_logl) return;
    // Deterministic reduction: fixed tree within the block, fixed-order sum of
    // block partials by the last block to finish.
    __shared__ double s_red[kThreads / 32];
    __shared__ bool s_last;
    double v = term;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) b += s_red[w];
        a.logl_part[blockIdx.x] = b;
        __threadfence();
        const unsigned int ticket = atomicAdd(a.counter, 1u);
        s_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double acc = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
        acc += ((volatile double *)a.logl_part)[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) tot += s_red[w];
        // loglikelihood returns -typemax(T) = -Inf when the sum is exactly zero
        // (fitting_base.jl:95).
        const double logl = (tot != 0.0) ? tot : -INFINITY;
        if (a.negLogL) *a.negLogL = a.logl_sign * -logl;
        *a.counter = 0u;  // re-arm for the next launch on this stream
    }
}

// ---------------------------------------------------------------- k_gemv_t (FP32 storage)
template <bool VEC>
__global__ void __launch_bounds__(kThreads)
k_gemv_t_f32(const float *__restrict__ M, int64_t nbins, int64_t nt, const float2 *__restrict__ w,
             int R, int CB, int ncolgroups, double *__restrict__ partG) {
    extern __shared__ float s_w[];
    float *swh = s_w, *swl = s_w + R;
    const int rc = blockIdx.y;
    const int64_t i0 = (int64_t)rc * R;
    const int rn = (int)min((int64_t)R, nbins - i0);
    for (int t = threadIdx.x; t < R; t += blockDim.x) {
        float2 v = make_float2(0.f, 0.f);
        if (t < rn) v = w[i0 + t];
        swh[t] = v.x;
        swl[t] = v.y;
    }
    __syncthreads();
    const int g = ncolgroups - 1 - (int)blockIdx.x;  // reverse of k_gemv_n's order
    const int64_t jb = (int64_t)g * CB;
    const int64_t je = min(nt, jb + CB);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t j = je - 1 - warp; j >= jb; j -= kThreads / 32) {
        const float *col = M + j * nbins + i0;
        float ah = 0.f, al = 0.f;
        if (VEC) {
            int ii = lane * 4;
            for (; ii + 384 < rn; ii += 512) {
                float4 m[4];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    m[u] = __ldg(reinterpret_cast<const float4 *>(col + ii + 128 * u));
                float s = 0.f;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float4 h = *reinterpret_cast<const float4 *>(swh + ii + 128 * u);
                    const float4 l = *reinterpret_cast<const float4 *>(swl + ii + 128 * u);
                    s = fmaf(m[u].x, h.x, fmaf(m[u].x, l.x, s));
                    s = fmaf(m[u].y, h.y, fmaf(m[u].y, l.y, s));
                    s = fmaf(m[u].z, h.z, fmaf(m[u].z, l.z, s));
                    s = fmaf(m[u].w, h.w, fmaf(m[u].w, l.w, s));
                }
                two_sum_acc(ah, al, s);
            }
            for (; ii < rn; ii += 128) {
                const float4 mv = __ldg(reinterpret_cast<const float4 *>(col + ii));
                const float4 h = *reinterpret_cast<const float4 *>(swh + ii);
                const float4 l = *reinterpret_cast<const float4 *>(swl + ii);
                float s = 0.f;
                s = fmaf(mv.x, h.x, fmaf(mv.x, l.x, s));
                s = fmaf(mv.y, h.y, fmaf(mv.y, l.y, s));
                s = fmaf(mv.z, h.z, fmaf(mv.z, l.z, s));
                s = fmaf(mv.w, h.w, fmaf(mv.w, l.w, s));
                two_sum_acc(ah, al, s);
            }
        } else {
            for (int ii = lane; ii < rn; ii += 32) {
                const float x = __ldg(col + ii);
                two_sum_acc(ah, al, fmaf(x, swh[ii], x * swl[ii]));
            }
        }
        double v = (double)ah + (double)al;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) partG[(int64_t)rc * nt + j] = v;
    }
}

// ---------------------------------------------------------------- k_gemv_t (FP64 storage)
__global__ void __launch_bounds__(kThreads)
k_gemv_t_f64(const double *__restrict__ M, int64_t nbins, int64_t nt, const double *__restrict__ w,
             int R, int CB, int ncolgroups, double *__restrict__ partG) {
    extern __shared__ double s_wd[];
    const int rc = blockIdx.y;
    const int64_t i0 = (int64_t)rc * R;
    const int rn = (int)min((int64_t)R, nbins - i0);
    for (int t = threadIdx.x; t < R; t += blockDim.x) s_wd[t] = (t < rn) ? w[i0 + t] : 0.0;
    __syncthreads();
    const int g = ncolgroups - 1 - (int)blockIdx.x;
    const int64_t jb = (int64_t)g * CB;
    const int64_t je = min(nt, jb + CB);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t j = je - 1 - warp; j >= jb; j -= kThreads / 32) {
        const double *col = M + j * nbins + i0;
        double acc = 0.0;
        for (int ii = lane; ii < rn; ii += 32) acc = fma(__ldg(col + ii), s_wd[ii], acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) partG[(int64_t)rc * nt + j] = acc;
    }
}

__global__ void k_reduce_g(const double *__restrict__ partG, int nchunks, int64_t nt, double sign,
                           double *__restrict__ G) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nt) return;
    double acc = 0.0;
    for (int c = 0; c < nchunks; ++c) acc += partG[(int64_t)c * nt + j];
    G[j] = sign * acc;
}


// ---------------------------------------------------------------- fused pass 1 (FP32 storage)
// m partials over template splits (register double-buffered loads).  The last split
// block to finish a row tile sums its rows' partials in split order, forms the FP64
// Poisson terms and w, and the last row tile sums the per-tile logL partials in tile
// order, so every result is deterministic.
struct Pass1Args {
    const float *M;
    int64_t nbins, nt;
    const double *r;
    int kchunk;
    float2 *part;  // (hi, lo) partial sums, ksplit x nbins
    const double *data;
    double eps;
    double *composite;
    float2 *w32;
    int want_logl, want_w;
    double *tile_logl;
    unsigned int *tile_cnt;
    unsigned int *all_cnt;
    double *negLogL;
    const sfh_df *tab;  // log table of the double-float Poisson terms
    float eps_f;        // eps(T) (a power of two) in FP32
    const float2 *rowb; // per bin (sum, max) of |M_ij|: the accumulation anchors' bound
};

__device__ __forceinline__ void block_sum_to(double v, double *s_red, double *out_tid0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += s_red[w];
        *out_tid0 = b;
    }
}

template <bool VEC>
__global__ void __launch_bounds__(kThreads) k_fg_pass1_f32(Pass1Args a) {
    extern __shared__ float s_r[];
    float *rhi = s_r, *rlo = s_r + a.kchunk;
    __shared__ double s_red[kThreads / 32];
    __shared__ bool s_last;
    // Grid: x = template split (fastest), y = row tile, so row tiles complete one after
    // another and their finalisation overlaps the streaming of later tiles.
    const int split = blockIdx.x, tile = blockIdx.y;
    const int nsplit = gridDim.x, ntile = gridDim.y;
    const int64_t j0 = (int64_t)split * a.kchunk;
    const int kn = (int)min((int64_t)a.kchunk, a.nt - j0);
    float rmx = 0.f, rsm = 0.f;
    for (int t = threadIdx.x; t < kn; t += blockDim.x) {
        const double v = a.r[j0 + t];
        const float h = __double2float_rn(v);
        rhi[t] = h;
        rlo[t] = __double2float_rn(v - (double)h);
        rmx = fmaxf(rmx, fabsf(h));
        rsm += fabsf(h);
    }
    // the chunk's max and sum of |r| for the anchors' bound
    __shared__ float s_rs[2][kThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        rmx = fmaxf(rmx, __shfl_xor_sync(0xffffffffu, rmx, o));
        rsm += __shfl_xor_sync(0xffffffffu, rsm, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s_rs[0][threadIdx.x >> 5] = rmx;
        s_rs[1][threadIdx.x >> 5] = rsm;
    }
    __syncthreads();
    float rmax = 0.f, rsum = 0.f;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) {
        rmax = fmaxf(rmax, s_rs[0][w]);
        rsum += s_rs[1][w];
    }
    const int64_t nbins = a.nbins;
    const int64_t i = ((int64_t)tile * blockDim.x + threadIdx.x) * 4;
    if (i < nbins) {
        // m r over the chunk, accumulated against each bin's power-of-two anchor (error-free
        // up to ~2^-47 of the anchor per term, sfh_anc_acc)
        const int nr = (int)min((int64_t)4, nbins - i);
        float sg[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float2 rb = q < nr ? __ldg(a.rowb + i + q) : make_float2(0.f, 0.f);
            sg[q] = sfh_anchor(sfh_row_bound(rb, rmax, rsum));
        }
        const float *colp = a.M + j0 * nbins + i;
        float2 *dst = a.part + (int64_t)split * nbins + i;
        if (VEC) {
            float2 a01 = make_float2(sg[0], sg[1]), a23 = make_float2(sg[2], sg[3]);
            float2 l01 = make_float2(0.f, 0.f), l23 = l01;
            int k = 0;
            for (; k + 8 <= kn; k += 8) {
                float4 v[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) v[u] = ld_stream4(colp + (int64_t)(k + u) * nbins);
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const float2 h2 = make_float2(rhi[k + u], rhi[k + u]);
                    const float2 l2 = make_float2(rlo[k + u], rlo[k + u]);
                    sfh_anc_acc2(a01, l01, make_float2(v[u].x, v[u].y), h2, l2);
                    sfh_anc_acc2(a23, l23, make_float2(v[u].z, v[u].w), h2, l2);
                }
            }
            for (; k < kn; ++k) {
                const float4 x = __ldg(reinterpret_cast<const float4 *>(colp + (int64_t)k * nbins));
                const float2 h2 = make_float2(rhi[k], rhi[k]), l2 = make_float2(rlo[k], rlo[k]);
                sfh_anc_acc2(a01, l01, make_float2(x.x, x.y), h2, l2);
                sfh_anc_acc2(a23, l23, make_float2(x.z, x.w), h2, l2);
            }
            const sfh_df c0 = sfh_anc_result(a01.x, l01.x, sg[0]), c1 = sfh_anc_result(a01.y, l01.y, sg[1]);
            const sfh_df c2 = sfh_anc_result(a23.x, l23.x, sg[2]), c3 = sfh_anc_result(a23.y, l23.y, sg[3]);
            *reinterpret_cast<float4 *>(dst) = make_float4(c0.h, c0.l, c1.h, c1.l);
            *reinterpret_cast<float4 *>(dst + 2) = make_float4(c2.h, c2.l, c3.h, c3.l);
        } else {
            float av[4] = {sg[0], sg[1], sg[2], sg[3]}, lv[4] = {0.f, 0.f, 0.f, 0.f};
            for (int k = 0; k < kn; ++k) {
                const float h = rhi[k], l = rlo[k];
                const float *c = colp + (int64_t)k * nbins;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (q < nr) sfh_anc_acc(av[q], lv[q], __ldg(c + q), h, l);
            }
            for (int q = 0; q < nr; ++q) {
                const sfh_df cq = sfh_anc_result(av[q], lv[q], sg[q]);
                dst[q] = make_float2(cq.h, cq.l);
            }
        }
    }
    // ---- the last split block of this row tile finalises the tile's rows
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int tk = atomicAdd(&a.tile_cnt[tile], 1u);
        s_last = (tk == nsplit - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const int ks = nsplit;
    const int64_t rbase = (int64_t)tile * blockDim.x * 4;
    __shared__ sfh_df s_tab[SFH_DF_TAB_ALL];
    if (a.want_logl) {
        for (int k = threadIdx.x; k < SFH_DF_TAB_ALL; k += blockDim.x) s_tab[k] = a.tab[k];
        __syncthreads();
    }
    // Poisson terms in double-float on the FP32 pipes (sfh_dfloat.cuh); eps(T) is a
    // power of two, exact in FP32.
    const float eps_f = a.eps_f;
    sfh_df term{0.f, 0.f};
    for (int q = 0; q < 4; ++q) {
        const int64_t ii = rbase + (int64_t)q * blockDim.x + threadIdx.x;
        if (ii >= nbins) continue;
        float mh = 0.f, ml = 0.f;
        int sp = 0;
        for (; sp + 16 <= ks; sp += 16) {
            float2 v[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) v[u] = __ldcg(a.part + (int64_t)(sp + u) * nbins + ii);
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                two_sum_acc(mh, ml, v[u].x);
                ml += v[u].y;
            }
        }
        for (; sp < ks; ++sp) {
            const float2 v = __ldcg(a.part + (int64_t)sp * nbins + ii);
            two_sum_acc(mh, ml, v.x);
            ml += v.y;
        }
        sfh_df c = df_fast_two_sum(mh, ml);
        if (!a.want_w) a.composite[ii] = sfh_f2d(c.h) + sfh_f2d(c.l);  // the model, unclamped
        if (!a.want_logl && !a.want_w) continue;  // composite only: data may be NULL
        if (c.h < eps_f || (c.h == eps_f && c.l < 0.f)) c = sfh_df{eps_f, 0.f};  // max(c, eps)
        float nh, nl;
        sfh_split_double(a.data[ii], nh, nl);
        if (a.want_logl)
            term = df_add(term, sfh_bin_term(c, nh, nl, s_tab));
        if (a.want_w) {
            const sfh_df diff = df_add(c, sfh_df{-nh, -nl});
            const float w = __fdiv_rn(diff.h, c.h);  // 1 - n/c
            a.composite[ii] = sfh_f2d(w);
            a.w32[ii] = make_float2(w, 0.f);
        }
    }
    double tile_sum = 0.0;
    sfh_df_block_sum(term, s_red, &tile_sum);
    if (threadIdx.x == 0) {
        a.tile_cnt[tile] = 0u;  // re-arm for the next launch on this stream
        s_last = false;
        if (a.want_logl) {
            a.tile_logl[tile] = tile_sum;
            __threadfence();
            const unsigned int tk = atomicAdd(a.all_cnt, 1u);
            s_last = (tk == ntile - 1);
        }
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double acc = 0.0;
    for (int b = threadIdx.x; b < ntile; b += blockDim.x) acc += __ldcg(a.tile_logl + b);
    double tot = 0.0;
    block_sum_to(acc, s_red, &tot);
    if (threadIdx.x == 0) {
        // loglikelihood returns -typemax(T) = -Inf when the sum is exactly zero (fitting_base.jl:95)
        const double logl = (tot != 0.0) ? tot : -INFINITY;
        if (a.negLogL) *a.negLogL = -logl;
        *a.all_cnt = 0u;
    }
}

// ---------------------------------------------------------------- fused pass 2 (FP32 storage)
// G partials over row chunks (w staged in shared memory); the last row-chunk block of a
// column group sums that group's partials in chunk order.
struct Pass2Args {
    const float *M;
    int64_t nbins, nt;
    const float2 *w;
    int R, CB, ncolgroups;
    double *partG;
    unsigned int *grp_cnt;
    double gsign;
    double *G;
};

template <bool VEC>
__global__ void __launch_bounds__(kThreads) k_fg_pass2_f32(Pass2Args a) {
    extern __shared__ float s_w[];
    __shared__ bool s_last;
    const int R = a.R;
    // Last row chunk first: pass 1 streamed the last row tiles most recently.
    const int rc = (int)gridDim.y - 1 - (int)blockIdx.y;
    const int64_t nbins = a.nbins, nt = a.nt;
    const int64_t i0 = (int64_t)rc * R;
    const int rn = (int)min((int64_t)R, nbins - i0);
    for (int t = threadIdx.x; t < R; t += blockDim.x) s_w[t] = (t < rn) ? a.w[i0 + t].x : 0.f;
    __syncthreads();
    const int g = a.ncolgroups - 1 - (int)blockIdx.x;
    const int64_t jb = (int64_t)g * a.CB;
    const int64_t je = min(nt, jb + a.CB);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t j = je - 1 - warp; j >= jb; j -= kThreads / 32) {
        const float *col = a.M + j * nbins + i0;
        float ah = 0.f, al = 0.f;
        if (VEC) {
            int ii = lane * 4;
            for (; ii + 896 < rn; ii += 1024) {
                float4 m[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) m[u] = ld_stream4(col + ii + 128 * u);
                float s0 = 0.f, s1 = 0.f;
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const float4 h = *reinterpret_cast<const float4 *>(s_w + ii + 128 * u);
                    float &sx = (u & 1) ? s1 : s0;
                    sx = fmaf(m[u].x, h.x, sx);
                    sx = fmaf(m[u].y, h.y, sx);
                    sx = fmaf(m[u].z, h.z, sx);
                    sx = fmaf(m[u].w, h.w, sx);
                }
                two_sum_acc(ah, al, s0);
                two_sum_acc(ah, al, s1);
            }
            for (; ii < rn; ii += 128) {
                const float4 mv = ld_stream4(col + ii);
                const float4 h = *reinterpret_cast<const float4 *>(s_w + ii);
                float sx = mv.x * h.x;
                sx = fmaf(mv.y, h.y, sx);
                sx = fmaf(mv.z, h.z, sx);
                sx = fmaf(mv.w, h.w, sx);
                two_sum_acc(ah, al, sx);
            }
        } else {
            for (int ii = lane; ii < rn; ii += 32) two_sum_acc(ah, al, __ldg(col + ii) * s_w[ii]);
        }
        // warp sum in double-float on the FP32 pipes, one conversion per column
        const sfh_df v = sfh_df_warp_sum(df_fast_two_sum(ah, al));
        if (lane == 0) a.partG[(int64_t)rc * nt + j] = sfh_f2d(v.h) + sfh_f2d(v.l);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int tk = atomicAdd(&a.grp_cnt[g], 1u);
        s_last = (tk == gridDim.y - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const int nch = (int)gridDim.y;
    for (int64_t j = jb + threadIdx.x; j < je; j += blockDim.x) {
        double acc = 0.0;
        int c = 0;
        for (; c + 8 <= nch; c += 8) {
            double v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = __ldcg(a.partG + (int64_t)(c + u) * nt + j);
#pragma unroll
            for (int u = 0; u < 8; ++u) acc += v[u];
        }
        for (; c < nch; ++c) acc += __ldcg(a.partG + (int64_t)c * nt + j);
        a.G[j] = a.gsign * acc;
    }
    if (threadIdx.x == 0) a.grp_cnt[g] = 0u;
}

struct Plan {
    int ksplit, kchunk, nrowblk;
    int R, CB, ncolgroups, nchunks;
    size_t off_part, off_w, off_partG, off_logl, total;
};

// Row chunk of the fused pass 2 (w staged in shared memory as FP32).
constexpr int kFusedR = 2048;

// Resident blocks per SM of the fused kernels (queried once per process).
struct FusedOcc {
    int p1 = 0, p2 = 0;
};
FusedOcc fused_occupancy(bool vec) {
    static FusedOcc cache[2];
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    FusedOcc &c = cache[vec ? 1 : 0];
    if (c.p1 == 0) {
        int a = 0, b = 0;
        if (vec) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_fg_pass1_f32<true>, kThreads, 8192);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fg_pass2_f32<true>, kThreads,
                                                          kFusedR * sizeof(float));
        } else {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_fg_pass1_f32<false>, kThreads, 8192);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fg_pass2_f32<false>, kThreads,
                                                          kFusedR * sizeof(float));
        }
        c.p1 = a > 0 ? a : 1;
        c.p2 = b > 0 ? b : 1;
    }
    return c;
}

Plan make_plan(const sfh_ctx *ctx, int64_t nbins, int64_t nt, bool f64, bool fused = false,
               const sfh_models *m = nullptr) {
    Plan p{};
    const int rows_per_block = f64 ? 2 * kThreads : 4 * kThreads;
    p.nrowblk = (int)((nbins + rows_per_block - 1) / rows_per_block);
    const int target = ctx->sm_count * 6;
    int ks = (target + p.nrowblk - 1) / p.nrowblk;
    p.R = f64 ? 2048 : 4096;
    p.nchunks = (int)((nbins + p.R - 1) / p.R);
    int groups = (target + p.nchunks - 1) / p.nchunks;
    if (fused) {
        // Pass 1: two whole waves of resident blocks.  Pass 2: 2,048-row chunks, column
        // groups of a multiple of 8 (every warp busy) sized to about one wave.  A plan
        // measured by sfh_models_autotune replaces these choices.
        const FusedOcc occ = fused_occupancy(nbins % 4 == 0);
        const int slots1 = occ.p1 * ctx->sm_count, slots2 = occ.p2 * ctx->sm_count;
        const int w2 = (m && m->tune_w2 > 0) ? m->tune_w2 : 1;
        // rounded down, so the grid fills whole waves (a few leftover blocks would run
        // as a nearly empty extra wave)
        ks = (m && m->tune_ks > 0) ? m->tune_ks : (2 * slots1) / p.nrowblk;
        p.R = (m && m->tune_R > 0) ? m->tune_R : kFusedR;
        p.nchunks = (int)((nbins + p.R - 1) / p.R);
        const double per_block = (double)nt * p.nchunks / ((double)w2 * slots2);
        const int cb8 = 8 * (int)ceil(per_block / 8.0);
        groups = (int)((nt + cb8 - 1) / cb8);
    }
    if (ks < 1) ks = 1;
    if (ks > 64) ks = 64;
    if (ks > nt) ks = (int)nt;
    p.kchunk = (int)((nt + ks - 1) / ks);
    p.ksplit = (int)((nt + p.kchunk - 1) / p.kchunk);
    if (groups < 1) groups = 1;
    int cb = (int)((nt + groups - 1) / groups);
    if (!fused) cb = ((cb + 7) / 8) * 8;
    p.CB = cb;
    p.ncolgroups = (int)((nt + cb - 1) / cb);
    const int nfin = (int)((nbins + kThreads - 1) / kThreads);
    p.off_part = 0;
    p.off_w = sfh_align256((size_t)p.ksplit * nbins * sizeof(double));
    p.off_partG = p.off_w + sfh_align256((size_t)nbins * (f64 ? sizeof(double) : sizeof(float2)));
    p.off_logl = p.off_partG + sfh_align256((size_t)p.nchunks * nt * sizeof(double));
    p.total = p.off_logl + sfh_align256((size_t)nfin * sizeof(double));
    return p;
}

}  // namespace

int sfh_launch_fg(sfh_ctx *ctx, const sfh_models *m, const FgArgs &a, cudaEvent_t *ev) {
    const bool f64 = (m->storage == SFH_F64);
    const void *Mptr = f64 ? m->d_col : (const void *)m->d_f32;
    if (!Mptr) return sfh_set_error(ctx, SFH_ERR_ARG, "models handle has no matrix");
    const int64_t nbins = m->nbins, nt = m->nt;
    // one-pass kernel (onepass.cu) for fg! with G on FP32 storage
    if (!f64 && a.mode == FG_MODE_FG && a.G && a.data &&
        (m->path == SFH_PATH_ONEPASS ||
         (m->path == SFH_PATH_AUTO && sfh_onepass_eligible(ctx, m)))) {
        int rc = sfh_scratch_reserve(ctx, sfh_onepass_scratch(ctx, m));
        if (rc) return rc;
        return sfh_launch_fg_onepass(ctx, const_cast<sfh_models *>(m), a.coeffs, a.data,
                                     a.composite, a.G, a.negLogL, a.eps, a.gsign, ctx->scratch, ev,
                                     a.skip, a.occ_key);
    }
    const bool fused_path = !f64 && (a.mode == FG_MODE_FG || a.mode == FG_MODE_COMPOSITE);
    const Plan p = make_plan(ctx, nbins, nt, f64, fused_path, m);
    int rc = sfh_scratch_reserve(ctx, p.total);
    if (rc) return rc;
    char *s = (char *)ctx->scratch;
    double *part = (double *)(s + p.off_part);
    double *partG = (double *)(s + p.off_partG);
    double *logl_part = (double *)(s + p.off_logl);
    float2 *w32 = f64 ? nullptr : (float2 *)(s + p.off_w);
    double *w64 = f64 ? (double *)(s + p.off_w) : nullptr;
    cudaStream_t st = ctx->stream;

    const bool from_coeffs = (a.mode == FG_MODE_FG || a.mode == FG_MODE_COMPOSITE);
    const bool want_g = (a.mode == FG_MODE_GRAD_GIVEN) || (a.mode == FG_MODE_FG && a.G);
    const bool want_l = (a.mode == FG_MODE_FG && a.negLogL);

    // FP32 storage from coefficients: two fused kernels (pass 1: m, logL, w; pass 2: G).
    if (!f64 && from_coeffs && p.nrowblk <= 32768 && p.ncolgroups <= 16384) {
        if (ev) SFH_CK(ctx, cudaEventRecord(ev[0], st));
        Pass1Args p1{};
        p1.M = (const float *)Mptr;
        p1.nbins = nbins;
        p1.nt = nt;
        p1.r = a.coeffs;
        p1.kchunk = p.kchunk;
        p1.part = reinterpret_cast<float2 *>(part);
        p1.data = a.data;
        p1.eps = a.eps;
        p1.composite = a.composite;
        p1.w32 = w32;
        p1.want_logl = want_l ? 1 : 0;
        p1.want_w = want_g ? 1 : 0;
        p1.tile_logl = logl_part;
        p1.tile_cnt = ctx->d_counters + SFH_CNT_ROWTILE;
        p1.all_cnt = ctx->d_counters + SFH_CNT_FG_LOGL;
        p1.negLogL = a.negLogL;
        p1.tab = ctx->d_df_tab;
        p1.eps_f = (float)a.eps;
        p1.rowb = m->d_rowb;
        if (!p1.rowb) return sfh_set_error(ctx, SFH_ERR_ARG, "models handle has no row statistics");
        dim3 grid(p.ksplit, p.nrowblk);
        const size_t sm = 2 * (size_t)p.kchunk * sizeof(float);
        if (nbins % 4 == 0)
            k_fg_pass1_f32<true><<<grid, kThreads, sm, st>>>(p1);
        else
            k_fg_pass1_f32<false><<<grid, kThreads, sm, st>>>(p1);
        SFH_LAUNCHED(ctx);
        if (ev) SFH_CK(ctx, cudaEventRecord(ev[1], st));
        if (ev) SFH_CK(ctx, cudaEventRecord(ev[2], st));
        if (want_g) {
            Pass2Args p2{};
            p2.M = (const float *)Mptr;
            p2.nbins = nbins;
            p2.nt = nt;
            p2.w = w32;
            p2.R = p.R;
            p2.CB = p.CB;
            p2.ncolgroups = p.ncolgroups;
            p2.partG = partG;
            p2.grp_cnt = ctx->d_counters + SFH_CNT_COLGROUP;
            p2.gsign = a.gsign;
            p2.G = a.G;
            dim3 gridt(p.ncolgroups, p.nchunks);
            const size_t smt = (size_t)p.R * sizeof(float);
            if (nbins % 4 == 0)
                k_fg_pass2_f32<true><<<gridt, kThreads, smt, st>>>(p2);
            else
                k_fg_pass2_f32<false><<<gridt, kThreads, smt, st>>>(p2);
            SFH_LAUNCHED(ctx);
        }
        if (ev) SFH_CK(ctx, cudaEventRecord(ev[3], st));
        if (ev) SFH_CK(ctx, cudaEventRecord(ev[4], st));
        return SFH_OK;
    }

    if (ev) SFH_CK(ctx, cudaEventRecord(ev[0], st));
    if (from_coeffs) {
        dim3 grid(p.nrowblk, p.ksplit);
        if (f64) {
            k_gemv_n_f64<<<grid, kThreads, 0, st>>>((const double *)Mptr, nbins, nt, a.coeffs,
                                                     p.kchunk, part);
        } else {
            const size_t sm = 2 * (size_t)p.kchunk * sizeof(float);
            if (nbins % 4 == 0)
                k_gemv_n_f32<true><<<grid, kThreads, sm, st>>>((const float *)Mptr, nbins, nt,
                                                               a.coeffs, p.kchunk, part);
            else
                k_gemv_n_f32<false><<<grid, kThreads, sm, st>>>((const float *)Mptr, nbins, nt,
                                                                a.coeffs, p.kchunk, part);
        }
        SFH_LAUNCHED(ctx);
    }
    FinArgs fa{};
    fa.part = from_coeffs ? part : nullptr;
    fa.ksplit = p.ksplit;
    fa.nbins = nbins;
    fa.data = a.data;
    fa.eps = a.eps;
    fa.composite = a.composite;
    fa.w32 = want_g ? w32 : nullptr;
    fa.w64 = want_g ? w64 : nullptr;
    fa.want_logl = want_l ? 1 : 0;
    fa.want_w = want_g ? 1 : 0;
    fa.write_m = from_coeffs ? 1 : 0;
    fa.logl_part = logl_part;
    fa.counter = ctx->d_counters + SFH_CNT_LOGL;
    fa.negLogL = a.negLogL;
    fa.logl_sign = 1.0;
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[1], st));
    const int nfin = (int)((nbins + kThreads - 1) / kThreads);
    k_finalize<<<nfin, kThreads, 0, st>>>(fa);
    SFH_LAUNCHED(ctx);
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[2], st));
    if (!want_g) return SFH_OK;
    dim3 gridt(p.ncolgroups, p.nchunks);
    if (f64) {
        k_gemv_t_f64<<<gridt, kThreads, (size_t)p.R * sizeof(double), st>>>(
            (const double *)Mptr, nbins, nt, w64, p.R, p.CB, p.ncolgroups, partG);
    } else {
        const size_t sm = 2 * (size_t)p.R * sizeof(float);
        if (nbins % 4 == 0)
            k_gemv_t_f32<true><<<gridt, kThreads, sm, st>>>((const float *)Mptr, nbins, nt, w32,
                                                            p.R, p.CB, p.ncolgroups, partG);
        else
            k_gemv_t_f32<false><<<gridt, kThreads, sm, st>>>((const float *)Mptr, nbins, nt, w32,
                                                             p.R, p.CB, p.ncolgroups, partG);
    }
    SFH_LAUNCHED(ctx);
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[3], st));
    k_reduce_g<<<(int)((nt + kThreads - 1) / kThreads), kThreads, 0, st>>>(partG, p.nchunks, nt,
                                                                            a.gsign, a.G);
    SFH_LAUNCHED(ctx);
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[4], st));
    return SFH_OK;
}

// Average per-kernel device time of `iters` fg! evaluations (telemetry for the
// roofline report): ms_out[0..3] = k_gemv_n, k_finalize, k_gemv_t, k_reduce_g.
extern "C" int sfh_fg_kernel_times(sfh_ctx *ctx, const sfh_models *m, const double *d_coeffs,
                                   const double *d_data, double *d_composite, double *d_G,
                                   double *d_negLogL, double eps, int iters, double *ms_out) {
    if (!ctx || !m || !d_coeffs || !d_data || !d_composite || !d_G || !ms_out || iters < 1)
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    cudaEvent_t ev[5];
    for (int k = 0; k < 5; ++k) SFH_CK(ctx, cudaEventCreate(&ev[k]));
    double acc[4] = {0, 0, 0, 0};
    FgArgs a{};
    a.coeffs = d_coeffs;
    a.data = d_data;
    a.composite = d_composite;
    a.G = d_G;
    a.negLogL = d_negLogL;
    a.eps = eps;
    a.gsign = 1.0;
    a.mode = FG_MODE_FG;
    int rc = SFH_OK;
    for (int it = 0; it < iters && rc == SFH_OK; ++it) {
        rc = sfh_launch_fg(ctx, m, a, ev);
        if (rc != SFH_OK) break;
        cudaError_t e = cudaEventSynchronize(ev[4]);
        if (e != cudaSuccess) { rc = sfh_cuda_error(ctx, e, "event sync"); break; }
        for (int k = 0; k < 4; ++k) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
            acc[k] += ms;
        }
    }
    for (int k = 0; k < 5; ++k) cudaEventDestroy(ev[k]);
    for (int k = 0; k < 4; ++k) ms_out[k] = acc[k] / iters;
    return rc;
}

extern "C" int sfh_models_autotune(sfh_ctx *ctx, sfh_models *m, const double *d_coeffs,
                                   const double *d_data, double eps, int iters, int *plan_out,
                                   double *ms_out) {
    if (!ctx || !m || !d_coeffs || !d_data || iters < 1) return SFH_ERR_ARG;
    if (m->storage == SFH_F64) return SFH_OK;  // the FP64 path has no tunable plan
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    double *buf = nullptr;  // composite, G, -logL of the trial runs
    SFH_CK(ctx, cudaMalloc(&buf, (size_t)(m->nbins + m->nt + 1) * sizeof(double)));
    cudaEvent_t ev[5];
    for (int k = 0; k < 5; ++k) {
        cudaError_t e = cudaEventCreate(&ev[k]);
        if (e != cudaSuccess) {
            for (int q = 0; q < k; ++q) cudaEventDestroy(ev[q]);
            cudaFree(buf);
            return sfh_cuda_error(ctx, e, "event create");
        }
    }
    FgArgs a{};
    a.coeffs = d_coeffs;
    a.data = d_data;
    a.composite = buf;
    a.G = buf + m->nbins;
    a.negLogL = buf + m->nbins + m->nt;
    a.eps = eps;
    a.gsign = 1.0;
    a.mode = FG_MODE_FG;
    // average pass-1 / pass-2 times of the current plan (after one untimed run)
    auto timed = [&](double &t1, double &t2) -> int {
        t1 = t2 = 0.0;
        for (int it = -1; it < iters; ++it) {
            int rc = sfh_launch_fg(ctx, m, a, ev);
            if (rc) return rc;
            cudaError_t e = cudaEventSynchronize(ev[4]);
            if (e != cudaSuccess) return sfh_cuda_error(ctx, e, "event sync");
            if (it < 0) continue;
            float x = 0.f, y = 0.f;
            cudaEventElapsedTime(&x, ev[0], ev[1]);
            cudaEventElapsedTime(&y, ev[2], ev[4]);
            t1 += x;
            t2 += y;
        }
        t1 /= iters;
        t2 /= iters;
        return SFH_OK;
    };
    // pass-1 candidates: template splits filling 1/2 to 4 whole waves of resident blocks
    const FusedOcc occ = fused_occupancy(m->nbins % 4 == 0);
    const int slots1 = occ.p1 * ctx->sm_count;
    const int nrowblk = (int)((m->nbins + 4 * kThreads - 1) / (4 * kThreads));
    int KS[8], nks = 0;
    for (int f2 : {1, 2, 3, 4, 6, 8}) {  // f2 / 2 waves
        int ks = (f2 * slots1) / (2 * nrowblk);
        ks = ks < 1 ? 1 : (ks > 64 ? 64 : ks);
        if (ks > m->nt) ks = (int)m->nt;
        bool dup = false;
        for (int q = 0; q < nks; ++q) dup = dup || KS[q] == ks;
        if (!dup) KS[nks++] = ks;
    }
    const int RR[] = {1024, 2048, 4096}, W2[] = {1, 2, 4};
    int best_ks = KS[0], best_R = kFusedR, best_w2 = 1;
    double b1 = 1e300, b2 = 1e300, t1 = 0, t2 = 0;
    int rc = SFH_OK;
    m->tune_R = best_R;
    m->tune_w2 = best_w2;
    m->path = SFH_PATH_TWOPASS;
    for (int q = 0; q < nks; ++q) {  // pass 1 (pass 2 fixed at the default)
        m->tune_ks = KS[q];
        if ((rc = timed(t1, t2))) break;
        if (t1 < b1) { b1 = t1; best_ks = KS[q]; }
    }
    m->tune_ks = best_ks;
    for (int r = 0; r < 3 && rc == SFH_OK; ++r)  // pass 2 with the chosen pass 1
        for (int w2 : W2) {
            m->tune_R = RR[r];
            m->tune_w2 = w2;
            if ((rc = timed(t1, t2))) break;
            if (t2 < b2) { b2 = t2; best_R = RR[r]; best_w2 = w2; }
        }
    m->tune_ks = best_ks;
    m->tune_R = best_R;
    m->tune_w2 = best_w2;
    m->onepass_ms = 0.0;
    if (rc == SFH_OK && sfh_onepass_eligible(ctx, m)) {  // one-pass tile widths against the best plan
        m->path = SFH_PATH_ONEPASS;
        double best_op = 1e300;
        int best_bins = 16, best_ctas = 1, best_skew = 0;
        // tile width, CTAs per SM, skewed schedule
        const int variants[4][3] = {{16, 1, 0}, {32, 1, 0}, {16, 2, 0}, {16, 1, 1}};
        for (const auto &v : variants) {
            m->onepass_bins = v[0];
            m->onepass_ctas = v[1];
            m->onepass_skew = v[2];
            if ((rc = timed(t1, t2)) != SFH_OK) break;
            if (t1 + t2 < best_op) {
                best_op = t1 + t2;
                best_bins = v[0];
                best_ctas = v[1];
                best_skew = v[2];
            }
        }
        m->onepass_bins = best_bins;
        m->onepass_ctas = best_ctas;
        m->onepass_skew = best_skew;
        if (rc == SFH_OK) {
            m->onepass_ms = best_op;
            if (best_op >= b1 + b2) m->path = SFH_PATH_TWOPASS;
        }
    }
    for (int k = 0; k < 5; ++k) cudaEventDestroy(ev[k]);
    cudaFree(buf);
    if (rc) {
        m->tune_ks = m->tune_R = m->tune_w2 = 0;
        m->path = SFH_PATH_AUTO;
        m->onepass_bins = m->onepass_ctas = m->onepass_skew = 0;
        m->onepass_lp = -1;
        return rc;
    }
    if (plan_out) {
        plan_out[0] = best_ks;
        plan_out[1] = best_R;
        plan_out[2] = best_w2;
    }
    if (ms_out) {
        ms_out[0] = b1;
        ms_out[1] = b2;
    }
    return SFH_OK;
}

int sfh_launch_loglikelihood(sfh_ctx *ctx, const double *composite, const double *data,
                             int64_t nbins, double eps, double *d_out) {
    const int nfin = (int)((nbins + kThreads - 1) / kThreads);
    int rc = sfh_scratch_reserve(ctx, sfh_align256((size_t)(nfin > 0 ? nfin : 1) * sizeof(double)));
    if (rc) return rc;
    if (nbins == 0) {
        const double v = -INFINITY;  // empty sum is exactly zero -> -typemax
        SFH_CK(ctx, cudaMemcpyAsync(d_out, &v, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
        return SFH_OK;
    }
    FinArgs fa{};
    fa.part = nullptr;
    fa.nbins = nbins;
    fa.data = data;
    fa.eps = eps;
    fa.composite = const_cast<double *>(composite);
    fa.want_logl = 1;
    fa.want_w = 0;
    fa.write_m = 0;
    fa.logl_part = (double *)ctx->scratch;
    fa.counter = ctx->d_counters + SFH_CNT_LOGL;
    fa.negLogL = d_out;
    fa.logl_sign = -1.0;  // store +logL
    k_finalize<<<nfin, kThreads, 0, ctx->stream>>>(fa);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

// ---------------------------------------------------------------- allocation-free fg!
// Some callers cannot call cudaMalloc at all: code running inside a CUDA-graph
// capture that must not allocate, plugins living inside a host application that
// owns the device memory budget (and forbids side allocations), or real-time loops
// where an allocation could stall.  sfh_fg_dev_noalloc serves them with the two-pass
// FP32 plan (m = M r with the Poisson terms and w, then G = -Mᵀ w): the same
// arithmetic as sfh_fg_dev's two-pass path, but not the one-pass kernel that
// sfh_fg_dev prefers for FP32 storage (that kernel keeps a blocked copy of the
// templates, an allocation), so on the production matrix it is about 1.6x slower
// than sfh_fg_dev.  Its scratch is this fixed, file-scope device array, so the call
// itself allocates nothing.  The array is 11 MiB and is held by every GPU that loads
// the library until the process exits.
namespace {
constexpr int64_t kNoAllocMaxBins = 131072;  // e.g. a 362 x 362 Hess grid
constexpr int64_t kNoAllocMaxTempl = 4096;
constexpr int kNoAllocMaxSplit = 8;
constexpr size_t kNoAllocBytes = 11u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// The array's device address differs per CUDA context (a host application may create
// its own driver-API contexts, and a reset device gets a new primary context), so the
// looked-up address is cached per context, not per device ordinal.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
CtxGetCurrentFn ctx_get_current() {
    static CtxGetCurrentFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (CtxGetCurrentFn)p;
    }
    return fn;
}
constexpr int kNoAllocCtxSlots = 64;
std::mutex g_noalloc_mu;
CUcontext g_noalloc_ctx[kNoAllocCtxSlots] = {nullptr};
void *g_noalloc_ptr[kNoAllocCtxSlots] = {nullptr};
}  // namespace

extern "C" int sfh_fg_dev_noalloc(void *stream, const float *d_models, int64_t nbins,
                                  int64_t ntempl, const double *d_coeffs, const double *d_data,
                                  double *d_composite, double *d_G, double *d_negLogL,
                                  double eps) {
    if (!d_models || !d_coeffs || !d_data || !d_composite || nbins < 1 || ntempl < 1)
        return SFH_ERR_ARG;
    if (nbins > kNoAllocMaxBins || ntempl > kNoAllocMaxTempl)
        return SFH_ERR_SHAPE;  // beyond the fixed scratch: use sfh_fg_dev instead
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return SFH_ERR_CUDA;
    // The context current on this thread (the caller's, or the runtime's primary
    // context, which cudaSetDevice binds to a thread that has not used it yet).
    CtxGetCurrentFn get_ctx = ctx_get_current();
    CUcontext cu = nullptr;
    if (!get_ctx || get_ctx(&cu) != CUDA_SUCCESS) return SFH_ERR_CUDA;
    if (!cu) {
        if (cudaSetDevice(dev) != cudaSuccess) return SFH_ERR_CUDA;
        if (get_ctx(&cu) != CUDA_SUCCESS || !cu) return SFH_ERR_CUDA;
    }
    void *base = nullptr;
    {
        // First call in this context: resolve the device address of the array (the
        // host-side symbol is only a stand-in).  Make that first call outside any
        // stream capture.
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        int slot = -1, free_slot = -1;
        for (int k = 0; k < kNoAllocCtxSlots; ++k) {
            if (g_noalloc_ctx[k] == cu) { slot = k; break; }
            if (!g_noalloc_ctx[k] && free_slot < 0) free_slot = k;
        }
        if (slot < 0) {
            if (free_slot < 0) return SFH_ERR_CUDA;  // more than 64 live contexts
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return SFH_ERR_CUDA;
            g_noalloc_ctx[free_slot] = cu;
            g_noalloc_ptr[free_slot] = p;
            slot = free_slot;
        }
        base = g_noalloc_ptr[slot];
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return SFH_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    // Launch plan as in make_plan, with the template split capped so the partials fit.
    const int rows_per_block = 4 * kThreads;
    const int nrowblk = (int)((nbins + rows_per_block - 1) / rows_per_block);
    const int target = sms * 6;
    int ks = (target + nrowblk - 1) / nrowblk;
    ks = ks < 1 ? 1 : (ks > kNoAllocMaxSplit ? kNoAllocMaxSplit : ks);
    if (ks > ntempl) ks = (int)ntempl;
    const int kchunk = (int)((ntempl + ks - 1) / ks);
    const int ksplit = (int)((ntempl + kchunk - 1) / kchunk);
    const int R = 4096;
    const int nchunks = (int)((nbins + R - 1) / R);
    int groups = (target + nchunks - 1) / nchunks;
    if (groups < 1) groups = 1;
    int cb = (int)((ntempl + groups - 1) / groups);
    cb = ((cb + 7) / 8) * 8;
    const int ncolgroups = (int)((ntempl + cb - 1) / cb);
    const int nfin = (int)((nbins + kThreads - 1) / kThreads);
    const size_t off_part = 0;
    const size_t off_w = sfh_align256((size_t)ksplit * nbins * sizeof(double));
    const size_t off_partG = off_w + sfh_align256((size_t)nbins * sizeof(float2));
    const size_t off_logl = off_partG + sfh_align256((size_t)nchunks * ntempl * sizeof(double));
    const size_t off_cnt = off_logl + sfh_align256((size_t)nfin * sizeof(double));
    if (off_cnt + 256 > kNoAllocBytes) return SFH_ERR_SHAPE;
    char *s = (char *)base;
    double *part = (double *)(s + off_part);
    float2 *w32 = (float2 *)(s + off_w);
    double *partG = (double *)(s + off_partG);
    double *logl_part = (double *)(s + off_logl);
    unsigned int *counter = (unsigned int *)(s + off_cnt);
    // The array keeps the previous call's contents: the reduction counter must start at 0.
    if (cudaMemsetAsync(counter, 0, sizeof(unsigned int), st) != cudaSuccess) return SFH_ERR_CUDA;

    dim3 grid(nrowblk, ksplit);
    const size_t sm_n = 2 * (size_t)kchunk * sizeof(float);
    // The float4 loads need every column to start on a 16-byte boundary: nbins a
    // multiple of 4 and a 16-byte-aligned base.  A caller's pointer is only known to be
    // float-aligned (a sliced or offset view), so check it.
    const bool vec = (nbins % 4 == 0) && (((uintptr_t)d_models & 15) == 0);
    if (vec)
        k_gemv_n_f32<true><<<grid, kThreads, sm_n, st>>>(d_models, nbins, ntempl, d_coeffs, kchunk,
                                                         part);
    else
        k_gemv_n_f32<false><<<grid, kThreads, sm_n, st>>>(d_models, nbins, ntempl, d_coeffs,
                                                          kchunk, part);
    if (cudaGetLastError() != cudaSuccess) return SFH_ERR_CUDA;
    const bool want_g = d_G != nullptr;
    FinArgs fa{};
    fa.part = part;
    fa.ksplit = ksplit;
    fa.nbins = nbins;
    fa.data = d_data;
    fa.eps = eps;
    fa.composite = d_composite;
    fa.w32 = want_g ? w32 : nullptr;
    fa.w64 = nullptr;
    fa.want_logl = d_negLogL ? 1 : 0;
    fa.want_w = want_g ? 1 : 0;
    fa.write_m = 1;
    fa.logl_part = logl_part;
    fa.counter = counter;
    fa.negLogL = d_negLogL;
    fa.logl_sign = 1.0;
    k_finalize<<<nfin, kThreads, 0, st>>>(fa);
    if (cudaGetLastError() != cudaSuccess) return SFH_ERR_CUDA;
    if (!want_g) return SFH_OK;
    dim3 gridt(ncolgroups, nchunks);
    const size_t sm_t = 2 * (size_t)R * sizeof(float);
    if (vec)
        k_gemv_t_f32<true><<<gridt, kThreads, sm_t, st>>>(d_models, nbins, ntempl, w32, R, cb,
                                                          ncolgroups, partG);
    else
        k_gemv_t_f32<false><<<gridt, kThreads, sm_t, st>>>(d_models, nbins, ntempl, w32, R, cb,
                                                           ncolgroups, partG);
    if (cudaGetLastError() != cudaSuccess) return SFH_ERR_CUDA;
    k_reduce_g<<<(int)((ntempl + kThreads - 1) / kThreads), kThreads, 0, st>>>(partG, nchunks,
                                                                                ntempl, 1.0, d_G);
    if (cudaGetLastError() != cudaSuccess) return SFH_ERR_CUDA;
    return SFH_OK;
}

extern "C" int sfh_models_set_path(sfh_ctx *ctx, sfh_models *m, int path) {
    if (!ctx || !m || path < SFH_PATH_AUTO || path > SFH_PATH_TWOPASS) return SFH_ERR_ARG;
    if (path == SFH_PATH_ONEPASS && !sfh_onepass_eligible(ctx, m))
        return sfh_set_error(ctx, SFH_ERR_UNSUPPORTED,
                             "one-pass fg! needs FP32 storage and nt <= 1536");
    m->path = path;
    return SFH_OK;
}

extern "C" int sfh_models_set_onepass_tile(sfh_ctx *ctx, sfh_models *m, int bins) {
    if (!ctx || !m || (bins != 16 && bins != 32)) return SFH_ERR_ARG;
    m->onepass_bins = bins;
    return SFH_OK;
}

extern "C" int sfh_models_set_onepass_ctas(sfh_ctx *ctx, sfh_models *m, int ctas_per_sm) {
    if (!ctx || !m || (ctas_per_sm != 1 && ctas_per_sm != 2)) return SFH_ERR_ARG;
    m->onepass_ctas = ctas_per_sm;
    return SFH_OK;
}

extern "C" int sfh_models_set_onepass_schedule(sfh_ctx *ctx, sfh_models *m, int skewed) {
    if (!ctx || !m || (skewed != 0 && skewed != 1)) return SFH_ERR_ARG;
    m->onepass_skew = skewed;
    return SFH_OK;
}

extern "C" int sfh_models_set_onepass_run(sfh_ctx *ctx, sfh_models *m, int boxes) {
    if (!ctx || !m || (boxes != 0 && boxes != 1 && boxes != 2 && boxes != 4)) return SFH_ERR_ARG;
    m->onepass_lp = boxes == 0 ? -1 : boxes == 1 ? 0 : boxes == 2 ? 1 : 2;
    return SFH_OK;
}

extern "C" int sfh_models_onepass_variant(sfh_ctx *ctx, const sfh_models *m, int *bins,
                                          int *ctas_per_sm, int *skewed, int *run_boxes) {
    if (!ctx || !m || !bins || !ctas_per_sm || !skewed || !run_boxes) return SFH_ERR_ARG;
    if (!sfh_onepass_eligible(ctx, m)) return sfh_set_error(ctx, SFH_ERR_UNSUPPORTED, "not one-pass eligible");
    OnePassChoice c{};
    sfh_onepass_choose(ctx, m, &c);
    *bins = c.bins;
    *ctas_per_sm = c.per_sm;
    *skewed = c.skew;
    *run_boxes = 1 << c.lp;
    return SFH_OK;
}

extern "C" int sfh_models_path(sfh_ctx *ctx, const sfh_models *m, int *path_out,
                               double *onepass_ms) {
    if (!ctx || !m) return SFH_ERR_ARG;
    const bool one = m->storage != SFH_F64 &&
                     (m->path == SFH_PATH_ONEPASS ||
                      (m->path == SFH_PATH_AUTO && sfh_onepass_eligible(ctx, m)));
    if (path_out) *path_out = one ? SFH_PATH_ONEPASS : SFH_PATH_TWOPASS;
    if (onepass_ms) *onepass_ms = m->onepass_ms;
    return SFH_OK;
}

int sfh_check_onepass(sfh_ctx *ctx) {
    unsigned int h = 0;
    SFH_CK(ctx, cudaMemcpyAsync(&h, ctx->d_counters + SFH_CNT_ONEPASS_ERR, sizeof(h),
                                cudaMemcpyDeviceToHost, ctx->stream));
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (h) {
        SFH_CK(ctx, cudaMemsetAsync(ctx->d_counters + SFH_CNT_ONEPASS_ERR, 0, sizeof(h), ctx->stream));
        SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
        return sfh_set_error(ctx, SFH_ERR_TIMEOUT, "one-pass fg! pipeline wait timed out");
    }
    return SFH_OK;
}
