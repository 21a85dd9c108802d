// batched_exact.cu -- the composite of many coefficient vectors, exact on the tensor cores.
//
// For logL at |ΔlogL| <= 1e-6 per 1e4 stars the composite C = R Mᵀ (composite!,
// src/fitting/fitting_base.jl:55-65, for every vector) must be close to FP64: the FP32
// accumulators of the tensor cores truncate, and the hi/lo BF16 form leaves C ~4e-6 low.
// Here C is formed from integer digit planes whose products and sums the tensor cores
// carry out exactly (the Ozaki scheme: Ozaki, Ogita, Oishi, Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59, 2012; on BF16/FP16 tensor
// cores with FP32 accumulation as in Mukunoki, Ozaki, Ogita, Imamura, ICCS 2020):
//
//   M_ij = 2^E_i  Σ_{q<5} e_q,ij 2^{-6(q+1)}   (per bin exponent E_i: max_j |M_ij| < 2^E_i)
//   R_bj = 2^S_b  Σ_{p<P} d_p,bj 2^{-6(p+1)}   (per vector exponent S_b, P = 6, 7 or 8)
//   digits: first in [-64, 64], the others in [-32, 32] (round to nearest), exact in BF16;
//   C_bi = 2^{E_i + S_b - 12} Σ_{s<P} 2^{-6s} A_s,bi,   A_s = Σ_{p+q=s} Σ_j d_p,bj e_q,ij.
// Each class sum A_s is an integer below 7168 * nt in magnitude, exact in an FP32
// accumulator for nt <= 2304 (< 2^24); the products (p, q) with p + q < P (20, 25 or 30)
// run as five MMAs per K step: A operand = M plane q (128 bins), B operand = R planes
// 0 .. P-1-q stacked (32 vectors each), accumulator offset 32 q columns, so R plane p
// lands in class p + q.  M is represented to 2^-31 of the bin's largest template value
// and R to 2^-(6P+1) of the vector's largest entry; P grows with the widest ratio of
// largest to smallest nonzero |R_bj| in the batch (6 up to 2^19, 7 up to 2^25, else 8) so
// that small coefficients keep their precision.  The classes from P on are dropped.  The
// composite then matches FP64 on the stored FP32 templates to ~1e-10 relative.
//
// The Poisson sum is split so the epilogue only forms logarithms (fitting_base.jl:84-96):
//   logL_b = Σ_{i: n_i>0} n_i log c_bi  -  Σ_j R_bj colsum_j  +  Σ_{i: n_i>0} (n_i - n_i log n_i),
// the middle term an FP64 dot product per vector with the templates' column sums (Σ_i c_bi
// for nonnegative templates and coefficients, where max(c, eps) moves a bin by < eps), the
// last a constant of the data.  With a negative template value or coefficient the
// epilogue subtracts each max(c, eps) itself instead.
//
// k_tc_exact: one CTA per SM, 320 threads, persistent over (bin tile of 128, vector tile
// of 32) units, vector tiles inner so concurrent CTAs share the template planes in L2:
//   warp 0     TMA producer: 2-stage ring of {5 M planes 128x64, P R planes 32x64}
//   warp 1     allocates 512 TMEM columns (two buffers of up to 8 classes x 32 columns);
//              lane 0 issues the MMAs (M=128, N = 32 (P - q), K=16)
//   warps 2-9  epilogue: per (bin, vector) the class sums combined in double-float (the
//              two leading classes by an error-free sum, the rest, below 2^-11 of the
//              composite, in FP32), scaled, n log c in double-float (sfh_dfloat.cuh) and
//              w = 1 - n/c (BF16 hi/lo, the A operand of G = W M); partial sums of n log c
//              per (bin tile, lane quarter, vector).
// Every mbarrier wait is bounded as in batched.cu.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>

#include "sfh_internal.cuh"
#include "sfh_ptx.cuh"

namespace {

constexpr int kQ = 5;          // M digit planes
constexpr int kPMax = 8;       // R digit planes (at most; P per launch in {6, 7, 8})
constexpr int XBM = 128;       // bins per tile (A rows)
constexpr int XBN = 32;        // vectors per tile (B rows per R plane)
constexpr int XBK = 64;        // templates per stage
constexpr int XSTAGES = 2;
constexpr int XA_PLANE = XBM * XBK * 2;                   // 16 KB
constexpr int XB_PLANE = XBN * XBK * 2;                   // 4 KB
constexpr int XSTAGE_BYTES = kQ * XA_PLANE + kPMax * XB_PLANE;  // 112 KB
constexpr int XCLS_COLS = kPMax * XBN;                     // 256 accumulator columns per buffer
constexpr int XTMEM_COLS = 512;
constexpr int kXThreads = 320;
constexpr int kXEpi = 256;
constexpr size_t kXSmem = 1024 + (size_t)XSTAGES * XSTAGE_BYTES + 256 +
                          (size_t)SFH_DF_TAB_LOG * sizeof(sfh_df);  // + the log table

// kind::f16 instruction descriptor: D F32, A = B = BF16, both K-major, N, M = 128.
__host__ __device__ constexpr uint32_t xidesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(XBM >> 4) << 24);
}

struct ExactParams {
    int n_mt, n_vt, kb_total;
    int64_t nbins, nbins_pad;  // nbins_pad: rows per M plane (multiple of 128)
    int B, B_pad;              // B_pad: rows per R plane (multiple of 32)
    const double *data;        // nbins
    const float *escale;       // nbins: 2^E_i
    const float *rscale;       // B_pad: 2^S_b
    const int *nplanes;        // P (device scalar, set by k_r_digits)
    const int *negflag;        // nonzero: a coefficient is negative (set by k_r_digits)
    int m_negative;            // the templates hold a negative value
    float eps;
    const sfh_df *tab;
    __nv_bfloat16 *W_hi, *W_lo;
    int64_t w_ld;
    int want_w;
    float2 *lpart;             // [n_mt * 4][B_pad]
    int *err;
};

__device__ __forceinline__ void xfence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void xfence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// K-major tile, 128-byte rows, 128-byte swizzle, 8-row core groups 1024 bytes apart.
__device__ __forceinline__ uint64_t xdesc(uint32_t addr) {
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

__device__ __forceinline__ void xmma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                     uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void xcommit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

// 8 consecutive FP32 accumulator columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void xld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}

__global__ void __launch_bounds__(kXThreads, 1)
k_tc_exact(const __grid_constant__ CUtensorMap tM, const __grid_constant__ CUtensorMap tR,
           const ExactParams P) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bar = (uint64_t *)(smem + (size_t)XSTAGES * XSTAGE_BYTES);
    uint64_t *full = bar, *empty = bar + XSTAGES, *tfull = bar + 2 * XSTAGES,
             *tempty = bar + 2 * XSTAGES + 2, *drain = bar + 2 * XSTAGES + 4;
    uint32_t *tmem_slot = (uint32_t *)(bar + 2 * XSTAGES + 5);
    volatile int *s_abort = (volatile int *)(tmem_slot + 1);
    sfh_df *s_tab = (sfh_df *)(smem + (size_t)XSTAGES * XSTAGE_BYTES + 256);  // log(1 + j/128)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k < SFH_DF_TAB_LOG; k += blockDim.x) s_tab[k] = P.tab[k];

    if (threadIdx.x == 0) {
        for (int s = 0; s < XSTAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], kXEpi);
        }
        mbar_init(drain, 1);
        *s_abort = 0;
        fence_barrier_init();
    }
    const int NP = min(kPMax, max(6, *P.nplanes));  // R planes this launch (uniform)
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(XTMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    xfence_before();
    __syncthreads();
    xfence_after();
    const uint32_t tmem_base = *tmem_slot;
    const int total = P.n_mt * P.n_vt;

    if (warp == 0) {
        // ---------------- TMA producer
        if (lane == 0) {
            int stage = 0, issued = 0;
            uint32_t phase = 0;
            for (int u = blockIdx.x; u < total && !*s_abort; u += gridDim.x) {
                const int mt = u / P.n_vt, vt = u - mt * P.n_vt;
                for (int kb = 0; kb < P.kb_total; ++kb) {
                    if (!mbar_wait(&empty[stage], phase ^ 1u, s_abort, P.err, 11)) break;
                    uint8_t *st = smem + (size_t)stage * XSTAGE_BYTES;
                    mbar_expect_tx(&full[stage], (uint32_t)(kQ * XA_PLANE + NP * XB_PLANE));
#pragma unroll
                    for (int q = 0; q < kQ; ++q)
                        tma_load_2d(st + q * XA_PLANE, &tM, kb * XBK,
                                    (int)(q * P.nbins_pad + (int64_t)mt * XBM), &full[stage]);
                    for (int p = 0; p < NP; ++p)
                        tma_load_2d(st + kQ * XA_PLANE + p * XB_PLANE, &tR, kb * XBK,
                                    p * P.B_pad + vt * XBN, &full[stage]);
                    ++issued;
                    if (++stage == XSTAGES) {
                        stage = 0;
                        phase ^= 1u;
                    }
                }
            }
            if (*s_abort) {
                volatile int never = 0;
                int dummy = 0;
                for (int k = 0; k < XSTAGES && k < issued; ++k) {
                    if (--stage < 0) {
                        stage = XSTAGES - 1;
                        phase ^= 1u;
                    }
                    mbar_wait(&full[stage], phase, &never, &dummy, 0);
                }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer
        if (lane == 0) {
            int stage = 0, lt = 0;
            uint32_t phase = 0;
            for (int u = blockIdx.x; u < total && !*s_abort; u += gridDim.x, ++lt) {
                const int buf = lt & 1;
                const uint32_t tph = (uint32_t)((lt >> 1) & 1);
                if (!mbar_wait(&tempty[buf], tph ^ 1u, s_abort, P.err, 12)) break;
                xfence_after();
                const uint32_t d0 = tmem_base + (uint32_t)(buf * XCLS_COLS);
                bool ok = true;
                for (int kb = 0; kb < P.kb_total; ++kb) {
                    if (!mbar_wait(&full[stage], phase, s_abort, P.err, 13)) { ok = false; break; }
                    xfence_after();
                    const uint32_t st = smem_u32(smem + (size_t)stage * XSTAGE_BYTES);
                    const uint64_t db = xdesc(st + kQ * XA_PLANE);
#pragma unroll
                    for (int kk = 0; kk < XBK / 16; ++kk) {
                        const uint64_t adv = (uint64_t)(kk * 2);  // 32 bytes per K=16 step
#pragma unroll
                        for (int q = 0; q < kQ; ++q) {
                            // M plane q against R planes 0 .. NP-1-q: class p + q at columns 32 (p + q)
                            const uint64_t da = xdesc(st + q * XA_PLANE);
                            xmma(d0 + (uint32_t)(q * XBN), da + adv, db + adv,
                                 xidesc((NP - q) * XBN), (kb > 0 || kk > 0 || q > 0) ? 1u : 0u);
                        }
                    }
                    xcommit(&empty[stage]);
                    if (++stage == XSTAGES) {
                        stage = 0;
                        phase ^= 1u;
                    }
                }
                if (!ok) break;
                xcommit(&tfull[buf]);
            }
            if (*s_abort) {
                xcommit(drain);
                volatile int never = 0;
                int dummy = 0;
                mbar_wait(drain, 0, &never, &dummy, 0);
            }
        }
    } else {
        // ---------------- epilogue (warps 2-9): warp covers TMEM lanes 32 (warp & 3) ..,
        // vectors 16 h .. 16 h + 15 of the tile
        const int qd = warp & 3, h = (warp - 2) >> 2;
        const bool per_c = P.m_negative || *P.negflag;  // Σ c from the column sums does not hold
        int lt = 0;
        for (int u = blockIdx.x; u < total; u += gridDim.x, ++lt) {
            const int mt = u / P.n_vt, vt = u - mt * P.n_vt;
            const int buf = lt & 1;
            const uint32_t tph = (uint32_t)((lt >> 1) & 1);
            const int64_t i = (int64_t)mt * XBM + 32 * qd + lane;  // this lane's bin
            const bool live = i < P.nbins;
            float nh = 0.f, nl = 0.f;
            if (live) sfh_split_double(__ldg(P.data + i), nh, nl);
            const float es = live ? __ldg(P.escale + i) : 0.f;
            float rsv[16];  // the 16 vectors' scales 2^S_b, loaded while the MMAs run
#pragma unroll
            for (int k = 0; k < 16; ++k) rsv[k] = __ldg(P.rscale + vt * XBN + 16 * h + k);
            if (!mbar_wait(&tfull[buf], tph, s_abort, P.err, 14)) break;
            __syncwarp();  // the lanes left the wait at different polls: reconverge for tcgen05.ld
            xfence_after();
            const uint32_t tb = tmem_base + ((uint32_t)(32 * qd) << 16) + (uint32_t)(buf * XCLS_COLS) +
                                (uint32_t)(16 * h);
            sfh_df tv[16];
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                __syncwarp();
                float acc[kPMax][8];
#pragma unroll
                for (int s = 0; s < kPMax; ++s) {
                    if (s < NP) {
                        xld8(tb + (uint32_t)(s * XBN + 8 * half), acc[s]);
                    } else {
#pragma unroll
                        for (int e = 0; e < 8; ++e) acc[s][e] = 0.f;
                    }
                }
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int vv = 16 * h + 8 * half + e;
                    const int b = vt * XBN + vv;
                    // Σ_s 2^{-6s} A_s (each A_s an exact integer): A_0 + 2^-6 A_1 error-free,
                    // the classes from 2 on (below 2^-11 of the sum) in FP32, then the
                    // power-of-two scale 2^{E_i + S_b - 12}
                    float tail = 0.f;
#pragma unroll
                    for (int s = kPMax - 1; s >= 2; --s)
                        if (s < NP) tail = fmaf(acc[s][e], __uint_as_float((uint32_t)(127 - 6 * s) << 23), tail);
                    sfh_df c = df_two_sum(acc[0][e], acc[1][e] * 0.015625f);
                    c = df_two_sum(c.h, c.l + tail);
                    const float sc = es * rsv[8 * half + e] * 2.44140625e-4f;  // 2^-12
                    c = sfh_df{c.h * sc, c.l * sc};
                    if (c.h < P.eps || (c.h == P.eps && c.l < 0.f)) c = sfh_df{P.eps, 0.f};
                    sfh_df t{0.f, 0.f};
                    float w = 0.f;  // padding bins carry w = 0 into G = W M
                    if (live && b < P.B) {
                        // w = 1 - n/c to FP32 accuracy (it enters G as BF16 hi + lo)
                        w = __fdividef(c.h - nh, c.h);
                        if (nh != 0.f || nl != 0.f) {  // n log c, the per-bin part of logL
                            sfh_df lc = df_log_f_fast(c.h, s_tab);  // c >= eps: a normal float
                            lc = df_add_f(lc, __fdividef(c.l, c.h));
                            t = df_mul(lc, sfh_df{nh, nl});
                        }
                        if (per_c) t = df_add(t, df_neg(c));  // -max(c, eps) per bin
                    }
                    if (P.want_w && b < P.B && i < P.w_ld) {
                        const __nv_bfloat16 wh = __float2bfloat16_rn(w);
                        P.W_hi[(int64_t)b * P.w_ld + i] = wh;
                        P.W_lo[(int64_t)b * P.w_ld + i] = __float2bfloat16_rn(w - __bfloat162float(wh));
                    }
                    tv[8 * half + e] = t;
                }
            }
            __syncwarp();
            // TMEM drained: the MMA warp may refill this buffer
            xfence_before();
            mbar_arrive(&tempty[buf]);
            // sum over the warp's 32 bins per vector: fold lanes l and l ^ 16, then recursive
            // halving (lane l ends with vector l & 15)
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                const sfh_df o{__shfl_xor_sync(0xffffffffu, tv[k].h, 16), __shfl_xor_sync(0xffffffffu, tv[k].l, 16)};
                tv[k] = df_add_fast(tv[k], o);
            }
#pragma unroll
            for (int o = 8; o >= 1; o >>= 1) {
                const bool upper = (lane & o) != 0;
#pragma unroll
                for (int k = 0; k < o; ++k) {
                    const sfh_df send = upper ? tv[k] : tv[k + o];
                    const sfh_df keep = upper ? tv[k + o] : tv[k];
                    const sfh_df got{__shfl_xor_sync(0xffffffffu, send.h, o), __shfl_xor_sync(0xffffffffu, send.l, o)};
                    tv[k] = df_add_fast(keep, got);
                }
            }
            // after the halving lane l holds vector (l & 15) of this warp's half: the bit
            // order of the halving makes the kept index equal to the lane's low bits.  One
            // partial per (bin tile, lane quarter, vector); no barrier among the epilogue warps
            if (lane < 16)
                P.lpart[((int64_t)mt * 4 + qd) * P.B_pad + vt * XBN + 16 * h + lane] =
                    make_float2(tv[0].h, tv[0].l);
        }
    }
    xfence_before();
    __syncthreads();
    if (warp == 1) {
        xfence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                     "r"(XTMEM_COLS)
                     : "memory");
    }
}

// M digit planes: plane q row i (bin) column j (template) = e_q,ij; rows nbins..nbins_pad
// and columns nt..nt_pad zero.  One thread per (bin, template) of a 32 x 32 tile, read
// through shared memory so both the column-major read and the row-major write coalesce.
__global__ void k_m_digits(const float *__restrict__ M, const float2 *__restrict__ rowb,
                           int64_t nbins, int64_t nt, int64_t nbins_pad, int64_t nt_pad,
                           __nv_bfloat16 *__restrict__ planes, float *__restrict__ escale) {
    __shared__ float tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    for (int r = ty; r < 32; r += 8) {
        const int64_t i = i0 + tx, j = j0 + r;
        tile[r][tx] = (i < nbins && j < nt) ? M[j * nbins + i] : 0.f;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int64_t i = i0 + r, j = j0 + tx;
        if (i >= nbins_pad || j >= nt_pad) continue;
        float mx = 0.f;
        if (i < nbins) mx = rowb[i].y;
        int e = 0;
        if (mx > 0.f) frexpf(mx, &e);  // mx < 2^e
        if (j == 0 && i < nbins) escale[i] = ldexpf(1.f, e);
        float x = ldexpf(tile[tx][r], -e) * 64.f;  // |x| < 64: exact
        for (int q = 0; q < kQ; ++q) {
            const float d = rintf(x);
            planes[(int64_t)q * nbins_pad * nt_pad + i * nt_pad + j] = __float2bfloat16_rn(d);
            x = (x - d) * 64.f;  // exact: |x - d| <= 1/2
        }
    }
}

// R digit planes: one block per vector b (B_pad blocks): S_b from max_j |R_bj|, then
// plane p row b column j = d_p,bj for p < 8 (balanced base-64 digits of R_bj / S_b to
// 2^-43, from integer arithmetic on the mantissa); padding rows and
// columns zero.  The planes a launch needs: P = 6 while the ratio of the largest to the
// smallest nonzero |R_bj| stays below 2^19, 7 below 2^25, else 8 (the maximum over the
// batch, by atomicMax into *nplanes, which the caller zeroes first).
__global__ void k_r_digits(const double *__restrict__ R, int64_t B, int64_t nt, int64_t B_pad,
                           int64_t nt_pad, __nv_bfloat16 *__restrict__ planes,
                           float *__restrict__ rscale, int *__restrict__ nplanes,
                           const double *__restrict__ colsum, double *__restrict__ csum,
                           int *__restrict__ negflag, const double *__restrict__ colsum_e,
                           double *__restrict__ csum_e) {
    // integer operations wherever the result is exact (max / min of |R| on the bit patterns,
    // the digits from the mantissa): FP64 is the slow pipe; the two dot products stay FP64
    __shared__ double s_d[2][32];
    __shared__ unsigned long long s_m[2][32];
    const int64_t b = blockIdx.x;
    unsigned long long mxb = 0ull, mnb = ~0ull;  // |R| bit patterns: monotone in the value
    double dot = 0.0, dote = 0.0;
    bool neg = false;
    if (b < B)
        for (int64_t j = threadIdx.x; j < nt; j += blockDim.x) {
            const double v = R[b * nt + j];
            const unsigned long long ab = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
            mxb = ab > mxb ? ab : mxb;
            if (ab) mnb = ab < mnb ? ab : mnb;
            dot = fma(v, colsum[j], dot);  // Σ_j R_bj Σ_i M_ij = Σ_i c_bi
            if (colsum_e) dote = fma(v, colsum_e[j], dote);  // Σ over a parent's empty bins
            neg |= __double_as_longlong(v) < 0 && ab;
        }
    if (neg) atomicOr(negflag, 1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long a1 = __shfl_xor_sync(0xffffffffu, mxb, o);
        const unsigned long long a2 = __shfl_xor_sync(0xffffffffu, mnb, o);
        mxb = a1 > mxb ? a1 : mxb;
        mnb = a2 < mnb ? a2 : mnb;
        dot += __shfl_xor_sync(0xffffffffu, dot, o);
        dote += __shfl_xor_sync(0xffffffffu, dote, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s_m[0][threadIdx.x >> 5] = mxb;
        s_m[1][threadIdx.x >> 5] = mnb;
        s_d[0][threadIdx.x >> 5] = dot;
        s_d[1][threadIdx.x >> 5] = dote;
    }
    __syncthreads();
    mxb = 0ull;
    mnb = ~0ull;
    dot = 0.0;
    dote = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        mxb = s_m[0][w] > mxb ? s_m[0][w] : mxb;
        mnb = s_m[1][w] < mnb ? s_m[1][w] : mnb;
        dot += s_d[0][w];
        dote += s_d[1][w];
    }
    if (threadIdx.x == 0) {
        csum[b] = dot;
        if (colsum_e) csum_e[b] = dote;
    }
    const double mx = __longlong_as_double((long long)mxb);
    int e = 0;
    if (mx > 0.0) frexp(mx, &e);  // mx = f 2^e, f in [0.5, 1): |R_bj| < 2^e
    if (e < -120) e = -120;  // the scale stays a normal float
    if (e > 120) e = 120;
    if (threadIdx.x == 0) {
        rscale[b] = ldexpf(1.f, e);
        if (b < B && mx > 0.0) {
            const double bits = log2(mx / __longlong_as_double((long long)mnb));
            atomicMax(nplanes, bits <= 19.0 ? 6 : bits <= 25.0 ? 7 : 8);
        }
    }
    // X = round(R_bj 2^(48 - e)) (|X| < 2^48: x = R 2^(6 - e) in units of 2^-42), then its
    // balanced base-64 digits from the top: d_p = round(X_p / 2^(42 - 6p)), X_{p+1} = X_p -
    // d_p 2^(42 - 6p); |d_0| <= 64, |d_p| <= 32, Σ_p d_p 64^-p = x to 2^-43
    for (int64_t j = threadIdx.x; j < nt_pad; j += blockDim.x) {
        long long X = 0;
        if (b < B && j < nt) {
            const unsigned long long vb = (unsigned long long)__double_as_longlong(R[b * nt + j]);
            const int E = (int)((vb >> 52) & 0x7ffu);
            if (E) {  // subnormals are far below 2^(e - 48) unless every entry is: zero
                const long long m = (long long)((vb & 0xfffffffffffffull) | (1ull << 52));
                // m 2^(E - 1075 + 48 - e) = m / 2^sh, sh >= 5 for |R| < 2^e (sh is held at 5
                // for coefficients beyond the clamped scale, 2^120)
                const int sh = max(5, 1075 - 48 + e - E);
                X = sh < 63 ? (m + (1ll << (sh - 1))) >> sh : 0;
                if (vb >> 63) X = -X;
            }
        }
        for (int p = 0; p < kPMax; ++p) {
            const int sh = 42 - 6 * p;
            const long long d = sh ? (X + (1ll << (sh - 1))) >> sh : X;
            X -= d << sh;
            planes[((int64_t)p * B_pad + b) * nt_pad + j] = __float2bfloat16_rn((float)d);
        }
    }
}

// -logL_b = -(Σ_tiles (hi + lo) - Σ_i c_bi + Σ_i (n_i - n_i log n_i)), fixed order; an
// exactly zero sum gives -typemax semantics (fitting_base.jl:95).
__global__ void k_logl_reduce_x(const float2 *__restrict__ part, int n_mt, int B, int B_pad,
                                const double *__restrict__ csum, const int *__restrict__ negflag,
                                int m_negative, const double *__restrict__ kn,
                                double *__restrict__ negLogL, const double *__restrict__ csum_e) {
    // one warp per vector: lane l sums partials l, l + 32, ... in double-float (FP32 pipes),
    // then a fixed shuffle tree
    const int b = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (b >= B) return;  // whole warps leave together
    sfh_df acc{0.f, 0.f};
    for (int t = lane; t < n_mt; t += 32) {
        const float2 v = part[(int64_t)t * B_pad + b];
        acc = df_add(acc, df_two_sum(v.x, v.y));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const sfh_df u{__shfl_down_sync(0xffffffffu, acc.h, o), __shfl_down_sync(0xffffffffu, acc.l, o)};
        acc = df_add(acc, u);
    }
    if (lane) return;
    double a = sfh_f2d(acc.h) + sfh_f2d(acc.l);
    if (!(m_negative || *negflag)) a -= csum[b];  // else the epilogue subtracted each c
    else if (csum_e) a -= csum_e[b];  // and a derived handle's parent's empty bins remain
    a += *kn;
    negLogL[b] = (a != 0.0) ? -a : INFINITY;
}

// Σ_{i: n_i > 0} (n_i - n_i log n_i) in FP64: each block a contiguous chunk (the log runs on
// the FP64 pipe, so the work is spread over the SMs), the last block sums the block partials
// in block order (fixed order, reproducible) and re-arms the ticket.
constexpr int kDcBlocks = 64;
__global__ void k_data_const(const double *__restrict__ n, int64_t nbins, double *__restrict__ part,
                             unsigned int *ticket, double *__restrict__ kn) {
    __shared__ double s[32];
    __shared__ bool last;
    const int64_t per = (nbins + gridDim.x - 1) / gridDim.x;
    const int64_t i0 = (int64_t)blockIdx.x * per, i1 = min(nbins, i0 + per);
    double a = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const double v = n[i];
        if (v > 0.0) a += v - v * log(v);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
        part[blockIdx.x] = t;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double t = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) t += ((volatile double *)part)[b];
        *kn = t;
        *ticket = 0u;
    }
}

// Column sums Σ_i M_ij in FP64 (one block per template) and whether any value is negative.
__global__ void k_colsum(const float *__restrict__ M, int64_t nbins, double *__restrict__ colsum,
                         int *__restrict__ negative) {
    __shared__ double s[32];
    const int64_t j = blockIdx.x;
    double a = 0.0;
    bool neg = false;
    for (int64_t i = threadIdx.x; i < nbins; i += blockDim.x) {
        const float v = M[j * nbins + i];
        a += (double)v;
        neg |= v < 0.f;
    }
    if (neg) atomicOr(negative, 1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
        colsum[j] = t;
    }
}

int xmake_map(sfh_ctx *ctx, CUtensorMap *map, const void *base, int64_t rows, int64_t cols,
              int box_rows) {
    auto enc = sfh_tensor_map_encoder();
    if (!enc) return sfh_set_error(ctx, SFH_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    if (((uintptr_t)base & 15) || ((cols * 2) & 15))
        return sfh_set_error(ctx, SFH_ERR_ARG, "tensor base/stride not 16-byte aligned");
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(cols * 2)};
    cuuint32_t box[2] = {(cuuint32_t)XBK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims,
                     strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return sfh_set_error(ctx, SFH_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    return SFH_OK;
}

}  // namespace

bool sfh_exact_supported(const sfh_models *m) {
    return m->digits && m->nt_pad <= 2304;
}

int sfh_build_digit_planes(sfh_ctx *ctx, sfh_models *m) {
    if (!m->d_f32 || !m->d_rowb) return sfh_set_error(ctx, SFH_ERR_ARG, "no FP32 templates");
    if (m->nt_pad == 0) m->nt_pad = ((m->nt + 63) / 64) * 64;
    if (m->nt_pad > 2304) return SFH_OK;  // class sums could pass 2^24: no exact planes
    m->nbins_pad128 = ((m->nbins + XBM - 1) / XBM) * XBM;
    const size_t n = (size_t)kQ * m->nbins_pad128 * m->nt_pad;
    SFH_CK(ctx, cudaMalloc(&m->digits, n * 2));
    SFH_CK(ctx, cudaMalloc(&m->escale, (size_t)m->nbins * sizeof(float)));
    dim3 grid((unsigned)(m->nbins_pad128 / 32), (unsigned)(m->nt_pad / 32)), block(32, 8);
    k_m_digits<<<grid, block, 0, ctx->stream>>>(m->d_f32, m->d_rowb, m->nbins, m->nt,
                                               m->nbins_pad128, m->nt_pad, m->digits, m->escale);
    SFH_LAUNCHED(ctx);
    // column sums (FP64) and, in the slot after them, whether any template value is negative
    const size_t o_flag = sfh_align256((size_t)m->nt * sizeof(double));
    SFH_CK(ctx, cudaMalloc(&m->colsum, o_flag + 256));
    int *neg = (int *)((char *)m->colsum + o_flag);
    SFH_CK(ctx, cudaMemsetAsync(neg, 0, sizeof(int), ctx->stream));
    k_colsum<<<(unsigned)m->nt, 256, 0, ctx->stream>>>(m->d_f32, m->nbins, m->colsum, neg);
    SFH_LAUNCHED(ctx);
    int hneg = 0;
    SFH_CK(ctx, cudaMemcpyAsync(&hneg, neg, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    m->m_negative = hneg;
    return SFH_OK;
}

size_t sfh_exact_scratch(const sfh_models *m, int64_t B, int64_t *B_pad_out) {
    const int64_t B_pad = ((B + XBN - 1) / XBN) * XBN;
    const int64_t n_mt = m->nbins_pad128 / XBM;
    if (B_pad_out) *B_pad_out = B_pad;
    return sfh_align256((size_t)kPMax * B_pad * m->nt_pad * 2) + sfh_align256((size_t)B_pad * 4) +
           256 + 2 * sfh_align256((size_t)B_pad * 8) + 256 + sfh_align256(kDcBlocks * 8) +
           sfh_align256((size_t)n_mt * 4 * B_pad * sizeof(float2));
}

int sfh_exact_prepare(sfh_ctx *ctx, const sfh_models *m, int64_t B, void *scratch,
                      SfhExactPlan *xp) {
    int64_t B_pad = 0;
    const size_t bytes = sfh_exact_scratch(m, B, &B_pad);
    (void)bytes;
    char *s = (char *)scratch;
    xp->B = B;
    xp->B_pad = B_pad;
    xp->n_mt = (int)(m->nbins_pad128 / XBM);
    xp->n_vt = (int)(B_pad / XBN);
    xp->Rd = (__nv_bfloat16 *)s;
    s += sfh_align256((size_t)kPMax * B_pad * m->nt_pad * 2);
    xp->rscale = (float *)s;
    s += sfh_align256((size_t)B_pad * 4);
    xp->nplanes = (int *)s;        // [0] planes, [1] negative-coefficient flag
    xp->kn = (double *)(s + 128);  // Σ (n - n log n)
    s += 256;
    xp->csum = (double *)s;
    s += sfh_align256((size_t)B_pad * 8);
    xp->csum_e = (double *)s;
    s += sfh_align256((size_t)B_pad * 8);
    xp->kpart = (double *)s;
    s += sfh_align256(kDcBlocks * 8);
    xp->lpart = (float2 *)s;
    int rc;
    if ((rc = xmake_map(ctx, &xp->maps[0], m->digits, (int64_t)kQ * m->nbins_pad128, m->nt_pad, XBM)))
        return rc;
    if ((rc = xmake_map(ctx, &xp->maps[1], xp->Rd, (int64_t)kPMax * B_pad, m->nt_pad, XBN))) return rc;
    return SFH_OK;
}

int sfh_exact_launch(sfh_ctx *ctx, const sfh_models *m, const SfhExactPlan &xp, const double *d_R,
                     const double *d_data, double *d_negLogL, __nv_bfloat16 *W_hi,
                     __nv_bfloat16 *W_lo, int64_t w_ld, int want_w, double eps, int *d_err) {
    static bool attr = false;
    if (!attr) {
        SFH_CK(ctx, cudaFuncSetAttribute(k_tc_exact, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kXSmem));
        attr = true;
    }
    cudaStream_t st = ctx->stream;
    SFH_CK(ctx, cudaMemsetAsync(xp.nplanes, 0, 3 * sizeof(int), st));  // planes, flag, ticket
    k_r_digits<<<(unsigned)xp.B_pad, 256, 0, st>>>(d_R, xp.B, m->nt, xp.B_pad, m->nt_pad, xp.Rd,
                                                    xp.rscale, xp.nplanes, m->colsum, xp.csum,
                                                    xp.nplanes + 1, m->colsum_e, xp.csum_e);
    SFH_LAUNCHED(ctx);
    if (d_negLogL) {
        k_data_const<<<kDcBlocks, 256, 0, st>>>(d_data, m->nbins, xp.kpart,
                                                (unsigned int *)(xp.nplanes + 2), xp.kn);
        SFH_LAUNCHED(ctx);
    }
    ExactParams P{};
    P.n_mt = xp.n_mt;
    P.n_vt = xp.n_vt;
    P.kb_total = (int)(m->nt_pad / XBK);
    P.nbins = m->nbins;
    P.nbins_pad = m->nbins_pad128;
    P.B = (int)xp.B;
    P.B_pad = (int)xp.B_pad;
    P.data = d_data;
    P.escale = m->escale;
    P.rscale = xp.rscale;
    P.nplanes = xp.nplanes;
    P.negflag = xp.nplanes + 1;
    P.m_negative = m->m_negative;
    P.eps = (float)fmax(eps, 1.1754943508222875e-38);
    P.tab = ctx->d_df_tab;
    P.W_hi = W_hi;
    P.W_lo = W_lo;
    P.w_ld = w_ld;
    P.want_w = want_w;
    P.lpart = xp.lpart;
    P.err = d_err;
    const int total = xp.n_mt * xp.n_vt;
    const int grid = total < ctx->sm_count ? total : ctx->sm_count;
    k_tc_exact<<<grid, kXThreads, kXSmem, st>>>(xp.maps[0], xp.maps[1], P);
    SFH_LAUNCHED(ctx);
    if (d_negLogL) {
        k_logl_reduce_x<<<(unsigned)((xp.B * 32 + 255) / 256), 256, 0, st>>>(
            xp.lpart, 4 * xp.n_mt, (int)xp.B, (int)xp.B_pad, xp.csum, xp.nplanes + 1, m->m_negative,
            xp.kn, d_negLogL, m->colsum_e ? xp.csum_e : nullptr);
        SFH_LAUNCHED(ctx);
    }
    return SFH_OK;
}
