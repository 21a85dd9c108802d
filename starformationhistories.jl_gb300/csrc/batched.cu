// batched.cu -- many coefficient vectors against one template matrix on the
// 5th-generation tensor cores (tcgen05, sm_103a).
//
// B coefficient vectors r_b (HMC chains, line-search probes) are evaluated at once:
//   C = R Mᵀ      (B x nbins)   composite!  for every vector      fitting_base.jl:55-65
//   W = 1 - N/max(C, eps)       ∇loglikelihood! weights            fitting_base.jl:274-280
//   logL_b = Σ_i term(C_bi, n_i)                                   fitting_base.jl:84-96
//   G = W M       (B x nt)      = -∇logL for every vector (fg!)    fitting_base.jl:283, solvers.jl:20-38
// Both products run as persistent tcgen05 GEMMs with BF16 operands split into hi/lo
// planes (x = hi + lo, 16 significant bits) and three products per k-step
// (hi·hi + hi·lo + lo·hi) accumulated in FP32 in tensor memory.
//
// Kernel structure (k_tc_gemm, one CTA per SM, 192 threads):
//   warp 0     TMA producer: 2-stage ring of {A_hi, A_lo, B_hi, B_lo} tiles (128B swizzle)
//   warp 1     allocates 512 TMEM columns; lane 0 issues tcgen05.mma (M=128, N=256, K=16)
//   warps 2-9  epilogue: tcgen05.ld of the finished accumulator (double-buffered in TMEM);
//              two warps per TMEM lane quarter, each taking half of the 256 columns
// Every mbarrier wait is bounded: on timeout the kernel records an error, stops the
// other roles through a shared flag, drains what it issued and frees its TMEM.
//
// Storage of the template matrix for this path (models with SFH_BF16X2):
//   row planes (nbins, nt_pad) row-major:  K = templates, the B operand of C = R Mᵀ
//   col planes (nt, nbins_pad) row-major:  K = bins,      the B operand of G = W M
// nt_pad / nbins_pad round up to 64; padding is zero.  Tiles that run past the last
// row are zero-filled by the TMA unit.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "sfh_internal.cuh"
#include "sfh_ptx.cuh"

namespace {

constexpr int BM = 128;   // rows of A per tile (coefficient vectors)
constexpr int BN = 256;   // rows of B per tile (bins or templates)
constexpr int BK = 64;    // K per stage (64 BF16 = one 128-byte swizzle span)
constexpr int STAGES = 2;
constexpr int A_BYTES = BM * BK * 2;               // 16 KB per plane
constexpr int B_BYTES = BN * BK * 2;               // 32 KB per plane
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;  // 96 KB
constexpr int TMEM_COLS = 512;                     // two 128 x 256 FP32 accumulators
constexpr int kGemmThreads = 320;  // producer, MMA, 8 epilogue warps
constexpr int kEpiThreads = 256;
constexpr size_t kGemmSmem = 1024 + (size_t)STAGES * STAGE_BYTES + 256;

// Instruction descriptor, kind::f16: D = F32 (bits 4-5), A = B = BF16 (bits 7-9, 10-12),
// both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

struct GemmParams {
    int m_tiles, n_tiles, ksplit, kb_total, kb_per_split;
    int epi;  // 0: composite epilogue (W, logL partials); 1: G partials
    // epilogue 0
    const float *data;
    int64_t nbins;
    int B, B_pad;
    float eps;
    __nv_bfloat16 *W_hi, *W_lo;
    int64_t w_ld;  // = nbins_pad
    int want_w, want_logl;
    float2 *logl_part;  // [n_tiles * 2][B_pad] (two column halves per tile)
    // epilogue 1
    float *Gpart;  // [ksplit][B_pad][nt]
    int64_t nt;
    int *err;
};

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major tile, rows of 128 bytes, 128-byte swizzle,
// 8-row core groups 1024 bytes apart (SBO), descriptor version 1 (bit 46).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;                 // LBO (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;       // SBO
    d |= (uint64_t)1 << 46;                 // version
    d |= (uint64_t)2 << 61;                 // SWIZZLE_128B
    return d;
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(kIdesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

// 32 consecutive FP32 accumulator columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
        "%28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void decode(const GemmParams &P, int u, int &m, int &n, int &ks) {
    if (P.epi == 0) {  // bins outer: concurrent tiles share one block of the template matrix
        n = u / P.m_tiles;
        m = u - n * P.m_tiles;
        ks = 0;
    } else {           // K slab outer, then vectors, templates inner
        const int per = P.m_tiles * P.n_tiles;
        ks = u / per;
        const int r = u - ks * per;
        m = r / P.n_tiles;
        n = r - m * P.n_tiles;
    }
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// ------------------------------------------------------------------ the GEMM kernel
__global__ void __launch_bounds__(kGemmThreads, 1)
k_tc_gemm(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
          const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl,
          const GemmParams P) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bar = (uint64_t *)(smem + (size_t)STAGES * STAGE_BYTES);
    uint64_t *full = bar, *empty = bar + STAGES, *tfull = bar + 2 * STAGES,
             *tempty = bar + 2 * STAGES + 2, *drain = bar + 2 * STAGES + 4;
    uint32_t *tmem_slot = (uint32_t *)(bar + 2 * STAGES + 5);
    volatile int *s_abort = (volatile int *)(tmem_slot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], kEpiThreads);
        }
        mbar_init(drain, 1);
        *s_abort = 0;
        fence_barrier_init();
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    const int total = P.ksplit * P.m_tiles * P.n_tiles;

    if (warp == 0) {
        // ---------------- TMA producer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            int issued = 0;
            for (int u = blockIdx.x; u < total && !*s_abort; u += gridDim.x) {
                int m, n, ks;
                decode(P, u, m, n, ks);
                const int kb0 = ks * P.kb_per_split;
                const int kb1 = min(P.kb_total, kb0 + P.kb_per_split);
                for (int kb = kb0; kb < kb1; ++kb) {
                    if (!mbar_wait(&empty[stage], phase ^ 1u, s_abort, P.err, 1)) break;
                    uint8_t *st = smem + (size_t)stage * STAGE_BYTES;
                    mbar_expect_tx(&full[stage], STAGE_BYTES);
                    tma_load_2d(st, &tAh, kb * BK, m * BM, &full[stage]);
                    tma_load_2d(st + A_BYTES, &tAl, kb * BK, m * BM, &full[stage]);
                    tma_load_2d(st + 2 * A_BYTES, &tBh, kb * BK, n * BN, &full[stage]);
                    tma_load_2d(st + 2 * A_BYTES + B_BYTES, &tBl, kb * BK, n * BN, &full[stage]);
                    ++issued;
                    if (++stage == STAGES) {
                        stage = 0;
                        phase ^= 1u;
                    }
                }
            }
            if (*s_abort) {
                // Drain: the last min(issued, STAGES) loads may still be landing.
                volatile int never = 0;
                int dummy = 0;
                for (int k = 0; k < STAGES && k < issued; ++k) {
                    if (--stage < 0) {
                        stage = STAGES - 1;
                        phase ^= 1u;
                    }
                    mbar_wait(&full[stage], phase, &never, &dummy, 0);
                }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            int lt = 0;
            for (int u = blockIdx.x; u < total && !*s_abort; u += gridDim.x, ++lt) {
                int m, n, ks;
                decode(P, u, m, n, ks);
                const int kb0 = ks * P.kb_per_split;
                const int kb1 = min(P.kb_total, kb0 + P.kb_per_split);
                const int buf = lt & 1;
                const uint32_t tph = (uint32_t)((lt >> 1) & 1);
                if (!mbar_wait(&tempty[buf], tph ^ 1u, s_abort, P.err, 2)) break;
                tc_fence_after();
                const uint32_t d_tmem = tmem_base + (uint32_t)(buf * BN);
                bool ok = true;
                for (int kb = kb0; kb < kb1; ++kb) {
                    if (!mbar_wait(&full[stage], phase, s_abort, P.err, 3)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t st = smem_u32(smem + (size_t)stage * STAGE_BYTES);
                    const uint64_t dah = smem_desc(st), dal = smem_desc(st + A_BYTES);
                    const uint64_t dbh = smem_desc(st + 2 * A_BYTES);
                    const uint64_t dbl = smem_desc(st + 2 * A_BYTES + B_BYTES);
#pragma unroll
                    for (int kk = 0; kk < BK / 16; ++kk) {
                        const uint64_t adv = (uint64_t)(kk * 2);  // 32 bytes per K=16 step
                        mma_bf16(d_tmem, dah + adv, dbh + adv, (kb > kb0 || kk > 0) ? 1u : 0u);
                        mma_bf16(d_tmem, dah + adv, dbl + adv, 1u);
                        mma_bf16(d_tmem, dal + adv, dbh + adv, 1u);
                    }
                    mma_commit(&empty[stage]);  // the stage is free once these MMAs finish
                    if (++stage == STAGES) {
                        stage = 0;
                        phase ^= 1u;
                    }
                }
                if (!ok) break;
                mma_commit(&tfull[buf]);
            }
            if (*s_abort) {
                // Make sure no MMA is still writing TMEM before it is freed.
                mma_commit(drain);
                volatile int never = 0;
                int dummy = 0;
                mbar_wait(drain, 0, &never, &dummy, 0);
            }
        }
    } else {
        // ---------------- epilogue (warps 2-9)
        const int q = warp & 3;                 // TMEM lane quarter this warp may access
        const int half = (warp - 2) >> 2;       // which 128 of the 256 columns
        const int row = 32 * q + lane;          // accumulator row = coefficient vector in tile
        int lt = 0;
        for (int u = blockIdx.x; u < total; u += gridDim.x, ++lt) {
            int m, n, ks;
            decode(P, u, m, n, ks);
            const int buf = lt & 1;
            const uint32_t tph = (uint32_t)((lt >> 1) & 1);
            if (!mbar_wait(&tfull[buf], tph, s_abort, P.err, 4)) break;
            tc_fence_after();
            const int b = m * BM + row;
            const uint32_t tbase = tmem_base + ((uint32_t)(32 * q) << 16) +
                                   (uint32_t)(buf * BN + half * (BN / 2));
            if (P.epi == 0) {
                const int64_t i0 = (int64_t)n * BN + half * (BN / 2);
                // four independent compensated sums keep the dependency chains short
                float th[4] = {0.f, 0.f, 0.f, 0.f}, tl[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
                for (int c = 0; c < BN / 64; ++c) {
                    float v[32];
                    tmem_ld32(tbase + (uint32_t)(c * 32), v);
                    const int64_t ic = i0 + c * 32;
                    float w[32];
#pragma unroll
                    for (int e = 0; e < 32; ++e) {
                        const int64_t i = ic + e;
                        w[e] = 0.f;
                        if (i < P.nbins) {
                            const float ni = __ldg(P.data + i);  // warp-uniform address
                            const float ci = fmaxf(v[e], P.eps);
                            const float df = ci - ni;
                            w[e] = __fdividef(df, ci);  // 1 - n/c
                            if (P.want_logl) {
                                const float t = (ni > 0.f)
                                                    ? ni * sfh_log1p_minus_id(__fdividef(df, ni), ci, ni)
                                                    : -ci;
                                sfh_two_sum_acc(th[e & 3], tl[e & 3], t);
                            }
                        }
                    }
                    if (P.want_w && b < P.B && ic < P.w_ld) {
                        __nv_bfloat16 *dh = P.W_hi + (int64_t)b * P.w_ld + ic;
                        __nv_bfloat16 *dl = P.W_lo + (int64_t)b * P.w_ld + ic;
#pragma unroll
                        for (int g = 0; g < 4; ++g) {
                            uint32_t hh[4], ll[4];
#pragma unroll
                            for (int h = 0; h < 4; ++h) {
                                const float a0 = w[8 * g + 2 * h], a1 = w[8 * g + 2 * h + 1];
                                const __nv_bfloat16 b0 = __float2bfloat16_rn(a0);
                                const __nv_bfloat16 b1 = __float2bfloat16_rn(a1);
                                hh[h] = pack_bf16(__bfloat162float(b0), __bfloat162float(b1));
                                ll[h] = pack_bf16(a0 - __bfloat162float(b0), a1 - __bfloat162float(b1));
                            }
                            if (ic + 8 * g + 8 <= P.w_ld) {
                                *reinterpret_cast<uint4 *>(dh + 8 * g) = make_uint4(hh[0], hh[1], hh[2], hh[3]);
                                *reinterpret_cast<uint4 *>(dl + 8 * g) = make_uint4(ll[0], ll[1], ll[2], ll[3]);
                            }
                        }
                    }
                }
                if (P.want_logl && b < P.B_pad) {
                    float h = 0.f, l = 0.f;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        sfh_two_sum_acc(h, l, th[k]);
                        l += tl[k];
                    }
                    P.logl_part[((int64_t)n * 2 + half) * P.B_pad + b] = make_float2(h, l);
                }
            } else {
                const int64_t j0 = (int64_t)n * BN + half * (BN / 2);
                float *dst = P.Gpart + ((int64_t)ks * P.B_pad + b) * P.nt;
#pragma unroll 1
                for (int c = 0; c < BN / 64; ++c) {
                    float v[32];
                    tmem_ld32(tbase + (uint32_t)(c * 32), v);
                    if (b < P.B) {
                        const int64_t jc = j0 + c * 32;
                        if ((P.nt & 3) == 0 && jc + 32 <= P.nt) {
#pragma unroll
                            for (int g = 0; g < 8; ++g)
                                *reinterpret_cast<float4 *>(dst + jc + 4 * g) =
                                    make_float4(v[4 * g], v[4 * g + 1], v[4 * g + 2], v[4 * g + 3]);
                        } else {
#pragma unroll
                            for (int e = 0; e < 32; ++e)
                                if (jc + e < P.nt) dst[jc + e] = v[e];
                        }
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(&tempty[buf]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                     "r"(TMEM_COLS)
                     : "memory");
    }
}

// ------------------------------------------------------------------ helper kernels
// Template planes: row planes (nbins, nt_pad) row-major and col planes (nt, nbins_pad)
// row-major, hi = bf16(M), lo = bf16(M - hi), zero padding.
__global__ void k_split_planes(const float *__restrict__ src, int64_t nbins, int64_t nt,
                               int64_t nbins_pad, int64_t nt_pad,
                               __nv_bfloat16 *__restrict__ col_hi, __nv_bfloat16 *__restrict__ col_lo,
                               __nv_bfloat16 *__restrict__ row_hi, __nv_bfloat16 *__restrict__ row_lo) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // over nt x nbins_pad
    if (idx >= nt * nbins_pad) return;
    const int64_t j = idx / nbins_pad, i = idx - j * nbins_pad;
    const float v = (i < nbins) ? src[j * nbins + i] : 0.f;
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
    col_hi[idx] = h;
    col_lo[idx] = l;
    if (i < nbins) {
        row_hi[i * nt_pad + j] = h;
        row_lo[i * nt_pad + j] = l;
    }
}

__global__ void k_zero_row_pad(__nv_bfloat16 *__restrict__ row_hi, __nv_bfloat16 *__restrict__ row_lo,
                               int64_t nbins, int64_t nt, int64_t nt_pad) {
    const int64_t w = nt_pad - nt;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w <= 0 || idx >= nbins * w) return;
    const int64_t i = idx / w, j = nt + (idx - i * w);
    row_hi[i * nt_pad + j] = __float2bfloat16_rn(0.f);
    row_lo[i * nt_pad + j] = __float2bfloat16_rn(0.f);
}

// Coefficient planes (B_pad, nt_pad): hi = bf16(r), lo = bf16(r - hi), zero padding.
__global__ void k_split_coeffs(const double *__restrict__ R, int64_t B, int64_t nt, int64_t B_pad,
                               int64_t nt_pad, __nv_bfloat16 *__restrict__ hi,
                               __nv_bfloat16 *__restrict__ lo) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B_pad * nt_pad) return;
    const int64_t b = idx / nt_pad, j = idx - b * nt_pad;
    const double r = (b < B && j < nt) ? R[b * nt + j] : 0.0;
    const __nv_bfloat16 h = __float2bfloat16_rn((float)r);
    hi[idx] = h;
    lo[idx] = __float2bfloat16_rn((float)(r - (double)__bfloat162float(h)));
}

__global__ void k_f64_to_f32(const double *__restrict__ x, float *__restrict__ y, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = (float)x[i];
}

// -logL_b = -Σ_tiles (hi + lo), fixed tile order; zero sum -> -typemax semantics.
__global__ void k_logl_reduce(const float2 *__restrict__ part, int n_tiles, int B, int B_pad,
                              double *__restrict__ negLogL) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    double acc = 0.0;
    for (int t = 0; t < n_tiles; ++t) {
        const float2 v = part[(int64_t)t * B_pad + b];
        acc += (double)v.x + (double)v.y;
    }
    negLogL[b] = (acc != 0.0) ? -acc : INFINITY;
}

// G = Σ_ks Gpart[ks], fixed order.
__global__ void k_g_reduce(const float *__restrict__ part, int ksplit, int64_t B, int64_t B_pad,
                           int64_t nt, float *__restrict__ G, const double *__restrict__ colsum_e) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B * nt) return;
    const int64_t b = idx / nt, j = idx - b * nt;
    float hi = 0.f, lo = 0.f;
    for (int s = 0; s < ksplit; ++s) sfh_two_sum_acc(hi, lo, part[((int64_t)s * B_pad + b) * nt + j]);
    // a derived occupied-bin handle: the parent's empty bins, w = 1, enter as E_j
    G[idx] = colsum_e ? (float)((double)hi + (double)lo + colsum_e[j]) : hi + lo;
}

// ------------------------------------------------------------------ host side
// 2-D BF16 tensor (rows x cols, row-major, leading dimension ld elements), box
// (64 columns x box_rows rows), 128-byte swizzle, zero fill outside.
int make_map(sfh_ctx *ctx, CUtensorMap *map, const void *base, int64_t rows, int64_t cols,
             int64_t ld, int box_rows) {
    auto enc = sfh_tensor_map_encoder();
    if (!enc) return sfh_set_error(ctx, SFH_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    if (((uintptr_t)base & 15) || ((ld * 2) & 15))
        return sfh_set_error(ctx, SFH_ERR_ARG, "tensor base/stride not 16-byte aligned");
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims,
                     strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return sfh_set_error(ctx, SFH_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    return SFH_OK;
}

int launch_gemm(sfh_ctx *ctx, const CUtensorMap &ah, const CUtensorMap &al, const CUtensorMap &bh,
                const CUtensorMap &bl, const GemmParams &P) {
    static bool attr = false;
    if (!attr) {
        SFH_CK(ctx, cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kGemmSmem));
        attr = true;
    }
    const int total = P.ksplit * P.m_tiles * P.n_tiles;
    const int grid = total < ctx->sm_count ? total : ctx->sm_count;
    k_tc_gemm<<<grid, kGemmThreads, kGemmSmem, ctx->stream>>>(ah, al, bh, bl, P);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

}  // namespace

int sfh_build_bf16_planes(sfh_ctx *ctx, sfh_models *m, const float *d_f32) {
    m->nbins_pad = ((m->nbins + 63) / 64) * 64;
    m->nt_pad = ((m->nt + 63) / 64) * 64;
    const size_t ncol = (size_t)m->nt * (size_t)m->nbins_pad;
    const size_t nrow = (size_t)m->nbins * (size_t)m->nt_pad;
    SFH_CK(ctx, cudaMalloc(&m->col_hi, ncol * 2));
    SFH_CK(ctx, cudaMalloc(&m->col_lo, ncol * 2));
    SFH_CK(ctx, cudaMalloc(&m->row_hi, nrow * 2));
    SFH_CK(ctx, cudaMalloc(&m->row_lo, nrow * 2));
    const int threads = 256;
    k_split_planes<<<(unsigned)((ncol + threads - 1) / threads), threads, 0, ctx->stream>>>(
        d_f32, m->nbins, m->nt, m->nbins_pad, m->nt_pad, m->col_hi, m->col_lo, m->row_hi, m->row_lo);
    SFH_LAUNCHED(ctx);
    const int64_t npad = m->nbins * (m->nt_pad - m->nt);
    if (npad > 0) {
        k_zero_row_pad<<<(unsigned)((npad + threads - 1) / threads), threads, 0, ctx->stream>>>(
            m->row_hi, m->row_lo, m->nbins, m->nt, m->nt_pad);
        SFH_LAUNCHED(ctx);
    }
    return SFH_OK;
}

int sfh_batched_prepare(sfh_ctx *ctx, const sfh_models *m, int64_t B, const double *d_data,
                        void *scratch, size_t scratch_bytes, SfhBatchedPlan *pl) {
    if (!m->row_hi || !m->col_hi)
        return sfh_set_error(ctx, SFH_ERR_ARG, "models have no BF16 hi/lo planes");
    if (B < 1 || B > (1 << 24)) return sfh_set_error(ctx, SFH_ERR_ARG, "bad number of coefficient vectors");
    const int64_t nbins = m->nbins, nt = m->nt, nbp = m->nbins_pad, ntp = m->nt_pad;
    SfhBatchedPlan P{};
    P.B = B;
    P.B_pad = ((B + BM - 1) / BM) * BM;
    P.m_tiles = (int)(P.B_pad / BM);
    P.n_tiles1 = (int)((nbins + BN - 1) / BN);
    P.n_tiles2 = (int)((nt + BN - 1) / BN);
    // G = W M split over K so that every SM gets work: pick the split that minimises
    // (rounds of work units) x (k-blocks per unit).
    const int kb2 = (int)(nbp / BK);
    int ks2 = 1;
    double best = 1e300;
    for (int ks = 1; ks <= 32 && ks <= kb2; ++ks) {
        const int per = (kb2 + ks - 1) / ks;
        const int units = ks * P.m_tiles * P.n_tiles2;
        const int rounds = (units + ctx->sm_count - 1) / ctx->sm_count;
        const double cost = (double)rounds * per * (1.0 + 0.01 * ks);
        if (cost < best) { best = cost; ks2 = ks; }
    }
    P.per2 = (kb2 + ks2 - 1) / ks2;
    P.ks2 = (kb2 + P.per2 - 1) / P.per2;  // no empty splits
    P.kb2 = kb2;
    const int64_t B_pad = P.B_pad;
    const size_t o_rh = 0, sz_r = sfh_align256((size_t)B_pad * ntp * 2);
    const size_t o_rl = o_rh + sz_r;
    const size_t sz_w = sfh_align256((size_t)B_pad * nbp * 2);
    const size_t o_wh = o_rl + sz_r, o_wl = o_wh + sz_w;
    const size_t o_lp = o_wl + sz_w, sz_lp = sfh_align256((size_t)P.n_tiles1 * 2 * B_pad * sizeof(float2));
    const size_t o_gp = o_lp + sz_lp, sz_gp = sfh_align256((size_t)P.ks2 * B_pad * nt * sizeof(float));
    const size_t o_data = o_gp + sz_gp, sz_data = sfh_align256((size_t)nbins * sizeof(float));
    const size_t o_err = o_data + sz_data;
    P.exact = sfh_exact_supported(m);
    const size_t o_x = o_err + 256;
    P.scratch_bytes = o_x + (P.exact ? sfh_exact_scratch(m, B, nullptr) : 0);
    if (!scratch) {  // size query
        *pl = P;
        return SFH_OK;
    }
    if (scratch_bytes < P.scratch_bytes) return sfh_set_error(ctx, SFH_ERR_ARG, "batched scratch too small");
    char *s = (char *)scratch;
    P.Rh = (__nv_bfloat16 *)(s + o_rh);
    P.Rl = (__nv_bfloat16 *)(s + o_rl);
    P.Wh = (__nv_bfloat16 *)(s + o_wh);
    P.Wl = (__nv_bfloat16 *)(s + o_wl);
    P.lp = (float2 *)(s + o_lp);
    P.gp = (float *)(s + o_gp);
    P.dataf = (float *)(s + o_data);
    P.err = (int *)(s + o_err);
    P.data = d_data;
    int rc;
    if (P.exact && (rc = sfh_exact_prepare(ctx, m, B, s + o_x, &P.xp))) return rc;
    cudaStream_t st = ctx->stream;
    SFH_CK(ctx, cudaMemsetAsync(P.err, 0, sizeof(int), st));
    // data as FP32 (counts are exact below 2^24)
    k_f64_to_f32<<<(unsigned)((nbins + 255) / 256), 256, 0, st>>>(d_data, P.dataf, nbins);
    SFH_LAUNCHED(ctx);
    CUtensorMap *mp = P.maps;
    if ((rc = make_map(ctx, &mp[0], P.Rh, B_pad, ntp, ntp, BM))) return rc;
    if ((rc = make_map(ctx, &mp[1], P.Rl, B_pad, ntp, ntp, BM))) return rc;
    if ((rc = make_map(ctx, &mp[2], m->row_hi, nbins, ntp, ntp, BN))) return rc;
    if ((rc = make_map(ctx, &mp[3], m->row_lo, nbins, ntp, ntp, BN))) return rc;
    if ((rc = make_map(ctx, &mp[4], P.Wh, B_pad, nbp, nbp, BM))) return rc;
    if ((rc = make_map(ctx, &mp[5], P.Wl, B_pad, nbp, nbp, BM))) return rc;
    if ((rc = make_map(ctx, &mp[6], m->col_hi, nt, nbp, nbp, BN))) return rc;
    if ((rc = make_map(ctx, &mp[7], m->col_lo, nt, nbp, nbp, BN))) return rc;
    *pl = P;
    return SFH_OK;
}

int sfh_batched_launch(sfh_ctx *ctx, const sfh_models *m, const SfhBatchedPlan &pl,
                       const double *d_R, double *d_negLogL, float *d_G, double eps) {
    const int64_t nbins = m->nbins, nt = m->nt, nbp = m->nbins_pad, ntp = m->nt_pad;
    const int64_t B = pl.B, B_pad = pl.B_pad;
    const bool want_g = d_G != nullptr, want_l = d_negLogL != nullptr;
    cudaStream_t st = ctx->stream;
    if (!(want_l && pl.exact)) {
        const int64_t n = B_pad * ntp;
        k_split_coeffs<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d_R, B, nt, B_pad, ntp, pl.Rh,
                                                                    pl.Rl);
        SFH_LAUNCHED(ctx);
    }
    int rc;
    if (want_l && pl.exact) {
        // composite, Poisson terms and w from the exact digit planes (GEMM 1 done)
        if ((rc = sfh_exact_launch(ctx, m, pl.xp, d_R, pl.data, d_negLogL, pl.Wh, pl.Wl, nbp,
                                   want_g ? 1 : 0, eps, pl.err)))
            return rc;
    } else {
    GemmParams P1{};
    P1.m_tiles = pl.m_tiles;
    P1.n_tiles = pl.n_tiles1;
    P1.ksplit = 1;
    P1.kb_total = (int)(ntp / BK);
    P1.kb_per_split = P1.kb_total;
    P1.epi = 0;
    P1.data = pl.dataf;
    P1.nbins = nbins;
    P1.B = (int)B;
    P1.B_pad = (int)B_pad;
    P1.eps = (float)fmax(eps, 1.1754943508222875e-38);
    P1.W_hi = pl.Wh;
    P1.W_lo = pl.Wl;
    P1.w_ld = nbp;
    P1.want_w = want_g ? 1 : 0;
    P1.want_logl = want_l ? 1 : 0;
    P1.logl_part = pl.lp;
    P1.err = pl.err;
    if ((rc = launch_gemm(ctx, pl.maps[0], pl.maps[1], pl.maps[2], pl.maps[3], P1))) return rc;
    if (want_l) {
        k_logl_reduce<<<(unsigned)((B + 255) / 256), 256, 0, st>>>(pl.lp, 2 * pl.n_tiles1, (int)B,
                                                                   (int)B_pad, d_negLogL);
        SFH_LAUNCHED(ctx);
    }
    }
    if (want_g) {
        GemmParams P2{};
        P2.m_tiles = pl.m_tiles;
        P2.n_tiles = pl.n_tiles2;
        P2.ksplit = pl.ks2;
        P2.kb_total = pl.kb2;
        P2.kb_per_split = pl.per2;
        P2.epi = 1;
        P2.B = (int)B;
        P2.B_pad = (int)B_pad;
        P2.Gpart = pl.gp;
        P2.nt = nt;
        P2.err = pl.err;
        if ((rc = launch_gemm(ctx, pl.maps[4], pl.maps[5], pl.maps[6], pl.maps[7], P2))) return rc;
        const int64_t n = B * nt;
        k_g_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(pl.gp, pl.ks2, B, B_pad, nt, d_G,
                                                                m->colsum_e);
        SFH_LAUNCHED(ctx);
    }
    (void)nbp;
    return SFH_OK;
}

int sfh_batched_check(sfh_ctx *ctx, const SfhBatchedPlan &pl) {
    int herr = 0;
    SFH_CK(ctx, cudaMemcpyAsync(&herr, pl.err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (herr) return sfh_set_error(ctx, SFH_ERR_TIMEOUT, "tensor-core pipeline wait timed out");
    return SFH_OK;
}

static int run_batched(sfh_ctx *ctx, const sfh_models *m, const double *d_R, int64_t B,
                       const double *d_data, double *d_negLogL, float *d_G, double eps) {
    SfhBatchedPlan pl{};
    int rc = sfh_batched_prepare(ctx, m, B, d_data, nullptr, 0, &pl);
    if (rc) return rc;
    if ((rc = sfh_scratch_reserve(ctx, pl.scratch_bytes))) return rc;
    if ((rc = sfh_batched_prepare(ctx, m, B, d_data, ctx->scratch, ctx->scratch_bytes, &pl))) return rc;
    if ((rc = sfh_batched_launch(ctx, m, pl, d_R, d_negLogL, d_G, eps))) return rc;
    return sfh_batched_check(ctx, pl);
}

int sfh_launch_fg_batched(sfh_ctx *ctx, const sfh_models *m, const double *d_R, int64_t B,
                          const double *d_data, double *d_negLogL, float *d_G, double eps) {
    // the occupied-bin plan's derived handle when the diagram leaves bins empty
    const sfh_models *mb = m;
    const double *db = d_data;
    SfhOccPlan *occ = nullptr;
    int rc = sfh_occ_batched(ctx, const_cast<sfh_models *>(m), d_data, d_negLogL != nullptr, &mb,
                             &db, &occ);
    if (rc) return rc;
    if ((rc = run_batched(ctx, mb, d_R, B, db, d_negLogL, d_G, eps))) return rc;
    if (occ && *occ->h_bviol) {  // a plan-empty bin holds counts now: the dense evaluation
        sfh_occ_retire(occ);
        rc = run_batched(ctx, m, d_R, B, d_data, d_negLogL, d_G, eps);
    }
    return rc;
}

PFN_cuTensorMapEncodeTiled_v12000 sfh_tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}
