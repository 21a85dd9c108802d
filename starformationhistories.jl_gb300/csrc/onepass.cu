// onepass.cu -- fg! for one coefficient vector with a single read of the template matrix
// (FP32 storage, column-major nbins x nt).
//
// fg! (src/fitting/solvers.jl:20-38: composite!, loglikelihood, ∇loglikelihood!,
// fitting_base.jl:55-96, 265-285) needs every template of a bin before w = 1 - n/max(m, eps)
// and G = Mᵀ w can be formed, so the two-kernel form reads M twice.  Here each SM keeps
// tiles of 32 bins x all templates (nt <= kMaxTemplates) in shared memory:
//
//   one persistent CTA per SM, 16 warps; tiles of BINS = 16 (or 32) bins;
//   warp 15 (4 lanes)  producers: boxes of BINS bins x 64 templates (bulk copies of the
//                      blocked copy) into a ring of shared-memory slots, full / empty
//                      mbarriers per slot; lane p issues every fourth box;
//   box c belongs to owner warp c % 14 in both phases; lane l reads its rows (one 16-byte
//   shared load per row and 4 bins; a warp load covers whole rows, conflict-free);
//   phase A   as its boxes land, an owner forms m r for the lane's 4 bins (r split hi + lo,
//             packed FP32 pairs, compensated per box) and sums the lanes that share bins;
//   finish    warp 14 sums the 14 owner partials (double-float, fixed order), forms
//             max(m, eps), w = 1 - n/m, the composite, and the Poisson term
//             (double-float, sfh_dfloat.cuh) one step later;
//   phase B   one tile behind phase A (so it overlaps the finish), an owner forms M w
//             over the lane's 4 bins for each of its rows, accumulated over the CTA's tiles
//             in per-lane double-float registers, and releases each box after reading it;
//             the lanes of a row are summed once, at the end.
// The kernel streams a blocked copy of the templates (one contiguous block per tile and
// box, tiles in order) with 1-D bulk copies, so every CTA reads long sequential runs of
// HBM; the copy is made once per handle and tile width (k_onepass_block).
// The CTAs' G and logL partials are summed after a grid barrier, in a fixed order, so
// results are reproducible.  M crosses HBM once per evaluation.  Every mbarrier wait is bounded:
// on timeout the CTA stops at a tile boundary (all warps together, so no CTA barrier is
// left waiting), drains its TMA loads, raises the error slot, and the reduction writes NaN
// to G and -logL.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>

#include "sfh_internal.cuh"
#include "sfh_ptx.cuh"

namespace {

constexpr int kBoxCols = 64;                      // templates per TMA box
constexpr int kOwners = 14;                       // warps that own boxes: box c -> warp c % 14
constexpr int kFinishWarp = kOwners;              // forms m, w and the Poisson terms
constexpr int kWarps = kOwners + 1;               // consumer warps
constexpr int kThreadsOP = (kWarps + 1) * 32;     // + producer warp (16 warps: 128 registers)
constexpr int kMaxBoxes = 24;                     // boxes per tile
constexpr int kBoxesPerWarp = (kMaxBoxes + kOwners - 1) / kOwners;  // 2
constexpr int kMaxTemplates = kMaxBoxes * kBoxCols;  // 1536
constexpr int kMaxSlots = 64;
constexpr int kProducers = 4;                     // issuing lanes of the producer warp

// Tile geometry for BINS bins per tile (16 or 32): a box is BINS x 64 floats; a template
// row of a box is BINS/4 lanes of one 16-byte load, so a warp load covers 32/(BINS/4) rows.
template <int BINS>
struct Geo {
    static constexpr int kBoxFloats = BINS * kBoxCols;
    static constexpr int kBoxBytes = kBoxFloats * 4;
    static constexpr int kLanesPerRow = BINS / 4;
    static constexpr int kRowsPerLoad = 32 / kLanesPerRow;
    static constexpr int kRows = kBoxCols / kRowsPerLoad;  // rows of a box per lane
};

struct OnePassArgs {
    const float *blk;  // blocked copy of the templates: box (t, c) at (t * nch + c) * box floats
    int64_t nbins, nt;
    int ntiles, nch, slots;
    const double *r, *data;
    double *composite;
    double *gpart;  // [gridDim.x][nt]
    double *lpart;  // [gridDim.x]
    unsigned int *err;
    unsigned int *bar;  // grid barrier: arrivals, generation
    const sfh_df *tab;  // double-float log / n log n tables (read through L1)
    float eps_f;
    int want_logl;
    double gsign;
    double *G, *negLogL;  // results (either may be NULL)
};

// Dynamic shared memory: ring | r (hi, lo) | s_part | s_w[2] | full | empty | flags.
__host__ __device__ inline size_t op_smem_bytes(int bins, int slots, int nch) {
    return 128 + (size_t)slots * bins * kBoxCols * 4 + (size_t)nch * kBoxCols * sizeof(float2) +
           (size_t)kOwners * bins * sizeof(sfh_df) + 2 * (size_t)bins * 4 + 2 * (size_t)slots * 8 +
           16;
}

// Bounded wait with an inline fast path (the box has usually landed already).
__device__ __forceinline__ bool op_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                        int *err, int code) {
    if (mbar_test(bar, parity)) return true;
    return mbar_wait_sleep(bar, parity, abort_flag, err, code);
}

// Steps over the CTA's tiles (k = 0, 1, ...), two named barriers per step.  LAG = true:
//   owners   phase A(k)   | bar 1 | phase B(k-1) with w(k-1)             | bar 2
//   finish   Poisson(k-1) | bar 1 | m(k), w(k) from the owners' partials | bar 2
// so the finish of one tile overlaps the G products of the previous one, with boxes of
// two tiles resident (the ring needs 2 nch slots plus prefetch).  LAG = false:
//   owners   phase A(k)   | bar 1 |                                      | bar 2 | phase B(k)
//   finish   Poisson(k-1) | bar 1 | m(k), w(k)                           | bar 2 |
// holds one tile (nch slots plus prefetch), leaving more of the ring to the stream.
template <int BINS, bool LAG>
__global__ void __launch_bounds__(kThreadsOP, 1)
k_fg_onepass(const OnePassArgs a) {
    using GE = Geo<BINS>;
    constexpr int LPR = GE::kLanesPerRow, RPL = GE::kRowsPerLoad, NR = GE::kRows;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // 128-byte aligned TMA destination; derived from the shared array by pointer arithmetic
    // so that every access below stays a shared-memory access
    unsigned char *base = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    const int slots = a.slots, nch = a.nch;
    float *ring = (float *)base;
    float2 *rr = (float2 *)(ring + (size_t)slots * GE::kBoxFloats);  // r split (hi, lo)
    sfh_df *s_part = (sfh_df *)(rr + nch * kBoxCols);                // [kOwners][BINS]
    float *s_w = (float *)(s_part + kOwners * BINS);                 // [2][BINS]
    uint64_t *full = (uint64_t *)(s_w + 2 * BINS);
    uint64_t *empty = full + slots;
    volatile int *s_abort = (volatile int *)(empty + slots);
    volatile int *s_stop = s_abort + 1;
    int *err = (int *)a.err;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k < nch * kBoxCols; k += blockDim.x) {
        const double v = k < a.nt ? a.r[k] : 0.0;
        const float h = __double2float_rn(v);
        rr[k] = make_float2(h, __double2float_rn(v - (double)h));
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < slots; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);  // the box's warp releases it
        }
        *s_abort = 0;
        *s_stop = 0;
        fence_barrier_init();
    }
    __syncthreads();

    // ------------------------------------------------------------ producers
    // kProducers lanes of the last warp; lane p issues the boxes whose sequence number
    // q = (local tile) * nch + c has q % kProducers == p (one bulk copy occupies its issuing
    // thread for a while, so several issuers keep more copies in flight).  slots is a
    // multiple of kProducers: a slot is always refilled by the same lane, which waits for
    // the release of that slot's previous box.
    if (warp == kWarps) {
        if (lane < kProducers) {
            const int64_t nq = (int64_t)((a.ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1) * nch;
            int64_t q = lane, last = -1;
            bool ok = true;
            for (; q < nq && ok; q += kProducers) {
                const int s = (int)(q % slots);
                const uint32_t ph = (uint32_t)(q / slots) & 1u;
                if (!op_wait(&empty[s], ph ^ 1u, s_abort, err, 1)) { ok = false; break; }
                const int64_t tl = q / nch, c = q - tl * nch;
                const int64_t t = (int64_t)blockIdx.x + tl * gridDim.x;
                mbar_expect_tx(&full[s], GE::kBoxBytes);
                bulk_load(ring + (size_t)s * GE::kBoxFloats,
                          a.blk + ((size_t)t * nch + c) * GE::kBoxFloats, GE::kBoxBytes, &full[s]);
                last = q;
            }
            // every box this lane requested has landed before the CTA exits
            volatile int never = 0;
            int dummy = 0;
            for (int64_t r = last; r >= 0 && r > last - slots; r -= kProducers)
                mbar_wait(&full[r % slots], (uint32_t)(r / slots) & 1u, &never, &dummy, 0);
        }
        return;
    }

    // ------------------------------------------------------------ consumers
    // Box c (templates 64c .. 64c+63) belongs to warp c % kOwners in both phases.  Lane l
    // reads rows g + RPL k (k < NR, g = l / LPR) and bins 4 quad .. 4 quad + 3
    // (quad = l % LPR): one 16-byte shared load per row, a warp load covering RPL whole
    // rows (512 contiguous bytes, conflict-free).
    const int g = lane / LPR, quad = lane % LPR;
    const int64_t nbins = a.nbins;
    const bool want_g = a.gpart != nullptr;
    const bool fin = warp == kFinishWarp;
    // G of template 64c + g + RPL k over this lane's 4 bins and all of the CTA's tiles
    float gh[kBoxesPerWarp][NR], gl[kBoxesPerWarp][NR];
#pragma unroll
    for (int b = 0; b < kBoxesPerWarp; ++b)
#pragma unroll
        for (int k = 0; k < NR; ++k) gh[b][k] = gl[b][k] = 0.f;
    // finish warp: lane = bin (lanes < BINS) + BINS * half; the Poisson term of the
    // previous tile is kept (pending) for the window after bar 2
    sfh_df term{0.f, 0.f}, pc{0.f, 0.f};
    float pnh = 0.f, pnl = 0.f;
    bool pending = false;
    int s0 = 0, sp = 0;  // first slot of the current / previous tile
    uint32_t ph0 = 0;    // use parity of the current tile's first slot
    bool ok = true, have_prev = false;
    // phase B of the tile whose first box is in slot sbase, with w at wsrc: M w over the
    // lane's 4 bins from the resident boxes (packed FP32 pairs), compensated per template
    // over the tiles; each box is released after its last read
    auto phase_b = [&](int sbase, const float *wsrc) {
        const float4 w4 = *(const float4 *)(wsrc + 4 * quad);
        const float2 w01 = make_float2(w4.x, w4.y), w23 = make_float2(w4.z, w4.w);
#pragma unroll
        for (int b = 0; b < kBoxesPerWarp; ++b) {
            const int c = warp + kOwners * b;
            if (c >= nch) break;
            int s = sbase + c;
            if (s >= slots) s -= slots;
            if (want_g) {
                const float *bp = ring + (size_t)s * GE::kBoxFloats + g * BINS + 4 * quad;
#pragma unroll
                for (int k = 0; k < NR; ++k) {
                    const float4 m = *(const float4 *)(bp + k * RPL * BINS);
                    const float2 p = __ffma2_rn(make_float2(m.z, m.w), w23,
                                                __fmul2_rn(make_float2(m.x, m.y), w01));
                    sfh_two_sum_acc(gh[b][k], gl[b][k], p.x + p.y);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[s]);
        }
    };
    for (int t = blockIdx.x, kk = 0;; t += gridDim.x, ++kk) {
        const bool have_cur = t < a.ntiles;
        if (!have_cur && (!LAG || !have_prev)) break;
        const int64_t i = (int64_t)t * BINS + (lane % BINS);
        double nd = 0.0;
        if (fin) {
            if (have_cur && lane < BINS && i < nbins) nd = a.data[i];  // loads while the boxes land
            if (pending) {
                term = df_add(term, sfh_bin_term(pc, pnh, pnl, a.tab));
                pending = false;
            }
        } else if (have_cur) {
            // phase A(k): m r over this warp's boxes for the lane's 4 bins (r split hi + lo,
            // packed FP32 pairs, two chains per bin pair; compensated per box)
            float ah[4] = {0.f, 0.f, 0.f, 0.f}, al[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int b = 0; b < kBoxesPerWarp; ++b) {
                const int c = warp + kOwners * b;
                if (c >= nch || !ok) break;
                int s = s0 + c;
                uint32_t ph = ph0;
                if (s >= slots) { s -= slots; ph ^= 1u; }
                if (!op_wait(&full[s], ph, s_abort, err, 2)) {
                    ok = false;
                    break;
                }
                const float *bp = ring + (size_t)s * GE::kBoxFloats + g * BINS + 4 * quad;
                const float2 *rp = rr + c * kBoxCols + g;
                float2 e01 = make_float2(0.f, 0.f), e23 = e01, o01 = e01, o23 = e01;
#pragma unroll
                for (int k = 0; k < NR; ++k) {
                    const float4 m = *(const float4 *)(bp + k * RPL * BINS);
                    const float2 rv = rp[RPL * k];
                    const float2 h2 = make_float2(rv.x, rv.x), l2 = make_float2(rv.y, rv.y);
                    const float2 m01 = make_float2(m.x, m.y), m23 = make_float2(m.z, m.w);
                    if (k & 1) {
                        o01 = __ffma2_rn(m01, h2, __ffma2_rn(m01, l2, o01));
                        o23 = __ffma2_rn(m23, h2, __ffma2_rn(m23, l2, o23));
                    } else {
                        e01 = __ffma2_rn(m01, h2, __ffma2_rn(m01, l2, e01));
                        e23 = __ffma2_rn(m23, h2, __ffma2_rn(m23, l2, e23));
                    }
                }
                sfh_two_sum_acc(ah[0], al[0], e01.x + o01.x);
                sfh_two_sum_acc(ah[1], al[1], e01.y + o01.y);
                sfh_two_sum_acc(ah[2], al[2], e23.x + o23.x);
                sfh_two_sum_acc(ah[3], al[3], e23.y + o23.y);
            }
            // sum over the lanes that hold the same bins (other rows)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                sfh_df v = df_fast_two_sum(ah[k], al[k]);
#pragma unroll
                for (int o = LPR; o <= 16; o <<= 1) {
                    const sfh_df u{__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
                    v = df_add_fast(v, u);
                }
                if (lane < LPR) s_part[warp * BINS + 4 * quad + k] = v;
            }
        }
        named_bar_sync(1, kWarps * 32);
        if (fin) {
            // m(k) and w(k): lane pair (bin, bin + BINS) sums the owners' partials of even /
            // odd owners, then the two halves are added
            if (have_cur) {
                const int b = lane % BINS, h = lane / BINS;  // BINS == 16: h in {0, 1}
                sfh_df cm{0.f, 0.f};
                if (BINS == 16) {
                    for (int w = h; w < kOwners; w += 2) cm = df_add_fast(cm, s_part[w * BINS + b]);
                    const sfh_df u{__shfl_xor_sync(0xffffffffu, cm.h, 16),
                                   __shfl_xor_sync(0xffffffffu, cm.l, 16)};
                    cm = h == 0 ? df_add_fast(cm, u) : df_add_fast(u, cm);
                } else {
                    for (int w = 0; w < kOwners; ++w) cm = df_add_fast(cm, s_part[w * BINS + b]);
                }
                float wv = 0.f;
                if (lane < BINS && i < nbins) {
                    if (!want_g) a.composite[i] = sfh_f2d(cm.h) + sfh_f2d(cm.l);  // the model, unclamped
                    // max(composite, eps(T)); eps(T) is a power of two, exact in FP32
                    if (cm.h < a.eps_f || (cm.h == a.eps_f && cm.l < 0.f)) cm = sfh_df{a.eps_f, 0.f};
                    float nh, nl;
                    sfh_split_double(nd, nh, nl);
                    if (want_g) {
                        wv = __fdiv_rn(df_add(cm, sfh_df{-nh, -nl}).h, cm.h);  // 1 - n/c
                        a.composite[i] = sfh_f2d(wv);
                    }
                    if (a.want_logl) {  // the term is formed in the next window
                        pc = cm;
                        pnh = nh;
                        pnl = nl;
                        pending = true;
                    }
                }
                if (lane < BINS) s_w[(kk & 1) * BINS + lane] = wv;
            }
            if (lane == 0) *s_stop = *s_abort;
        } else if (LAG && have_prev) {
            phase_b(sp, s_w + ((kk - 1) & 1) * BINS);
        }
        named_bar_sync(1, kWarps * 32);
        if (*s_stop) break;  // the same decision in every consumer warp
        if (!LAG && !fin && have_cur) phase_b(s0, s_w + (kk & 1) * BINS);
        have_prev = have_cur;
        sp = s0;
        if (have_cur) {
            s0 += nch;  // nch <= slots: at most one wrap
            if (s0 >= slots) { s0 -= slots; ph0 ^= 1u; }
        }
    }
    if (fin && pending) term = df_add(term, sfh_bin_term(pc, pnh, pnl, a.tab));
    // per-CTA partials of G: the lanes of a row (bin quads) summed once
    if (want_g && !fin) {
#pragma unroll
        for (int b = 0; b < kBoxesPerWarp; ++b) {
            const int c = warp + kOwners * b;
            if (c >= nch) break;
#pragma unroll
            for (int k = 0; k < NR; ++k) {
                sfh_df v = df_fast_two_sum(gh[b][k], gl[b][k]);
#pragma unroll
                for (int o = 1; o < LPR; o <<= 1) {
                    const sfh_df u{__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
                    v = df_add(v, u);
                }
                const int64_t col = (int64_t)c * kBoxCols + g + RPL * k;
                if (quad == 0 && col < a.nt)
                    a.gpart[(int64_t)blockIdx.x * a.nt + col] = sfh_f2d(v.h) + sfh_f2d(v.l);
            }
        }
    }
    if (a.want_logl && fin) {
        const sfh_df tot = sfh_df_warp_sum(term);
        if (lane == 0) a.lpart[blockIdx.x] = sfh_f2d(tot.h) + sfh_f2d(tot.l);
    }

    // ------------------------------------------------------------ grid reduction
    // Every CTA of the launch is resident (one per SM): after a grid barrier CTA b sums
    // columns [b per, (b+1) per) of G over all CTAs' partials (one warp per column, lanes
    // over CTAs, a fixed shuffle tree) and CTA 0 sums -logL: a fixed order, so results are
    // reproducible.  The barrier's wait is bounded like the pipeline's.
    named_bar_sync(1, kWarps * 32);  // this CTA's partials are written
    if (threadIdx.x == 0) {
        __threadfence();
        volatile unsigned int *gen = a.bar + 1;
        const unsigned int g0 = *gen;
        if (atomicAdd(a.bar, 1u) == gridDim.x - 1) {
            *a.bar = 0u;  // re-armed for the next launch
            __threadfence();
            atomicAdd(a.bar + 1, 1u);
        } else {
            const long long t0 = clock64();
            while (*gen == g0) {
                if (clock64() - t0 > kSfhWaitBudget) {
                    atomicExch(err, 3);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    named_bar_sync(1, kWarps * 32);
    const bool bad = *(volatile unsigned int *)a.err != 0u;
    if (a.G) {  // warp w sums columns j0 + w, j0 + w + kWarps, ...: lane l takes CTAs
                // l, l + 32, ..., then a fixed shuffle tree
        const int per = (int)((a.nt + gridDim.x - 1) / gridDim.x);
        for (int cw = warp; cw < per; cw += kWarps) {
            const int64_t j = (int64_t)blockIdx.x * per + cw;
            if (j >= a.nt) break;
            double acc = 0.0;
            for (int p = lane; p < (int)gridDim.x; p += 32) acc += __ldcg(a.gpart + (int64_t)p * a.nt + j);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (lane == 0) a.G[j] = bad ? NAN : a.gsign * acc;
        }
    }
    if (a.negLogL && blockIdx.x == 0 && warp == 0) {
        double acc = 0.0;
        for (int p = lane; p < (int)gridDim.x; p += 32) acc += __ldcg(a.lpart + p);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        // loglikelihood returns -typemax(T) = -Inf when the sum is exactly zero (fitting_base.jl:95)
        if (lane == 0) *a.negLogL = bad ? NAN : -((acc != 0.0) ? acc : -INFINITY);
    }
}

// Blocked copy for BINS-bin tiles: blk[((t * nch + c) * 64 + j) * BINS + b] =
// M[(64 c + j) * nbins + BINS t + b], zero outside the matrix.  One thread per output
// float (b fastest: reads BINS contiguous floats of a template column, writes contiguous).
__global__ void k_onepass_block(const float *__restrict__ M, int64_t nbins, int64_t nt, int bins,
                                int nch, int64_t total, float *__restrict__ blk) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int64_t b = idx % bins, rest = idx / bins;
    const int64_t j = rest % kBoxCols, tc = rest / kBoxCols;
    const int64_t c = tc % nch, t = tc / nch;
    const int64_t bin = t * bins + b, col = c * kBoxCols + j;
    blk[idx] = (bin < nbins && col < nt) ? M[col * nbins + bin] : 0.f;
}

int op_max_smem(sfh_ctx *ctx) {
    static int cached = -1;
    if (cached < 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device) !=
            cudaSuccess)
            v = 0;
        cached = v;
    }
    return cached;
}

// Ring slots for BINS-bin tiles of a matrix with nch boxes per tile, one or (lag) two tiles
// resident (0 if it does not fit).
int op_slots(sfh_ctx *ctx, int bins, int nch, bool lag) {
    const int maxs = op_max_smem(ctx);
    int slots = kMaxSlots;
    while (slots > 0 && op_smem_bytes(bins, slots, nch) > (size_t)maxs) --slots;
    slots -= slots % kProducers;  // each slot is refilled by one producer lane
    return slots >= (lag ? 2 : 1) * nch + 2 ? slots : 0;  // resident tiles plus prefetch
}

template <int BINS, bool LAG>
int launch_onepass(sfh_ctx *ctx, const OnePassArgs &a0, int grid, cudaStream_t st) {
    static size_t attr_set = 0;
    const size_t smem = op_smem_bytes(BINS, a0.slots, a0.nch);
    if (smem > attr_set) {
        SFH_CK(ctx, cudaFuncSetAttribute(k_fg_onepass<BINS, LAG>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = smem;
    }
    // grid <= SM count and one CTA per SM (shared memory): the CTAs are resident together,
    // as the in-kernel grid reduction needs; its barrier wait is bounded all the same
    k_fg_onepass<BINS, LAG><<<grid, kThreadsOP, smem, st>>>(a0);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

}  // namespace

bool sfh_onepass_eligible(sfh_ctx *ctx, const sfh_models *m) {
    if (!m || m->storage == SFH_F64 || !m->d_f32) return false;
    if (m->nbins > INT32_MAX - 64 || m->nt > kMaxTemplates) return false;
    const int nch = (int)((m->nt + kBoxCols - 1) / kBoxCols);
    return op_slots(ctx, 16, nch, false) > 0;
}

size_t sfh_onepass_scratch(const sfh_ctx *ctx, const sfh_models *m) {
    return sfh_align256((size_t)ctx->sm_count * (size_t)m->nt * 8) +
           sfh_align256((size_t)ctx->sm_count * 8);
}

int sfh_launch_fg_onepass(sfh_ctx *ctx, sfh_models *m, const double *d_coeffs,
                          const double *d_data, double *d_composite, double *d_G,
                          double *d_negLogL, double eps, double gsign, void *scratch,
                          cudaEvent_t *ev) {
    const int64_t nbins = m->nbins, nt = m->nt;
    const int nch = (int)((nt + kBoxCols - 1) / kBoxCols);
    // the handle's variant, else the nearest one the shape fits (16-bin, no lag always fits
    // an eligible shape)
    int bins = m->onepass_bins == 32 ? 32 : 16;
    bool lag = m->onepass_lag != 0;
    int slots = op_slots(ctx, bins, nch, lag);
    if (!slots && lag) slots = op_slots(ctx, bins, nch, lag = false);
    if (!slots && bins == 32) slots = op_slots(ctx, bins = 16, nch, lag);
    if (!slots) return sfh_set_error(ctx, SFH_ERR_UNSUPPORTED, "one-pass fg!: shape does not fit");
    const int mi = bins == 16 ? 0 : 1;
    const int ntiles = (int)((nbins + bins - 1) / bins);
    if (!m->d_blk[mi]) {  // the blocked copy, once per handle and tile width
        const int64_t total = (int64_t)ntiles * nch * kBoxCols * bins;
        SFH_CK(ctx, cudaMalloc(&m->d_blk[mi], (size_t)total * sizeof(float)));
        k_onepass_block<<<(unsigned)((total + 255) / 256), 256, 0, ctx->stream>>>(
            m->d_f32, nbins, nt, bins, nch, total, m->d_blk[mi]);
        SFH_LAUNCHED(ctx);
    }
    const int grid = ntiles < ctx->sm_count ? ntiles : ctx->sm_count;
    OnePassArgs a{};
    a.blk = m->d_blk[mi];
    a.nbins = nbins;
    a.nt = nt;
    a.ntiles = ntiles;
    a.nch = nch;
    a.slots = slots;
    a.r = d_coeffs;
    a.data = d_data;
    a.composite = d_composite;
    a.gpart = d_G ? (double *)scratch : nullptr;
    a.lpart = (double *)((char *)scratch + sfh_align256((size_t)ctx->sm_count * (size_t)nt * 8));
    a.err = ctx->d_counters + SFH_CNT_ONEPASS_ERR;
    a.bar = ctx->d_counters + SFH_CNT_ONEPASS_BAR;
    a.tab = ctx->d_df_tab;
    a.eps_f = (float)eps;
    a.want_logl = d_negLogL ? 1 : 0;
    a.gsign = gsign;
    a.G = d_G;
    a.negLogL = d_negLogL;
    cudaStream_t st = ctx->stream;
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[0], st));
    int rc = bins == 16 ? (lag ? launch_onepass<16, true>(ctx, a, grid, st)
                               : launch_onepass<16, false>(ctx, a, grid, st))
                        : (lag ? launch_onepass<32, true>(ctx, a, grid, st)
                               : launch_onepass<32, false>(ctx, a, grid, st));
    if (rc) return rc;
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[1], st));
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[2], st));
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[3], st));
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[4], st));
    return SFH_OK;
}
