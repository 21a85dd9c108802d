// onepass.cu -- fg! for one coefficient vector with a single read of the template matrix
// (FP32 storage).
//
// fg! (src/fitting/solvers.jl:20-38: composite!, loglikelihood, ∇loglikelihood!,
// fitting_base.jl:55-96, 265-285) needs every template of a bin before w = 1 - n/max(m, eps)
// and G = Mᵀ w can be formed, so the two-kernel form reads M twice.  Here each SM keeps
// a tile of BINS bins (16 or 32) x all templates (nt <= 1536) in shared memory:
//
//   one persistent CTA per SM, 16 warps;
//   warp 15, 4 lanes    producers: boxes of BINS bins x 64 templates (a blocked copy of the
//                       matrix, the boxes of a tile contiguous), moved as runs of up to 1, 2
//                       or 4 consecutive boxes per 1-D bulk copy into a ring of shared-memory
//                       run-slots with full / empty mbarriers; lane p issues every fourth
//                       run, so four copies are in issue concurrently;
//   warps 0-13          owners: half-box unit u (32 template rows of box u / 2) belongs to
//                       owner u % 14 (one 16-byte shared load per lane: 4 bins of a row);
//   warp 14             the Poisson terms.
// Per tile, two named barriers:
//   phase A   owners form m r for their units as the boxes land (r split hi + lo, packed
//             FP32 pairs accumulated error-free against a power-of-two anchor per bin,
//             sfh_anc_acc2) and sum the lanes that share bins;
//   bar 1
//   finish    owners 0-7: each bin's 14 owner partials summed by a group of lanes (fixed
//             shuffle tree, double-float), max(m, eps), w = 1 - n/m, the composite;
//   bar 2
//   phase B   owners form M w over their units, accumulated over the CTA's tiles in
//             per-lane packed FP32 registers, and release each unit's box (two owners
//             per box); warp 14 forms the tile's Poisson terms (double-float,
//             sfh_dfloat.cuh) meanwhile.
// After the last tile the CTAs' G and logL partials are summed after a grid barrier in a
// fixed order, so results are reproducible.  M crosses HBM once per evaluation.  Every
// wait is bounded: on timeout the CTA stops at a tile boundary (all warps together, so no
// CTA barrier is left waiting), drains its copies, raises the error slot, and G and -logL
// become NaN.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "sfh_internal.cuh"
#include "sfh_ptx.cuh"

namespace {

constexpr int kBoxCols = 64;                      // templates per box
constexpr int kMaxBoxes = 24;                     // boxes per tile
constexpr int kMaxTemplates = kMaxBoxes * kBoxCols;  // 1536
constexpr int kMaxSlots = 64;
constexpr int kProducers = 4;                     // issuing lanes of the producer warp

// Kernel shape for BINS bins per tile and OWN owner warps.  A box is [64 rows][BINS]
// floats; a row is LPR lanes of one 16-byte load, a warp load covers RPL rows, a half-box
// unit (32 rows) GU loads.  Warps 0 .. OWN-1 own units, warp OWN forms the Poisson terms,
// warp OWN+1 produces; OWN = 14 runs one CTA per SM, OWN = 6 two (half the registers and
// shared memory each, so the two CTAs' per-tile latencies overlap).
template <int BINS, int OWN>
struct Geo {
    static constexpr int kBoxFloats = BINS * kBoxCols;
    static constexpr int kBoxBytes = kBoxFloats * 4;
    static constexpr int LPR = BINS / 4;
    static constexpr int RPL = 32 / LPR;
    static constexpr int GU = 32 / RPL;               // row groups of a half-box unit
    static constexpr int kOwners = OWN;
    static constexpr int kPoissonWarp = OWN;
    static constexpr int kWarps = OWN + 1;            // consumer warps (named barriers)
    static constexpr int kThreads = (kWarps + 1) * 32;
    static constexpr int kFinishers = OWN >= 8 ? 8 : 4;  // owners that also finish the bins
    static constexpr int LB = kFinishers * 32 / BINS;    // lanes per bin in the finish
    static constexpr int kUnits = (2 * kMaxBoxes + OWN - 1) / OWN;  // units per owner
    static constexpr int kMinBlocks = OWN >= 8 ? 1 : 2;  // CTAs per SM
};

struct OnePassArgs {
    const float *blk;  // blocked copy of the templates: box (t, c) at (t * nch + c) * box floats
    int64_t nbins, nt;
    int ntiles, nch, slots;
    int runs, lp;      // run-slots of the ring (slots = runs << lp), log2 boxes per run
    const double *r, *data;
    double *composite;
    float2 *gpart;  // [gridDim.x][nt] double-float partials of G
    double *lpart;  // [gridDim.x]
    unsigned int *err;
    unsigned int *bar;  // grid barrier: arrivals, generation
    const sfh_df *tab;  // double-float log / n log n tables (copied to shared memory)
    float eps_f;
    int want_logl;
    double gsign;
    double *G, *negLogL;  // results (either may be NULL)
    const int *skip;      // device flag: nonzero makes every CTA return at once (may be NULL)
    const float2 *rowb;   // per bin: (sum, max) of |M_ij| over the templates (the anchors' bound)
    long long budget;     // SM cycles a device wait may take before the launch gives up
    int drop_copy;        // test-only: producer lane 0 skips its first bulk copy
    // Launched as a programmatic dependent of the previous kernel in the stream: the
    // consumers wait for it to complete (griddepcontrol.wait) before they touch inputs or
    // outputs; the producers stream the blocked matrix, which no kernel writes, at once.
    // Every CTA lets the next such launch start after the last grid barrier (all CTAs are
    // resident then, so a dependent cannot take an SM a CTA of this launch still needs).
    int pdl;
    // Occupied-bin plan (all NULL for the dense kernel).  Tile bin p is bin occ[p] (nbins
    // above counts the tile bins); empty[0 .. nempty) are the plan's empty bins; colsum_e
    // their per-template column sums E_j; viol counts empty bins found occupied in this
    // launch (reset by the launch), flag is set for the host when one was; mcol is the
    // (nbins_all, nt) column-major FP32 matrix the in-launch correction reads.
    const int *occ;
    const int *empty;
    int64_t nempty, nbins_all;
    const double *colsum_e;
    unsigned int *viol;
    unsigned int *flag;
    const float *mcol;
};

// Grid barrier over the launch's resident CTAs (arrivals a.bar[0], generation a.bar[1]),
// called by one thread per CTA after a CTA barrier; bounded like the pipeline's waits.  The
// arrival is an acquire-release atomic, so the last CTA to arrive sees every CTA's writes;
// it re-arms the count and publishes the next generation with a release, which the others
// poll with acquire loads.
__device__ __forceinline__ void op_grid_barrier(const OnePassArgs &a) {
    unsigned int *arr = a.bar, *gen = a.bar + 1;
    unsigned int g0, old;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(g0) : "l"(gen) : "memory");
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(arr) : "memory");
    if (old == gridDim.x - 1) {
        asm volatile("st.relaxed.gpu.global.u32 [%0], 0;" ::"l"(arr) : "memory");  // re-armed
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(gen) : "memory");
        return;
    }
    const long long t0 = clock64();
    for (;;) {
        unsigned int g;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(g) : "l"(gen) : "memory");
        if (g != g0) break;
        if (clock64() - t0 > a.budget) {
            atomicExch(a.err, 3u);
            break;
        }
    }
}

// Dynamic shared memory: ring | r (hi, lo) | s_part | s_w | s_cn | s_tab | full | empty |
// flags.
__host__ __device__ inline size_t op_smem_bytes(int bins, int owners, int slots, int nch) {
    return 128 + (size_t)slots * bins * kBoxCols * 4 + (size_t)nch * kBoxCols * sizeof(float2) +
           (size_t)owners * bins * sizeof(sfh_df) + (size_t)bins * 4 + (size_t)bins * 16 +
           (size_t)SFH_DF_TAB_ALL * sizeof(sfh_df) + 2 * (size_t)slots * 8 + 16;
}

// Bounded wait with an inline fast path (the box has usually landed already).
__device__ __forceinline__ bool op_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                        int *err, int code, long long budget) {
    if (mbar_test(bar, parity)) return true;
    return mbar_wait_sleep(bar, parity, abort_flag, err, code, budget);
}

// Anchors of bins i0 .. i0 + 3 (power-of-two accumulator starts, sfh_anc_acc2) from the
// handle's row statistics and the coefficients' max and sum of |r|.
__device__ __forceinline__ void op_anchors(const OnePassArgs &a, int64_t i0, float rmax, float rsum,
                                           float2 &sg01, float2 &sg23) {
    float sg[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float2 rb = (i0 + q < a.nbins) ? __ldg(a.rowb + i0 + q) : make_float2(0.f, 0.f);
        sg[q] = sfh_anchor(sfh_row_bound(rb, rmax, rsum));
    }
    sg01 = make_float2(sg[0], sg[1]);
    sg23 = make_float2(sg[2], sg[3]);
}

// Empty bins of the plan that this call's data occupies (the CTA's share of a.empty, as
// checked in the prologue): each becomes a tile bin after the fact.  Per bin the consumer
// threads form c = Σ_j M_ij r_j in FP64 (a fixed reduction tree), thread 0 applies the
// finish's arithmetic (clamp, w in FP32, the Poisson term) and adds t_i + c_i to the
// CTA's logL partial (the plan subtracted c_i through E_j), and G's partial gets
// M_ij (w_i - 1) (E_j counted the bin with w = 1).  Slow, exact, and rare: the next call
// builds a plan for the new data.  `red` holds at least 32 doubles of shared memory.
__device__ __noinline__ void op_fold_occupied(const OnePassArgs &a, const sfh_df *s_tab, double *red) {
    const int nthr = (int)(blockDim.x - 32);  // the consumer threads
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5, nwarps = nthr >> 5;
    __shared__ float s_wfold;
    double lcorr = 0.0;
    for (int64_t k0 = (int64_t)blockIdx.x * nthr; k0 < a.nempty; k0 += (int64_t)gridDim.x * nthr) {
        for (int q = 0; q < nthr && k0 + q < a.nempty; ++q) {  // the share's bins in order
            const int i = __ldg(a.empty + k0 + q);
            const double n = a.data[i];
            if (n == 0.0) continue;  // the same value in every thread
            double c = 0.0;
            for (int64_t j = t; j < a.nt; j += nthr) c = fma((double)a.mcol[j * a.nbins_all + i], a.r[j], c);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
            if (lane == 0) red[warp] = c;
            named_bar_sync(1, nthr);
            if (t == 0) {
                double tot = 0.0;
                for (int w = 0; w < nwarps; ++w) tot += red[w];
                const float ch = __double2float_rn(tot);
                sfh_df cm{ch, __double2float_rn(tot - (double)ch)};
                if (cm.h < a.eps_f || (cm.h == a.eps_f && cm.l < 0.f)) cm = sfh_df{a.eps_f, 0.f};
                float nh, nl;
                sfh_split_double(n, nh, nl);
                const float wv = __fdiv_rn(df_add(cm, sfh_df{-nh, -nl}).h, cm.h);
                a.composite[i] = sfh_f2d(wv);
                s_wfold = wv;
                if (a.want_logl) {
                    const sfh_df tt = sfh_bin_term(cm, nh, nl, s_tab);
                    lcorr += (sfh_f2d(tt.h) + sfh_f2d(tt.l)) + tot;
                }
            }
            named_bar_sync(1, nthr);
            if (a.gpart) {
                const double wm1 = (double)s_wfold - 1.0;
                for (int64_t j = t; j < a.nt; j += nthr) {
                    float2 &gp = a.gpart[(int64_t)blockIdx.x * a.nt + j];
                    const double gv = sfh_f2d(gp.x) + sfh_f2d(gp.y) +
                                      (double)a.mcol[j * a.nbins_all + i] * wm1;
                    float gh, gl;
                    sfh_split_double(gv, gh, gl);
                    gp = make_float2(gh, gl);
                }
            }
            named_bar_sync(1, nthr);
        }
    }
    if (t == 0 && a.want_logl) a.lpart[blockIdx.x] += lcorr;
}

template <int BINS, int OWN, bool SKEW>
__global__ void __launch_bounds__(Geo<BINS, OWN>::kThreads, Geo<BINS, OWN>::kMinBlocks)
k_fg_onepass(const OnePassArgs a) {
    using GE = Geo<BINS, OWN>;
    // a finished device-side driver turns the evaluations still queued into no-ops; every
    // CTA reads the same flag, so none waits at the grid barrier
    if (a.skip && *a.skip) return;
    constexpr int LPR = GE::LPR, RPL = GE::RPL, GU = GE::GU, LB = GE::LB;
    constexpr int kOwners = GE::kOwners, kWarps = GE::kWarps, kFinishers = GE::kFinishers;
    constexpr int kUnits = GE::kUnits, kPoissonWarp = GE::kPoissonWarp;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // 128-byte aligned copy destination; derived from the shared array by pointer arithmetic
    // so that every access below stays a shared-memory access
    unsigned char *base = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    const int slots = a.slots, nch = a.nch, runs = a.runs, lp = a.lp, P = 1 << lp;
    const int nr = (nch + P - 1) >> lp;             // runs (bulk copies) per tile
    const int short_extra = 2 * ((nr << lp) - nch);  // releases the tile's last run lacks
    float *ring = (float *)base;
    float2 *rr = (float2 *)(ring + (size_t)slots * GE::kBoxFloats);  // r split (hi, lo)
    sfh_df *s_part = (sfh_df *)(rr + nch * kBoxCols);                // [kOwners][BINS]
    float *s_w = (float *)(s_part + kOwners * BINS);                 // [BINS]
    float4 *s_cn = (float4 *)(s_w + BINS);                           // [BINS] (m hi, lo, n hi, lo)
    sfh_df *s_tab = (sfh_df *)(s_cn + BINS);                         // log / n log n tables
    uint64_t *full = (uint64_t *)(s_tab + SFH_DF_TAB_ALL);
    uint64_t *empty = full + runs;
    volatile int *s_abort = (volatile int *)(empty + runs);
    volatile int *s_stop = s_abort + 1;
    int *err = (int *)a.err;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == kWarps) {  // the producer warp initialises the ring's barriers
        for (int s = lane; s < runs; s += 32) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 2 * P);  // the owners of the run's box halves release it
        }
        if (lane == 0) {
            *s_abort = 0;
            *s_stop = 0;
        }
        fence_barrier_init();
    }
    __syncthreads();
    // the first copies are issued now; the consumers stage r and the tables meanwhile and
    // meet at a consumer-only barrier before their first tile
    __shared__ float s_rstat[2][32];  // per consumer warp: max and sum of |r|
    __shared__ unsigned int s_nviol;  // the CTA's empty bins found occupied
    if (warp < kWarps) {
        if (a.pdl) asm volatile("griddepcontrol.wait;" ::: "memory");
        const int nk = nch * kBoxCols, ct = kWarps * 32;
        float rmx = 0.f, rsm = 0.f;
        for (int k0 = threadIdx.x; k0 < nk; k0 += 4 * ct) {
            double v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int k = k0 + q * ct;
                v[q] = (k < nk && k < a.nt) ? a.r[k] : 0.0;
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int k = k0 + q * ct;
                float h, l;
                sfh_split_any(v[q], h, l);  // integer operations: FP64 is the slow pipe
                if (k < nk) rr[k] = make_float2(h, l);
                rmx = fmaxf(rmx, fabsf(h));
                rsm += fabsf(h);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            rmx = fmaxf(rmx, __shfl_xor_sync(0xffffffffu, rmx, o));
            rsm += __shfl_xor_sync(0xffffffffu, rsm, o);
        }
        if (lane == 0) {
            s_rstat[0][warp] = rmx;
            s_rstat[1][warp] = rsm;
        }
        if (a.want_logl)
            for (int k = threadIdx.x; k < SFH_DF_TAB_ALL; k += ct) s_tab[k] = a.tab[k];
        if (a.empty) {
            // the plan's empty bins: w = 1 in the output, and a check that n is still <= 0
            // (each thread one bin of the CTA's share per pass, loads issued together)
            if (threadIdx.x == 0) s_nviol = 0;
            named_bar_sync(1, kWarps * 32);
            unsigned int nv = 0;
            for (int64_t k0 = (int64_t)blockIdx.x * ct; k0 < a.nempty; k0 += (int64_t)gridDim.x * ct) {
                const int64_t k = k0 + threadIdx.x;
                if (k < a.nempty) {
                    const int i = __ldg(a.empty + k);
                    a.composite[i] = 1.0;
                    // w = 1 needs n = 0 exactly (+-0; an integer test of the bits)
                    nv += (__double_as_longlong(a.data[i]) << 1) != 0ll ? 1u : 0u;
                }
            }
            if (nv) atomicAdd(&s_nviol, nv);
        }
        named_bar_sync(1, kWarps * 32);
        if (a.empty && threadIdx.x == 0 && s_nviol) atomicAdd(a.viol, s_nviol);
    }

    // ------------------------------------------------------------ producers
    // A run is up to P consecutive boxes of a tile (contiguous in the blocked copy and in
    // the ring): one bulk copy, one full and one empty barrier per run-slot.  Lane p issues
    // the runs whose sequence number q = (local tile) * nr + k has q % kProducers == p;
    // runs is a multiple of kProducers, so a run-slot is always refilled by the same lane,
    // which waits for the release of that run-slot's previous run.
    if (warp == kWarps) {
        if (lane < kProducers) {
            const int64_t nq = (int64_t)((a.ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1) * nr;
            int64_t last = -1;
            int s = lane, k = lane;  // run-slot and run within the tile of q
            uint32_t ph = 0;
            int64_t tl = 0;
            while (k >= nr) { k -= nr; ++tl; }
            for (int64_t q = lane; q < nq; q += kProducers) {
                if (!op_wait(&empty[s], ph ^ 1u, s_abort, err, 1, a.budget)) break;
                const int64_t t = (int64_t)blockIdx.x + tl * gridDim.x;
                const int c0 = k << lp, nb = min(P, nch - c0);
                if (!(a.drop_copy && q == 0)) {  // the injected failure: this copy never lands
                    mbar_expect_tx(&full[s], (uint32_t)(nb * GE::kBoxBytes));
                    bulk_load(ring + ((size_t)s << lp) * GE::kBoxFloats,
                              a.blk + ((size_t)t * nch + c0) * GE::kBoxFloats,
                              (uint32_t)(nb * GE::kBoxBytes), &full[s]);
                }
                last = q;
                s += kProducers;
                if (s >= runs) { s -= runs; ph ^= 1u; }
                k += kProducers;
                while (k >= nr) { k -= nr; ++tl; }
            }
            // every run this lane requested has landed before the CTA exits
            volatile int never = 0;
            int dummy = 0;
            for (int64_t q = last; q >= 0 && q > last - runs; q -= kProducers)
                if (!(a.drop_copy && q == 0))
                    mbar_wait_sleep(&full[q % runs], (uint32_t)(q / runs) & 1u, &never, &dummy, 0,
                                    a.budget);
        }
        return;
    }

    // ------------------------------------------------------------ consumers
    // Unit u = (box c, half h) = 2c + h (rows 32h .. 32h + 31 of box c) belongs to owner
    // u % kOwners in both phases.  Lane l reads rows 32h + g + RPL k (g = l / LPR, k < GU)
    // and bins 4 quad .. 4 quad + 3 (quad = l % LPR): one 16-byte shared load per row, a
    // warp load covering RPL whole rows (512 contiguous bytes, conflict-free).
    const int g = lane / LPR, quad = lane % LPR;
    const int64_t nbins = a.nbins;
    const bool want_g = a.gpart != nullptr;
    const bool owner = warp < kOwners;
    const int nunits = 2 * nch;
    // finish: warp fw < kFinishers, lanes of bin fb = fw * (32 / LB) + lane / LB
    const bool finisher = warp < kFinishers;
    const int fb = warp * (32 / LB) + lane / LB, fl = lane % LB;
    // G of the lane's rows of unit j over its 4 bins (packed pairs: bins 0, 2 and 1, 3) and
    // all of the CTA's tiles
    float2 g2[kUnits][GU];
#pragma unroll
    for (int j = 0; j < kUnits; ++j)
#pragma unroll
        for (int k = 0; k < GU; ++k) g2[j][k] = make_float2(0.f, 0.f);
    // bound of the coefficients for the anchors: max and sum of |r_hi| (FP32 sum of
    // nt <= 1536 terms, relative rounding below 1e-4)
    float rmax = 0.f, rsum = 0.f;
    for (int w = 0; w < kWarps; ++w) {
        rmax = fmaxf(rmax, s_rstat[0][w]);
        rsum += s_rstat[1][w];
    }
    sfh_df term{0.f, 0.f};
    int s0 = 0;        // slot of the tile's first box
    uint32_t ph0 = 0;  // its use parity
    bool ok = true;
    if constexpr (!SKEW)
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const int64_t tb = (int64_t)t * BINS;
        double nd = 0.0;
        int64_t ib = tb + fb;  // the finisher lane's bin (through the plan's map)
        if (finisher && fl == 0 && tb + fb < nbins) {  // loads while boxes land
            if (a.occ) ib = __ldg(a.occ + tb + fb);
            nd = a.data[ib];
        }
        __syncwarp();  // lane-dependent code ends: reconverge the warp (here and below)
        if (owner) {
            // phase A: m r over the owner's units for the lane's 4 bins (r split hi + lo,
            // packed FP32 pairs accumulated against the bins' anchors: error-free up to
            // ~2^-47 of the anchor per term)
            float2 sg01, sg23;
            op_anchors(a, tb + 4 * quad, rmax, rsum, sg01, sg23);
            float2 a01 = sg01, a23 = sg23, l01 = make_float2(0.f, 0.f), l23 = l01;
#pragma unroll
            for (int j = 0; j < kUnits; ++j) {
                const int u = warp + kOwners * j;
                if (u >= nunits || !ok) break;
                const int c = u >> 1, h = u & 1;
                int rs = s0 + (c >> lp);
                uint32_t ph = ph0;
                if (rs >= runs) { rs -= runs; ph ^= 1u; }
                const int s = (rs << lp) + (c & (P - 1));
                if (!op_wait(&full[rs], ph, s_abort, err, 2, a.budget)) { ok = false; break; }
                const float *bp = ring + (size_t)s * GE::kBoxFloats + (32 * h + g) * BINS + 4 * quad;
                const float2 *rp = rr + c * kBoxCols + 32 * h + g;
#pragma unroll
                for (int k = 0; k < GU; ++k) {
                    const float4 m = *(const float4 *)(bp + k * RPL * BINS);
                    const float2 rv = rp[RPL * k];
                    const float2 h2 = make_float2(rv.x, rv.x), l2 = make_float2(rv.y, rv.y);
                    sfh_anc_acc2(a01, l01, make_float2(m.x, m.y), h2, l2);
                    sfh_anc_acc2(a23, l23, make_float2(m.z, m.w), h2, l2);
                }
            }
            __syncwarp();
            const sfh_df av[4] = {sfh_anc_result(a01.x, l01.x, sg01.x), sfh_anc_result(a01.y, l01.y, sg01.y),
                                  sfh_anc_result(a23.x, l23.x, sg23.x), sfh_anc_result(a23.y, l23.y, sg23.y)};
            // sum over the lanes that hold the same bins (other rows)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                sfh_df v = av[k];
#pragma unroll
                for (int o = LPR; o <= 16; o <<= 1) {
                    const sfh_df u{__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
                    v = df_add_fast(v, u);
                }
                if (lane < LPR) s_part[warp * BINS + 4 * quad + k] = v;
            }
            __syncwarp();
        }
        named_bar_sync(1, kWarps * 32);
        if (finisher) {
            // the bin's owner partials: lane fl takes owners fl, fl + LB, ...; a fixed
            // butterfly over the LB lanes; lane fl == 0 keeps the total
            sfh_df cm{0.f, 0.f};
#pragma unroll
            for (int o = 0; o < kOwners; o += LB)
                if (o + fl < kOwners) cm = df_add_fast(cm, s_part[(o + fl) * BINS + fb]);
#pragma unroll
            for (int o = LB / 2; o >= 1; o >>= 1) {
                const sfh_df u{__shfl_xor_sync(0xffffffffu, cm.h, o), __shfl_xor_sync(0xffffffffu, cm.l, o)};
                cm = df_add_fast(cm, u);
            }
            const int64_t i = tb + fb;
            if (fl == 0) {
                float wv = 0.f;
                if (i < nbins) {
                    if (!want_g) a.composite[ib] = sfh_f2d(cm.h) + sfh_f2d(cm.l);  // the model, unclamped
                    // max(composite, eps(T)); eps(T) is a power of two, exact in FP32
                    if (cm.h < a.eps_f || (cm.h == a.eps_f && cm.l < 0.f)) cm = sfh_df{a.eps_f, 0.f};
                    float nh, nl;
                    sfh_split_double(nd, nh, nl);
                    if (want_g) {
                        wv = __fdiv_rn(df_add(cm, sfh_df{-nh, -nl}).h, cm.h);  // 1 - n/c
                        a.composite[ib] = sfh_f2d(wv);
                    }
                    s_cn[fb] = make_float4(cm.h, cm.l, nh, nl);
                }
                s_w[fb] = wv;
            }
            if (threadIdx.x == 0) *s_stop = *s_abort;
            __syncwarp();
        }
        named_bar_sync(1, kWarps * 32);
        if (*s_stop) break;  // the same decision in every consumer warp
        if (owner) {
            // phase B: M w over the owner's units from the resident boxes (packed FP32 pairs),
            // compensated per row over the tiles; each unit's box is released after its read
            const float4 w4 = *(const float4 *)(s_w + 4 * quad);
            const float2 w01 = make_float2(w4.x, w4.y), w23 = make_float2(w4.z, w4.w);
#pragma unroll
            for (int j = 0; j < kUnits; ++j) {
                const int u = warp + kOwners * j;
                if (u >= nunits) break;
                const int c = u >> 1, h = u & 1;
                int rs = s0 + (c >> lp);
                if (rs >= runs) rs -= runs;
                const int s = (rs << lp) + (c & (P - 1));
                if (want_g) {
                    const float *bp = ring + (size_t)s * GE::kBoxFloats + (32 * h + g) * BINS + 4 * quad;
#pragma unroll
                    for (int k = 0; k < GU; ++k) {
                        const float4 m = *(const float4 *)(bp + k * RPL * BINS);
                        g2[j][k] = __ffma2_rn(make_float2(m.z, m.w), w23,
                                              __ffma2_rn(make_float2(m.x, m.y), w01, g2[j][k]));
                    }
                }
                __syncwarp();
                if (lane == 0) {
                    mbar_arrive(&empty[rs]);
                    if (u == nunits - 1 && short_extra) mbar_arrive_n(&empty[rs], short_extra);
                }
                __syncwarp();
            }
        } else {
            // warp 14: the tile's Poisson terms
            if (a.want_logl && lane < BINS && tb + lane < nbins) {
                const float4 cn = s_cn[lane];
                term = df_add(term, sfh_bin_term(sfh_df{cn.x, cn.y}, cn.z, cn.w, s_tab));
            }
            __syncwarp();
        }
        s0 += nr;  // nr <= runs: at most one wrap
        if (s0 >= runs) { s0 -= runs; ph0 ^= 1u; }
    }
    else {
    // Skewed schedule (runs >= 2 nr): iteration it runs phase B of the CTA's tile it - 1
    // and phase A of its tile it in the same barrier interval, so the two phases' latency
    // chains overlap, then finishes tile it.  Per unit the owner reads the resident box of
    // tile it - 1 (phase B) and releases it before waiting for tile it's box (phase A);
    // the two tiles occupy disjoint slots.
    const int nloc = (a.ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1;
    int sB = 0;        // first slot of tile it - 1
    for (int it = 0; it <= nloc; ++it) {
        const bool doA = it < nloc, doB = it > 0;  // the same in every warp
        const int64_t tb = ((int64_t)blockIdx.x + (int64_t)it * gridDim.x) * BINS;  // tile it
        double nd = 0.0;
        int64_t ib = tb + fb;
        if (doA && finisher && fl == 0 && tb + fb < nbins) {
            if (a.occ) ib = __ldg(a.occ + tb + fb);
            nd = a.data[ib];
        }
        __syncwarp();
        if (owner) {
            float2 sg01 = make_float2(1.f, 1.f), sg23 = sg01;
            if (doA) op_anchors(a, tb + 4 * quad, rmax, rsum, sg01, sg23);
            float2 a01 = sg01, a23 = sg23, l01 = make_float2(0.f, 0.f), l23 = l01;
            float2 w01 = make_float2(0.f, 0.f), w23 = w01;
            if (doB) {
                const float4 w4 = *(const float4 *)(s_w + 4 * quad);
                w01 = make_float2(w4.x, w4.y);
                w23 = make_float2(w4.z, w4.w);
            }
#pragma unroll
            for (int j = 0; j < kUnits; ++j) {
                const int u = warp + kOwners * j;
                if (u >= nunits) break;
                const int c = u >> 1, h = u & 1;
                const int rowoff = (32 * h + g) * BINS + 4 * quad;
                if (doB) {  // phase B of tile it - 1
                    int rs = sB + (c >> lp);
                    if (rs >= runs) rs -= runs;
                    const int s = (rs << lp) + (c & (P - 1));
                    if (want_g) {
                        const float *bp = ring + (size_t)s * GE::kBoxFloats + rowoff;
#pragma unroll
                        for (int k = 0; k < GU; ++k) {
                            const float4 m = *(const float4 *)(bp + k * RPL * BINS);
                            g2[j][k] = __ffma2_rn(make_float2(m.z, m.w), w23,
                                                  __ffma2_rn(make_float2(m.x, m.y), w01, g2[j][k]));
                        }
                    }
                    __syncwarp();
                    if (lane == 0) {
                        mbar_arrive(&empty[rs]);
                        if (u == nunits - 1 && short_extra) mbar_arrive_n(&empty[rs], short_extra);
                    }
                    __syncwarp();
                }
                if (doA && ok) {  // phase A of tile it
                    int rs = s0 + (c >> lp);
                    uint32_t ph = ph0;
                    if (rs >= runs) { rs -= runs; ph ^= 1u; }
                    const int s = (rs << lp) + (c & (P - 1));
                    if (!op_wait(&full[rs], ph, s_abort, err, 2, a.budget)) {
                        ok = false;
                    } else {
                        const float *bp = ring + (size_t)s * GE::kBoxFloats + rowoff;
                        const float2 *rp = rr + c * kBoxCols + 32 * h + g;
#pragma unroll
                        for (int k = 0; k < GU; ++k) {
                            const float4 m = *(const float4 *)(bp + k * RPL * BINS);
                            const float2 rv = rp[RPL * k];
                            const float2 h2 = make_float2(rv.x, rv.x), l2 = make_float2(rv.y, rv.y);
                            sfh_anc_acc2(a01, l01, make_float2(m.x, m.y), h2, l2);
                            sfh_anc_acc2(a23, l23, make_float2(m.z, m.w), h2, l2);
                        }
                    }
                    __syncwarp();
                }
            }
            if (doA) {
                const sfh_df av[4] = {sfh_anc_result(a01.x, l01.x, sg01.x), sfh_anc_result(a01.y, l01.y, sg01.y),
                                      sfh_anc_result(a23.x, l23.x, sg23.x), sfh_anc_result(a23.y, l23.y, sg23.y)};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    sfh_df v = av[k];
#pragma unroll
                    for (int o = LPR; o <= 16; o <<= 1) {
                        const sfh_df uu{__shfl_xor_sync(0xffffffffu, v.h, o),
                                        __shfl_xor_sync(0xffffffffu, v.l, o)};
                        v = df_add_fast(v, uu);
                    }
                    if (lane < LPR) s_part[warp * BINS + 4 * quad + k] = v;
                }
            }
            __syncwarp();
        } else {
            // warp OWN: the Poisson terms of tile it - 1 (s_cn from its finish)
            const int64_t tbB = tb - (int64_t)gridDim.x * BINS;
            if (doB && a.want_logl && lane < BINS && tbB + lane < nbins) {
                const float4 cn = s_cn[lane];
                term = df_add(term, sfh_bin_term(sfh_df{cn.x, cn.y}, cn.z, cn.w, s_tab));
            }
            __syncwarp();
        }
        if (!doA) break;
        named_bar_sync(1, kWarps * 32);
        if (finisher) {
            sfh_df cm{0.f, 0.f};
#pragma unroll
            for (int o = 0; o < kOwners; o += LB)
                if (o + fl < kOwners) cm = df_add_fast(cm, s_part[(o + fl) * BINS + fb]);
#pragma unroll
            for (int o = LB / 2; o >= 1; o >>= 1) {
                const sfh_df uu{__shfl_xor_sync(0xffffffffu, cm.h, o), __shfl_xor_sync(0xffffffffu, cm.l, o)};
                cm = df_add_fast(cm, uu);
            }
            const int64_t i = tb + fb;
            if (fl == 0) {
                float wv = 0.f;
                if (i < nbins) {
                    if (!want_g) a.composite[ib] = sfh_f2d(cm.h) + sfh_f2d(cm.l);
                    if (cm.h < a.eps_f || (cm.h == a.eps_f && cm.l < 0.f)) cm = sfh_df{a.eps_f, 0.f};
                    float nh, nl;
                    sfh_split_double(nd, nh, nl);
                    if (want_g) {
                        wv = __fdiv_rn(df_add(cm, sfh_df{-nh, -nl}).h, cm.h);
                        a.composite[ib] = sfh_f2d(wv);
                    }
                    s_cn[fb] = make_float4(cm.h, cm.l, nh, nl);
                }
                s_w[fb] = wv;
            }
            if (threadIdx.x == 0) *s_stop = *s_abort;
            __syncwarp();
        }
        named_bar_sync(1, kWarps * 32);
        if (*s_stop) break;
        sB = s0;
        s0 += nr;  // 2 nr <= runs: at most one wrap
        if (s0 >= runs) { s0 -= runs; ph0 ^= 1u; }
    }
    }
    // per-CTA partials of G: the lanes of a row (bin quads) summed once
    if (want_g && owner) {
#pragma unroll
        for (int j = 0; j < kUnits; ++j) {
            const int u = warp + kOwners * j;
            if (u >= nunits) break;
#pragma unroll
            for (int k = 0; k < GU; ++k) {
                // FP32 sums of the lanes' packed partials (2 LPR terms, 2^-24 relative each,
                // below the FP32 accumulation over the tiles); double-float across the CTAs
                float v = g2[j][k].x + g2[j][k].y;
#pragma unroll
                for (int o = 1; o < LPR; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                const int64_t col = (int64_t)(u >> 1) * kBoxCols + 32 * (u & 1) + g + RPL * k;
                if (quad == 0 && col < a.nt)
                    a.gpart[(int64_t)blockIdx.x * a.nt + col] = make_float2(v, 0.f);
            }
        }
    }
    if (a.want_logl && warp == kPoissonWarp) {
        const sfh_df tot = sfh_df_warp_sum(term);
        // the plan's empty bins: -Σ_j r_j E_j over this CTA's share of the columns (the
        // share it reduces below)
        double te = 0.0;
        if (a.colsum_e) {
            const int per = (int)((a.nt + gridDim.x - 1) / gridDim.x);
            for (int c = lane; c < per; c += 32) {
                const int64_t j = (int64_t)blockIdx.x * per + c;
                if (j < a.nt) te = fma(a.r[j], a.colsum_e[j], te);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) te += __shfl_down_sync(0xffffffffu, te, o);
        }
        if (lane == 0) a.lpart[blockIdx.x] = (sfh_f2d(tot.h) + sfh_f2d(tot.l)) - te;
    }

    // ------------------------------------------------------------ grid reduction
    // Every CTA of the launch is resident (one per SM): after a grid barrier CTA b sums
    // columns [b per, (b+1) per) of G over all CTAs' partials (one warp per column, lanes
    // over CTAs, a fixed shuffle tree) and CTA 0 sums -logL: a fixed order, so results are
    // reproducible.  The barrier's wait is bounded like the pipeline's.
    named_bar_sync(1, kWarps * 32);  // this CTA's partials are written
    if (threadIdx.x == 0) op_grid_barrier(a);
    named_bar_sync(1, kWarps * 32);
    if (a.empty && *(volatile unsigned int *)a.viol != 0u) {
        // some plan-empty bin is occupied in this call's data: every CTA folds in the ones
        // of its share exactly (the same arithmetic as a tile bin), then a second barrier
        op_fold_occupied(a, s_tab, (double *)s_part);
        named_bar_sync(1, kWarps * 32);
        if (threadIdx.x == 0) op_grid_barrier(a);
        named_bar_sync(1, kWarps * 32);
        if (blockIdx.x == 0 && threadIdx.x == 0) {  // every CTA read the count before
            *(volatile unsigned int *)a.viol = 0u;  // the second barrier
            *(volatile unsigned int *)a.flag = 1u;  // the host builds a new plan
        }
    }
    // every CTA is past the last grid barrier: the next dependent launch may start
    if (a.pdl) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const bool bad = *(volatile unsigned int *)a.err != 0u;
    if (a.G) {  // warp w sums columns j0 + w, j0 + w + kWarps, ...: lane l takes CTAs
                // l, l + 32, ..., then a fixed shuffle tree
        const int per = (int)((a.nt + gridDim.x - 1) / gridDim.x);
        for (int cw = warp; cw < per; cw += kWarps) {
            const int64_t j = (int64_t)blockIdx.x * per + cw;
            if (j >= a.nt) break;
            // up to 12 CTAs' partials per lane (grid <= 2 x SMs <= 384), loads issued together;
            // double-float sums on the FP32 pipes, one FP64 add per column at the end
            float2 v[12];
#pragma unroll
            for (int q = 0; q < 12; ++q) {
                const int p = lane + 32 * q;
                v[q] = p < (int)gridDim.x ? __ldcg(a.gpart + (int64_t)p * a.nt + j)
                                          : make_float2(0.f, 0.f);
            }
            sfh_df acc{0.f, 0.f};
#pragma unroll
            for (int q = 0; q < 12; ++q) acc = df_add(acc, sfh_df{v[q].x, v[q].y});
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const sfh_df u{__shfl_down_sync(0xffffffffu, acc.h, o),
                               __shfl_down_sync(0xffffffffu, acc.l, o)};
                acc = df_add(acc, u);
            }
            if (lane == 0) {
                double gj = sfh_f2d(acc.h) + sfh_f2d(acc.l);
                if (a.colsum_e) gj += a.colsum_e[j];  // the empty bins, w = 1
                a.G[j] = bad ? NAN : a.gsign * gj;
            }
        }
    }
    if (a.negLogL && blockIdx.x == 0 && warp == 0) {
        double v[12];
#pragma unroll
        for (int q = 0; q < 12; ++q) {
            const int p = lane + 32 * q;
            v[q] = p < (int)gridDim.x ? __ldcg(a.lpart + p) : 0.0;
        }
        double acc = 0.0;
#pragma unroll
        for (int q = 0; q < 12; ++q) acc += v[q];
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

// Blocked copy of a plan's occupied rows for BINS-bin tiles: as k_onepass_block with tile
// bin p standing for bin occ[p] (occ[p] < 0: padding, zero).
__global__ void k_occ_block(const float *__restrict__ M, int64_t nbins, int64_t nt, int bins,
                            int nch, int64_t total, const int *__restrict__ occ,
                            float *__restrict__ blk) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int64_t b = idx % bins, rest = idx / bins;
    const int64_t j = rest % kBoxCols, tc = rest / kBoxCols;
    const int64_t c = tc % nch, t = tc / nch;
    const int bin = occ[t * bins + b];
    const int64_t col = c * kBoxCols + j;
    blk[idx] = (bin >= 0 && col < nt) ? M[col * nbins + bin] : 0.f;
}

// Row statistics of the tile bins (zero for padding).
__global__ void k_occ_rowb(const float2 *__restrict__ rowb, const int *__restrict__ occ, int64_t n,
                           float2 *__restrict__ out) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int bin = occ[p];
    out[p] = bin >= 0 ? rowb[bin] : make_float2(0.f, 0.f);
}

// E_j = Σ over the empty bins of M_ij in FP64, one block per template (fixed tree).
__global__ void k_occ_colsum(const float *__restrict__ M, int64_t nbins,
                             const int *__restrict__ empty, int64_t nempty,
                             double *__restrict__ out) {
    __shared__ double s_red[32];
    const int64_t j = blockIdx.x;
    double acc = 0.0;
    for (int64_t k = threadIdx.x; k < nempty; k += blockDim.x) acc += (double)M[j * nbins + empty[k]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += s_red[w];
        out[j] = tot;
    }
}

// Counts of the occupied bins for the derived handle (out[p] = data[rows[p]]) and the check
// that the plan's empty bins are still empty (their count into *viol).
__global__ void k_occ_gather(const double *__restrict__ data, const int *__restrict__ rows,
                             int64_t nocc, const int *__restrict__ empty, int64_t nempty,
                             double *__restrict__ out, unsigned int *viol) {
    unsigned int nv = 0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nocc || k < nempty;
         k += (int64_t)gridDim.x * blockDim.x) {
        if (k < nocc) out[k] = data[rows[k]];
        if (k < nempty) nv += data[empty[k]] != 0.0 ? 1u : 0u;
    }
    if (nv) atomicAdd(viol, nv);
}

// Shared memory a CTA may use when `per_sm` CTAs share an SM.
int op_max_smem(sfh_ctx *ctx, int per_sm) {
    static int optin = -1, per_smp = 0, reserved = 0;
    if (optin < 0) {
        int v = 0, w = 0, r = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device) != cudaSuccess) v = 0;
        if (cudaDeviceGetAttribute(&w, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device) != cudaSuccess) w = 0;
        if (cudaDeviceGetAttribute(&r, cudaDevAttrReservedSharedMemoryPerBlock, ctx->device) != cudaSuccess) r = 0;
        optin = v;
        per_smp = w;
        reserved = r;
    }
    if (per_sm <= 1) return optin;
    const int share = per_smp / per_sm - reserved;
    return share < optin ? share : optin;
}

// Run-slots (of 2^lp boxes each) for BINS-bin tiles of a matrix with nch boxes per tile, with
// tiles_resident tiles held at once, and `owners` owner
// warps: the resident tile plus prefetch (0 if it does not fit).
int op_runs(sfh_ctx *ctx, int bins, int owners, int nch, int lp, int tiles_resident) {
    const int maxs = op_max_smem(ctx, owners >= 8 ? 1 : 2);
    int slots = kMaxSlots;
    while (slots > 0 && op_smem_bytes(bins, owners, slots, nch) > (size_t)maxs) --slots;
    int runs = slots >> lp;
    runs -= runs % kProducers;  // each run-slot is refilled by one producer lane
    const int nr = (nch + (1 << lp) - 1) >> lp;
    // the resident tiles' runs plus one in flight
    return runs >= tiles_resident * nr + 1 ? runs : 0;
}

template <int BINS, int OWN, bool SKEW>
int launch_onepass(sfh_ctx *ctx, const OnePassArgs &a0, int grid, cudaStream_t st) {
    using GE = Geo<BINS, OWN>;
    static size_t attr_set = 0;
    const size_t smem = op_smem_bytes(BINS, OWN, a0.slots, a0.nch);
    if (smem > attr_set) {
        SFH_CK(ctx, cudaFuncSetAttribute(k_fg_onepass<BINS, OWN, SKEW>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = smem;
    }
    // grid <= SMs x kMinBlocks and that many CTAs fit an SM (checked by the caller): the
    // CTAs are resident together, as the in-kernel grid reduction needs; its barrier wait
    // is bounded all the same
    if (a0.pdl) {
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3(GE::kThreads);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        SFH_CK(ctx, cudaLaunchKernelEx(&cfg, k_fg_onepass<BINS, OWN, SKEW>, a0));
    } else {
        k_fg_onepass<BINS, OWN, SKEW><<<grid, GE::kThreads, smem, st>>>(a0);
    }
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

// CTAs of the variant an SM holds at once with `smem` bytes (occupancy query, cached).
template <int BINS, int OWN>
int op_resident(size_t smem) {
    static size_t q_smem = 0;
    static int q_blocks = 0;
    if (smem != q_smem) {
        cudaFuncSetAttribute(k_fg_onepass<BINS, OWN, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fg_onepass<BINS, OWN, false>,
                                                          Geo<BINS, OWN>::kThreads, smem) != cudaSuccess)
            b = 0;
        q_smem = smem;
        q_blocks = b;
    }
    return q_blocks;
}

}  // namespace

bool sfh_onepass_eligible(sfh_ctx *ctx, const sfh_models *m) {
    if (!m || m->storage == SFH_F64 || !m->d_f32) return false;
    if (m->nbins > INT32_MAX - 64 || m->nt > kMaxTemplates) return false;
    const int nch = (int)((m->nt + kBoxCols - 1) / kBoxCols);
    return op_runs(ctx, 16, 14, nch, 0, 1) > 0;
}

// The variant later launches take on this handle: the requested tile width, CTAs per SM,
// schedule and boxes per run where they fit, else the nearest that does (fewer boxes per
// run, the phased schedule, 16-bin tiles on one CTA per SM).  Returns false when nothing
// fits.
bool sfh_onepass_choose(sfh_ctx *ctx, const sfh_models *m, OnePassChoice *c) {
    const int nch = (int)((m->nt + kBoxCols - 1) / kBoxCols);
    int bins = m->onepass_bins == 32 ? 32 : 16;
    int per_sm = (m->onepass_ctas == 2 && bins == 16) ? 2 : 1;
    bool skew = m->onepass_skew == 1 && bins == 16 && per_sm == 1;
    int runs = 0, lp = 0;
    auto pick = [&](int b, int owners, int resident) {
        const int pref = m->onepass_lp >= 0 ? m->onepass_lp : (b == 16 ? 2 : 1);
        for (int l = pref; l >= 0; --l) {
            const int r = op_runs(ctx, b, owners, nch, l, resident);
            if (r) { runs = r; lp = l; return; }
        }
        runs = 0;
    };
    pick(bins, per_sm == 2 ? 6 : 14, skew ? 2 : 1);
    if (runs && per_sm == 2 &&  // two CTAs must fit an SM
        op_resident<16, 6>(op_smem_bytes(16, 6, runs << lp, nch)) < 2)
        runs = 0;
    if (!runs && skew) {
        skew = false;
        pick(bins, 14, 1);
    }
    if (!runs) {
        bins = 16;
        per_sm = 1;
        skew = false;
        pick(16, 14, 1);
    }
    c->bins = bins;
    c->per_sm = per_sm;
    c->skew = skew ? 1 : 0;
    c->runs = runs;
    c->lp = lp;
    return runs > 0;
}

// ------------------------------------------------------------------ occupied-bin plans
static void occ_plan_free(SfhOccPlan &p) {
    for (int k = 0; k < 2; ++k) {
        if (p.d_occ[k]) cudaFree(p.d_occ[k]);
        if (p.d_blk[k]) cudaFree(p.d_blk[k]);
        if (p.d_rowb[k]) cudaFree(p.d_rowb[k]);
    }
    if (p.d_empty) cudaFree(p.d_empty);
    if (p.d_colsum_e) cudaFree(p.d_colsum_e);
    if (p.d_viol) cudaFree(p.d_viol);
    if (p.h_flag) cudaFreeHost((void *)p.h_flag);
    if (p.sub) sfh_models_free(p.sub);
    if (p.d_rows) cudaFree(p.d_rows);
    if (p.d_nocc) cudaFree(p.d_nocc);
    if (p.h_bviol) cudaFreeHost((void *)p.h_bviol);
    p = SfhOccPlan{};
}

void sfh_occ_plans_free(sfh_models *m) {
    for (int k = 0; k < m->nocc_plans; ++k) occ_plan_free(m->occ[k]);
    m->nocc_plans = 0;
}

// A new plan for the diagram at d_data (device, mapped or host-page-table memory): one
// synchronous copy of the counts to the host, the bin lists, E_j.  The per-width parts
// come from occ_plan_width, from the same snapshot.
static int occ_plan_build(sfh_ctx *ctx, sfh_models *m, const void *key, const double *d_data,
                          int streak, SfhOccPlan &p) {
    const auto t0 = std::chrono::steady_clock::now();
    const int64_t nbins = m->nbins, nt = m->nt;
    std::vector<double> h((size_t)nbins);
    SFH_CK(ctx, cudaMemcpyAsync(h.data(), d_data, (size_t)nbins * 8, cudaMemcpyDefault, ctx->stream));
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<int> empty, occ;
    for (int64_t i = 0; i < nbins; ++i) {
        if (h[i] != 0.0) occ.push_back((int)i);  // NaN and negative counts stay tile bins
        else empty.push_back((int)i);
    }
    p = SfhOccPlan{};
    p.key = key;
    p.streak = streak;
    p.nocc = (int64_t)occ.size();
    p.nempty = (int64_t)empty.size();
    const bool some = p.nocc > 0 && p.nempty > 0;
    p.sparse = some && streak < 3 &&
               (m->occ_mode == SFH_OCC_ON || (double)p.nocc <= 0.6 * (double)nbins);
    if (p.sparse) {
        p.occ_host = std::move(occ);
        SFH_CK(ctx, cudaMalloc(&p.d_empty, (size_t)p.nempty * sizeof(int)));
        SFH_CK(ctx, cudaMalloc(&p.d_colsum_e, (size_t)nt * sizeof(double)));
        SFH_CK(ctx, cudaMalloc(&p.d_viol, sizeof(unsigned int)));
        void *hf = nullptr;
        SFH_CK(ctx, cudaHostAlloc(&hf, sizeof(unsigned int), cudaHostAllocMapped));
        p.h_flag = (volatile unsigned int *)hf;
        *p.h_flag = 0u;
        SFH_CK(ctx, cudaHostGetDevicePointer((void **)&p.d_flag, hf, 0));
        SFH_CK(ctx, cudaMemcpyAsync(p.d_empty, empty.data(), (size_t)p.nempty * sizeof(int),
                                    cudaMemcpyHostToDevice, ctx->stream));
        SFH_CK(ctx, cudaMemsetAsync(p.d_viol, 0, sizeof(unsigned int), ctx->stream));
        k_occ_colsum<<<(unsigned)nt, 256, 0, ctx->stream>>>(m->d_f32, nbins, p.d_empty, p.nempty,
                                                          p.d_colsum_e);
        SFH_LAUNCHED(ctx);
        SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));  // `empty` leaves scope
    }
    m->occ_build_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return SFH_OK;
}

// The tile-width parts of a sparse plan (occupied bins padded to whole tiles, their
// blocked rows and row statistics), built on first use of the width.
static int occ_plan_width(sfh_ctx *ctx, sfh_models *m, SfhOccPlan &p, int bins, int mi, int nch) {
    if (p.d_blk[mi]) return SFH_OK;
    const int64_t nbins = m->nbins, nt = m->nt;
    const int64_t ntiles = (p.nocc + bins - 1) / bins;
    std::vector<int> occ((size_t)(ntiles * bins), -1);
    std::copy(p.occ_host.begin(), p.occ_host.end(), occ.begin());
    const int64_t total = ntiles * nch * kBoxCols * bins;
    SFH_CK(ctx, cudaMalloc(&p.d_occ[mi], occ.size() * sizeof(int)));
    SFH_CK(ctx, cudaMalloc(&p.d_rowb[mi], occ.size() * sizeof(float2)));
    SFH_CK(ctx, cudaMalloc(&p.d_blk[mi], (size_t)total * sizeof(float)));
    SFH_CK(ctx, cudaMemcpyAsync(p.d_occ[mi], occ.data(), occ.size() * sizeof(int),
                                cudaMemcpyHostToDevice, ctx->stream));
    k_occ_rowb<<<(unsigned)((occ.size() + 255) / 256), 256, 0, ctx->stream>>>(
        m->d_rowb, p.d_occ[mi], (int64_t)occ.size(), p.d_rowb[mi]);
    SFH_LAUNCHED(ctx);
    k_occ_block<<<(unsigned)((total + 255) / 256), 256, 0, ctx->stream>>>(
        m->d_f32, nbins, nt, bins, nch, total, p.d_occ[mi], p.d_blk[mi]);
    SFH_LAUNCHED(ctx);
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));  // `occ` leaves scope
    return SFH_OK;
}

// The sparse plan serving `key` (the data pointer, or the handle's host-array slot) at
// this tile width, or NULL for the dense kernel.  A plan whose launches saw an occupied
// empty bin is retired and replaced; with every slot taken the least recently used plan
// that no capture holds is freed.  During stream capture only an existing, complete plan
// is used (and is then kept for the handle's lifetime).
static SfhOccPlan *occ_plan_get(sfh_ctx *ctx, sfh_models *m, const void *key,
                                const double *d_data, int bins, int mi, int nch, int *rc) {
    *rc = SFH_OK;
    if (m->occ_mode == SFH_OCC_OFF || !m->d_rowb || !key) return nullptr;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess) return nullptr;
    const bool capturing = cs != cudaStreamCaptureStatusNone;
    SfhOccPlan *p = nullptr;
    for (int k = 0; k < m->nocc_plans; ++k)
        if (!m->occ[k].retired && m->occ[k].key == key) p = &m->occ[k];
    int streak = 0;
    if (p && p->sparse && !capturing && *p->h_flag) {
        p->retired = true;
        streak = p->streak + 1;
        p = nullptr;
    }
    if (!p) {
        if (capturing) return nullptr;
        int slot = -1;
        if (m->nocc_plans < kSfhOccPlans) {
            slot = m->nocc_plans++;
        } else {  // evict: retired first, then the least recently used
            uint64_t best = UINT64_MAX;
            for (int k = 0; k < kSfhOccPlans; ++k) {
                const SfhOccPlan &q = m->occ[k];
                if (q.captured) continue;
                const uint64_t age = q.retired ? 0 : q.last_use + 1;
                if (age < best) { best = age; slot = k; }
            }
            if (slot < 0) return nullptr;  // every plan is held by a capture
            cudaError_t e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) {
                *rc = sfh_cuda_error(ctx, e, "occupied-bin plan eviction");
                return nullptr;
            }
            occ_plan_free(m->occ[slot]);
        }
        if ((*rc = occ_plan_build(ctx, m, key, d_data, streak, m->occ[slot]))) {
            occ_plan_free(m->occ[slot]);
            m->occ[slot].retired = true;
            return nullptr;
        }
        p = &m->occ[slot];
    }
    p->last_use = ++m->occ_clock;
    if (!p->sparse) return nullptr;
    if (!p->d_blk[mi]) {
        if (capturing) return nullptr;
        if ((*rc = occ_plan_width(ctx, m, *p, bins, mi, nch))) return nullptr;
    }
    if (capturing && !ctx->internal_capture) p->captured = true;
    return p;
}

// The batched path's part of a plan: the occupied bins, the derived handle of their rows,
// the gathered counts and the mapped check count (built on first use).
static int occ_plan_batched_parts(sfh_ctx *ctx, sfh_models *m, SfhOccPlan &p) {
    if (p.sub) return SFH_OK;
    SFH_CK(ctx, cudaMalloc(&p.d_rows, (size_t)p.nocc * sizeof(int)));
    SFH_CK(ctx, cudaMalloc(&p.d_nocc, (size_t)p.nocc * sizeof(double)));
    void *hv = nullptr;
    SFH_CK(ctx, cudaHostAlloc(&hv, sizeof(unsigned int), cudaHostAllocMapped));
    p.h_bviol = (volatile unsigned int *)hv;
    *p.h_bviol = 0u;
    SFH_CK(ctx, cudaHostGetDevicePointer((void **)&p.d_bviol, hv, 0));
    SFH_CK(ctx, cudaMemcpyAsync(p.d_rows, p.occ_host.data(), (size_t)p.nocc * sizeof(int),
                                cudaMemcpyHostToDevice, ctx->stream));
    return sfh_models_derive_rows(ctx, m, p.d_rows, p.nocc, p.d_colsum_e, &p.sub);  // syncs
}

void sfh_occ_retire(SfhOccPlan *p) {
    if (p) p->retired = true;
}

int sfh_occ_batched(sfh_ctx *ctx, sfh_models *m, const double *d_data, bool want_l,
                    const sfh_models **mb, const double **db, SfhOccPlan **plan) {
    *mb = m;
    *db = d_data;
    *plan = nullptr;
    if (m->occ_mode == SFH_OCC_OFF || m->storage != SFH_BF16X2 || !m->colsum || !m->d_f32)
        return SFH_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
        return SFH_OK;
    SfhOccPlan *p = nullptr;
    for (int k = 0; k < m->nocc_plans; ++k)
        if (!m->occ[k].retired && m->occ[k].key == d_data) p = &m->occ[k];
    int streak = 0;
    if (p && p->sparse && (*p->h_flag || (p->h_bviol && *p->h_bviol))) {
        p->retired = true;
        streak = p->streak + 1;
        p = nullptr;
    }
    if (!p) {
        int slot = -1;
        if (m->nocc_plans < kSfhOccPlans) {
            slot = m->nocc_plans++;
        } else {
            uint64_t best = UINT64_MAX;
            for (int k = 0; k < kSfhOccPlans; ++k) {
                const SfhOccPlan &q = m->occ[k];
                if (q.captured) continue;
                const uint64_t age = q.retired ? 0 : q.last_use + 1;
                if (age < best) { best = age; slot = k; }
            }
            if (slot < 0) return SFH_OK;
            SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
            occ_plan_free(m->occ[slot]);
        }
        int rc = occ_plan_build(ctx, m, d_data, d_data, streak, m->occ[slot]);
        if (rc) {
            occ_plan_free(m->occ[slot]);
            m->occ[slot].retired = true;
            return rc;
        }
        p = &m->occ[slot];
    }
    p->last_use = ++m->occ_clock;
    if (!p->sparse) return SFH_OK;
    int rc = occ_plan_batched_parts(ctx, m, *p);
    if (rc) {
        p->retired = true;
        return rc;
    }
    if (want_l && !sfh_exact_supported(p->sub)) return SFH_OK;  // the split logL needs it
    *p->h_bviol = 0u;  // the previous batched call on this plan has completed (it synced)
    const int64_t n = p->nocc > p->nempty ? p->nocc : p->nempty;
    k_occ_gather<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, ctx->stream>>>(
        d_data, p->d_rows, p->nocc, p->d_empty, p->nempty, p->d_nocc, p->d_bviol);
    SFH_LAUNCHED(ctx);
    *mb = p->sub;
    *db = p->d_nocc;
    *plan = p;
    return SFH_OK;
}

extern "C" int sfh_models_set_occupied(sfh_ctx *ctx, sfh_models *m, int mode) {
    if (!ctx || !m || mode < SFH_OCC_OFF || mode > SFH_OCC_ON) return SFH_ERR_ARG;
    if (mode != m->occ_mode)  // plans were chosen under the old mode
        for (int k = 0; k < m->nocc_plans; ++k) m->occ[k].retired = true;
    m->occ_mode = mode;
    return SFH_OK;
}

extern "C" int sfh_models_occupied_info(sfh_ctx *ctx, const sfh_models *m, const double *d_data,
                                        int64_t *nocc_out, int *sparse_out, double *build_ms_out) {
    if (!ctx || !m) return SFH_ERR_ARG;
    const SfhOccPlan *p = nullptr;
    for (int k = 0; k < m->nocc_plans; ++k)
        if (!m->occ[k].retired && m->occ[k].key == d_data) p = &m->occ[k];
    if (nocc_out) *nocc_out = p ? p->nocc : -1;
    if (sparse_out) *sparse_out = p && p->sparse ? 1 : 0;
    if (build_ms_out) *build_ms_out = m->occ_build_ms;
    return SFH_OK;
}

size_t sfh_onepass_scratch(const sfh_ctx *ctx, const sfh_models *m) {  // up to 2 CTAs per SM
    return sfh_align256((size_t)2 * ctx->sm_count * (size_t)m->nt * 8) +
           sfh_align256((size_t)2 * ctx->sm_count * 8);
}

int sfh_launch_fg_onepass(sfh_ctx *ctx, sfh_models *m, const double *d_coeffs,
                          const double *d_data, double *d_composite, double *d_G,
                          double *d_negLogL, double eps, double gsign, void *scratch,
                          cudaEvent_t *ev, const int *d_skip, const void *occ_key) {
    const int64_t nbins = m->nbins, nt = m->nt;
    const int nch = (int)((nt + kBoxCols - 1) / kBoxCols);
    OnePassChoice ch{};
    if (!sfh_onepass_choose(ctx, m, &ch))
        return sfh_set_error(ctx, SFH_ERR_UNSUPPORTED, "one-pass fg!: shape does not fit");
    const int bins = ch.bins, per_sm = ch.per_sm;
    const bool skew = ch.skew != 0;  // 16-bin tiles, one CTA per SM, two tiles resident
    const int mi = bins == 16 ? 0 : 1;
    int prc = SFH_OK;
    SfhOccPlan *pl =
        d_G ? occ_plan_get(ctx, m, occ_key ? occ_key : d_data, d_data, bins, mi, nch, &prc) : nullptr;
    if (prc) return prc;
    const int ntiles = (int)(((pl ? pl->nocc : nbins) + bins - 1) / bins);
    bool built = false;  // a kernel of this call writes the blocked copy
    if (!pl && !m->d_blk[mi]) {  // the blocked copy, once per handle and tile width
        built = true;
        const int64_t total = (int64_t)ntiles * nch * kBoxCols * bins;
        SFH_CK(ctx, cudaMalloc(&m->d_blk[mi], (size_t)total * sizeof(float)));
        k_onepass_block<<<(unsigned)((total + 255) / 256), 256, 0, ctx->stream>>>(
            m->d_f32, nbins, nt, bins, nch, total, m->d_blk[mi]);
        SFH_LAUNCHED(ctx);
    }
    // the grid reduction takes at most 384 CTAs' partials per column
    const int cap = ctx->sm_count * per_sm < 384 ? ctx->sm_count * per_sm : 384;
    const int grid = ntiles < cap ? ntiles : cap;
    OnePassArgs a{};
    a.blk = pl ? pl->d_blk[mi] : m->d_blk[mi];
    a.nbins = pl ? pl->nocc : nbins;
    a.nbins_all = nbins;
    if (pl) {
        a.occ = pl->d_occ[mi];
        a.empty = pl->d_empty;
        a.nempty = pl->nempty;
        a.colsum_e = pl->d_colsum_e;
        a.viol = pl->d_viol;
        a.flag = pl->d_flag;
        a.mcol = m->d_f32;
    }
    a.nt = nt;
    a.ntiles = ntiles;
    a.nch = nch;
    a.slots = ch.runs << ch.lp;
    a.runs = ch.runs;
    a.lp = ch.lp;
    a.r = d_coeffs;
    a.data = d_data;
    a.composite = d_composite;
    a.gpart = d_G ? (float2 *)scratch : nullptr;
    a.lpart = (double *)((char *)scratch + sfh_align256((size_t)2 * ctx->sm_count * (size_t)nt * 8));
    a.err = ctx->d_counters + SFH_CNT_ONEPASS_ERR;
    a.bar = ctx->d_counters + SFH_CNT_ONEPASS_BAR;
    a.tab = ctx->d_df_tab;
    a.eps_f = (float)eps;
    a.want_logl = d_negLogL ? 1 : 0;
    a.gsign = gsign;
    a.G = d_G;
    a.negLogL = d_negLogL;
    a.skip = d_skip;
    a.rowb = pl ? pl->d_rowb[mi] : m->d_rowb;
    a.budget = ctx->wait_budget;
    a.drop_copy = ctx->inject == SFH_INJECT_DROP_COPY ? 1 : 0;
    {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        const bool capturing = cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess ||
                               cs != cudaStreamCaptureStatusNone;
        a.pdl = (ctx->pdl && !built && !d_skip && !capturing && !ev) ? 1 : 0;
    }
    if (a.drop_copy) ctx->inject = SFH_INJECT_NONE;  // one shot
    if (!a.rowb) return sfh_set_error(ctx, SFH_ERR_ARG, "models handle has no row statistics");
    cudaStream_t st = ctx->stream;
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[0], st));
    int rc = per_sm == 2 ? launch_onepass<16, 6, false>(ctx, a, grid, st)
             : skew       ? launch_onepass<16, 14, true>(ctx, a, grid, st)
             : bins == 16 ? launch_onepass<16, 14, false>(ctx, a, grid, st)
                          : launch_onepass<32, 14, false>(ctx, a, grid, st);
    if (rc) return rc;
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[1], st));
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[2], st));
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[3], st));
    if (ev) SFH_CK(ctx, cudaEventRecord(ev[4], st));
    return SFH_OK;
}
