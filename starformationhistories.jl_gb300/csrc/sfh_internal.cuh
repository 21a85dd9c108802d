// sfh_internal.cuh -- shared declarations of the sm_103a Hess-diagram library.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <functional>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sfhgpu.h"
#include "sfh_dfloat.cuh"

struct sfh_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    // Growable device scratch arena (one per context; single stream => no races).
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    // Device staging used by the host-array entry points.
    void *stage = nullptr;
    size_t stage_bytes = 0;
    // Mapped pinned host staging of the host-array entry points and its device alias.
    void *h_stage = nullptr, *d_h_stage = nullptr;
    size_t h_stage_bytes = 0;
    // Zero-initialised counters for last-block reductions (reset by the last block).
    unsigned int *d_counters = nullptr;
    // log(1 + j/128), j = 0..128, then n - n log n, n = 0..255, as double-float pairs
    // (sfh_dfloat.cuh), for the Poisson terms evaluated on the FP32 pipes.
    sfh_df *d_df_tab = nullptr;
    int64_t launches = 0;
    // Budget of the single-vector pipeline's device waits (SM cycles) and the one-shot
    // failure injection of the error-path tests (SFH_INJECT_*).
    long long wait_budget = 4000000000LL;
    int inject = 0;
    // The device reads pageable host memory through the host's page tables (a coherent
    // host link): the host-array fg! then hands the caller's own arrays to the kernels.
    bool pageable_direct = false;
    // Set while the library captures a graph that it destroys before returning (resources
    // such a graph uses need no pin beyond the call).
    bool internal_capture = false;
    // Single-vector one-pass launches overlap the previous one's tail (programmatic
    // dependent launch); sfh_ctx_set_overlap turns it off.
    bool pdl = true;
    int host_access = SFH_HOST_ACCESS_AUTO;  // sfh_ctx_set_host_access
    // Completion word of the host-array calls (sfh_host_call_wait): after a call's kernels
    // the stream writes a sequence number into mapped pinned memory with a stream memory
    // operation, which fences the kernels' writes first, and the host polls the word
    // instead of synchronising the stream.  write_value32 NULL: plain synchronisation.
    volatile unsigned int *h_done = nullptr;
    void *d_done = nullptr;
    unsigned int done_seq = 0;
    void *write_value32 = nullptr;  // cuStreamWriteValue32 (driver entry point)
};

// Waits for the work queued on ctx->stream by a host-array call (see sfh_ctx::h_done):
// polls the completion word for up to 2 ms, then falls back to cudaStreamSynchronize,
// which also reports any error the stream met.
cudaError_t sfh_host_call_wait(sfh_ctx *ctx);

// Occupied-bin plan of the single-vector fg! (onepass.cu).  With G requested, fg! needs the
// composite only where n_i > 0: an empty bin (n_i <= 0) has w_i = 1 - 0/max(c_i, eps) = 1
// exactly and contributes -max(c_i, eps) to logL, so its terms are sums over the template
// column: Σ_{i empty} M_ij w_i = E_j and Σ_{i empty} c_i = Σ_j r_j E_j (to eps per bin).
// The plan keeps, for one observed Hess diagram, the occupied bins, a blocked copy of their
// template rows and E_j; the kernel streams only those rows and checks every call that the
// empty bins are still empty (a bin that is not is corrected inside the same launch, and
// the next call builds a new plan).
struct SfhOccPlan {
    const void *key = nullptr;    // the data pointer the plan was built for
    bool retired = false;         // superseded by a newer plan for the same key
    bool captured = false;        // launched under stream capture: a graph may hold it, so
                                  // it is never freed before the handle
    bool sparse = false;          // false: the dense kernel serves this data
    int streak = 0;               // plans retired in a row for this key (3: stay dense)
    uint64_t last_use = 0;
    int64_t nocc = 0, nempty = 0;
    std::vector<int> occ_host;    // the occupied bins of the snapshot the plan was built from
    // batched path (BF16X2 storage): a derived handle of the occupied rows, the occupied
    // bins, the counts gathered for it, and a mapped pinned count of plan-empty bins found
    // occupied by the last gather
    sfh_models *sub = nullptr;
    int *d_rows = nullptr;
    double *d_nocc = nullptr;
    volatile unsigned int *h_bviol = nullptr;
    unsigned int *d_bviol = nullptr;
    int *d_occ[2] = {nullptr, nullptr};   // per tile width: occupied bins, -1 padded to tiles
    float *d_blk[2] = {nullptr, nullptr};  // per tile width: blocked copy of the occupied rows
    float2 *d_rowb[2] = {nullptr, nullptr};  // per tile width: their row statistics
    int *d_empty = nullptr;       // empty bins (ascending)
    double *d_colsum_e = nullptr;  // E_j = Σ_{i empty} M_ij (FP64)
    unsigned int *d_viol = nullptr;  // violations seen in the current launch (reset in-kernel)
    volatile unsigned int *h_flag = nullptr;  // mapped pinned: set when a launch saw one
    unsigned int *d_flag = nullptr;           // its device alias
};
constexpr int kSfhOccPlans = 4;

struct sfh_models {
    int device = 0;
    int64_t nbins = 0, nt = 0;
    int storage = SFH_F32;
    // F64/F32: (nbins, nt) column-major.  BF16X2: unused.
    void *d_col = nullptr;
    // BF16X2 planes for the batched tensor-core path:
    //  col_hi/col_lo: (nbins_pad, nt_pad) column-major (K = bins contiguous) for G = Mᵀ W
    //  row_hi/row_lo: (nbins_pad, nt_pad) row-major    (K = templates contiguous) for C = M R
    __nv_bfloat16 *col_hi = nullptr, *col_lo = nullptr, *row_hi = nullptr, *row_lo = nullptr;
    // FP32 copy kept with BF16X2 storage so single-vector calls still work.
    float *d_f32 = nullptr;
    // Per bin (sum, max) of |M_ij| over the templates (FP32 and BF16X2 storage): the bound
    // from which the single-vector kernels pick their accumulation anchors.
    float2 *d_rowb = nullptr;
    int64_t nbins_pad = 0, nt_pad = 0;
    // Exact batched composite (batched_exact.cu): 5 BF16 digit planes of the templates,
    // plane q row i column j (rows padded to nbins_pad128, columns to nt_pad), and the
    // per-bin power-of-two scales 2^E_i (NULL when nt_pad > 2304).
    __nv_bfloat16 *digits = nullptr;
    float *escale = nullptr;
    int64_t nbins_pad128 = 0;
    double *colsum = nullptr;  // Σ_i M_ij per template (FP64)
    int m_negative = 0;        // a template value is negative
    // A handle derived from a parent's occupied rows (batched occupied-bin path): E_j, the
    // parent's column sums over its empty bins (borrowed from the parent's plan), added to
    // G; colsum above is the parent's full column sum.
    const double *colsum_e = nullptr;
    // Single-vector launch plan chosen by sfh_models_autotune (0 = built-in heuristics):
    // pass-1 template splits, pass-2 row chunk, pass-2 waves.
    int tune_ks = 0, tune_R = 0, tune_w2 = 0;
    // Single-vector fg! path (SFH_PATH_*): AUTO takes the one-pass kernel when the
    // shape fits it; sfh_models_autotune replaces AUTO by the faster measured path.
    int path = SFH_PATH_AUTO;
    double onepass_ms = 0.0;  // measured by sfh_models_autotune (0: not measured)
    // One-pass tile width (16 or 32 bins; 0: 16) and, per width, the blocked copy of d_f32
    // it streams (built on first use): for tile t and box c (64 templates) one contiguous
    // block of [64 templates][bins] floats, blocks in (tile, box) order, zero padded.
    int onepass_bins = 0;
    int onepass_ctas = 0;
    int onepass_skew = 0;  // 1: skewed schedule (phase B of one tile beside phase A of the next)
    int onepass_lp = -1;   // log2 boxes per bulk copy (-1: 2 for 16-bin tiles, 1 for 32-bin)  // one-pass CTAs per SM: 1 (14 owner warps) or 2 (6 each); 0: 1
    float *d_blk[2] = {nullptr, nullptr};
    // Occupied-bin plans (SFH_OCC_*): up to kSfhOccPlans observed diagrams, kept until the
    // handle is freed.
    int occ_mode = SFH_OCC_AUTO;
    SfhOccPlan occ[kSfhOccPlans];
    int nocc_plans = 0;
    uint64_t occ_clock = 0;
    double occ_build_ms = 0.0;  // host wall time of the last plan build
};

// Counter slots in sfh_ctx::d_counters (zeroed at context creation; every kernel that
// takes a ticket from a slot resets it before it exits).
enum {
    SFH_CNT_LOGL = 0,          // k_finalize last-block reduction
    SFH_CNT_BATCH = 1,
    SFH_CNT_FG_LOGL = 2,       // fused pass 1: last row tile
    SFH_CNT_ONEPASS_ERR = 3,   // one-pass fg!: a wait timed out (cleared by the host check)
    SFH_CNT_ONEPASS_BAR = 4,   // one-pass fg! grid barrier: arrivals (4), generation (5)
    SFH_CNT_ROWTILE = 256,     // fused pass 1: one per row tile (<= 32768)
    SFH_CNT_COLGROUP = 256 + 32768,  // fused pass 2: one per column group (<= 16384)
    SFH_CNT_SLOTS = 65536
};

// ------------------------------------------------------------------ error helpers
int sfh_set_error(sfh_ctx *ctx, int code, const std::string &msg);
int sfh_cuda_error(sfh_ctx *ctx, cudaError_t e, const char *what);

#define SFH_CK(ctx, call)                                                     \
    do {                                                                      \
        cudaError_t _e = (call);                                              \
        if (_e != cudaSuccess) return sfh_cuda_error((ctx), _e, #call);       \
    } while (0)

#define SFH_LAUNCHED(ctx)                                                     \
    do {                                                                      \
        (ctx)->launches++;                                                    \
        cudaError_t _e = cudaGetLastError();                                  \
        if (_e != cudaSuccess) return sfh_cuda_error((ctx), _e, "kernel launch"); \
    } while (0)

// Ensures ctx->scratch holds at least `bytes` (256-byte aligned sub-allocations).
int sfh_scratch_reserve(sfh_ctx *ctx, size_t bytes);
int sfh_stage_reserve(sfh_ctx *ctx, size_t bytes);
int sfh_host_stage_reserve(sfh_ctx *ctx, size_t bytes);

static inline size_t sfh_align256(size_t b) { return (b + 255) & ~size_t(255); }

// ------------------------------------------------------------------ shared device math
// Compensated FP32 accumulation: (hi, lo) += x.
__device__ __forceinline__ void sfh_two_sum_acc(float &hi, float &lo, float x) {
    const float s = __fadd_rn(hi, x);
    const float bp = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    hi = s;
    lo = __fadd_rn(lo, err);
}

// ------------------------------------------------------------------ anchored sums
// Error-free accumulation of products m*r (r = h + l, two FP32 numbers) against a
// power-of-two anchor.  The accumulator a starts at sigma, a power of two with
// |sum of all terms| <= sigma/2, so every intermediate a lies in [sigma/2, 2 sigma):
//   s  = fma(m, h, a)          one rounding, at ulp(sigma)
//   nu = a - s                 exact (Sterbenz: a and s are within a factor 2)
//   e  = fma(m, h, nu)         = (m h + a) - s, the rounding error of s, to 2^-24 of itself
//   lo = fma(m, l, lo + e)     the error and the low product, both ~2^-24 of the terms
// The sum is (a - sigma) + lo, a - sigma exact; its error is ~2^-47 sigma per term
// instead of the 2^-25 |partial| of a plain FP32 chain, so the composite carries
// ~1e-12 relative error for sigma within a few powers of two of it.  (The anchor is the
// "extraction against a power of two" of error-free vector transformations: Rump, Ogita,
// Oishi, "Accurate floating-point summation", SIAM J. Sci. Comput. 31(1), 2008.)
__device__ __forceinline__ void sfh_anc_acc(float &a, float &lo, float m, float h, float l) {
    const float s = __fmaf_rn(m, h, a);
    const float e = __fmaf_rn(m, h, __fsub_rn(a, s));
    lo = __fmaf_rn(m, l, __fadd_rn(lo, e));
    a = s;
}
// The same on packed pairs (two bins at once, FFMA2 / FADD2).
__device__ __forceinline__ void sfh_anc_acc2(float2 &a, float2 &lo, float2 m, float2 h, float2 l) {
    const float2 s = __ffma2_rn(m, h, a);
    const float2 nu = __ffma2_rn(s, make_float2(-1.f, -1.f), a);  // a - s, exact
    const float2 e = __ffma2_rn(m, h, nu);
    lo = __ffma2_rn(m, l, __fadd2_rn(lo, e));
    a = s;
}
// Anchor for a sum bounded by b >= 0: the power of two 2^(E+3) where b < 2^(E+1), i.e.
// at least 4 b (so a bound a little short of the true one still leaves the factor-2
// margin); 2^-124 for b = 0 or subnormal b (all terms then vanish or stay below it).
__device__ __forceinline__ float sfh_anchor(float b) {
    const int ex = (int)((__float_as_uint(b) >> 23) & 0xffu);  // b >= 0
    return __uint_as_float((unsigned int)min(ex + 3, 254) << 23);
}
// Bound of |sum_j M_ij r_j| for bin i from the handle's row statistics (sum and max of
// |M_ij| over j) and the coefficients' max and sum of |r_j|, inflated for the rounding of
// those FP32 statistics.
__device__ __forceinline__ float sfh_row_bound(float2 rowb, float rmax, float rsum) {
    return fminf(rmax * rowb.x, rsum * rowb.y) * 1.0009765625f;
}
// (a - sigma) + lo as a normalised double-float (a - sigma is exact).
__device__ __forceinline__ sfh_df sfh_anc_result(float a, float lo, float sigma) {
    return df_two_sum(__fsub_rn(a, sigma), lo);
}

// log1p(d) - d for d = c/n - 1 > -1, in FP32 without cancellation (relative error
// < 6e-7 for eps <= c <= 1e30, checked against 40-digit arithmetic).  With
// z = d / (2 + d):  log1p(d) = 2 atanh(z)  and  d - 2z = d z, hence
// log1p(d) - d = -d z + 2 z^3 (1/3 + z^2/5 + z^4/7 + ...).
__device__ __forceinline__ float sfh_log1p_minus_id(float d, float c, float n) {
    if (fabsf(d) <= 0.5f) {
        const float z = __fdividef(d, 2.0f + d);
        const float z2 = z * z;
        float S = 1.0f / 17.0f;
        S = fmaf(S, z2, 1.0f / 15.0f);
        S = fmaf(S, z2, 1.0f / 13.0f);
        S = fmaf(S, z2, 1.0f / 11.0f);
        S = fmaf(S, z2, 1.0f / 9.0f);
        S = fmaf(S, z2, 1.0f / 7.0f);
        S = fmaf(S, z2, 1.0f / 5.0f);
        S = fmaf(S, z2, 1.0f / 3.0f);
        return fmaf(2.0f * z * z2, S, -d * z);
    }
    if (d < 0.0f) return logf(__fdividef(c, n)) - d;  // c/n < 1/2: log of the ratio itself
    return log1pf(d) - d;
}

// Conversions between double and float without the FP64 pipe (GB300 retires FP64 and
// FP64<->FP32 conversions at a small fraction of its FP32 rate).  Exact bit moves for the
// common cases -- a double that holds a float value (counts), a normal float -- and the
// ordinary conversion otherwise.
static __device__ __noinline__ void sfh_split_double_slow(double x, float &h, float &l) {
    h = __double2float_rn(x);
    l = __double2float_rn(x - (double)h);
}
static __device__ __noinline__ double sfh_f2d_slow(float f) { return (double)f; }
__device__ __forceinline__ void sfh_split_double(double x, float &h, float &l) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned int e = (unsigned int)(b >> 52) & 0x7ffu;
    if ((b << 1) == 0ull) {  // +-0
        h = __uint_as_float((unsigned int)(b >> 32));
        l = 0.f;
    } else if ((b & 0x1fffffffull) == 0ull && e >= 897u && e <= 1150u) {  // a normal float
        h = __uint_as_float(((unsigned int)(b >> 32) & 0x80000000u) | ((e - 896u) << 23) |
                            (unsigned int)((b >> 29) & 0x7fffffull));
        l = 0.f;
    } else {  // not a float value: the ordinary conversion, kept out of line
        sfh_split_double_slow(x, h, l);
    }
}
// x = h + l for any double in the normal float range, with integer operations only: h
// keeps the top 24 significant bits (truncated), l is the remaining 29 bits rounded to a
// float (|h + l - x| <= 2^-47 |x|, |l| < 2^-23 |h|); the FP64 conversions otherwise.
__device__ __forceinline__ void sfh_split_any(double x, float &h, float &l) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned int e = (unsigned int)(b >> 52) & 0x7ffu;
    if (e >= 960u && e <= 1150u) {  // 2^-63 <= |x| < 2^128
        const unsigned int sg = (unsigned int)(b >> 32) & 0x80000000u;
        h = __uint_as_float(sg | ((e - 896u) << 23) | (unsigned int)((b >> 29) & 0x7fffffull));
        const float lm = __fmul_rn(__uint2float_rn((unsigned int)(b & 0x1fffffffull)),
                                   __uint_as_float((e - 948u) << 23));  // rem 2^(e - 1075)
        l = __uint_as_float(__float_as_uint(lm) | sg);
    } else {
        sfh_split_double(x, h, l);
    }
}
__device__ __forceinline__ double sfh_f2d(float f) {
    const unsigned int u = __float_as_uint(f);
    const unsigned int e = (u >> 23) & 0xffu;
    const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
    if ((u << 1) == 0u) return __longlong_as_double((long long)s);  // +-0
    if (e == 0u || e == 0xffu) return sfh_f2d_slow(f);               // subnormal, inf, nan
    return __longlong_as_double((long long)(s | ((unsigned long long)(e + 896u) << 52) |
                                            ((unsigned long long)(u & 0x7fffffu) << 29)));
}

// Poisson term of one bin for the kernels: the branch-free double-float form, skipped as a
// whole when no active lane of the warp holds counts (empty bins give -c).
__device__ __forceinline__ sfh_df sfh_bin_term(sfh_df c, float nh, float nl, const sfh_df *s_tab) {
    if (!__any_sync(__activemask(), nh != 0.0f || nl != 0.0f)) return df_neg(c);
    return df_poisson_term_bf(c, nh, nl, s_tab, s_tab + SFH_DF_TAB_LOG);
}

// Sum of a double-float over the warp (all lanes receive it), FP32 operations only.
__device__ __forceinline__ sfh_df sfh_df_warp_sum(sfh_df v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const sfh_df u{__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
        v = df_add(v, u);
    }
    return v;
}

// Block sum of a double-float into a double at *out (thread 0); s_red holds one double per
// warp.  Every thread of the block must call it.
__device__ __forceinline__ void sfh_df_block_sum(sfh_df v, double *s_red, double *out) {
    v = sfh_df_warp_sum(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = sfh_f2d(v.h) + sfh_f2d(v.l);
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += s_red[w];
        *out = b;
    }
}

// ------------------------------------------------------------------ internal launchers
// Single-vector objective on device arrays (likelihood.cu).
struct FgArgs {
    const double *coeffs;   // nt (may be NULL when only loglikelihood/grad of a given composite)
    const double *data;     // nbins
    double *composite;      // nbins (in/out per mode)
    double *G;              // nt or NULL
    double *negLogL;        // device scalar or NULL
    double eps;
    double gsign;           // +1: gradient of -logL (fg!), -1: ∇loglikelihood!
    int mode;               // see FG_MODE_*
    const int *skip;        // device flag that turns the one-pass kernel into a no-op (or NULL)
    // key of the occupied-bin plan (NULL: the data pointer; the host-array entry passes
    // its handle slot, since its staging pointer is shared by every diagram)
    const void *occ_key;
};
enum {
    FG_MODE_FG = 0,          // composite from coeffs, then logL/G as requested
    FG_MODE_COMPOSITE = 1,   // composite only
    FG_MODE_GRAD_GIVEN = 2   // ∇loglikelihood! from a given composite
};
int sfh_launch_fg(sfh_ctx *ctx, const sfh_models *m, const FgArgs &a, cudaEvent_t *ev = nullptr);
// One-pass single-vector fg! (onepass.cu): FP32 storage, nt <= 1536.
bool sfh_onepass_eligible(sfh_ctx *ctx, const sfh_models *m);
size_t sfh_onepass_scratch(const sfh_ctx *ctx, const sfh_models *m);
int sfh_launch_fg_onepass(sfh_ctx *ctx, sfh_models *m, const double *d_coeffs,
                          const double *d_data, double *d_composite, double *d_G,
                          double *d_negLogL, double eps, double gsign, void *scratch,
                          cudaEvent_t *ev, const int *d_skip = nullptr,
                          const void *occ_key = nullptr);
void sfh_occ_plans_free(sfh_models *m);
// Batched occupied-bin path: the handle and counts the batched kernels take for the
// diagram at d_data (the parent's derived handle and the gathered counts, or m and d_data
// themselves), and the plan whose gather check the caller reads after its sync (NULL when
// dense).  Not during stream capture.
int sfh_occ_batched(sfh_ctx *ctx, sfh_models *m, const double *d_data, bool want_l,
                    const sfh_models **mb, const double **db, SfhOccPlan **plan);
// Retires a plan whose gather found a plan-empty bin occupied.
void sfh_occ_retire(SfhOccPlan *p);
// A BF16X2 handle of rows d_rows[0 .. nrows) of parent's FP32 matrix, with the parent's
// full column sums, its negative flag, and colsum_e as E_j.
int sfh_models_derive_rows(sfh_ctx *ctx, const sfh_models *parent, const int *d_rows,
                           int64_t nrows, const double *colsum_e, sfh_models **out);
struct OnePassChoice {
    int bins, per_sm, skew, runs, lp;
};
bool sfh_onepass_choose(sfh_ctx *ctx, const sfh_models *m, OnePassChoice *c);
// Reads and clears the one-pass timeout slot (synchronises the stream).
int sfh_check_onepass(sfh_ctx *ctx);
int sfh_launch_loglikelihood(sfh_ctx *ctx, const double *composite, const double *data,
                             int64_t nbins, double eps, double *d_out);

// Exact batched composite (batched_exact.cu): digit planes of the coefficients, their
// scales and the logL partials live in the batched plan's scratch.
#include <cuda.h>
struct SfhExactPlan {
    int64_t B = 0, B_pad = 0;
    int n_mt = 0, n_vt = 0;
    __nv_bfloat16 *Rd = nullptr;
    float *rscale = nullptr;
    int *nplanes = nullptr;   // [0] R planes, [1] negative-coefficient flag, [2] ticket
    double *kn = nullptr;     // Σ_{n>0} (n - n log n)
    double *csum = nullptr;   // per vector Σ_j R_bj colsum_j
    double *csum_e = nullptr; // per vector Σ_j R_bj E_j (derived occupied-bin handles)
    double *kpart = nullptr;  // block partials of Σ (n - n log n)
    float2 *lpart = nullptr;
    CUtensorMap maps[2];
};
bool sfh_exact_supported(const sfh_models *m);
int sfh_build_digit_planes(sfh_ctx *ctx, sfh_models *m);
size_t sfh_exact_scratch(const sfh_models *m, int64_t B, int64_t *B_pad_out);
int sfh_exact_prepare(sfh_ctx *ctx, const sfh_models *m, int64_t B, void *scratch, SfhExactPlan *xp);
int sfh_exact_launch(sfh_ctx *ctx, const sfh_models *m, const SfhExactPlan &xp, const double *d_R,
                     const double *d_data, double *d_negLogL, __nv_bfloat16 *W_hi,
                     __nv_bfloat16 *W_lo, int64_t w_ld, int want_w, double eps, int *d_err);

// Batched objective (batched.cu).  prepare() sizes/lays out scratch (scratch == NULL
// is a size query), converts the data and encodes the tensor maps; launch() only
// enqueues kernels (capturable in a CUDA graph); check() reads the timeout flag.
// With logL requested and exact planes available, the composite and the Poisson terms
// come from the exact digit-plane kernel; gradient-only calls keep the hi/lo form.
struct SfhBatchedPlan {
    int64_t B = 0, B_pad = 0;
    int m_tiles = 0, n_tiles1 = 0, n_tiles2 = 0, ks2 = 1, per2 = 0, kb2 = 0;
    size_t scratch_bytes = 0;
    __nv_bfloat16 *Rh = nullptr, *Rl = nullptr, *Wh = nullptr, *Wl = nullptr;
    float2 *lp = nullptr;
    float *gp = nullptr, *dataf = nullptr;
    int *err = nullptr;
    CUtensorMap maps[8];
    const double *data = nullptr;  // FP64 counts (the exact epilogue splits them itself)
    bool exact = false;
    SfhExactPlan xp;
};
int sfh_batched_prepare(sfh_ctx *ctx, const sfh_models *m, int64_t B, const double *d_data,
                        void *scratch, size_t scratch_bytes, SfhBatchedPlan *pl);
int sfh_batched_launch(sfh_ctx *ctx, const sfh_models *m, const SfhBatchedPlan &pl,
                       const double *d_R, double *d_negLogL, float *d_G, double eps);
int sfh_batched_check(sfh_ctx *ctx, const SfhBatchedPlan &pl);
int sfh_launch_fg_batched(sfh_ctx *ctx, const sfh_models *m, const double *d_R, int64_t B,
                          const double *d_data, double *d_negLogL, float *d_G, double eps);
// Device BFGS loop (fit.cu) over an objective that enqueues its evaluation at θt on the
// context stream: for the transforms of fit_templates it gets r = transform(θt) and writes
// fg!'s -logL and raw gradient; with transform kFitObjective (100) it writes f(θt) to f and
// ∇f(θt) to grad.  `skip` is a device flag set once the loop has finished (queued slots
// may turn into no-ops).
using SfhFitObjective = std::function<int(const double *theta_t, double *r, double *grad,
                                          double *f, const int *skip)>;
constexpr int SFH_FIT_OBJECTIVE = 100;
int sfh_bfgs_run(sfh_ctx *ctx, int64_t nvar, const double *d_theta0, const sfh_fit_options *opt,
                 int transform, const SfhFitObjective &objective, double *d_theta_out,
                 double *d_invH, sfh_fit_result *res);

// Per-bin (sum, max) of |M_ij| of an FP32 (nbins, nt) column-major matrix (core.cu).
int sfh_row_stats(sfh_ctx *ctx, const float *d_M, int64_t nbins, int64_t nt, float2 *d_out);
// Builds the BF16 hi/lo planes from an FP32 column-major matrix (batched.cu).
int sfh_build_bf16_planes(sfh_ctx *ctx, sfh_models *m, const float *d_f32);

// Templates (templates.cu).
int sfh_launch_stamps(sfh_ctx *ctx, const double *d_x, const double *d_y, const double *d_sx,
                      const double *d_sy, const double *d_w, const int64_t *d_start,
                      const int32_t *d_count, const int32_t *d_cov, int64_t ntempl,
                      double xf, double xs, int64_t nx, double yf, double ys, int64_t ny,
                      float *d_out);
