// simulate.cu -- model_cmd (src/simulate.jl:621-680): mock observation of a catalogue of
// stellar magnitudes.  Star i is kept when a uniform draw u_i <= c_i (the product of its
// single-filter completeness values, evaluated by the caller like the reference's
// callables); a kept star's magnitudes become m_ij + z_ij σ_ij + b_ij with standard normal
// z_ij.  The kept stars keep their input order (the reference's findall).
//
// Draws are counter-based (Philox4x32-10 keyed by the seed; u_i from counter (i, 0), the
// normals of star i from counter (i, 1 + pair of filters), Box-Muller), so a star's draws
// do not depend on the launch shape or on which other stars are kept.  Three launches:
// per-chunk keep counts, an exclusive scan of the counts, and an order-preserving scatter
// (per-chunk prefix by warp ballots).
#include <algorithm>
#include <cmath>

#include "sfh_internal.cuh"
#include "sfh_philox.cuh"

namespace {

constexpr int kMcThreads = 256;
constexpr int kMcPer = 8;                           // stars per thread
constexpr int kMcChunk = kMcThreads * kMcPer;       // stars per block
constexpr int kMcMaxFilters = 8;

__device__ __forceinline__ bool mc_keep(uint64_t seed, int64_t i, double c) {
    const sfh_rng::u4 r = sfh_rng::philox(sfh_rng::u4{(uint32_t)i, (uint32_t)(i >> 32), 0u, 0u},
                                          (uint32_t)seed, (uint32_t)(seed >> 32));
    return sfh_rng::u01(r.x, r.y) <= c;
}

// Keep counts per chunk of kMcChunk stars (thread t takes stars base + t*kMcPer + k).
__global__ void __launch_bounds__(kMcThreads)
k_mc_count(const double *__restrict__ compl_, int64_t n, uint64_t seed, int64_t *__restrict__ counts) {
    __shared__ int s_red[kMcThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kMcChunk + (int64_t)threadIdx.x * kMcPer;
    int c = 0;
#pragma unroll
    for (int k = 0; k < kMcPer; ++k) {
        const int64_t i = base + k;
        if (i < n && mc_keep(seed, i, compl_[i])) ++c;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int tot = 0;
        for (int w = 0; w < kMcThreads / 32; ++w) tot += s_red[w];
        counts[blockIdx.x] = tot;
    }
}

// Exclusive scan of the chunk counts in place (one block, sequential over 1,024-wide
// pieces); total kept into *total.
__global__ void __launch_bounds__(1024) k_mc_scan(int64_t *__restrict__ counts, int64_t nchunks,
                                                  int64_t *__restrict__ total) {
    __shared__ int64_t s[1024];
    __shared__ int64_t s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int64_t b0 = 0; b0 < nchunks; b0 += 1024) {
        const int64_t b = b0 + threadIdx.x;
        const int64_t v = b < nchunks ? counts[b] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
            const int64_t add = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
            __syncthreads();
            s[threadIdx.x] += add;
            __syncthreads();
        }
        if (b < nchunks) counts[b] = s_carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) s_carry += s[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = s_carry;
}

// Order-preserving scatter of the kept stars with their errors and biases applied.
__global__ void __launch_bounds__(kMcThreads)
k_mc_scatter(const double *__restrict__ mags, const double *__restrict__ sigma,
             const double *__restrict__ bias, const double *__restrict__ compl_, int64_t n,
             int nf, uint64_t seed, const int64_t *__restrict__ offsets,
             double *__restrict__ out, int64_t *__restrict__ idx) {
    __shared__ int s_warp[kMcThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kMcChunk + (int64_t)threadIdx.x * kMcPer;
    bool keep[kMcPer];
    int c = 0;
#pragma unroll
    for (int k = 0; k < kMcPer; ++k) {
        const int64_t i = base + k;
        keep[k] = i < n && mc_keep(seed, i, compl_[i]);
        c += keep[k] ? 1 : 0;
    }
    // exclusive prefix of c over the block (threads in star order)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    int wbase = 0;
    for (int w = 0; w < warp; ++w) wbase += s_warp[w];
    int64_t pos = offsets[blockIdx.x] + wbase + incl - c;
#pragma unroll
    for (int k = 0; k < kMcPer; ++k) {
        if (!keep[k]) continue;
        const int64_t i = base + k;
        for (int f = 0; f < nf; f += 2) {
            const sfh_rng::u4 r = sfh_rng::philox(
                sfh_rng::u4{(uint32_t)i, (uint32_t)(i >> 32), 1u + (uint32_t)(f >> 1), 0u},
                (uint32_t)seed, (uint32_t)(seed >> 32));
            const double rad = sqrt(-2.0 * log(sfh_rng::u01(r.x, r.y)));
            const double ang = 2.0 * sfh_rng::u01(r.z, r.w);
            const double z0 = rad * cospi(ang), z1 = rad * sinpi(ang);
            const int64_t a = i * nf + f;
            out[pos * nf + f] = mags[a] + z0 * sigma[a] + (bias ? bias[a] : 0.0);
            if (f + 1 < nf)
                out[pos * nf + f + 1] = mags[a + 1] + z1 * sigma[a + 1] + (bias ? bias[a + 1] : 0.0);
        }
        idx[pos] = i;
        ++pos;
    }
}

}  // namespace

// Device buffers, ordered on the context's stream: d_mags, d_sigma, d_bias (NULL = no bias)
// are n x nf row-major (star-major, as the reference's vector of per-star vectors);
// d_compl (n) the stars' detection probabilities.  d_out (n x nf capacity) and d_idx (n
// capacity, 0-based input indices) receive the kept stars in input order; *n_out their
// number (the call synchronises to read it).
extern "C" int sfh_model_cmd_dev(sfh_ctx *ctx, const double *d_mags, const double *d_sigma,
                                 const double *d_bias, const double *d_compl, int64_t n, int nf,
                                 uint64_t seed, double *d_out, int64_t *d_idx, int64_t *n_out) {
    if (!ctx || !n_out || n < 0 || nf < 1 || nf > kMcMaxFilters ||
        (n > 0 && (!d_mags || !d_sigma || !d_compl || !d_out || !d_idx)))
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    *n_out = 0;
    if (n == 0) return SFH_OK;
    const int64_t nchunks = (n + kMcChunk - 1) / kMcChunk;
    if (nchunks > INT32_MAX) return sfh_set_error(ctx, SFH_ERR_SHAPE, "model_cmd: too many stars");
    int rc = sfh_scratch_reserve(ctx, sfh_align256((size_t)(nchunks + 1) * 8));
    if (rc) return rc;
    int64_t *counts = (int64_t *)ctx->scratch, *total = counts + nchunks;
    cudaStream_t st = ctx->stream;
    k_mc_count<<<(unsigned)nchunks, kMcThreads, 0, st>>>(d_compl, n, seed, counts);
    SFH_LAUNCHED(ctx);
    k_mc_scan<<<1, 1024, 0, st>>>(counts, nchunks, total);
    SFH_LAUNCHED(ctx);
    k_mc_scatter<<<(unsigned)nchunks, kMcThreads, 0, st>>>(d_mags, d_sigma, d_bias, d_compl, n, nf,
                                                          seed, counts, d_out, d_idx);
    SFH_LAUNCHED(ctx);
    if ((rc = sfh_host_stage_reserve(ctx, 8))) return rc;
    SFH_CK(ctx, cudaMemcpyAsync(ctx->h_stage, total, 8, cudaMemcpyDeviceToHost, st));
    SFH_CK(ctx, cudaStreamSynchronize(st));
    *n_out = *(const int64_t *)ctx->h_stage;
    return SFH_OK;
}

// Host arrays, as sfh_model_cmd_dev (out and idx with capacity n x nf and n).
extern "C" int sfh_model_cmd(sfh_ctx *ctx, const double *mags, const double *sigma,
                             const double *bias, const double *compl_, int64_t n, int nf,
                             uint64_t seed, double *out, int64_t *idx, int64_t *n_out) {
    if (!ctx || !n_out || n < 0 || nf < 1 || nf > kMcMaxFilters ||
        (n > 0 && (!mags || !sigma || !compl_ || !out || !idx)))
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    *n_out = 0;
    if (n == 0) return SFH_OK;
    const size_t mat = sfh_align256((size_t)n * nf * 8), vec = sfh_align256((size_t)n * 8);
    const size_t o_s = mat, o_b = 2 * mat, o_c = 3 * mat, o_o = 3 * mat + vec,
                 o_i = 4 * mat + vec, total = o_i + vec;
    int rc = sfh_stage_reserve(ctx, total);
    if (rc) return rc;
    char *b = (char *)ctx->stage;
    cudaStream_t st = ctx->stream;
    SFH_CK(ctx, cudaMemcpyAsync(b, mags, (size_t)n * nf * 8, cudaMemcpyHostToDevice, st));
    SFH_CK(ctx, cudaMemcpyAsync(b + o_s, sigma, (size_t)n * nf * 8, cudaMemcpyHostToDevice, st));
    if (bias) SFH_CK(ctx, cudaMemcpyAsync(b + o_b, bias, (size_t)n * nf * 8, cudaMemcpyHostToDevice, st));
    SFH_CK(ctx, cudaMemcpyAsync(b + o_c, compl_, (size_t)n * 8, cudaMemcpyHostToDevice, st));
    int64_t m = 0;
    rc = sfh_model_cmd_dev(ctx, (const double *)b, (const double *)(b + o_s),
                           bias ? (const double *)(b + o_b) : nullptr, (const double *)(b + o_c), n,
                           nf, seed, (double *)(b + o_o), (int64_t *)(b + o_i), &m);
    if (rc) return rc;
    if (m > 0) {
        SFH_CK(ctx, cudaMemcpyAsync(out, b + o_o, (size_t)m * nf * 8, cudaMemcpyDeviceToHost, st));
        SFH_CK(ctx, cudaMemcpyAsync(idx, b + o_i, (size_t)m * 8, cudaMemcpyDeviceToHost, st));
        SFH_CK(ctx, cudaStreamSynchronize(st));
    }
    *n_out = m;
    return SFH_OK;
}
