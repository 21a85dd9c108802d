// core.cu -- contexts, template-matrix handles, scratch, and the host-array
// entry points of the C ABI (include/sfhgpu.h).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <vector>

#include "sfh_internal.cuh"

// ------------------------------------------------------------------ errors
int sfh_set_error(sfh_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

int sfh_cuda_error(sfh_ctx *ctx, cudaError_t e, const char *what) {
    std::string msg = std::string(what) + ": " + cudaGetErrorName(e) + " (" +
                      cudaGetErrorString(e) + ")";
    return sfh_set_error(ctx, e == cudaErrorMemoryAllocation ? SFH_ERR_NOMEM : SFH_ERR_CUDA, msg);
}

extern "C" int sfh_abi_version(void) { return SFH_ABI_VERSION; }

extern "C" const char *sfh_status_string(int status) {
    switch (status) {
        case SFH_OK: return "ok";
        case SFH_ERR_ARG: return "invalid argument";
        case SFH_ERR_SHAPE: return "shape mismatch";
        case SFH_ERR_CUDA: return "CUDA error";
        case SFH_ERR_TIMEOUT: return "device wait timed out";
        case SFH_ERR_NOMEM: return "device out of memory";
        case SFH_ERR_UNSUPPORTED: return "unsupported device or configuration";
        case SFH_ERR_NUMERIC: return "non-finite input";
        default: return "unknown status";
    }
}

// ------------------------------------------------------------------ context
// The completion word (sfh_ctx::h_done): best effort, the context works without it.
static void sfh_done_init(sfh_ctx *ctx) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuStreamWriteValue32", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
        return;
    void *h = nullptr, *d = nullptr;
    if (cudaHostAlloc(&h, 64, cudaHostAllocMapped) != cudaSuccess) return;
    if (cudaHostGetDevicePointer(&d, h, 0) != cudaSuccess || !d) {
        cudaFreeHost(h);
        return;
    }
    *(volatile unsigned int *)h = 0u;
    ctx->h_done = (volatile unsigned int *)h;
    ctx->d_done = d;
    ctx->write_value32 = fn;
}

cudaError_t sfh_host_call_wait(sfh_ctx *ctx) {
    typedef CUresult (*WriteValue32)(CUstream, CUdeviceptr, cuuint32_t, unsigned int);
    if (!ctx->write_value32) return cudaStreamSynchronize(ctx->stream);
    const unsigned int seq = ++ctx->done_seq;
    if (((WriteValue32)ctx->write_value32)((CUstream)ctx->stream, (CUdeviceptr)ctx->d_done, seq,
                                           0u) != CUDA_SUCCESS) {
        ctx->write_value32 = nullptr;  // not available here: synchronise from now on
        return cudaStreamSynchronize(ctx->stream);
    }
    const auto t0 = std::chrono::steady_clock::now();
    for (unsigned int it = 1;; ++it) {
        if (__atomic_load_n((const unsigned int *)ctx->h_done, __ATOMIC_ACQUIRE) == seq)
            return cudaSuccess;
        if ((it & 255u) == 0u &&
            std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(2000))
            return cudaStreamSynchronize(ctx->stream);
    }
}

extern "C" int sfh_ctx_create(int device, sfh_ctx **out) {
    if (!out) return SFH_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return SFH_ERR_CUDA;
    if (device < 0 || device >= ndev) return SFH_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return SFH_ERR_CUDA;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return SFH_ERR_CUDA;
    // The library is compiled for sm_103a only (GB300).
    if (!(prop.major == 10 && prop.minor == 3)) return SFH_ERR_UNSUPPORTED;
    sfh_ctx *ctx = new sfh_ctx();
    ctx->device = device;
    ctx->sm_count = prop.multiProcessorCount;
    int pma = 0, pma_host = 0;
    if (cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, device) == cudaSuccess &&
        cudaDeviceGetAttribute(&pma_host, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                               device) == cudaSuccess)
        ctx->pageable_direct = pma && pma_host;
    sfh_df tab[SFH_DF_TAB_ALL];
    sfh_df_log_table(tab);
    sfh_df_nlogn_table(tab + SFH_DF_TAB_LOG);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&ctx->d_counters, sizeof(unsigned int) * SFH_CNT_SLOTS) != cudaSuccess ||
        cudaMemset(ctx->d_counters, 0, sizeof(unsigned int) * SFH_CNT_SLOTS) != cudaSuccess ||
        cudaMalloc(&ctx->d_df_tab, sizeof(tab)) != cudaSuccess ||
        cudaMemcpy(ctx->d_df_tab, tab, sizeof(tab), cudaMemcpyHostToDevice) != cudaSuccess) {
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        if (ctx->d_counters) cudaFree(ctx->d_counters);
        if (ctx->d_df_tab) cudaFree(ctx->d_df_tab);
        delete ctx;
        return SFH_ERR_CUDA;
    }
    sfh_done_init(ctx);
    *out = ctx;
    return SFH_OK;
}

extern "C" int sfh_ctx_destroy(sfh_ctx *ctx) {
    if (!ctx) return SFH_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->stage) cudaFree(ctx->stage);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    if (ctx->h_done) cudaFreeHost((void *)ctx->h_done);
    if (ctx->d_counters) cudaFree(ctx->d_counters);
    if (ctx->d_df_tab) cudaFree(ctx->d_df_tab);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SFH_OK;
}

extern "C" const char *sfh_ctx_last_error(const sfh_ctx *ctx) {
    return ctx ? ctx->last_error.c_str() : "null context";
}

extern "C" int sfh_ctx_synchronize(sfh_ctx *ctx) {
    if (!ctx) return SFH_ERR_ARG;
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return sfh_check_onepass(ctx);  // a timed-out one-pass fg! since the last check
}

extern "C" int sfh_ctx_set_wait_budget(sfh_ctx *ctx, int64_t cycles) {
    if (!ctx || cycles < 0 || (cycles > 0 && cycles < 100000)) return SFH_ERR_ARG;
    ctx->wait_budget = cycles ? (long long)cycles : 4000000000LL;
    return SFH_OK;
}

extern "C" int sfh_ctx_set_overlap(sfh_ctx *ctx, int on) {
    if (!ctx) return SFH_ERR_ARG;
    ctx->pdl = on != 0;
    return SFH_OK;
}

extern "C" int sfh_ctx_set_host_access(sfh_ctx *ctx, int mode) {
    if (!ctx || mode < SFH_HOST_ACCESS_AUTO || mode > SFH_HOST_ACCESS_DIRECT) return SFH_ERR_ARG;
    if (mode == SFH_HOST_ACCESS_DIRECT && !ctx->pageable_direct)
        return sfh_set_error(ctx, SFH_ERR_UNSUPPORTED,
                             "direct host access needs pageable memory access through the "
                             "host page tables");
    ctx->host_access = mode;
    return SFH_OK;
}

extern "C" int sfh_ctx_host_access(const sfh_ctx *ctx, int *mode_out) {
    if (!ctx || !mode_out) return SFH_ERR_ARG;
    *mode_out = ctx->host_access == SFH_HOST_ACCESS_AUTO
                    ? (ctx->pageable_direct ? SFH_HOST_ACCESS_DIRECT : SFH_HOST_ACCESS_STAGED)
                    : ctx->host_access;
    return SFH_OK;
}

extern "C" int sfh_ctx_inject_fault(sfh_ctx *ctx, int what) {
    if (!ctx || what < SFH_INJECT_NONE || what > SFH_INJECT_ALLOC_FAIL) return SFH_ERR_ARG;
    ctx->inject = what;
    return SFH_OK;
}

extern "C" int sfh_ctx_stream(sfh_ctx *ctx, void **stream_out) {
    if (!ctx || !stream_out) return SFH_ERR_ARG;
    *stream_out = (void *)ctx->stream;
    return SFH_OK;
}

extern "C" int sfh_ctx_launch_count(const sfh_ctx *ctx, int64_t *count_out) {
    if (!ctx || !count_out) return SFH_ERR_ARG;
    *count_out = ctx->launches;
    return SFH_OK;
}

// A one-shot injected allocation failure (SFH_INJECT_ALLOC_FAIL), refused on the host.
static int injected_alloc_failure(sfh_ctx *ctx) {
    if (ctx->inject != SFH_INJECT_ALLOC_FAIL) return SFH_OK;
    ctx->inject = SFH_INJECT_NONE;
    return sfh_set_error(ctx, SFH_ERR_NOMEM, "allocation refused (injected failure)");
}

static int reserve(sfh_ctx *ctx, void **buf, size_t *cur, size_t bytes) {
    if (bytes <= *cur) return SFH_OK;
    if (int rc = injected_alloc_failure(ctx)) return rc;
    // Growth is rare: drain the stream so the old buffer is no longer in use.
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (*buf) cudaFree(*buf);
    *buf = nullptr;
    *cur = 0;
    size_t want = bytes + bytes / 4;
    SFH_CK(ctx, cudaMalloc(buf, want));
    *cur = want;
    return SFH_OK;
}

int sfh_scratch_reserve(sfh_ctx *ctx, size_t bytes) {
    return reserve(ctx, &ctx->scratch, &ctx->scratch_bytes, bytes);
}
int sfh_stage_reserve(sfh_ctx *ctx, size_t bytes) {
    return reserve(ctx, &ctx->stage, &ctx->stage_bytes, bytes);
}
int sfh_host_stage_reserve(sfh_ctx *ctx, size_t bytes) {
    if (bytes <= ctx->h_stage_bytes) return SFH_OK;
    if (int rc = injected_alloc_failure(ctx)) return rc;
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    ctx->h_stage = nullptr;
    ctx->d_h_stage = nullptr;
    ctx->h_stage_bytes = 0;
    const size_t want = bytes + bytes / 4;
    // mapped pinned memory: kernels of the host-array entry points read their inputs from it
    // and write their outputs into it through its device alias (no separate DMA steps)
    SFH_CK(ctx, cudaHostAlloc(&ctx->h_stage, want, cudaHostAllocMapped));
    SFH_CK(ctx, cudaHostGetDevicePointer(&ctx->d_h_stage, ctx->h_stage, 0));
    ctx->h_stage_bytes = want;
    return SFH_OK;
}

// ------------------------------------------------------------------ models
static void free_models(sfh_models *m) {
    if (!m) return;
    cudaSetDevice(m->device);
    if (m->d_col) cudaFree(m->d_col);
    if (m->d_f32 && m->d_f32 != m->d_col) cudaFree(m->d_f32);
    if (m->col_hi) cudaFree(m->col_hi);
    if (m->col_lo) cudaFree(m->col_lo);
    if (m->row_hi) cudaFree(m->row_hi);
    if (m->row_lo) cudaFree(m->row_lo);
    for (float *b : m->d_blk)
        if (b) cudaFree(b);
    if (m->d_rowb) cudaFree(m->d_rowb);
    if (m->digits) cudaFree(m->digits);
    if (m->escale) cudaFree(m->escale);
    if (m->colsum) cudaFree(m->colsum);
    sfh_occ_plans_free(m);
    delete m;
}

extern "C" int sfh_models_free(sfh_models *m) {
    if (!m) return SFH_ERR_ARG;
    free_models(m);
    return SFH_OK;
}

extern "C" int sfh_models_info(const sfh_models *m, int64_t *nbins, int64_t *nt, int *storage) {
    if (!m) return SFH_ERR_ARG;
    if (nbins) *nbins = m->nbins;
    if (nt) *nt = m->nt;
    if (storage) *storage = m->storage;
    return SFH_OK;
}

namespace {
// One thread per bin: (sum, max) of |M_ij| over j (a warp reads 32 consecutive bins of a
// column: coalesced).  The sum is an FP32 sum of nonnegative terms (relative rounding below
// nt 2^-24, covered by the inflation in sfh_row_bound).
__global__ void k_row_stats(const float *__restrict__ M, int64_t nbins, int64_t nt,
                            float2 *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbins) return;
    float s = 0.f, mx = 0.f;
    for (int64_t j = 0; j < nt; ++j) {
        const float v = fabsf(__ldg(M + j * nbins + i));
        s += v;
        mx = fmaxf(mx, v);
    }
    // rounding of a long FP32 sum: bound it from above by the max times the count too
    out[i] = make_float2(fminf(s * (1.0f + 1e-3f), mx * (float)nt), mx);
}
}  // namespace

int sfh_row_stats(sfh_ctx *ctx, const float *d_M, int64_t nbins, int64_t nt, float2 *d_out) {
    k_row_stats<<<(unsigned)((nbins + 255) / 256), 256, 0, ctx->stream>>>(d_M, nbins, nt, d_out);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

// Finishes a handle whose FP32 column-major copy is in m->d_f32.
static int finish_models(sfh_ctx *ctx, sfh_models *m) {
    SFH_CK(ctx, cudaMalloc(&m->d_rowb, (size_t)m->nbins * sizeof(float2)));
    int rc0 = sfh_row_stats(ctx, m->d_f32, m->nbins, m->nt, m->d_rowb);
    if (rc0 != SFH_OK) return rc0;
    if (m->storage == SFH_F32) {
        m->d_col = m->d_f32;
    } else if (m->storage == SFH_BF16X2) {
        int rc = sfh_build_bf16_planes(ctx, m, m->d_f32);
        if (rc != SFH_OK) return rc;
        // digit planes of the exact logL path (batched_exact.cu)
        if ((rc = sfh_build_digit_planes(ctx, m)) != SFH_OK) return rc;
    }
    return SFH_OK;
}

extern "C" int sfh_models_upload(sfh_ctx *ctx, const void *host, int src_dtype, int64_t nbins,
                                 int64_t nt, int storage, sfh_models **out) {
    if (!ctx || !host || !out || nbins <= 0 || nt <= 0) return SFH_ERR_ARG;
    if (src_dtype != SFH_F64 && src_dtype != SFH_F32) return SFH_ERR_ARG;
    if (storage != SFH_F64 && storage != SFH_F32 && storage != SFH_BF16X2) return SFH_ERR_ARG;
    *out = nullptr;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    sfh_models *m = new sfh_models();
    m->device = ctx->device;
    m->nbins = nbins;
    m->nt = nt;
    m->storage = storage;
    const size_t n = (size_t)nbins * (size_t)nt;
    cudaError_t e;
    if (storage == SFH_F64) {
        e = cudaMalloc(&m->d_col, n * sizeof(double));
        if (e != cudaSuccess) { free_models(m); return sfh_cuda_error(ctx, e, "cudaMalloc models"); }
        if (src_dtype == SFH_F64) {
            e = cudaMemcpy(m->d_col, host, n * sizeof(double), cudaMemcpyHostToDevice);
        } else {
            std::vector<double> tmp(n);
            const float *src = (const float *)host;
            for (size_t i = 0; i < n; ++i) tmp[i] = src[i];
            e = cudaMemcpy(m->d_col, tmp.data(), n * sizeof(double), cudaMemcpyHostToDevice);
        }
        if (e != cudaSuccess) { free_models(m); return sfh_cuda_error(ctx, e, "upload models"); }
        *out = m;
        return SFH_OK;
    }
    e = cudaMalloc(&m->d_f32, n * sizeof(float));
    if (e != cudaSuccess) { free_models(m); return sfh_cuda_error(ctx, e, "cudaMalloc models"); }
    if (src_dtype == SFH_F32) {
        e = cudaMemcpy(m->d_f32, host, n * sizeof(float), cudaMemcpyHostToDevice);
    } else {
        // Round-to-nearest FP64 -> FP32 on the host, chunked to bound the temporary.
        const double *src = (const double *)host;
        const size_t chunk = (size_t)1 << 24;
        std::vector<float> tmp(n < chunk ? n : chunk);
        e = cudaSuccess;
        for (size_t off = 0; off < n && e == cudaSuccess; off += chunk) {
            const size_t cnt = (n - off) < chunk ? (n - off) : chunk;
            for (size_t i = 0; i < cnt; ++i) tmp[i] = (float)src[off + i];
            e = cudaMemcpy(m->d_f32 + off, tmp.data(), cnt * sizeof(float), cudaMemcpyHostToDevice);
        }
    }
    if (e != cudaSuccess) { free_models(m); return sfh_cuda_error(ctx, e, "upload models"); }
    int rc = finish_models(ctx, m);
    if (rc != SFH_OK) { free_models(m); return rc; }
    *out = m;
    return SFH_OK;
}

namespace {
// out[j nrows + p] = M[j nbins + rows[p]] (column-major gather of rows).
__global__ void k_gather_rows(const float *__restrict__ M, int64_t nbins, int64_t nt,
                              const int *__restrict__ rows, int64_t nrows, float *__restrict__ out) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nrows * nt) return;
    const int64_t j = idx / nrows, p = idx - j * nrows;
    out[idx] = M[j * nbins + rows[p]];
}
}  // namespace

int sfh_models_derive_rows(sfh_ctx *ctx, const sfh_models *parent, const int *d_rows,
                           int64_t nrows, const double *colsum_e, sfh_models **out) {
    *out = nullptr;
    if (!parent->d_f32 || nrows <= 0) return sfh_set_error(ctx, SFH_ERR_ARG, "derive_rows");
    sfh_models *m = new sfh_models();
    m->device = ctx->device;
    m->nbins = nrows;
    m->nt = parent->nt;
    m->storage = parent->storage;
    m->occ_mode = SFH_OCC_OFF;
    const int64_t n = nrows * parent->nt;
    cudaError_t e = cudaMalloc(&m->d_f32, (size_t)n * sizeof(float));
    if (e != cudaSuccess) { free_models(m); return sfh_cuda_error(ctx, e, "derive_rows alloc"); }
    k_gather_rows<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(parent->d_f32, parent->nbins,
                                                                      parent->nt, d_rows, nrows, m->d_f32);
    e = cudaGetLastError();
    if (e != cudaSuccess) { free_models(m); return sfh_cuda_error(ctx, e, "k_gather_rows"); }
    ctx->launches++;
    int rc = finish_models(ctx, m);
    if (rc == SFH_OK && parent->colsum && m->colsum)
        if ((e = cudaMemcpyAsync(m->colsum, parent->colsum, (size_t)m->nt * 8, cudaMemcpyDeviceToDevice,
                                 ctx->stream)) != cudaSuccess)
            rc = sfh_cuda_error(ctx, e, "derive_rows colsum");
    if (rc == SFH_OK && (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
        rc = sfh_cuda_error(ctx, e, "derive_rows sync");
    if (rc != SFH_OK) { free_models(m); return rc; }
    m->m_negative = parent->m_negative;
    m->colsum_e = colsum_e;
    *out = m;
    return SFH_OK;
}

extern "C" int sfh_models_from_device(sfh_ctx *ctx, const float *dev, int64_t nbins, int64_t nt,
                                      int storage, sfh_models **out) {
    if (!ctx || !dev || !out || nbins <= 0 || nt <= 0) return SFH_ERR_ARG;
    if (storage != SFH_F32 && storage != SFH_BF16X2) return SFH_ERR_ARG;
    *out = nullptr;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    sfh_models *m = new sfh_models();
    m->device = ctx->device;
    m->nbins = nbins;
    m->nt = nt;
    m->storage = storage;
    const size_t n = (size_t)nbins * (size_t)nt;
    cudaError_t e = cudaMalloc(&m->d_f32, n * sizeof(float));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(m->d_f32, dev, n * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) { free_models(m); return sfh_cuda_error(ctx, e, "copy models"); }
    int rc = finish_models(ctx, m);
    if (rc == SFH_OK) {
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = sfh_cuda_error(ctx, e, "models_from_device sync");
    }
    if (rc != SFH_OK) { free_models(m); return rc; }
    *out = m;
    return SFH_OK;
}

// ------------------------------------------------------------------ combined templates
namespace {
// out[:, g] = Σ_{q in group g} w_q M[:, col_q] for FP32 (nbins, nt) column-major M; one
// thread per bin, compensated FP32 accumulation of the FP32 products w_q M (w split hi/lo).
__global__ void k_combine_columns(const float *__restrict__ M, int64_t nbins,
                                  const int64_t *__restrict__ goff, const int32_t *__restrict__ cols,
                                  const float2 *__restrict__ w, int64_t ngroups,
                                  float *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbins) return;
    for (int64_t g = 0; g < ngroups; ++g) {
        float h = 0.f, l = 0.f;
        for (int64_t q = goff[g]; q < goff[g + 1]; ++q) {
            const float2 wq = w[q];  // weight as an FP32 hi/lo pair
            const float m = __ldg(M + (int64_t)cols[q] * nbins + i);
            sfh_two_sum_acc(h, l, fmaf(m, wq.x, m * wq.y));
        }
        out[g * nbins + i] = h + l;
    }
}
}  // namespace

extern "C" int sfh_models_combine(sfh_ctx *ctx, const sfh_models *models, int64_t ngroups,
                                  const int64_t *h_group_off, const int32_t *h_cols,
                                  const double *h_weights, int storage, sfh_models **out) {
    if (!ctx || !models || !h_group_off || !h_cols || !h_weights || !out || ngroups < 1)
        return SFH_ERR_ARG;
    *out = nullptr;
    if (!models->d_f32) return sfh_set_error(ctx, SFH_ERR_UNSUPPORTED, "needs FP32 template storage");
    if (storage != SFH_F32 && storage != SFH_BF16X2) return SFH_ERR_ARG;
    const int64_t nq = h_group_off[ngroups];
    if (h_group_off[0] != 0 || nq < 1) return sfh_set_error(ctx, SFH_ERR_ARG, "bad group offsets");
    for (int64_t g = 0; g < ngroups; ++g)
        if (h_group_off[g + 1] < h_group_off[g]) return sfh_set_error(ctx, SFH_ERR_ARG, "bad group offsets");
    for (int64_t q = 0; q < nq; ++q)
        if (h_cols[q] < 0 || h_cols[q] >= models->nt)
            return sfh_set_error(ctx, SFH_ERR_SHAPE, "template index out of range");
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const int64_t nbins = models->nbins;
    std::vector<float2> wf((size_t)nq);  // weights split into FP32 hi/lo on the host
    for (int64_t q = 0; q < nq; ++q) {
        const float wh = (float)h_weights[q];
        wf[(size_t)q] = make_float2(wh, (float)(h_weights[q] - (double)wh));
    }
    void *buf = nullptr;
    const size_t o_off = 0, o_cols = sfh_align256((size_t)(ngroups + 1) * 8);
    const size_t o_w = o_cols + sfh_align256((size_t)nq * 4);
    const size_t o_out = o_w + sfh_align256((size_t)nq * 8);
    const size_t total = o_out + (size_t)ngroups * nbins * sizeof(float);
    SFH_CK(ctx, cudaMalloc(&buf, total));
    char *b = (char *)buf;
    cudaError_t e = cudaMemcpyAsync(b + o_off, h_group_off, (size_t)(ngroups + 1) * 8,
                                    cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b + o_cols, h_cols, (size_t)nq * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b + o_w, wf.data(), (size_t)nq * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) {
        cudaFree(buf);
        return sfh_cuda_error(ctx, e, "combine upload");
    }
    k_combine_columns<<<(unsigned)((nbins + 255) / 256), 256, 0, ctx->stream>>>(
        models->d_f32, nbins, (const int64_t *)(b + o_off), (const int32_t *)(b + o_cols),
        (const float2 *)(b + o_w), ngroups, (float *)(b + o_out));
    ctx->launches++;
    e = cudaGetLastError();
    int rc = e == cudaSuccess ? SFH_OK : sfh_cuda_error(ctx, e, "k_combine_columns");
    if (rc == SFH_OK) rc = sfh_models_from_device(ctx, (const float *)(b + o_out), nbins, ngroups,
                                                  storage, out);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(buf);
    return rc;
}

// ------------------------------------------------------------------ host-array entry points
namespace {

// Copies a host array of `dtype` elements into device doubles.
int h2d_as_double(sfh_ctx *ctx, double *dst, const void *src, int dtype, int64_t n,
                  std::vector<double> &tmp) {
    if (n == 0) return SFH_OK;
    const void *p = src;
    if (dtype == SFH_F32) {
        tmp.resize((size_t)n);
        const float *s = (const float *)src;
        for (int64_t i = 0; i < n; ++i) tmp[(size_t)i] = s[i];
        p = tmp.data();
    }
    SFH_CK(ctx, cudaMemcpyAsync(dst, p, (size_t)n * sizeof(double), cudaMemcpyHostToDevice,
                                ctx->stream));
    // The temporary must outlive the copy: pageable copies are staged by the driver
    // before cudaMemcpyAsync returns, so reusing `tmp` afterwards is safe.
    return SFH_OK;
}

int d2h_from_double(sfh_ctx *ctx, void *dst, const double *src, int dtype, int64_t n) {
    if (n == 0) return SFH_OK;
    if (dtype == SFH_F64) {
        SFH_CK(ctx, cudaMemcpyAsync(dst, src, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost,
                                    ctx->stream));
        SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
        return SFH_OK;
    }
    std::vector<double> tmp((size_t)n);
    SFH_CK(ctx, cudaMemcpyAsync(tmp.data(), src, (size_t)n * sizeof(double),
                                cudaMemcpyDeviceToHost, ctx->stream));
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    float *d = (float *)dst;
    for (int64_t i = 0; i < n; ++i) d[i] = (float)tmp[(size_t)i];
    return SFH_OK;
}

double eps_of(int dtype) { return dtype == SFH_F32 ? 1.1920928955078125e-7 : 2.220446049250313e-16; }

bool dtype_ok(int dtype) { return dtype == SFH_F64 || dtype == SFH_F32; }

}  // namespace

extern "C" int sfh_composite(sfh_ctx *ctx, const sfh_models *m, int dtype, const void *coeffs,
                             void *composite_out) {
    if (!ctx || !m || !coeffs || !composite_out || !dtype_ok(dtype)) return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const int64_t nb = m->nbins, nt = m->nt;
    int rc = sfh_stage_reserve(ctx, sfh_align256(nt * 8) + sfh_align256(nb * 8));
    if (rc) return rc;
    double *d_r = (double *)ctx->stage;
    double *d_c = (double *)((char *)ctx->stage + sfh_align256(nt * 8));
    std::vector<double> tmp;
    if ((rc = h2d_as_double(ctx, d_r, coeffs, dtype, nt, tmp))) return rc;
    FgArgs a{};
    a.coeffs = d_r;
    a.composite = d_c;
    a.eps = eps_of(dtype);
    a.mode = FG_MODE_COMPOSITE;
    if ((rc = sfh_launch_fg(ctx, m, a))) return rc;
    return d2h_from_double(ctx, composite_out, d_c, dtype, nb);
}

extern "C" int sfh_loglikelihood(sfh_ctx *ctx, int dtype, const void *composite, const void *data,
                                 int64_t nbins, double *out) {
    if (!ctx || !composite || !data || !out || nbins < 0 || !dtype_ok(dtype)) return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    int rc = sfh_stage_reserve(ctx, 2 * sfh_align256(nbins * 8) + 256);
    if (rc) return rc;
    double *d_c = (double *)ctx->stage;
    double *d_n = (double *)((char *)ctx->stage + sfh_align256(nbins * 8));
    double *d_o = (double *)((char *)ctx->stage + 2 * sfh_align256(nbins * 8));
    std::vector<double> t1, t2;
    if ((rc = h2d_as_double(ctx, d_c, composite, dtype, nbins, t1))) return rc;
    if ((rc = h2d_as_double(ctx, d_n, data, dtype, nbins, t2))) return rc;
    if ((rc = sfh_launch_loglikelihood(ctx, d_c, d_n, nbins, eps_of(dtype), d_o))) return rc;
    double v = 0;
    SFH_CK(ctx, cudaMemcpyAsync(&v, d_o, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    // The reference returns T-typed results; round to Float32 for dtype F32.
    *out = dtype == SFH_F32 ? (double)(float)v : v;
    return SFH_OK;
}

extern "C" int sfh_grad_loglikelihood(sfh_ctx *ctx, const sfh_models *m, int dtype,
                                      void *composite_inout, const void *data, void *G) {
    if (!ctx || !m || !composite_inout || !data || !G || !dtype_ok(dtype)) return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const int64_t nb = m->nbins, nt = m->nt;
    int rc = sfh_stage_reserve(ctx, 2 * sfh_align256(nb * 8) + sfh_align256(nt * 8));
    if (rc) return rc;
    double *d_c = (double *)ctx->stage;
    double *d_n = (double *)((char *)ctx->stage + sfh_align256(nb * 8));
    double *d_G = (double *)((char *)ctx->stage + 2 * sfh_align256(nb * 8));
    std::vector<double> t1, t2;
    if ((rc = h2d_as_double(ctx, d_c, composite_inout, dtype, nb, t1))) return rc;
    if ((rc = h2d_as_double(ctx, d_n, data, dtype, nb, t2))) return rc;
    FgArgs a{};
    a.data = d_n;
    a.composite = d_c;
    a.G = d_G;
    a.eps = eps_of(dtype);
    a.gsign = -1.0;
    a.mode = FG_MODE_GRAD_GIVEN;
    if ((rc = sfh_launch_fg(ctx, m, a))) return rc;
    if ((rc = d2h_from_double(ctx, composite_inout, d_c, dtype, nb))) return rc;
    return d2h_from_double(ctx, G, d_G, dtype, nt);
}

extern "C" int sfh_fg(sfh_ctx *ctx, const sfh_models *m, int dtype, const void *coeffs,
                      const void *data, void *composite, void *G, double *negLogL) {
    if (!ctx || !m || !coeffs || !data || !dtype_ok(dtype)) return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const int64_t nb = m->nbins, nt = m->nt;
    // Non-finite coefficients: the reference's arithmetic would return NaN; report it
    // without a launch (the outputs carry the NaN a caller ignoring the status would see).
    bool finite = true;
    for (int64_t j = 0; j < nt && finite; ++j)
        finite = std::isfinite(dtype == SFH_F64 ? ((const double *)coeffs)[j]
                                                : (double)((const float *)coeffs)[j]);
    if (!finite) {
        if (negLogL) *negLogL = NAN;
        for (int64_t j = 0; G && j < nt; ++j) {
            if (dtype == SFH_F64) ((double *)G)[j] = NAN;
            else ((float *)G)[j] = NAN;
        }
        return sfh_set_error(ctx, SFH_ERR_NUMERIC, "fg!: non-finite coefficients");
    }
    int rc;
    int access = SFH_HOST_ACCESS_STAGED;
    sfh_ctx_host_access(ctx, &access);
    const auto al8 = [](const void *p) { return ((uintptr_t)p & 7u) == 0; };
    if (access == SFH_HOST_ACCESS_DIRECT && dtype == SFH_F64 && composite && al8(coeffs) &&
        al8(data) && al8(composite) && (!G || al8(G))) {
        // the kernels read r and n and write the composite, G and -logL in the caller's own
        // arrays through the host page tables: one launch and one stream sync, no copies
        // (-logL goes through the staging slot, which a caller's stack variable can share
        // a page with while the kernel runs).  The host touches both ends of every array
        // first, so a bad pointer fails here rather than on the device.
        volatile double sink = ((const double *)data)[0] + ((const double *)data)[nb - 1];
        (void)sink;
        ((double *)composite)[0] = 0.0;
        ((double *)composite)[nb - 1] = 0.0;
        if (G) {
            ((double *)G)[0] = 0.0;
            ((double *)G)[nt - 1] = 0.0;
        }
        if ((rc = sfh_host_stage_reserve(ctx, 256))) return rc;
        double *hl = (double *)ctx->h_stage;
        FgArgs a{};
        a.coeffs = (const double *)coeffs;
        a.data = (const double *)data;
        a.composite = (double *)composite;
        a.G = (double *)G;
        a.negLogL = negLogL ? (double *)ctx->d_h_stage : nullptr;
        a.eps = eps_of(dtype);
        a.gsign = 1.0;
        a.mode = FG_MODE_FG;
        a.occ_key = m;  // one plan slot for the host-array calls on this handle
        if ((rc = sfh_launch_fg(ctx, m, a))) return rc;
        SFH_CK(ctx, sfh_host_call_wait(ctx));
        if (negLogL) {
            const double v = *(volatile double *)hl;
            if (std::isnan(v) && (rc = sfh_check_onepass(ctx))) return rc;
            *negLogL = v;
        }
        return SFH_OK;
    }
    // inputs [r | n] and outputs [composite | G | -logL] in the mapped pinned staging area:
    // the kernels read the inputs and write the outputs across the host link themselves, so
    // a call is one copy in, one launch, one stream sync and one copy out
    const size_t o_r = 0, o_n = sfh_align256(nt * 8), o_c = o_n + sfh_align256(nb * 8),
                 o_g = o_c + sfh_align256(nb * 8), o_l = o_g + sfh_align256(nt * 8),
                 o_end = o_l + 8;
    if ((rc = sfh_host_stage_reserve(ctx, o_end + 256))) return rc;
    char *base = (char *)ctx->d_h_stage, *hb = (char *)ctx->h_stage;
    double *hr = (double *)(hb + o_r), *hn = (double *)(hb + o_n);
    if (dtype == SFH_F64) {
        memcpy(hr, coeffs, (size_t)nt * 8);
        memcpy(hn, data, (size_t)nb * 8);
    } else {
        const float *cf = (const float *)coeffs, *df = (const float *)data;
        for (int64_t i = 0; i < nt; ++i) hr[i] = cf[i];
        for (int64_t i = 0; i < nb; ++i) hn[i] = df[i];
    }
    FgArgs a{};
    a.coeffs = (const double *)(base + o_r);
    a.data = (const double *)(base + o_n);
    a.composite = (double *)(base + o_c);
    a.G = G ? (double *)(base + o_g) : nullptr;
    a.negLogL = negLogL ? (double *)(base + o_l) : nullptr;
    a.eps = eps_of(dtype);
    a.gsign = 1.0;
    a.mode = FG_MODE_FG;
    a.occ_key = m;
    if ((rc = sfh_launch_fg(ctx, m, a))) return rc;
    SFH_CK(ctx, sfh_host_call_wait(ctx));
    if (negLogL) {
        double v;
        memcpy(&v, hb + o_l, 8);
        if (std::isnan(v) && (rc = sfh_check_onepass(ctx))) return rc;  // timed-out one-pass
        *negLogL = dtype == SFH_F32 ? (double)(float)v : v;
    }
    const double *hc = (const double *)(hb + o_c), *hg = (const double *)(hb + o_g);
    if (dtype == SFH_F64) {
        if (G) memcpy(G, hg, (size_t)nt * 8);
        if (composite) memcpy(composite, hc, (size_t)nb * 8);
    } else {
        if (G)
            for (int64_t i = 0; i < nt; ++i) ((float *)G)[i] = (float)hg[i];
        if (composite)
            for (int64_t i = 0; i < nb; ++i) ((float *)composite)[i] = (float)hc[i];
    }
    return SFH_OK;
}

extern "C" int sfh_fg_dev(sfh_ctx *ctx, const sfh_models *m, const double *d_coeffs,
                          const double *d_data, double *d_composite, double *d_G,
                          double *d_negLogL, double eps) {
    if (!ctx || !m || !d_coeffs || !d_data || !d_composite) return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    FgArgs a{};
    a.coeffs = d_coeffs;
    a.data = d_data;
    a.composite = d_composite;
    a.G = d_G;
    a.negLogL = d_negLogL;
    a.eps = eps;
    a.gsign = 1.0;
    a.mode = FG_MODE_FG;
    return sfh_launch_fg(ctx, m, a);
}

extern "C" int sfh_fg_batched_dev(sfh_ctx *ctx, const sfh_models *m, const double *d_R, int64_t B,
                                  const double *d_data, double *d_negLogL, float *d_G, double eps) {
    if (!ctx || !m || !d_R || !d_data || B <= 0) return SFH_ERR_ARG;
    if (m->storage != SFH_BF16X2)
        return sfh_set_error(ctx, SFH_ERR_ARG, "sfh_fg_batched_dev needs SFH_BF16X2 storage");
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    return sfh_launch_fg_batched(ctx, m, d_R, B, d_data, d_negLogL, d_G, eps);
}
