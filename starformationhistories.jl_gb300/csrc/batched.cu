// batched.cu -- many coefficient vectors against one template matrix.
//
// Storage for the tensor-core path: every template value M is split as
// M = hi + lo with hi = bf16(M), lo = bf16(M - hi) (16 significant bits), in two
// layouts so that both products read K-major operands:
//   row planes  (nbins_pad, nt_pad) row-major: A of C = M R   (K = templates)
//   col planes  (nbins_pad, nt_pad) col-major: A of G = Mᵀ W  (K = bins)
// Padding rows/columns are zero.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "sfh_internal.cuh"

namespace {

__global__ void k_split_planes(const float *__restrict__ src, int64_t nbins, int64_t nt,
                               int64_t nbins_pad, int64_t nt_pad, __nv_bfloat16 *__restrict__ col_hi,
                               __nv_bfloat16 *__restrict__ col_lo, __nv_bfloat16 *__restrict__ row_hi,
                               __nv_bfloat16 *__restrict__ row_lo) {
    // One thread per (bin, template) of the padded matrix; src is column-major.
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = nbins_pad * nt_pad;
    if (idx >= total) return;
    const int64_t j = idx / nbins_pad, i = idx - j * nbins_pad;
    float v = 0.f;
    if (i < nbins && j < nt) v = src[j * nbins + i];
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
    col_hi[idx] = h;
    col_lo[idx] = l;
    row_hi[i * nt_pad + j] = h;
    row_lo[i * nt_pad + j] = l;
}

}  // namespace

int sfh_build_bf16_planes(sfh_ctx *ctx, sfh_models *m, const float *d_f32) {
    m->nbins_pad = ((m->nbins + 127) / 128) * 128;
    m->nt_pad = ((m->nt + 127) / 128) * 128;
    const size_t n = (size_t)m->nbins_pad * (size_t)m->nt_pad;
    SFH_CK(ctx, cudaMalloc(&m->col_hi, n * 2));
    SFH_CK(ctx, cudaMalloc(&m->col_lo, n * 2));
    SFH_CK(ctx, cudaMalloc(&m->row_hi, n * 2));
    SFH_CK(ctx, cudaMalloc(&m->row_lo, n * 2));
    const int threads = 256;
    const int64_t blocks = ((int64_t)n + threads - 1) / threads;
    k_split_planes<<<(unsigned)blocks, threads, 0, ctx->stream>>>(
        d_f32, m->nbins, m->nt, m->nbins_pad, m->nt_pad, m->col_hi, m->col_lo, m->row_hi, m->row_lo);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

int sfh_launch_fg_batched(sfh_ctx *ctx, const sfh_models *m, const double *d_R, int64_t B,
                          const double *d_data, double *d_negLogL, float *d_G, double eps) {
    (void)m; (void)d_R; (void)B; (void)d_data; (void)d_negLogL; (void)d_G; (void)eps;
    return sfh_set_error(ctx, SFH_ERR_UNSUPPORTED, "batched objective not built yet");
}
