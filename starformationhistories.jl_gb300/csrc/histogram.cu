// histogram.cu -- hard-binned Hess diagrams: bin_cmd (src/StarFormationHistories.jl:544-553),
// StatsBase's fit(Histogram, (colors, mags), Weights(w), edges; closed=:left).
//
// Bin k of an axis holds e[k] <= v < e[k+1] against the STORED edge values (StatsBase
// searches the range's own elements; a Julia range such as 0.0:0.1:1.0 holds 0.3 exactly,
// not 0 + 3 * 0.1).  A point on the last edge, below the first, or NaN is dropped.  One
// thread per point finds its bin from the mean step and corrects the guess against the
// edge values; blocks accumulate a private FP64 histogram in shared memory when the grid
// fits (dense photometric catalogues pile up in few bins) and flush it with global atomics.
#include <algorithm>
#include <cmath>

#include "sfh_internal.cuh"

namespace {

constexpr int kHistThreads = 256;
constexpr int64_t kHistSmemBins = 12288;  // 96 KB of FP64 bins per block

// The bin of v among n bins with increasing edges e[0..n], or -1.
__device__ __forceinline__ int edge_bin(double v, const double *__restrict__ e, int n,
                                        double inv_step) {
    const double e0 = e[0];
    if (!(v >= e0) || !(v < e[n])) return -1;
    int k = (int)fmin(fmax(floor((v - e0) * inv_step), 0.0), (double)(n - 1));
    while (k > 0 && v < e[k]) --k;
    while (k < n - 1 && v >= e[k + 1]) ++k;
    return k;
}

struct HistAxes {
    const double *ex, *ey;
    int nx, ny;
};

__global__ void __launch_bounds__(kHistThreads)
k_bin_cmd_global(const double *__restrict__ x, const double *__restrict__ y,
                 const double *__restrict__ w, int64_t n, HistAxes A, double *__restrict__ out) {
    const double ixs = A.nx / (A.ex[A.nx] - A.ex[0]), iys = A.ny / (A.ey[A.ny] - A.ey[0]);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = edge_bin(x[i], A.ex, A.nx, ixs);
        if (ix < 0) continue;
        const int iy = edge_bin(y[i], A.ey, A.ny, iys);
        if (iy < 0) continue;
        atomicAdd(out + ix + (int64_t)A.nx * iy, w ? w[i] : 1.0);
    }
}

__global__ void __launch_bounds__(kHistThreads)
k_bin_cmd_shared(const double *__restrict__ x, const double *__restrict__ y,
                 const double *__restrict__ w, int64_t n, HistAxes A, double *__restrict__ out) {
    extern __shared__ double s_hist[];
    const int nb = A.nx * A.ny;
    const double ixs = A.nx / (A.ex[A.nx] - A.ex[0]), iys = A.ny / (A.ey[A.ny] - A.ey[0]);
    for (int k = threadIdx.x; k < nb; k += blockDim.x) s_hist[k] = 0.0;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = edge_bin(x[i], A.ex, A.nx, ixs);
        if (ix < 0) continue;
        const int iy = edge_bin(y[i], A.ey, A.ny, iys);
        if (iy < 0) continue;
        atomicAdd(s_hist + ix + A.nx * iy, w ? w[i] : 1.0);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nb; k += blockDim.x)
        if (s_hist[k] != 0.0) atomicAdd(out + k, s_hist[k]);
}

int check_edges(sfh_ctx *ctx, const double *e, int64_t n) {
    for (int64_t k = 0; k <= n; ++k)
        if (!std::isfinite(e[k]) || (k > 0 && !(e[k] > e[k - 1])))
            return sfh_set_error(ctx, SFH_ERR_ARG, "bin edges must be finite and increasing");
    return SFH_OK;
}

}  // namespace

// Stream-ordered on ctx's stream; d_hist_out (nx * ny, column-major like the reference's
// Histogram weights) is overwritten.  Edges must be increasing (sfh_bin_cmd checks them;
// here the bin search stays inside the edge arrays whatever they hold).
extern "C" int sfh_bin_cmd_dev(sfh_ctx *ctx, const double *d_x, const double *d_y,
                               const double *d_w, int64_t n, const double *d_xedges, int64_t nx,
                               const double *d_yedges, int64_t ny, double *d_hist_out) {
    if (!ctx || !d_hist_out || !d_xedges || !d_yedges || n < 0 || nx < 1 || ny < 1 ||
        nx * ny > INT32_MAX || (n > 0 && (!d_x || !d_y)))
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const int64_t nb = nx * ny;
    SFH_CK(ctx, cudaMemsetAsync(d_hist_out, 0, nb * 8, ctx->stream));
    if (n == 0) return SFH_OK;
    HistAxes A{d_xedges, d_yedges, (int)nx, (int)ny};
    const int64_t want = (n + kHistThreads * 8 - 1) / (kHistThreads * 8);
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, 4 * (int64_t)ctx->sm_count));
    if (nb <= kHistSmemBins) {
        const size_t smem = (size_t)nb * 8;
        if (smem > 48 * 1024)
            SFH_CK(ctx, cudaFuncSetAttribute(k_bin_cmd_shared,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(kHistSmemBins * 8)));
        k_bin_cmd_shared<<<grid, kHistThreads, smem, ctx->stream>>>(d_x, d_y, d_w, n, A,
                                                                   d_hist_out);
    } else {
        k_bin_cmd_global<<<grid, kHistThreads, 0, ctx->stream>>>(d_x, d_y, d_w, n, A,
                                                                d_hist_out);
    }
    SFH_CK(ctx, cudaGetLastError());
    ctx->launches++;
    return SFH_OK;
}

// Host buffers: x, y, w (NULL = unit weights) of n points; xedges (nx + 1 values), yedges
// (ny + 1 values); hist_out (nx * ny).  Synchronous.
extern "C" int sfh_bin_cmd(sfh_ctx *ctx, const double *x, const double *y, const double *w,
                           int64_t n, const double *xedges, int64_t nx, const double *yedges,
                           int64_t ny, double *hist_out) {
    if (!ctx || !hist_out || !xedges || !yedges || n < 0 || nx < 1 || ny < 1 ||
        nx * ny > INT32_MAX || (n > 0 && (!x || !y)))
        return SFH_ERR_ARG;
    int rc = check_edges(ctx, xedges, nx);
    if (!rc) rc = check_edges(ctx, yedges, ny);
    if (rc) return rc;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const int64_t nb = nx * ny;
    const size_t a = sfh_align256((size_t)(n > 0 ? n : 1) * 8);
    const size_t o_ex = 3 * a, o_ey = o_ex + sfh_align256((nx + 1) * 8),
                 o_out = o_ey + sfh_align256((ny + 1) * 8), total = o_out + nb * 8;
    rc = sfh_stage_reserve(ctx, total);
    if (rc) return rc;
    char *b = (char *)ctx->stage;
    if (n > 0) {
        SFH_CK(ctx, cudaMemcpyAsync(b, x, n * 8, cudaMemcpyHostToDevice, ctx->stream));
        SFH_CK(ctx, cudaMemcpyAsync(b + a, y, n * 8, cudaMemcpyHostToDevice, ctx->stream));
        if (w) SFH_CK(ctx, cudaMemcpyAsync(b + 2 * a, w, n * 8, cudaMemcpyHostToDevice, ctx->stream));
    }
    SFH_CK(ctx, cudaMemcpyAsync(b + o_ex, xedges, (nx + 1) * 8, cudaMemcpyHostToDevice, ctx->stream));
    SFH_CK(ctx, cudaMemcpyAsync(b + o_ey, yedges, (ny + 1) * 8, cudaMemcpyHostToDevice, ctx->stream));
    double *d_out = (double *)(b + o_out);
    rc = sfh_bin_cmd_dev(ctx, (const double *)b, (const double *)(b + a),
                         w ? (const double *)(b + 2 * a) : nullptr, n, (const double *)(b + o_ex),
                         nx, (const double *)(b + o_ey), ny, d_out);
    if (rc) return rc;
    SFH_CK(ctx, cudaMemcpyAsync(hist_out, d_out, nb * 8, cudaMemcpyDeviceToHost, ctx->stream));
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return SFH_OK;
}
