// ragged.cu -- fg! over many independent galaxies with uneven Hess grids, one batch.
//
// fg! (src/fitting/solvers.jl:20-38: composite!, loglikelihood, ∇loglikelihood!,
// fitting_base.jl:55-96, 265-285) for every galaxy g with its own template matrix
// (nbins_g x ntempl_g, column-major FP32, packed in one device array), coefficients,
// data, composite and gradient.  Two launches cover the whole batch:
//   pass 1  one CTA per (galaxy, 256-bin row tile): m = M r with the coefficient split
//           into FP32 hi + lo, groups of 8 products summed error-free against a
//           power-of-two anchor (sfh_anc_acc) and folded compensated, the Poisson terms
//           (FP64-light form), w = 1 - n / max(m, eps) written over the composite;
//   pass 2  one CTA per (galaxy, 8-template column group): G = Mᵀ w (fg!'s G .*= -1 of
//           -Mᵀ w), compensated FP32 per column, FP64 block reduction;
// then a per-galaxy reduction of the row-tile logL partials (fixed order, so results
// are reproducible).  Column groups are issued largest galaxy first.
// Galaxies with at most kFuseMax templates take one fused pass instead: each thread
// walks kFuseRows bins, keeps each bin's row of M in registers, forms m, the Poisson
// term and w, and accumulates the per-template products M w; these are summed across
// the warp by a recursive-halving transpose (31 shuffles for 32 templates), across the
// CTA in shared memory and across tiles by a fixed-order per-galaxy finish.  M is then
// read once per evaluation.  Fused galaxies are launched by register class (nt <= 8,
// <= 16, <= 32), so a batch with a few wide galaxies does not widen every tile.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "sfh_internal.cuh"

struct sfh_galaxies {
    int device;
    int64_t ngal, total_bins, total_templ, n_row_tiles, n_col_tiles, max_nt;
    int64_t n_fused_tiles;  // tiles of galaxies with <= kFuseMax templates
    int64_t n_fused_gal, n_big_gal, max_fused_nt;
    int64_t n_fused_class[3];  // fused tiles with nt <= 8, <= 16, <= 32 (in that order)
    void *d_desc;       // GalDesc[ngal]
    void *d_rows;       // RowTile[n_row_tiles] (two-pass galaxies)
    void *d_cols;       // ColTile[n_col_tiles] (two-pass galaxies)
    void *d_fused;      // RowTile[n_fused_tiles] (fused galaxies)
    void *d_fused_ids;  // int32[n_fused_gal]
    void *d_big_ids;    // int32[n_big_gal]
    const float *d_models;
};

namespace {

constexpr int kRT = 256;       // threads per CTA, rows per pass-1 tile
constexpr int kColGroup = 8;   // templates per pass-2 CTA
constexpr int kRChunk = 2048;  // coefficients staged in shared memory at a time
constexpr int kFuseMax = 32;   // templates per galaxy held in registers by the fused pass
constexpr int kFuseRows = 4;   // bins per thread in the fused pass (tile = kFuseRows * kRT rows)

constexpr int64_t kFuseStep = (int64_t)kRT * kFuseRows;
__host__ __device__ inline int fused_class(int64_t nt) { return nt <= 8 ? 0 : nt <= 16 ? 1 : 2; }

struct GalDesc {
    int64_t moff, nbins, nt, boff, toff, tile0, ntiles;
    int64_t fused;  // 1: tiles are in the fused list, 0: two-pass lists
};
struct RowTile {
    int32_t g, row0;
};
struct ColTile {
    int32_t g, j0;
};

__device__ __forceinline__ void block_sum(double v, double *s_red, double *out) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += s_red[w];
        *out = b;
    }
}

// One bin's share of fg!: the model m = ah + al (compensated), the Poisson term in
// double-float (sfh_dfloat.cuh) and w = 1 - n / max(m, eps) (fitting_base.jl:90-93,
// 274-280); composite receives w when the gradient is wanted, the model otherwise.
__device__ __forceinline__ void bin_terms(float ah, float al, const double *__restrict__ data,
                                          int64_t ii, float eps_f, int want_logl, int want_w,
                                          const sfh_df *s_tab, double *__restrict__ composite,
                                          sfh_df &term, float &w) {
    sfh_df c = df_fast_two_sum(ah, al);
    if (!want_w) composite[ii] = sfh_f2d(c.h) + sfh_f2d(c.l);  // the model, unclamped
    if (!want_logl && !want_w) return;
    // max(composite, eps(T)); eps(T) is a power of two, exact in FP32
    if (c.h < eps_f || (c.h == eps_f && c.l < 0.f)) c = sfh_df{eps_f, 0.f};
    float nh, nl;
    sfh_split_double(data[ii], nh, nl);
    if (want_logl)
        term = df_add(term, sfh_bin_term(c, nh, nl, s_tab));
    if (want_w) {
        w = __fdiv_rn(df_add(c, sfh_df{-nh, -nl}).h, c.h);
        composite[ii] = sfh_f2d(w);
    }
}

__global__ void __launch_bounds__(kRT)
k_ragged_pass1(const float *__restrict__ M, const GalDesc *__restrict__ gals,
               const RowTile *__restrict__ tiles, const double *__restrict__ coeffs,
               const double *__restrict__ data, double *__restrict__ composite,
               float *__restrict__ w32, double *__restrict__ tile_logl, float eps,
               int want_logl, int want_w, const sfh_df *__restrict__ tab) {
    __shared__ float rhi[kRChunk], rlo[kRChunk];
    __shared__ double s_red[kRT / 32];
    __shared__ sfh_df s_tab[SFH_DF_TAB_ALL];
    for (int k = threadIdx.x; k < SFH_DF_TAB_ALL; k += kRT) s_tab[k] = tab[k];
    const RowTile tile = tiles[blockIdx.x];
    const GalDesc G = gals[tile.g];
    const int64_t i = (int64_t)tile.row0 + threadIdx.x;
    const bool live = i < G.nbins;
    float ah = 0.f, al = 0.f;
    for (int64_t j0 = 0; j0 < G.nt; j0 += kRChunk) {
        const int kn = (int)min((int64_t)kRChunk, G.nt - j0);
        __syncthreads();
        for (int t = threadIdx.x; t < kn; t += kRT) {
            const double v = coeffs[G.toff + j0 + t];
            const float h = __double2float_rn(v);
            rhi[t] = h;
            rlo[t] = __double2float_rn(v - (double)h);
        }
        __syncthreads();
        if (!live) continue;
        const float *col = M + G.moff + j0 * G.nbins + i;
        // groups of 8 templates summed error-free against the group's own power-of-two
        // anchor (sfh_anc_acc), folded into the compensated pair
        for (int k = 0; k < kn; k += 8) {
            const int kk = min(8, kn - k);
            float v[8], hv[8], lv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                v[u] = u < kk ? __ldg(col + (int64_t)(k + u) * G.nbins) : 0.f;
                hv[u] = u < kk ? rhi[k + u] : 0.f;
                lv[u] = u < kk ? rlo[k + u] : 0.f;
            }
            float b = 0.f;
#pragma unroll
            for (int u = 0; u < 8; ++u) b = fmaf(fabsf(v[u]), fabsf(hv[u]), b);
            const float sg = sfh_anchor(b * 1.0009765625f);
            float a = sg, lo = 0.f;
#pragma unroll
            for (int u = 0; u < 8; ++u) sfh_anc_acc(a, lo, v[u], hv[u], lv[u]);
            sfh_two_sum_acc(ah, al, __fsub_rn(a, sg));
            al = __fadd_rn(al, lo);
        }
    }
    sfh_df term{0.f, 0.f};
    if (live) {
        const int64_t ii = G.boff + i;
        float w = 0.f;
        bin_terms(ah, al, data, ii, eps, want_logl, want_w, s_tab, composite, term, w);
        if (want_w) w32[ii] = w;
    }
    if (want_logl) {
        double tsum = 0.0;
        sfh_df_block_sum(term, s_red, &tsum);
        if (threadIdx.x == 0) tile_logl[blockIdx.x] = tsum;
    }
}

__global__ void __launch_bounds__(kRT)
k_ragged_logl(const GalDesc *__restrict__ gals, const int32_t *__restrict__ ids,
              const double *__restrict__ tile_logl, double *__restrict__ negLogL) {
    __shared__ double s_red[kRT / 32];
    const int g = ids[blockIdx.x];
    const GalDesc G = gals[g];
    double acc = 0.0;
    for (int64_t k = threadIdx.x; k < G.ntiles; k += kRT) acc += tile_logl[G.tile0 + k];
    double tot = 0.0;
    block_sum(acc, s_red, &tot);
    // loglikelihood returns -typemax(T) = -Inf when the sum is exactly zero (fitting_base.jl:95)
    if (threadIdx.x == 0) negLogL[g] = -((tot != 0.0) ? tot : -INFINITY);
}

__global__ void __launch_bounds__(kRT)
k_ragged_pass2(const float *__restrict__ M, const GalDesc *__restrict__ gals,
               const ColTile *__restrict__ tiles, const float *__restrict__ w32,
               double *__restrict__ Gout) {
    __shared__ double s_red[kRT / 32];
    const ColTile tile = tiles[blockIdx.x];
    const GalDesc G = gals[tile.g];
    const int nc = (int)min((int64_t)kColGroup, G.nt - tile.j0);
    float ah[kColGroup], al[kColGroup];
#pragma unroll
    for (int c = 0; c < kColGroup; ++c) ah[c] = al[c] = 0.f;
    const float *base = M + G.moff + (int64_t)tile.j0 * G.nbins;
    const float *w = w32 + G.boff;
    for (int64_t i = threadIdx.x; i < G.nbins; i += kRT) {
        const float wi = __ldg(w + i);
#pragma unroll
        for (int c = 0; c < kColGroup; ++c)
            if (c < nc) sfh_two_sum_acc(ah[c], al[c], __ldg(base + (int64_t)c * G.nbins + i) * wi);
    }
    for (int c = 0; c < nc; ++c) {
        double tot = 0.0;
        block_sum((double)ah[c] + (double)al[c], s_red, &tot);
        if (threadIdx.x == 0) Gout[G.toff + tile.j0 + c] = tot;
    }
}

// One fused fg! pass for galaxies with nt <= kFuseMax: m, Poisson terms, w and the
// tile's partial G = Mᵀ w (gpart, kFuseMax doubles per tile).  Tiles tile_base + blockIdx.x
// of the fused list; each thread takes kFuseRows bins (rows row0 + r * kRT + tid), so the
// table load, the block reduction and the transpose are paid once per kFuseRows * kRT bins.
template <int NT>
__global__ void __launch_bounds__(kRT, NT <= 8 ? 4 : NT <= 16 ? 3 : 2)
k_ragged_fused(const float *__restrict__ M, const GalDesc *__restrict__ gals,
               const RowTile *__restrict__ tiles, const double *__restrict__ coeffs,
               const double *__restrict__ data, double *__restrict__ composite,
               double *__restrict__ tile_logl, double *__restrict__ gpart, float eps,
               int want_logl, int want_g, const sfh_df *__restrict__ tab, int tile_base) {
    __shared__ float rhi[NT], rlo[NT];
    __shared__ double s_red[kRT / 32];
    __shared__ float s_g[kRT / 32][NT];
    __shared__ sfh_df s_tab[SFH_DF_TAB_ALL];
    for (int k = threadIdx.x; k < SFH_DF_TAB_ALL; k += kRT) s_tab[k] = tab[k];
    const int64_t t = (int64_t)tile_base + blockIdx.x;
    const RowTile tile = tiles[t];
    const GalDesc G = gals[tile.g];
    const int nt = (int)G.nt;
    if (threadIdx.x < NT) {
        const double v = threadIdx.x < nt ? coeffs[G.toff + threadIdx.x] : 0.0;
        const float h = __double2float_rn(v);
        rhi[threadIdx.x] = h;
        rlo[threadIdx.x] = __double2float_rn(v - (double)h);
    }
    __syncthreads();
    sfh_df term{0.f, 0.f};
    float v[NT];
#pragma unroll
    for (int j = 0; j < NT; ++j) v[j] = 0.f;
#pragma unroll 1
    for (int r = 0; r < kFuseRows; ++r) {
        if ((int64_t)tile.row0 + r * kRT >= G.nbins) break;  // uniform over the CTA
        const int64_t i = (int64_t)tile.row0 + r * kRT + threadIdx.x;
        const bool live = i < G.nbins;
        const float *col = M + G.moff + i;
        // templates in groups of four behind branches that are uniform over the CTA (one
        // galaxy per tile): a galaxy with nt < NT issues no loads or products for the rest
        float m[NT];
#pragma unroll
        for (int j0 = 0; j0 < NT; j0 += 4)
#pragma unroll
            for (int u = 0; u < 4; ++u)
                m[j0 + u] = (j0 < nt && live && j0 + u < nt)
                                ? __ldg(col + (int64_t)(j0 + u) * G.nbins) : 0.f;
        // the bin's products summed error-free against a power-of-two anchor from the bin's
        // own bound sum_j |M_ij| |r_j| (sfh_anc_acc)
        float b = 0.f;
#pragma unroll
        for (int j0 = 0; j0 < NT; j0 += 4) {
            if (j0 >= nt) break;
#pragma unroll
            for (int u = 0; u < 4; ++u) b = fmaf(fabsf(m[j0 + u]), fabsf(rhi[j0 + u]), b);
        }
        const float sg = sfh_anchor(b * 1.0009765625f);
        float aa = sg, lo = 0.f;
#pragma unroll
        for (int j0 = 0; j0 < NT; j0 += 4) {
            if (j0 >= nt) break;
#pragma unroll
            for (int u = 0; u < 4; ++u) sfh_anc_acc(aa, lo, m[j0 + u], rhi[j0 + u], rlo[j0 + u]);
        }
        const sfh_df cm = sfh_anc_result(aa, lo, sg);
        const float ah = cm.h, al = cm.l;
        float w = 0.f;
        if (live) bin_terms(ah, al, data, G.boff + i, eps, want_logl, want_g, s_tab, composite, term, w);
        __syncwarp();  // reconverge after the lane-dependent tail
#pragma unroll
        for (int j0 = 0; j0 < NT; j0 += 4) {
            if (j0 >= nt) break;
#pragma unroll
            for (int u = 0; u < 4; ++u) v[j0 + u] = fmaf(m[j0 + u], w, v[j0 + u]);
        }
    }
    if (want_logl) {
        double tsum = 0.0;
        sfh_df_block_sum(term, s_red, &tsum);
        if (threadIdx.x == 0) tile_logl[t] = tsum;
    }
    if (!want_g) return;
    // warp transpose-reduce over NT templates: after the step with offset o (o < NT)
    // each lane keeps o partial column sums; lanes that differ only in bits >= log2(NT)
    // hold the same columns and are folded first.  Lane l then holds template l % NT.
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o >= NT; o >>= 1)
#pragma unroll
        for (int k = 0; k < NT; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
#pragma unroll
    for (int o = NT / 2; o >= 1; o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int k = 0; k < o; ++k) {
            const float send = upper ? v[k] : v[k + o];
            const float keep = upper ? v[k + o] : v[k];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    if (lane < NT) s_g[warp][lane] = v[0];
    __syncthreads();
    if (threadIdx.x < NT) {
        sfh_df acc{0.f, 0.f};
#pragma unroll
        for (int wgi = 0; wgi < kRT / 32; ++wgi) acc = df_add_f(acc, s_g[wgi][threadIdx.x]);
        gpart[t * kFuseMax + threadIdx.x] = sfh_f2d(acc.h) + sfh_f2d(acc.l);
    }
}

// Per fused galaxy: -logL from its tile partials and G from its tile G partials.  Warp w
// sums tiles w, w + 8, ... (lane = template, coalesced), then the eight warp sums are
// added in warp order: a fixed order, so results are reproducible.
__global__ void __launch_bounds__(kRT)
k_ragged_finish(const GalDesc *__restrict__ gals, const int32_t *__restrict__ fused_ids,
                const double *__restrict__ tile_logl, const double *__restrict__ gpart,
                double *__restrict__ negLogL, double *__restrict__ Gout) {
    __shared__ double s_red[kRT / 32];
    __shared__ double s_g[kRT / 32][kFuseMax];
    const int g = fused_ids[blockIdx.x];
    const GalDesc G = gals[g];
    if (negLogL) {
        double acc = 0.0;
        for (int64_t k = threadIdx.x; k < G.ntiles; k += kRT) acc += tile_logl[G.tile0 + k];
        double tot = 0.0;
        block_sum(acc, s_red, &tot);
        if (threadIdx.x == 0) negLogL[g] = -((tot != 0.0) ? tot : -INFINITY);  // :95
    }
    if (!Gout) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double acc = 0.0;
    if (lane < G.nt)
        for (int64_t k = warp; k < G.ntiles; k += kRT / 32)
            acc += gpart[(G.tile0 + k) * kFuseMax + lane];
    s_g[warp][lane] = acc;
    __syncthreads();
    if (threadIdx.x < G.nt) {
        double t = 0.0;
#pragma unroll
        for (int w = 0; w < kRT / 32; ++w) t += s_g[w][threadIdx.x];
        Gout[G.toff + threadIdx.x] = t;
    }
}

}  // namespace

extern "C" int sfh_galaxies_create(sfh_ctx *ctx, const float *d_models, int64_t models_len,
                                   const sfh_galaxy *h_gal, int64_t ngal, sfh_galaxies **out) {
    if (!ctx || !d_models || !h_gal || !out || ngal < 1 || ngal > (1 << 24) || models_len < 1)
        return SFH_ERR_ARG;
    *out = nullptr;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    std::vector<GalDesc> desc((size_t)ngal);
    std::vector<RowTile> rows, fused;
    std::vector<ColTile> cols;
    std::vector<int32_t> fused_ids, big_ids;
    int64_t tb = 0, tt = 0, maxnt = 0, maxfnt = 0;
    for (int64_t g = 0; g < ngal; ++g) {
        const sfh_galaxy &h = h_gal[g];
        if (h.nbins < 1 || h.ntempl < 1 || h.nbins > INT32_MAX || h.ntempl > INT32_MAX ||
            h.model_offset < 0 || h.bin_offset < 0 || h.templ_offset < 0)
            return sfh_set_error(ctx, SFH_ERR_ARG, "galaxy descriptor out of range");
        if (h.nbins > models_len / h.ntempl || h.model_offset > models_len - h.nbins * h.ntempl)
            return sfh_set_error(ctx, SFH_ERR_SHAPE, "galaxy templates outside the model array");
        GalDesc &d = desc[(size_t)g];
        d.moff = h.model_offset;
        d.nbins = h.nbins;
        d.nt = h.ntempl;
        d.boff = h.bin_offset;
        d.toff = h.templ_offset;
        d.fused = h.ntempl <= kFuseMax ? 1 : 0;
        if (!d.fused) {
            d.ntiles = (h.nbins + kRT - 1) / kRT;
            d.tile0 = (int64_t)rows.size();
            for (int64_t r0 = 0; r0 < h.nbins; r0 += kRT) rows.push_back(RowTile{(int32_t)g, (int32_t)r0});
            big_ids.push_back((int32_t)g);
        } else {
            d.ntiles = (h.nbins + kFuseStep - 1) / kFuseStep;
            fused_ids.push_back((int32_t)g);
            maxfnt = std::max(maxfnt, h.ntempl);
        }
        tb = std::max(tb, h.bin_offset + h.nbins);
        tt = std::max(tt, h.templ_offset + h.ntempl);
        maxnt = std::max(maxnt, h.ntempl);
    }
    // fused tiles grouped by register class (nt <= 8, <= 16, <= 32): one launch per class
    int64_t ncls[3] = {0, 0, 0};
    for (int c = 0; c < 3; ++c) {
        const int64_t before = (int64_t)fused.size();
        for (int32_t g : fused_ids) {
            GalDesc &d = desc[(size_t)g];
            if (fused_class(d.nt) != c) continue;
            d.tile0 = (int64_t)fused.size();
            for (int64_t r0 = 0; r0 < d.nbins; r0 += kFuseStep)
                fused.push_back(RowTile{(int32_t)g, (int32_t)r0});
        }
        ncls[c] = (int64_t)fused.size() - before;
    }
    // column groups of the two-pass galaxies, largest galaxy first (shortens the tail)
    std::vector<int32_t> order(big_ids);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
        return desc[(size_t)a].nbins > desc[(size_t)b].nbins;
    });
    for (int32_t g : order)
        for (int64_t j0 = 0; j0 < desc[(size_t)g].nt; j0 += kColGroup)
            cols.push_back(ColTile{g, (int32_t)j0});
    if (rows.size() > 0x7fffffffu || cols.size() > 0x7fffffffu || fused.size() > 0x7fffffffu)
        return sfh_set_error(ctx, SFH_ERR_UNSUPPORTED, "too many tiles");
    sfh_galaxies *G = new sfh_galaxies{};
    G->device = ctx->device;
    G->ngal = ngal;
    G->total_bins = tb;
    G->total_templ = tt;
    G->n_row_tiles = (int64_t)rows.size();
    G->n_col_tiles = (int64_t)cols.size();
    G->n_fused_tiles = (int64_t)fused.size();
    G->n_fused_gal = (int64_t)fused_ids.size();
    G->n_big_gal = (int64_t)big_ids.size();
    G->max_nt = maxnt;
    G->max_fused_nt = maxfnt;
    for (int c = 0; c < 3; ++c) G->n_fused_class[c] = ncls[c];
    G->d_models = d_models;
    void **bufs[] = {&G->d_desc, &G->d_rows, &G->d_cols, &G->d_fused, &G->d_fused_ids, &G->d_big_ids};
    const void *src[] = {desc.data(), rows.data(), cols.data(), fused.data(), fused_ids.data(),
                         big_ids.data()};
    const size_t bytes[] = {desc.size() * sizeof(GalDesc), rows.size() * sizeof(RowTile),
                            cols.size() * sizeof(ColTile), fused.size() * sizeof(RowTile),
                            fused_ids.size() * 4, big_ids.size() * 4};
    for (int k = 0; k < 6; ++k) {
        cudaError_t e = cudaSuccess;
        if (bytes[k] && (e = cudaMalloc(bufs[k], bytes[k])) == cudaSuccess)
            e = cudaMemcpy(*bufs[k], src[k], bytes[k], cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            for (int q = 0; q < 6; ++q) cudaFree(*bufs[q]);
            delete G;
            return sfh_cuda_error(ctx, e, "galaxies upload");
        }
    }
    *out = G;
    return SFH_OK;
}

extern "C" int sfh_galaxies_free(sfh_galaxies *g) {
    if (!g) return SFH_OK;
    cudaSetDevice(g->device);
    cudaFree(g->d_desc);
    cudaFree(g->d_rows);
    cudaFree(g->d_cols);
    cudaFree(g->d_fused);
    cudaFree(g->d_fused_ids);
    cudaFree(g->d_big_ids);
    delete g;
    return SFH_OK;
}

extern "C" int sfh_galaxies_info(const sfh_galaxies *g, int64_t *ngal, int64_t *total_bins,
                                 int64_t *total_templ) {
    if (!g) return SFH_ERR_ARG;
    if (ngal) *ngal = g->ngal;
    if (total_bins) *total_bins = g->total_bins;
    if (total_templ) *total_templ = g->total_templ;
    return SFH_OK;
}

extern "C" int sfh_fg_ragged_dev(sfh_ctx *ctx, const sfh_galaxies *gal, const double *d_coeffs,
                                 const double *d_data, double *d_composite, double *d_G,
                                 double *d_negLogL, double eps) {
    if (!ctx || !gal || !d_coeffs || !d_composite) return SFH_ERR_ARG;
    if ((d_G || d_negLogL) && !d_data) return SFH_ERR_ARG;
    if (gal->device != ctx->device)
        return sfh_set_error(ctx, SFH_ERR_ARG, "galaxies belong to another device");
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const bool want_w = d_G != nullptr, want_logl = d_negLogL != nullptr;
    const size_t o_w = 0;
    const size_t o_tl = o_w + (gal->n_big_gal ? sfh_align256((size_t)gal->total_bins * 4) : 0);
    const size_t o_tf = o_tl + sfh_align256((size_t)gal->n_row_tiles * 8 + 8);
    const size_t o_gp = o_tf + sfh_align256((size_t)gal->n_fused_tiles * 8 + 8);
    const size_t o_end = o_gp + sfh_align256((size_t)gal->n_fused_tiles * kFuseMax * 8 + 8);
    int rc = sfh_scratch_reserve(ctx, o_end);
    if (rc) return rc;
    char *b = (char *)ctx->scratch;
    float *w32 = (float *)(b + o_w);
    double *tl = (double *)(b + o_tl), *tf = (double *)(b + o_tf), *gp = (double *)(b + o_gp);
    const GalDesc *desc = (const GalDesc *)gal->d_desc;
    cudaStream_t st = ctx->stream;
    if (gal->n_fused_gal) {
        decltype(&k_ragged_fused<8>) kerns[3] = {k_ragged_fused<8>, k_ragged_fused<16>,
                                                 k_ragged_fused<32>};
        int64_t base = 0;
        for (int c = 0; c < 3; ++c) {
            const int64_t n = gal->n_fused_class[c];
            if (!n) continue;
            kerns[c]<<<(unsigned)n, kRT, 0, st>>>(
                gal->d_models, desc, (const RowTile *)gal->d_fused, d_coeffs, d_data, d_composite,
                tf, gp, (float)eps, want_logl ? 1 : 0, want_w ? 1 : 0, ctx->d_df_tab, (int)base);
            SFH_LAUNCHED(ctx);
            base += n;
        }
        if (want_logl || want_w) {
            k_ragged_finish<<<(unsigned)gal->n_fused_gal, kRT, 0, st>>>(
                desc, (const int32_t *)gal->d_fused_ids, tf, gp, want_logl ? d_negLogL : nullptr,
                want_w ? d_G : nullptr);
            SFH_LAUNCHED(ctx);
        }
    }
    if (gal->n_big_gal) {
        k_ragged_pass1<<<(unsigned)gal->n_row_tiles, kRT, 0, st>>>(
            gal->d_models, desc, (const RowTile *)gal->d_rows, d_coeffs, d_data, d_composite, w32,
            tl, (float)eps, want_logl ? 1 : 0, want_w ? 1 : 0, ctx->d_df_tab);
        SFH_LAUNCHED(ctx);
        if (want_logl) {
            k_ragged_logl<<<(unsigned)gal->n_big_gal, kRT, 0, st>>>(
                desc, (const int32_t *)gal->d_big_ids, tl, d_negLogL);
            SFH_LAUNCHED(ctx);
        }
        if (want_w) {
            k_ragged_pass2<<<(unsigned)gal->n_col_tiles, kRT, 0, st>>>(
                gal->d_models, desc, (const ColTile *)gal->d_cols, w32, d_G);
            SFH_LAUNCHED(ctx);
        }
    }
    return SFH_OK;
}
