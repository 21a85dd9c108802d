// emulator.cu -- learned template emulator: MLP on a PCA basis of templates.
//
// No counterpart in the reference (new component): (log age, [M/H], distance modulus)
// -> MLP 3 -> 256 -> 256 -> 64 (GELU) -> standardised PCA coefficients -> template
// = mean + Σ_k c_k v_k.  The exact partial_cmd_smooth template is the arbiter (Poisson
// deviance per star) and the fallback.
//
// Kernels: tiled GEMMs with BF16-rounded operands and FP32 accumulation (the MLP's
// "BF16 matmuls" over FP32 master weights), bias + GELU, GELU backward, MSE loss
// gradient, Adam; reconstruction of templates from coefficients; the deviance score.  The
// training loop runs on the device: each step draws its minibatch indices with Philox.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "sfh_internal.cuh"

namespace {

constexpr int GBM = 64, GBN = 64, GBK = 16, GTHREADS = 256;

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// C[M x N] = alpha op(A) op(B) (+ C when accum), for each GEMM of a strided batch.  op(A) is M x K: A stored (M x K) row-major
// (ta = 0) or (K x M) row-major (ta = 1); op(B) is K x N: B stored (K x N) (tb = 0) or
// (N x K) (tb = 1).  FP32 accumulation; ROUND rounds every operand to BF16 first (the
// MLP's BF16 matmuls over FP32 master weights).  64 x 64 tiles, 16 x 16 threads with
// 4 x 4 outputs each; loads run along each operand's contiguous dimension.
template <bool ROUND>
__global__ void __launch_bounds__(GTHREADS)
k_gemm(const float *__restrict__ A, const float *__restrict__ B, float *__restrict__ C, int M, int N,
       int K, int ta, int tb, int accum, float alpha, int64_t strideA, int64_t strideB,
       int64_t strideC) {
    // blockIdx.z selects one GEMM of a strided batch (one per MLP group)
    A += blockIdx.z * strideA;
    B += blockIdx.z * strideB;
    C += blockIdx.z * strideC;
    __shared__ float sA[GBK][GBM + 4];
    __shared__ float sB[GBK][GBN + 4];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int row0 = blockIdx.y * GBM, col0 = blockIdx.x * GBN;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int k0 = 0; k0 < K; k0 += GBK) {
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const int l = tid + GTHREADS * p;
            int kl, ml;
            float v = 0.f;
            if (!ta) { kl = l & 15; ml = l >> 4; } else { ml = l & 63; kl = l >> 6; }
            const int m = row0 + ml, k = k0 + kl;
            if (m < M && k < K) v = ta ? A[(int64_t)k * M + m] : A[(int64_t)m * K + k];
            sA[kl][ml] = ROUND ? bf16r(v) : v;
            int nl;
            v = 0.f;
            if (!tb) { nl = l & 63; kl = l >> 6; } else { kl = l & 15; nl = l >> 4; }
            const int n = col0 + nl, kk = k0 + kl;
            if (n < N && kk < K) v = tb ? B[(int64_t)n * K + kk] : B[(int64_t)kk * N + n];
            sB[kl][nl] = ROUND ? bf16r(v) : v;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < GBK; ++k) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = sA[k][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = sB[k][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = row0 + ty + 16 * i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = col0 + tx + 16 * j;
            if (n < N) {
                float *c = C + (int64_t)m * N + n;
                *c = accum ? fmaf(alpha, acc[i][j], *c) : alpha * acc[i][j];
            }
        }
    }
}

__device__ __forceinline__ float gelu(float z) {
    return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) +
           z * 0.3989422804014327f * expf(-0.5f * z * z);
}

// Z += b (per column; rows come in groups of rpg, group g's bias at b + g * pstride);
// A = GELU(Z) when act.
__global__ void k_bias_act(float *__restrict__ Z, float *__restrict__ A, const float *__restrict__ b,
                           int64_t M, int N, int act, int64_t rpg, int64_t pstride) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M * N) return;
    const float z = Z[k] + b[(k / N / rpg) * pstride + k % N];
    Z[k] = z;
    if (act) A[k] = gelu(z);
}

// dZ = dA * GELU'(Z)
__global__ void k_gelu_back(float *__restrict__ dA, const float *__restrict__ Z, int64_t n) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dA[k] *= gelu_grad(Z[k]);
}

// Column sums of each group of rpg rows of X (G*rpg x N): out[g * pstride + n].
__global__ void k_colsum(const float *__restrict__ X, int64_t rpg, int64_t N, int64_t G,
                         float *__restrict__ out, int64_t pstride, float scale) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= G * N) return;
    const int64_t g = t / N, n = t % N;
    float h = 0.f, l = 0.f;
    for (int64_t m = g * rpg; m < (g + 1) * rpg; ++m) sfh_two_sum_acc(h, l, X[m * N + n]);
    out[g * pstride + n] = (h + l) * scale;
}

// MSE: dY = 2 (Y - T) / (M N); per-block partial loss
__global__ void k_mse(const float *__restrict__ Y, const float *__restrict__ T, int64_t n,
                      float scale, float *__restrict__ dY, float *__restrict__ loss_part) {
    __shared__ float s[256];
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (k < n) {
        const float d = Y[k] - T[k];
        dY[k] = 2.0f * d * scale;
        l = d * d * scale;
    }
    s[threadIdx.x] = l;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss_part[blockIdx.x] = s[0];
}

__global__ void k_sum(const float *__restrict__ x, int n, float *__restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        float h = 0.f, l = 0.f;
        for (int i = 0; i < n; ++i) sfh_two_sum_acc(h, l, x[i]);
        *out = h + l;
    }
}

// Adam (Kingma & Ba 2015), bias-corrected, on FP32 master weights.
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float gk = g[k];
    const float mk = b1 * m[k] + (1.0f - b1) * gk;
    const float vk = b2 * v[k] + (1.0f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    w[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
}

struct u4 {
    uint32_t x, y, z, w;
};
__device__ __forceinline__ u4 philox(u4 c, uint32_t k0, uint32_t k1) {  // Salmon et al. 2011
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = u4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Minibatch gather: row i of group g's batch = sample off[g] + floor(u * (off[g+1] - off[g]))
// for a Philox uniform u (off == NULL: one group over all N samples).
__global__ void k_gather(const float *__restrict__ X, const float *__restrict__ T, int64_t N,
                         const int64_t *__restrict__ off, int din, int dout, int B, uint64_t seed,
                         int64_t step, float *__restrict__ Xb, float *__restrict__ Tb) {
    const int i = blockIdx.x, g = blockIdx.y;
    const u4 r = philox(u4{(uint32_t)i, (uint32_t)step, (uint32_t)(step >> 32), 7u ^ ((uint32_t)g << 8)},
                        (uint32_t)seed, (uint32_t)(seed >> 32));
    const int64_t lo = off ? off[g] : 0, cnt = off ? off[g + 1] - off[g] : N;
    const int64_t s = lo + (int64_t)(((uint64_t)r.x * (uint64_t)cnt) >> 32);
    const int64_t row = (int64_t)g * B + i;
    for (int j = threadIdx.x; j < din; j += blockDim.x) Xb[row * din + j] = X[s * din + j];
    for (int j = threadIdx.x; j < dout; j += blockDim.x) Tb[row * dout + j] = T[s * dout + j];
}

// Variance-stabilising transform of templates, in place: y = sqrt(t) (mode 1) or y = t.
__global__ void k_transform(float *__restrict__ Y, int64_t n, int mode) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n && mode == 1) Y[k] = sqrtf(fmaxf(Y[k], 0.f));
}

// Y[r, :] -= mean (row-major rows x cols)
__global__ void k_center(float *__restrict__ Y, int64_t rows, int64_t cols,
                         const float *__restrict__ mean) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < rows * cols) Y[k] -= mean[k % cols];
}

// out = inverse transform of (offset + out): max(0, .)^2 for mode 1, max(0, .) for mode 0.
__global__ void k_finish(float *__restrict__ out, int64_t rows, int64_t cols,
                         const float *__restrict__ offset, int mode) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= rows * cols) return;
    const float y = fmaxf(out[k] + offset[k % cols], 0.f);
    out[k] = mode == 1 ? y * y : y;
}

// Score: Poisson deviance per star of emulated e against exact t,
// 2 Σ_i [e_i - t_i + t_i log(t_i / e_i)] / Σ_i t_i  (e clamped to a tiny floor).
__global__ void k_deviance(const float *__restrict__ exact, const float *__restrict__ emul,
                           int64_t nbins, double *__restrict__ dev) {
    __shared__ double s1[256], s2[256];
    const int t = blockIdx.x;
    double d = 0.0, tot = 0.0;
    for (int64_t i = threadIdx.x; i < nbins; i += blockDim.x) {
        const double tv = exact[(int64_t)t * nbins + i];
        const double ev = fmax((double)emul[(int64_t)t * nbins + i], 1e-30);
        d += ev - tv + (tv > 0.0 ? tv * log(tv / ev) : 0.0);
        tot += tv;
    }
    s1[threadIdx.x] = d;
    s2[threadIdx.x] = tot;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s1[threadIdx.x] += s1[threadIdx.x + o];
            s2[threadIdx.x] += s2[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) dev[t] = s2[0] > 0.0 ? 2.0 * s1[0] / s2[0] : 0.0;
}

// Parameter block layout (floats): W1 (H1 x IN), b1, W2 (H2 x H1), b2, W3 (OUT x H2), b3.
struct MlpShape {
    int in, h1, h2, out;
    int64_t oW1, ob1, oW2, ob2, oW3, ob3, n;
};
MlpShape mlp_shape(int in, int h1, int h2, int out) {
    MlpShape s{in, h1, h2, out, 0, 0, 0, 0, 0, 0, 0};
    s.oW1 = 0;
    s.ob1 = s.oW1 + (int64_t)h1 * in;
    s.oW2 = s.ob1 + h1;
    s.ob2 = s.oW2 + (int64_t)h2 * h1;
    s.oW3 = s.ob2 + h2;
    s.ob3 = s.oW3 + (int64_t)out * h2;
    s.n = s.ob3 + out;
    return s;
}

// One row per CTA, each row with its own group's parameters (inference over rows that
// belong to different groups).  Same arithmetic as the GEMM path: BF16-rounded operands,
// FP32 products accumulated in k order, bias added last, GELU after the hidden layers.
__global__ void k_mlp_rows(const float *__restrict__ P, int64_t pstride, int64_t ngroups, MlpShape S,
                           const float *__restrict__ X, const int32_t *__restrict__ group,
                           float *__restrict__ Y) {
    extern __shared__ float sm[];
    float *x = sm, *a1 = sm + S.in, *a2 = a1 + S.h1;
    const int64_t row = blockIdx.x;
    const int64_t g = group ? (int64_t)group[row] : 0;
    if (g < 0 || g >= ngroups) {  // invalid group: NaN row, no out-of-range read
        for (int j = threadIdx.x; j < S.out; j += blockDim.x) Y[row * S.out + j] = __int_as_float(0x7fc00000);
        return;
    }
    const float *p = P + g * pstride;
    for (int j = threadIdx.x; j < S.in; j += blockDim.x) x[j] = bf16r(X[row * S.in + j]);
    __syncthreads();
    for (int j = threadIdx.x; j < S.h1; j += blockDim.x) {
        const float *w = p + S.oW1 + (int64_t)j * S.in;
        float acc = 0.f;
        for (int k = 0; k < S.in; ++k) acc = fmaf(x[k], bf16r(w[k]), acc);
        a1[j] = bf16r(gelu(acc + p[S.ob1 + j]));
    }
    __syncthreads();
    for (int j = threadIdx.x; j < S.h2; j += blockDim.x) {
        const float *w = p + S.oW2 + (int64_t)j * S.h1;
        float acc = 0.f;
        for (int k = 0; k < S.h1; ++k) acc = fmaf(a1[k], bf16r(w[k]), acc);
        a2[j] = bf16r(gelu(acc + p[S.ob2 + j]));
    }
    __syncthreads();
    for (int j = threadIdx.x; j < S.out; j += blockDim.x) {
        const float *w = p + S.oW3 + (int64_t)j * S.h2;
        float acc = 0.f;
        for (int k = 0; k < S.h2; ++k) acc = fmaf(a2[k], bf16r(w[k]), acc);
        Y[row * S.out + j] = acc + p[S.ob3 + j];
    }
}

// Templates from coefficients with a basis per row's group:
// out[b, i] = inverse transform of (offset[g, i] + Σ_k coef[b, k] basis[g, k, i]), g = group[b].
__global__ void k_recon_rows(const float *__restrict__ coef, const int32_t *__restrict__ group,
                             int64_t ngroups, const float *__restrict__ basis,
                             const float *__restrict__ offset, int K, int64_t nbins, int mode,
                             float *__restrict__ out) {
    extern __shared__ float sc[];
    const int64_t b = blockIdx.y;
    const int64_t g = group ? group[b] : 0;
    if (g < 0 || g >= ngroups) {  // invalid group: NaN row, no out-of-range read
        const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (i < nbins) out[b * nbins + i] = __int_as_float(0x7fc00000);
        return;
    }
    for (int k = threadIdx.x; k < K; k += blockDim.x) sc[k] = coef[b * K + k];
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbins) return;
    const float *v = basis + g * K * nbins + i;
    float acc = 0.f;
    for (int k = 0; k < K; ++k) acc = fmaf(sc[k], v[(int64_t)k * nbins], acc);
    const float y = fmaxf(acc + offset[g * nbins + i], 0.f);
    out[b * nbins + i] = mode == 1 ? y * y : y;
}

// Templates of one group's rows at a time: a segment (group g, rows d_rows[start .. start +
// count), count <= kRecRows) reads its group's basis once for all of its rows, so a batch
// costs (segments x K x nbins + B x nbins) x 4 bytes instead of B x K x nbins x 4.  Each
// thread owns V consecutive bins and R row accumulators; R is the segment's row count
// rounded up to 4, 8 or 16 (block-uniform).  Coefficients of the segment sit in shared
// memory, zero past count.
constexpr int kRecRows = 16;
constexpr int kRecThreads = 256;

template <int R, int V>
__device__ __forceinline__ void recon_segment(const float *__restrict__ sc, int K,
                                              const float *__restrict__ vb,
                                              const float *__restrict__ off, int64_t nbins,
                                              int64_t i0, const int32_t *__restrict__ srow,
                                              int cnt, int mode, float *__restrict__ out) {
    float acc[R][V];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int v = 0; v < V; ++v) acc[r][v] = 0.f;
    if (V == 4) {
        // four basis rows in flight per thread: one 16-byte load at a time leaves the
        // kernel latency-bound at the two blocks per SM its registers allow
#pragma unroll 4
        for (int k = 0; k < K; ++k) {
            const float4 b = __ldg(reinterpret_cast<const float4 *>(vb + (int64_t)k * nbins + i0));
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const float c = sc[r * K + k];
                acc[r][0] = fmaf(c, b.x, acc[r][0]);
                acc[r][1] = fmaf(c, b.y, acc[r][1]);
                acc[r][2] = fmaf(c, b.z, acc[r][2]);
                acc[r][3] = fmaf(c, b.w, acc[r][3]);
            }
        }
    } else {
        for (int k = 0; k < K; ++k) {
            float b[V];
#pragma unroll
            for (int v = 0; v < V; ++v)
                b[v] = i0 + v < nbins ? __ldg(vb + (int64_t)k * nbins + i0 + v) : 0.f;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const float c = sc[r * K + k];
#pragma unroll
                for (int v = 0; v < V; ++v) acc[r][v] = fmaf(c, b[v], acc[r][v]);
            }
        }
    }
    float o[V];
#pragma unroll
    for (int v = 0; v < V; ++v) o[v] = i0 + v < nbins ? __ldg(off + i0 + v) : 0.f;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (r >= cnt) break;
        float *dst = out + (int64_t)srow[r] * nbins + i0;
        float y[V];
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const float t = fmaxf(acc[r][v] + o[v], 0.f);
            y[v] = mode == 1 ? t * t : t;
        }
        if (V == 4) {
            *reinterpret_cast<float4 *>(dst) = make_float4(y[0], y[1], y[2], y[3]);
        } else {
#pragma unroll
            for (int v = 0; v < V; ++v)
                if (i0 + v < nbins) dst[v] = y[v];
        }
    }
}

// seg: nseg x 3 int32 (group, start, count).  A segment whose group, start or count is out
// of range writes NaN to the rows it can address and nothing else; a row index outside
// [0, B) ends its segment at that row.
template <int V>
__global__ void __launch_bounds__(kRecThreads)
k_recon_groups(const float *__restrict__ coef, const int32_t *__restrict__ rows,
               const int32_t *__restrict__ seg, int64_t B, int64_t ngroups,
               const float *__restrict__ basis, const float *__restrict__ offset, int K,
               int64_t nbins, int mode, float *__restrict__ out) {
    extern __shared__ float sc[];  // kRecRows x K
    __shared__ int32_t srow[kRecRows];
    const int s = blockIdx.y;
    const int g = seg[3 * s], start = seg[3 * s + 1];
    int cnt = seg[3 * s + 2];
    const bool bad = g < 0 || g >= ngroups || start < 0 || cnt < 1 || cnt > kRecRows ||
                     (int64_t)start + cnt > B;
    if (threadIdx.x < kRecRows) {
        int32_t r = -1;
        if (start >= 0 && (int64_t)start + threadIdx.x < B && (int)threadIdx.x < cnt)
            r = rows[start + threadIdx.x];
        srow[threadIdx.x] = (r >= 0 && r < B) ? r : -1;
    }
    __syncthreads();
    const int64_t i0 = ((int64_t)blockIdx.x * kRecThreads + threadIdx.x) * V;
    if (bad) {
        for (int r = 0; r < kRecRows; ++r)
            if (srow[r] >= 0 && i0 < nbins)
                for (int v = 0; v < V && i0 + v < nbins; ++v)
                    out[(int64_t)srow[r] * nbins + i0 + v] = __int_as_float(0x7fc00000);
        return;
    }
    for (int r = 0; r < kRecRows; ++r)
        if (srow[r] < 0 && r < cnt) cnt = r;  // a row index out of range ends the segment
    for (int t = threadIdx.x; t < kRecRows * K; t += kRecThreads) {
        const int r = t / K;
        sc[t] = r < cnt ? coef[(int64_t)srow[r] * K + (t - r * K)] : 0.f;
    }
    __syncthreads();
    if (i0 >= nbins) return;
    const float *vb = basis + (int64_t)g * K * nbins;
    const float *off = offset + (int64_t)g * nbins;
    if (cnt <= 4)
        recon_segment<4, V>(sc, K, vb, off, nbins, i0, srow, cnt, mode, out);
    else if (cnt <= 8)
        recon_segment<8, V>(sc, K, vb, off, nbins, i0, srow, cnt, mode, out);
    else
        recon_segment<16, V>(sc, K, vb, off, nbins, i0, srow, cnt, mode, out);
}

struct Acts {  // activations of one batch (G groups x B rows)
    float *Z1, *A1, *Z2, *A2, *Y;
};

int gemm(sfh_ctx *ctx, const float *A, const float *B, float *C, int M, int N, int K, int ta,
         int tb, int accum, bool round = true, float alpha = 1.0f, int batch = 1,
         int64_t sA = 0, int64_t sB = 0, int64_t sC = 0) {
    if (M < 1 || N < 1 || K < 1 || batch < 1) return SFH_OK;
    dim3 grid((N + GBN - 1) / GBN, (M + GBM - 1) / GBM, batch);
    if (grid.y > 65535 || batch > 65535)
        return sfh_set_error(ctx, SFH_ERR_SHAPE, "GEMM too many row tiles or groups");
    if (round)
        k_gemm<true><<<grid, GTHREADS, 0, ctx->stream>>>(A, B, C, M, N, K, ta, tb, accum, alpha, sA,
                                                         sB, sC);
    else
        k_gemm<false><<<grid, GTHREADS, 0, ctx->stream>>>(A, B, C, M, N, K, ta, tb, accum, alpha, sA,
                                                          sB, sC);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

int bias_act(sfh_ctx *ctx, float *Z, float *A, const float *b, int64_t rows, int N, int act,
             int64_t rpg, int64_t pstride) {
    k_bias_act<<<(unsigned)((rows * N + 255) / 256), 256, 0, ctx->stream>>>(Z, A, b, rows, N, act,
                                                                           rpg, pstride);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

int colsum(sfh_ctx *ctx, const float *X, int64_t rpg, int64_t N, int64_t G, float *out,
           int64_t pstride) {
    k_colsum<<<(unsigned)((G * N + 255) / 256), 256, 0, ctx->stream>>>(X, rpg, N, G, out, pstride,
                                                                       1.0f);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

int gelu_back(sfh_ctx *ctx, float *dA, const float *Z, int64_t n) {
    k_gelu_back<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(dA, Z, n);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

// Forward pass of G independent MLPs (parameters P + g * S.n), B rows each; X is G*B x in.
int forward(sfh_ctx *ctx, const MlpShape &S, const float *P, int G, const float *X, int B,
            Acts &a) {
    int rc;
    const int64_t rows = (int64_t)G * B;
    if ((rc = gemm(ctx, X, P + S.oW1, a.Z1, B, S.h1, S.in, 0, 1, 0, true, 1.f, G,
                   (int64_t)B * S.in, S.n, (int64_t)B * S.h1)))
        return rc;
    if ((rc = bias_act(ctx, a.Z1, a.A1, P + S.ob1, rows, S.h1, 1, B, S.n))) return rc;
    if ((rc = gemm(ctx, a.A1, P + S.oW2, a.Z2, B, S.h2, S.h1, 0, 1, 0, true, 1.f, G,
                   (int64_t)B * S.h1, S.n, (int64_t)B * S.h2)))
        return rc;
    if ((rc = bias_act(ctx, a.Z2, a.A2, P + S.ob2, rows, S.h2, 1, B, S.n))) return rc;
    if ((rc = gemm(ctx, a.A2, P + S.oW3, a.Y, B, S.out, S.h2, 0, 1, 0, true, 1.f, G,
                   (int64_t)B * S.h2, S.n, (int64_t)B * S.out)))
        return rc;
    return bias_act(ctx, a.Y, nullptr, P + S.ob3, rows, S.out, 0, B, S.n);
}

// Gradient of the MSE loss w.r.t. all G parameter blocks into Gr (G x S.n); dY is consumed.
int backward(sfh_ctx *ctx, const MlpShape &S, const float *P, int G, const float *X, int B,
             Acts &a, float *dY, float *dA2, float *dA1, float *Gr) {
    int rc;
    const int64_t b = B;
    // layer 3: dW3 = dYᵀ A2, db3 = Σ dY, dA2 = dY W3
    if ((rc = gemm(ctx, dY, a.A2, Gr + S.oW3, S.out, S.h2, B, 1, 0, 0, true, 1.f, G, b * S.out,
                   b * S.h2, S.n)))
        return rc;
    if ((rc = colsum(ctx, dY, B, S.out, G, Gr + S.ob3, S.n))) return rc;
    if ((rc = gemm(ctx, dY, P + S.oW3, dA2, B, S.h2, S.out, 0, 0, 0, true, 1.f, G, b * S.out, S.n,
                   b * S.h2)))
        return rc;
    if ((rc = gelu_back(ctx, dA2, a.Z2, (int64_t)G * b * S.h2))) return rc;
    // layer 2
    if ((rc = gemm(ctx, dA2, a.A1, Gr + S.oW2, S.h2, S.h1, B, 1, 0, 0, true, 1.f, G, b * S.h2,
                   b * S.h1, S.n)))
        return rc;
    if ((rc = colsum(ctx, dA2, B, S.h2, G, Gr + S.ob2, S.n))) return rc;
    if ((rc = gemm(ctx, dA2, P + S.oW2, dA1, B, S.h1, S.h2, 0, 0, 0, true, 1.f, G, b * S.h2, S.n,
                   b * S.h1)))
        return rc;
    if ((rc = gelu_back(ctx, dA1, a.Z1, (int64_t)G * b * S.h1))) return rc;
    // layer 1
    if ((rc = gemm(ctx, dA1, X, Gr + S.oW1, S.h1, S.in, B, 1, 0, 0, true, 1.f, G, b * S.h1,
                   b * S.in, S.n)))
        return rc;
    return colsum(ctx, dA1, B, S.h1, G, Gr + S.ob1, S.n);
}

struct Work {
    Acts a{};
    float *dY = nullptr, *dA2 = nullptr, *dA1 = nullptr, *lp = nullptr;
    float *Xb = nullptr, *Tb = nullptr, *Gr = nullptr;  // training only
    int64_t *off = nullptr;                              // grouped training only
};

// Carves the MLP buffers for G groups of B rows out of the context scratch: no allocation
// once the scratch is large enough, so repeated calls cost only their kernels.
int make_work(sfh_ctx *ctx, Work &w, const MlpShape &S, int G, int B, bool train) {
    const size_t b = (size_t)G * (size_t)B;
    struct Item {
        void *p;
        size_t bytes;
    } items[] = {{&w.a.Z1, b * S.h1 * 4}, {&w.a.A1, b * S.h1 * 4}, {&w.a.Z2, b * S.h2 * 4},
                 {&w.a.A2, b * S.h2 * 4}, {&w.a.Y, b * S.out * 4}, {&w.dY, b * S.out * 4},
                 {&w.dA2, b * S.h2 * 4}, {&w.dA1, b * S.h1 * 4},
                 {&w.lp, ((b * S.out + 255) / 256 + 1) * 4},
                 {&w.Xb, train ? b * S.in * 4 : 0}, {&w.Tb, train ? b * S.out * 4 : 0},
                 {&w.Gr, train ? (size_t)G * S.n * 4 : 0},
                 {&w.off, train ? ((size_t)G + 1) * 8 : 0}};
    size_t total = 0;
    for (const Item &it : items) total += sfh_align256(it.bytes ? it.bytes : 4);
    int rc = sfh_scratch_reserve(ctx, total);
    if (rc) return rc;
    char *base = (char *)ctx->scratch;
    size_t o = 0;
    for (const Item &it : items) {
        *(void **)it.p = it.bytes ? (void *)(base + o) : nullptr;
        o += sfh_align256(it.bytes ? it.bytes : 4);
    }
    return SFH_OK;
}

int loss_grad(sfh_ctx *ctx, const MlpShape &S, const float *P, int G, const float *X,
              const float *Tg, int B, Work &w, float *Gr, float *d_loss) {
    int rc = forward(ctx, S, P, G, X, B, w.a);
    if (rc) return rc;
    const int64_t n = (int64_t)G * B * S.out;
    const int nb = (int)((n + 255) / 256);
    k_mse<<<nb, 256, 0, ctx->stream>>>(w.a.Y, Tg, n, 1.0f / (float)n, w.dY, w.lp);
    SFH_LAUNCHED(ctx);
    if (d_loss) {
        k_sum<<<1, 32, 0, ctx->stream>>>(w.lp, nb, d_loss);
        SFH_LAUNCHED(ctx);
    }
    return backward(ctx, S, P, G, X, B, w.a, w.dY, w.dA2, w.dA1, Gr);
}

bool bad_shape(int in, int h1, int h2, int out) {
    return in < 1 || h1 < 1 || h2 < 1 || out < 1 || in > 1024 || h1 > 1024 || h2 > 1024 ||
           out > 1024;
}

// Adam steps over minibatches drawn per group; G == 1 with off == NULL draws from all rows.
int train(sfh_ctx *ctx, const MlpShape &S, int G, float *d_params, float *d_m, float *d_v,
          int64_t step0, const float *d_X, const float *d_T, int64_t nsamples,
          const int64_t *h_off, int batch, int64_t nsteps, float lr, uint64_t seed,
          float *d_loss_trace) {
    Work w;
    int rc = make_work(ctx, w, S, G, batch, true);
    if (rc) return rc;
    cudaStream_t st = ctx->stream;
    if (h_off) SFH_CK(ctx, cudaMemcpyAsync(w.off, h_off, ((size_t)G + 1) * 8, cudaMemcpyHostToDevice, st));
    const float b1 = 0.9f, b2 = 0.999f;
    const int64_t np = (int64_t)G * S.n;
    for (int64_t it = 0; it < nsteps; ++it) {
        const int64_t step = step0 + it + 1;
        k_gather<<<dim3((unsigned)batch, (unsigned)G), 64, 0, st>>>(
            d_X, d_T, nsamples, h_off ? w.off : nullptr, S.in, S.out, batch, seed, step, w.Xb, w.Tb);
        SFH_LAUNCHED(ctx);
        rc = loss_grad(ctx, S, d_params, G, w.Xb, w.Tb, batch, w, w.Gr,
                       d_loss_trace ? d_loss_trace + it : nullptr);
        if (rc) return rc;
        const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
        k_adam<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(d_params, w.Gr, d_m, d_v, np, lr, b1, b2,
                                                             1e-8f, c1, c2);
        SFH_LAUNCHED(ctx);
    }
    SFH_CK(ctx, cudaStreamSynchronize(st));
    return SFH_OK;
}

}  // namespace

extern "C" int sfh_mlp_param_count(int in, int h1, int h2, int out, int64_t *n) {
    if (!n || bad_shape(in, h1, h2, out)) return SFH_ERR_ARG;
    *n = mlp_shape(in, h1, h2, out).n;
    return SFH_OK;
}

extern "C" int sfh_mlp_forward(sfh_ctx *ctx, int in, int h1, int h2, int out, const float *d_params,
                               const float *d_X, int B, float *d_Y) {
    if (!ctx || !d_params || !d_X || !d_Y || B < 1 || bad_shape(in, h1, h2, out)) return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const MlpShape S = mlp_shape(in, h1, h2, out);
    Work w;
    int rc = make_work(ctx, w, S, 1, B, false);
    if (rc) return rc;
    if ((rc = forward(ctx, S, d_params, 1, d_X, B, w.a))) return rc;
    SFH_CK(ctx, cudaMemcpyAsync(d_Y, w.a.Y, (size_t)B * out * sizeof(float), cudaMemcpyDeviceToDevice,
                                ctx->stream));
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return SFH_OK;
}

extern "C" int sfh_mlp_forward_rows(sfh_ctx *ctx, int in, int h1, int h2, int out,
                                    const float *d_params, int64_t ngroups, const float *d_X,
                                    const int32_t *d_group, int64_t B, float *d_Y) {
    if (!ctx || !d_params || !d_X || !d_Y || B < 1 || B > INT32_MAX || ngroups < 1 ||
        bad_shape(in, h1, h2, out) || (ngroups > 1 && !d_group))
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const MlpShape S = mlp_shape(in, h1, h2, out);
    const size_t smem = (size_t)(in + h1 + h2) * sizeof(float);
    k_mlp_rows<<<(unsigned)B, 256, smem, ctx->stream>>>(d_params, S.n, ngroups, S, d_X, d_group,
                                                        d_Y);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

extern "C" int sfh_mlp_loss_grad(sfh_ctx *ctx, int in, int h1, int h2, int out,
                                 const float *d_params, const float *d_X, const float *d_T, int B,
                                 float *d_grad, float *d_loss) {
    if (!ctx || !d_params || !d_X || !d_T || !d_grad || B < 1 || bad_shape(in, h1, h2, out))
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const MlpShape S = mlp_shape(in, h1, h2, out);
    Work w;
    int rc = make_work(ctx, w, S, 1, B, false);
    if (rc) return rc;
    if ((rc = loss_grad(ctx, S, d_params, 1, d_X, d_T, B, w, d_grad, d_loss))) return rc;
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return SFH_OK;
}

extern "C" int sfh_mlp_train(sfh_ctx *ctx, int in, int h1, int h2, int out, float *d_params,
                             float *d_adam_m, float *d_adam_v, int64_t step0, const float *d_X,
                             const float *d_T, int64_t nsamples, int batch, int64_t nsteps,
                             float lr, uint64_t seed, float *d_loss_trace) {
    if (!ctx || !d_params || !d_adam_m || !d_adam_v || !d_X || !d_T || nsamples < 1 || batch < 1 ||
        batch > 65535 || nsteps < 0 || !(lr > 0) || bad_shape(in, h1, h2, out))
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    return train(ctx, mlp_shape(in, h1, h2, out), 1, d_params, d_adam_m, d_adam_v, step0, d_X, d_T,
                 nsamples, nullptr, batch, nsteps, lr, seed, d_loss_trace);
}

extern "C" int sfh_mlp_train_grouped(sfh_ctx *ctx, int in, int h1, int h2, int out,
                                     int64_t ngroups, float *d_params, float *d_adam_m,
                                     float *d_adam_v, int64_t step0, const float *d_X,
                                     const float *d_T, const int64_t *h_group_off,
                                     int batch_per_group, int64_t nsteps, float lr,
                                     uint64_t seed, float *d_loss_trace) {
    if (!ctx || !d_params || !d_adam_m || !d_adam_v || !d_X || !d_T || !h_group_off ||
        ngroups < 1 || ngroups > 65535 || batch_per_group < 1 || batch_per_group > 65535 ||
        nsteps < 0 || !(lr > 0) || bad_shape(in, h1, h2, out))
        return SFH_ERR_ARG;
    if (h_group_off[0] != 0) return sfh_set_error(ctx, SFH_ERR_ARG, "group offsets must start at 0");
    for (int64_t g = 0; g < ngroups; ++g)
        if (h_group_off[g + 1] <= h_group_off[g])
            return sfh_set_error(ctx, SFH_ERR_ARG, "every group needs at least one sample");
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    return train(ctx, mlp_shape(in, h1, h2, out), (int)ngroups, d_params, d_adam_m, d_adam_v,
                 step0, d_X, d_T, h_group_off[ngroups], h_group_off, batch_per_group, nsteps, lr,
                 seed, d_loss_trace);
}

extern "C" int sfh_gemm_f32(sfh_ctx *ctx, const float *d_A, const float *d_B, float *d_C, int64_t M,
                            int64_t N, int64_t K, int ta, int tb, int accum, float alpha, int bf16) {
    if (!ctx || !d_A || !d_B || !d_C || M < 1 || N < 1 || K < 1 || M > INT32_MAX ||
        N > INT32_MAX || K > INT32_MAX)
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    return gemm(ctx, d_A, d_B, d_C, (int)M, (int)N, (int)K, ta, tb, accum, bf16 != 0, alpha);
}

extern "C" int sfh_emu_prepare(sfh_ctx *ctx, float *d_Y, int64_t rows, int64_t cols, int mode,
                               float *d_mean) {
    if (!ctx || !d_Y || !d_mean || rows < 1 || cols < 1 || (mode != 0 && mode != 1))
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const int64_t n = rows * cols;
    const unsigned nb = (unsigned)((n + 255) / 256);
    k_transform<<<nb, 256, 0, ctx->stream>>>(d_Y, n, mode);
    SFH_LAUNCHED(ctx);
    k_colsum<<<(unsigned)((cols + 255) / 256), 256, 0, ctx->stream>>>(d_Y, rows, cols, 1, d_mean, 0,
                                                                     1.0f / (float)rows);
    SFH_LAUNCHED(ctx);
    k_center<<<nb, 256, 0, ctx->stream>>>(d_Y, rows, cols, d_mean);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

extern "C" int sfh_emu_reconstruct(sfh_ctx *ctx, const float *d_coef, const float *d_basis,
                                   const float *d_offset, int K, int64_t nbins, int64_t B,
                                   int mode, float *d_out) {
    if (!ctx || !d_coef || !d_basis || !d_offset || !d_out || K < 1 || nbins < 1 || B < 1 ||
        nbins > INT32_MAX || B > INT32_MAX || (mode != 0 && mode != 1))
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    int rc = gemm(ctx, d_coef, d_basis, d_out, (int)B, (int)nbins, K, 0, 0, 0, false);
    if (rc) return rc;
    k_finish<<<(unsigned)((B * nbins + 255) / 256), 256, 0, ctx->stream>>>(d_out, B, nbins, d_offset,
                                                                           mode);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

extern "C" int sfh_emu_reconstruct_rows(sfh_ctx *ctx, const float *d_coef, const int32_t *d_group,
                                        int64_t ngroups, const float *d_basis,
                                        const float *d_offset, int K, int64_t nbins, int64_t B,
                                        int mode, float *d_out) {
    if (!ctx || !d_coef || !d_basis || !d_offset || !d_out || K < 1 || K > 4096 || nbins < 1 ||
        B < 1 || B > 65535 || ngroups < 1 || (ngroups > 1 && !d_group) || (mode != 0 && mode != 1))
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    dim3 grid((unsigned)((nbins + 255) / 256), (unsigned)B);
    k_recon_rows<<<grid, 256, (size_t)K * sizeof(float), ctx->stream>>>(
        d_coef, d_group, ngroups, d_basis, d_offset, K, nbins, mode, d_out);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

extern "C" int sfh_emu_reconstruct_groups(sfh_ctx *ctx, const float *d_coef,
                                          const int32_t *d_rows, const int32_t *d_seg,
                                          int64_t nseg, int64_t ngroups, const float *d_basis,
                                          const float *d_offset, int K, int64_t nbins, int64_t B,
                                          int mode, float *d_out) {
    if (!ctx || !d_coef || !d_rows || !d_seg || !d_basis || !d_offset || !d_out || K < 1 ||
        K > 1024 || nbins < 1 || B < 1 || B > INT32_MAX || nseg < 1 || nseg > 65535 ||
        ngroups < 1 || (mode != 0 && mode != 1))
        return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const size_t shm = (size_t)kRecRows * K * sizeof(float);
    // float4 rows need every basis, offset and output row on a 16-byte boundary
    const bool vec = nbins % 4 == 0 && ((uintptr_t)d_basis | (uintptr_t)d_offset |
                                        (uintptr_t)d_out) % 16 == 0;
    if (vec) {
        if (shm > 48 * 1024)
            SFH_CK(ctx, cudaFuncSetAttribute(k_recon_groups<4>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)shm));
        dim3 grid((unsigned)((nbins + 4 * kRecThreads - 1) / (4 * kRecThreads)), (unsigned)nseg);
        k_recon_groups<4><<<grid, kRecThreads, shm, ctx->stream>>>(
            d_coef, d_rows, d_seg, B, ngroups, d_basis, d_offset, K, nbins, mode, d_out);
    } else {
        if (shm > 48 * 1024)
            SFH_CK(ctx, cudaFuncSetAttribute(k_recon_groups<1>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)shm));
        dim3 grid((unsigned)((nbins + kRecThreads - 1) / kRecThreads), (unsigned)nseg);
        k_recon_groups<1><<<grid, kRecThreads, shm, ctx->stream>>>(
            d_coef, d_rows, d_seg, B, ngroups, d_basis, d_offset, K, nbins, mode, d_out);
    }
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

extern "C" int sfh_poisson_deviance(sfh_ctx *ctx, const float *d_exact, const float *d_emul,
                                    int64_t nbins, int B, double *d_dev) {
    if (!ctx || !d_exact || !d_emul || !d_dev || nbins < 1 || B < 1) return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    k_deviance<<<B, 256, 0, ctx->stream>>>(d_exact, d_emul, nbins, d_dev);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}
