// hmc.cu -- many HMC chains at once on the batched tensor-core objective.
//
// Replaces the per-chain DynamicHMC loop of hmc_sample (src/fitting/hmc_sample.jl:105-141,
// log density :24-37) and of sample_sfh with a PowerLawMZR + GaussianDispersion model
// (src/fitting/hierarchical/generic_fitting.jl:90-199, mzr.jl:50-215): all chains advance
// together, every leapfrog step evaluates all gradients with one batched call.
//
//   direct model (hmc_sample):  θ = log r, log p(θ) = logL(exp θ) + Σ θ,
//                               ∇ = -G ⊙ r + 1 with G = -∂logL/∂r (hmc_sample.jl:34-36)
//   MZR model (sample_sfh):     θ = (log R_j, log α | β, log σ) for the free parameters,
//                               r = calculate_coeffs(...) (mzr.jl:50-79), chain rule as
//                               mzr.jl:131-209, Jacobian terms as generic_fitting.jl:143-157
//
// Sampler: fixed-length HMC (nleap leapfrog steps per trajectory), Metropolis accept,
// per-chain dual-averaging step size during warmup (Hoffman & Gelman 2014, Alg. 5),
// diagonal inverse mass set once at half of warmup from the variance of θ pooled over
// all chains, Welford posterior mean/variance of the natural parameters after warmup.
// Random numbers: Philox4x32-10 (Salmon et al., SC'11) keyed by the seed, counter =
// (element, chain, trajectory, stream).  One trajectory is captured in a CUDA graph and
// replayed; the trajectory counter lives on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "sfh_internal.cuh"
#include "sfh_philox.cuh"

namespace {

constexpr int kT = 256;
// fewer chains than this adapt the diagonal metric from their own warmup windows rather
// than from the spread of positions across chains
constexpr int kPoolMin = 16;

using sfh_rng::philox;
using sfh_rng::u01;
using sfh_rng::u4;

__device__ __forceinline__ double normal(uint64_t seed, uint32_t e, uint32_t b, uint32_t t,
                                         uint32_t stream) {
    const u4 r = philox(u4{e, b, t, stream}, (uint32_t)seed, (uint32_t)(seed >> 32));
    const double u1 = u01(r.x, r.y), u2 = u01(r.z, r.w);
    return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

__device__ __forceinline__ double block_sum(double v, double *s_red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += s_red[w];
    __syncthreads();
    return tot;
}

// Per-chain sampler state.
struct ChainState {
    double *theta, *p, *g, *theta0, *g0;  // B x D
    double *logd, *logd0, *kin0;          // B
    double *eps;                          // B step sizes
    double *da;                           // B x 4 dual averaging: mu, Hbar, log_eps_bar, m
    double *acc_sum;                      // B: sum of acceptance probabilities (sampling)
    double *mean, *m2;                    // B x D Welford of the natural parameters
    double *minv;                         // D inverse mass (diagonal)
    int64_t *t;                           // trajectory counter (device)
    float *draws;                         // optional B x ndraws x D
};

struct HmcConst {
    int B, D;
    int64_t nwarm, nsamp;
    int nleap;
    double target;
    uint64_t seed;
    int thin;
    int64_t ndraws;
    int model;   // 0 direct, 1 PowerLawMZR, 2 LinearAMR, 3 LogarithmicAMR
    int nages;
    int alpha_free, beta_free, sigma_free;
    double alpha, beta, sigma, logM0;
    double T_max;  // LinearAMR / LogarithmicAMR: earliest lookback time (Gyr)
    int jac;       // 1: log p carries the Jacobian terms of the log transforms (MAP, sampling)
};

// ---------------------------------------------------------------- trajectory kernels
__global__ void k_refresh(ChainState s, HmcConst c) {
    __shared__ double s_red[kT / 32];
    const int b = blockIdx.x;
    const int64_t t = *s.t;
    double kin = 0.0;
    for (int d = threadIdx.x; d < c.D; d += blockDim.x) {
        const int64_t k = (int64_t)b * c.D + d;
        const double mi = s.minv[d];
        const double pk = normal(c.seed, (uint32_t)d, (uint32_t)b, (uint32_t)t, 1u) / sqrt(mi);
        s.p[k] = pk;
        s.theta0[k] = s.theta[k];
        s.g0[k] = s.g[k];
        kin += 0.5 * pk * pk * mi;
    }
    kin = block_sum(kin, s_red);
    if (threadIdx.x == 0) {
        s.kin0[b] = kin;
        s.logd0[b] = s.logd[b];
    }
}

// p += frac * eps * g; then (drift) θ += eps * minv * p
__global__ void k_kick_drift(ChainState s, HmcConst c, double frac, int drift) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (int64_t)c.B * c.D) return;
    const int b = (int)(k / c.D), d = (int)(k - (int64_t)b * c.D);
    const double e = s.eps[b];
    double pk = s.p[k] + frac * e * s.g[k];
    s.p[k] = pk;
    if (drift) s.theta[k] += e * s.minv[d] * pk;
}

// Dual averaging (Hoffman & Gelman 2014): gamma 0.05, t0 10, kappa 0.75.
__device__ void dual_average(double *da, double *eps, double alpha, double target) {
    const double m = da[3] + 1.0;
    da[3] = m;
    da[1] = (1.0 - 1.0 / (m + 10.0)) * da[1] + (target - alpha) / (m + 10.0);
    const double log_eps = da[0] - sqrt(m) / 0.05 * da[1];
    const double eta = pow(m, -0.75);
    da[2] = eta * log_eps + (1.0 - eta) * da[2];
    *eps = exp(fmin(fmax(log_eps, -30.0), 5.0));
}

__device__ double nat_param(const HmcConst &c, const double *th, int d) {
    if (c.model == 0) return exp(th[d]);
    if (d < c.nages) return exp(th[d]);
    int q = c.nages;
    if (c.alpha_free) { if (d == q) return exp(th[d]); ++q; }
    if (c.beta_free) { if (d == q) return th[d]; ++q; }
    return exp(th[d]);  // sigma
}

__global__ void k_accept(ChainState s, HmcConst c) {
    __shared__ double s_red[kT / 32];
    __shared__ int s_acc;
    const int b = blockIdx.x;
    const int64_t t = *s.t;
    double kin = 0.0;
    for (int d = threadIdx.x; d < c.D; d += blockDim.x) {
        const double pk = s.p[(int64_t)b * c.D + d];
        kin += 0.5 * pk * pk * s.minv[d];
    }
    kin = block_sum(kin, s_red);
    if (threadIdx.x == 0) {
        const double H0 = -s.logd0[b] + s.kin0[b];
        const double H1 = -s.logd[b] + kin;
        const double dH = H0 - H1;
        // A divergent trajectory (non-finite energy) is rejected; fmin would drop a NaN.
        const double a = (dH == dH && dH > -1e300) ? exp(fmin(0.0, dH)) : 0.0;
        const u4 r = philox(u4{0xFFFFFFFFu, (uint32_t)b, (uint32_t)t, 2u}, (uint32_t)c.seed,
                            (uint32_t)(c.seed >> 32));
        const int acc = u01(r.x, r.y) < a;
        s_acc = acc;
        if (!acc) s.logd[b] = s.logd0[b];
        if (t < c.nwarm) {
            dual_average(s.da + 4 * b, s.eps + b, a, c.target);
            if (t == c.nwarm - 1) s.eps[b] = exp(s.da[4 * b + 2]);
        } else {
            s.acc_sum[b] += a;
        }
    }
    __syncthreads();
    const int acc = s_acc;
    const int64_t ts = t - c.nwarm;  // sampling index
    for (int d = threadIdx.x; d < c.D; d += blockDim.x) {
        const int64_t k = (int64_t)b * c.D + d;
        if (!acc) {
            s.theta[k] = s.theta0[k];
            s.g[k] = s.g0[k];
        }
        if (ts < 0 && c.B < kPoolMin && c.nwarm >= 20 && t >= c.nwarm / 4 &&
            t < c.nwarm / 2) {
            // too few chains to pool over: each chain's own window of warmup positions
            // (the second quarter of warmup) gives its variance; the sums are cleared when
            // the metric is set
            const double x = s.theta[k];
            const double n1 = (double)(t - c.nwarm / 4 + 1);
            const double delta = x - s.mean[k];
            s.mean[k] += delta / n1;
            s.m2[k] += delta * (x - s.mean[k]);
        }
        if (ts >= 0) {
            const double x = nat_param(c, s.theta + (int64_t)b * c.D, d);
            const double n1 = (double)(ts + 1);
            const double delta = x - s.mean[k];
            s.mean[k] += delta / n1;
            s.m2[k] += delta * (x - s.mean[k]);
            if (s.draws && c.thin > 0 && ts % c.thin == 0 && ts / c.thin < c.ndraws)
                s.draws[((int64_t)b * c.ndraws + ts / c.thin) * c.D + d] = (float)x;
        }
    }
}

// At half of warmup: inverse mass = variance of θ pooled over chains (at least kPoolMin of
// them), else the chains' own variances over the second quarter of warmup (DynamicHMC
// adapts each chain from its own draws); restart dual averaging around the current steps.
__global__ void k_adapt_mass(ChainState s, HmcConst c) {
    const int64_t t = *s.t;
    if (c.nwarm < 20 || t != c.nwarm / 2) return;
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d < c.D && c.B < kPoolMin) {
        // the chains' own window variances (second quarter of warmup), averaged over the
        // chains and regularised by the window length; then the sums are cleared for the
        // sampling statistics
        const double nw = (double)(c.nwarm / 2 - c.nwarm / 4);
        double v = 0.0;
        for (int b = 0; b < c.B; ++b) {
            const int64_t k = (int64_t)b * c.D + d;
            v += nw > 1.0 ? s.m2[k] / (nw - 1.0) : 1.0;
            s.mean[k] = 0.0;
            s.m2[k] = 0.0;
        }
        s.minv[d] = (nw / (nw + 5.0)) * (v / c.B) + 1e-3 * (5.0 / (nw + 5.0));
    } else if (d < c.D) {
        double m = 0.0, q = 0.0;
        for (int b = 0; b < c.B; ++b) {
            const double x = s.theta[(int64_t)b * c.D + d];
            const double dl = x - m;
            m += dl / (b + 1);
            q += dl * (x - m);
        }
        const double var = c.B > 1 ? q / (c.B - 1) : 1.0;
        // regularised towards 1e-3 as in common practice for few samples
        s.minv[d] = (c.B / (c.B + 5.0)) * var + 1e-3 * (5.0 / (c.B + 5.0));
    }
    if (d < c.B) {
        double *da = s.da + 4 * d;
        da[0] = log(10.0 * s.eps[d]);
        da[1] = 0.0;
        da[2] = 0.0;
        da[3] = 0.0;
    }
}

__global__ void k_next_traj(ChainState s) { *s.t += 1; }

// ---------------------------------------------------------------- model maps
__global__ void k_direct_map(const double *__restrict__ theta, int64_t n, double *__restrict__ r) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) r[k] = exp(theta[k]);
}

// log p = -negLogL + Σ θ;  ∇ = -G ⊙ r + 1   (hmc_sample.jl:34-36)
template <typename GT>  // float: the batched gradient; double: the single-vector one
__global__ void k_direct_grad(const double *__restrict__ theta, const double *__restrict__ r,
                              const GT *__restrict__ G, const double *__restrict__ negL, int D,
                              double *__restrict__ g, double *__restrict__ logd, int want_logd) {
    __shared__ double s_red[kT / 32];
    const int b = blockIdx.x;
    double st = 0.0;
    for (int d = threadIdx.x; d < D; d += blockDim.x) {
        const int64_t k = (int64_t)b * D + d;
        g[k] = -(double)G[k] * r[k] + 1.0;
        st += theta[k];
    }
    if (want_logd) {
        st = block_sum(st, s_red);
        if (threadIdx.x == 0) logd[b] = -negL[b] + st;
    }
}

struct MzrDev {
    int nt, nages;
    const int *jidx;         // template -> age
    const double *MH;        // template [M/H]
    const int *age_off;      // CSR: templates of age j
    const int *age_tmpl;
    const int *sorted;       // ages by decreasing logAge (sortperm(unique_logAge; rev=true))
    const double *tage;      // LinearAMR: lookback time of each age in Gyr, 10^(logAge - 9)
    double *aux;             // B x (4 nages): cum, mu, Asum, R_j / Asum_j
    const int *uni;          // per age: its templates (CSR order = ascending [M/H]) are
                             // evenly spaced in [M/H], so A follows a product recurrence
    double *A;               // B x nt Gaussian weights A_jk
};

// MH_from_Z and dMH_dZ with the package defaults (solZ 0.01524, Y_p 0.2485, γ 1.78),
// src/utilities.jl:117-155: [M/H] of a metal mass fraction Z for LogarithmicAMR.
__device__ __forceinline__ double mh_from_z(double Z) {
    const double Yp = 0.2485, g = 1.78, solZ = 0.01524;
    const double X = 1.0 - (Yp + g * Z + Z), Xsol = 1.0 - (Yp + g * solZ + solZ);
    return X > 0.0 ? log10(Z / (X * solZ) * Xsol) : NAN;
}
__device__ __forceinline__ double dmh_dz(double Z) {
    const double Yp = 0.2485, g = 1.78;
    return (Yp - 1.0) / (2.302585092994046 * Z * (Yp + Z + g * Z - 1.0));
}

// calculate_coeffs (mzr.jl:50-79, amr.jl:50-72) per chain: one block per chain.
__global__ void k_mzr_map(const double *__restrict__ theta, HmcConst c, MzrDev z,
                          double *__restrict__ r) {
    // per-age work (exp R_j, μ_j, the normalisation) is done once per age, in parallel; per
    // template one FP64 exp (the Gaussian weight) and one multiply: FP64 is the slow pipe
    const int b = blockIdx.x;
    const double *th = theta + (int64_t)b * c.D;
    double *cum = z.aux + (int64_t)b * 4 * z.nages, *mu = cum + z.nages, *Asum = mu + z.nages;
    double *f = Asum + z.nages;  // R_j, then R_j / Σ_k A_jk
    double alpha = c.alpha, beta = c.beta, sigma = c.sigma;
    int q = z.nages;
    if (c.alpha_free) alpha = exp(th[q++]);
    if (c.beta_free) beta = (c.model == 3) ? exp(th[q++]) : th[q++];  // LogarithmicAMR: β > 0
    if (c.sigma_free) sigma = exp(th[q++]);
    for (int j = threadIdx.x; j < z.nages; j += blockDim.x) f[j] = exp(th[j]);
    __syncthreads();
    if (c.model == 2 || c.model == 3) {
        // LinearAMR: μ_j = β + α (T_max - t_j), amr.jl:205; LogarithmicAMR: μ_j =
        // MH_from_Z(β + α (T_max - t_j)), amr.jl:278
        for (int j = threadIdx.x; j < z.nages; j += blockDim.x) {
            const double x = beta + alpha * (c.T_max - z.tage[j]);
            mu[j] = c.model == 2 ? x : mh_from_z(x);
        }
    } else {
        if (threadIdx.x == 0) {
            double acc = 0.0;  // cumsum in decreasing-age order
            for (int p = 0; p < z.nages; ++p) {
                const int j = z.sorted[p];
                acc += f[j];
                cum[j] = acc;
            }
        }
        __syncthreads();
        for (int j = threadIdx.x; j < z.nages; j += blockDim.x)
            mu[j] = beta + alpha * (log10(cum[j]) - c.logM0);
    }
    __syncthreads();
    double *A = z.A + (int64_t)b * z.nt;
    const double hinv = 0.5 / (sigma * sigma);
    for (int k = threadIdx.x; k < z.nt; k += blockDim.x) {
        if (z.uni[z.jidx[k]]) continue;
        const double dd = z.MH[k] - mu[z.jidx[k]];
        A[k] = exp(-dd * dd * hinv);  // dispersion_models.jl:92
    }
    // evenly spaced [M/H] (step Δ): A_{k±1} / A_k = exp(-h (±2 x_k Δ + Δ²)), x_k = MH_k - μ,
    // and successive ratios differ by the factor exp(-2 h Δ²): three exps and two products
    // per template instead of one exp each (FP64 is the slow pipe), from the template
    // nearest μ outwards, where every ratio is at most 1
    for (int j = threadIdx.x; j < z.nages; j += blockDim.x) {
        if (!z.uni[j]) continue;
        const int a0 = z.age_off[j], n = z.age_off[j + 1] - a0;
        const double m = mu[j];
        const double mh0 = z.MH[z.age_tmpl[a0]];
        const double dl = (z.MH[z.age_tmpl[a0 + n - 1]] - mh0) / (double)(n - 1);
        int ks = (int)rint((m - mh0) / dl);
        ks = ks < 0 ? 0 : (ks > n - 1 ? n - 1 : ks);
        const double x = z.MH[z.age_tmpl[a0 + ks]] - m;
        const double Ak = exp(-x * x * hinv), c2 = exp(-2.0 * dl * dl * hinv);
        A[z.age_tmpl[a0 + ks]] = Ak;
        double q = exp(-(2.0 * x * dl + dl * dl) * hinv), Au = Ak;
        for (int k = ks + 1; k < n; ++k) {
            Au *= q;
            q *= c2;
            A[z.age_tmpl[a0 + k]] = Au;
        }
        double qd = exp(-(dl * dl - 2.0 * x * dl) * hinv), Ad = Ak;
        for (int k = ks - 1; k >= 0; --k) {
            Ad *= qd;
            qd *= c2;
            A[z.age_tmpl[a0 + k]] = Ad;
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < z.nages; j += blockDim.x) {
        double sA = 0.0;
        for (int q2 = z.age_off[j]; q2 < z.age_off[j + 1]; ++q2) sA += A[z.age_tmpl[q2]];
        Asum[j] = sA;
        f[j] = f[j] / sA;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < z.nt; k += blockDim.x)
        r[(int64_t)b * z.nt + k] = A[k] * f[z.jidx[k]];
}

// Chain rule of mzr.jl:131-209 (gradient of -logL w.r.t. R_j, α, β, σ) followed by the
// transforms and Jacobian terms of generic_fitting.jl:143-171; writes ∇ log p and log p.
// For LinearAMR (amr.jl:122-157) μ_j depends on the age only: ∂μ/∂R = 0 removes the
// cross-age terms and ∂μ/∂α = T_max - t_j.
template <typename GT>  // float: the batched gradient; double: the single-vector one
__global__ void k_mzr_grad(const double *__restrict__ theta, const double *__restrict__ r,
                           const GT *__restrict__ Gfg, const double *__restrict__ negL,
                           HmcConst c, MzrDev z, double *__restrict__ g, double *__restrict__ logd,
                           int want_logd) {
    extern __shared__ double sm[];
    const int b = blockIdx.x;
    const int na = z.nages;
    double *Gv = sm;                 // na + 3: gradient of -logL w.r.t. (R, α, β, σ)
    double *ksR = Gv + na + 3;       // per age: Σ dA/dR
    double *ksMu = ksR + na;         // Σ dA/dμ
    double *ksS = ksMu + na;         // Σ dA/dσ
    double *ksDr = ksS + na;         // Σ drjk/dRj
    double *t1 = ksDr + na;          // Σ fullG (r/R + ...)
    double *ps = t1 + na;            // psum per age
    double *ss = ps + na;            // ssum per age
    double *Rv = ss + na;            // R_j
    double *lc = Rv + na;            // log10(cum_j) - logM0 (MZR)
    const double *th = theta + (int64_t)b * c.D;
    const double *cum = z.aux + (int64_t)b * 4 * na, *mu = cum + na, *Asum = mu + na;
    const double *fR = Asum + na;    // R_j / Asum_j (k_mzr_map)
    const double *A = z.A + (int64_t)b * z.nt;
    const GT *G = Gfg + (int64_t)b * z.nt;
    double alpha = c.alpha, beta = c.beta, sigma = c.sigma;
    {
        int q = na;
        if (c.alpha_free) alpha = exp(th[q++]);
        if (c.beta_free) beta = (c.model == 3) ? exp(th[q++]) : th[q++];
        if (c.sigma_free) sigma = exp(th[q++]);
    }
    (void)r;
    const double ln10 = 2.302585092994046;
    // The per-template products run in GT: FP32 for the batched sampler, whose gradient
    // only steers the leapfrog (the log density that accepts or weights a state is
    // computed separately, in full precision), FP64 for the single-vector fit.
    using CT = GT;
    const CT is2 = (CT)(1.0 / (sigma * sigma)), is3 = (CT)(1.0 / (sigma * sigma * sigma));
    // per-age sums in fixed template order (deterministic); the divisions are hoisted out of
    // the template loops (FP64 division is slow on this part)
    for (int j = threadIdx.x; j < na; j += blockDim.x) {
        const double Rj = exp(th[j]);
        Rv[j] = Rj;
        if (c.model < 2) lc[j] = log10(cum[j]) - c.logM0;
        const CT dmu_dR = (CT)((c.model >= 2) ? 0.0 : alpha / (cum[j] * ln10));
        CT sR = 0, sM = 0, sS = 0;
        const CT mj = (CT)mu[j];
        for (int q2 = z.age_off[j]; q2 < z.age_off[j + 1]; ++q2) {
            const int k = z.age_tmpl[q2];
            const CT d = (CT)z.MH[k] - mj;
            const CT Ad = (CT)A[k] * d;
            const CT dAmu = Ad * is2;
            sR += dAmu * dmu_dR;
            sM += dAmu;
            sS += Ad * d * is3;
        }
        ksR[j] = sR;
        ksMu[j] = sM;
        ksS[j] = sS;
        CT dr = 0, tt = 0, psum = 0, ssum = 0;
        const CT iAv = (CT)(1.0 / Asum[j]), f = (CT)fR[j];  // f = R_j / Asum_j
        for (int q2 = z.age_off[j]; q2 < z.age_off[j + 1]; ++q2) {
            const int k = z.age_tmpl[q2];
            const CT fullG = -(CT)G[k];  // ∂logL/∂r_k
            const CT d = (CT)z.MH[k] - mj;
            const CT Ak = (CT)A[k];
            const CT Ad = Ak * d;
            const CT dAmu = Ad * is2;
            const CT dAR = dAmu * dmu_dR;
            const CT dAs = Ad * d * is3;
            const CT a = Ak * iAv;  // A_jk / Asum_j = r_k / R_j
            dr += fullG * (f * (dAR - a * sR));
            tt += fullG * (a + (dAR - sR * a) * f);
            psum -= fullG * f * (dAmu - a * sM);
            ssum += fullG * f * (dAs - a * sS);
        }
        ksDr[j] = dr;
        t1[j] = tt;
        ps[j] = psum;
        ss[j] = ssum;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < na + 3; ++q) Gv[q] = 0.0;
        double acc = 0.0;  // reverse cumulative sum over the decreasing-age order
        for (int p = na - 1; p >= 1; --p) {
            acc += ksDr[z.sorted[p]];
            Gv[z.sorted[p - 1]] -= acc;
        }
        for (int j = 0; j < na; ++j) {
            Gv[j] -= t1[j];
            // ∂μ/∂α and ∂μ/∂β: mzr.jl:279-281, amr.jl:207-209, amr.jl:280-288
            const double dt = c.T_max - z.tage[j];
            const double dz = (c.model == 3) ? dmh_dz(beta + alpha * dt) : 1.0;
            Gv[na] += ps[j] * ((c.model >= 2) ? dz * dt : lc[j]);
            Gv[na + 1] += ps[j] * dz;
            Gv[na + 2] -= ss[j];
        }
        // ∇ log p over the free variables; log p = logL + Σ log(positive x) with the
        // Jacobian terms (generic_fitting.jl:143-171), logL alone without them (the MLE)
        double* gb = g + (int64_t)b * c.D;
        const double jf = c.jac ? 1.0 : 0.0;
        double jac = 0.0;
        for (int j = 0; j < na; ++j) {
            const double Rj = Rv[j];
            gb[j] = -Gv[j] * Rj + jf;
            jac += th[j];
        }
        int q = na;
        if (c.alpha_free) { gb[q] = -Gv[na] * alpha + jf; jac += th[q]; ++q; }
        if (c.beta_free) {
            if (c.model == 3) { gb[q] = -Gv[na + 1] * beta + jf; jac += th[q]; }  // log β
            else gb[q] = -Gv[na + 1];
            ++q;
        }
        if (c.sigma_free) { gb[q] = -Gv[na + 2] * sigma + jf; jac += th[q]; ++q; }
        if (want_logd) logd[b] = -negL[b] + jf * jac;
    }
}

struct HmcRun {
    HmcConst c;
    ChainState s;
    MzrDev z;
    SfhBatchedPlan plan;
    const sfh_models *mb = nullptr;  // the handle the batched evaluations use
    double *d_r = nullptr, *d_negL = nullptr;
    float *d_G = nullptr;
    double eps_abs;
    // one chain: the single-vector fg! (the plain path) instead of the batched GEMMs
    bool single = false;
    const double *d_data = nullptr;
    double *d_Gd = nullptr, *d_comp = nullptr;
};

// The run's pending device errors: the batched pipeline's flag, or the single-vector one.
int run_check(sfh_ctx *ctx, const HmcRun &h) {
    if (!h.single) return sfh_batched_check(ctx, h.plan);
    SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return sfh_check_onepass(ctx);
}

int launch_eval(sfh_ctx *ctx, const sfh_models *m, HmcRun &h, bool want_logd) {
    cudaStream_t st = ctx->stream;
    const int64_t n = (int64_t)h.c.B * m->nt;
    if (h.c.model == 0) {
        k_direct_map<<<(unsigned)((n + kT - 1) / kT), kT, 0, st>>>(h.s.theta, n, h.d_r);
    } else {
        k_mzr_map<<<h.c.B, kT, 0, st>>>(h.s.theta, h.c, h.z, h.d_r);
    }
    SFH_LAUNCHED(ctx);
    if (h.single) {  // one chain: the single-vector fg! on the FP32 templates
        FgArgs a{};
        a.coeffs = h.d_r;
        a.data = h.d_data;
        a.composite = h.d_comp;
        a.G = h.d_Gd;
        a.negLogL = h.d_negL;
        a.eps = h.eps_abs;
        a.gsign = 1.0;
        a.mode = FG_MODE_FG;
        int rc = sfh_launch_fg(ctx, m, a);
        if (rc) return rc;
        if (h.c.model == 0) {
            k_direct_grad<double><<<1, kT, 0, st>>>(h.s.theta, h.d_r, h.d_Gd, h.d_negL, h.c.D,
                                                    h.s.g, h.s.logd, want_logd ? 1 : 0);
        } else {
            const size_t sm = (size_t)(h.z.nages * 10 + 3) * sizeof(double);
            if (sm > 48 * 1024)
                SFH_CK(ctx, cudaFuncSetAttribute(k_mzr_grad<double>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            k_mzr_grad<double><<<1, 64, sm, st>>>(h.s.theta, h.d_r, h.d_Gd, h.d_negL, h.c, h.z,
                                                  h.s.g, h.s.logd, want_logd ? 1 : 0);
        }
        SFH_LAUNCHED(ctx);
        return SFH_OK;
    }
    int rc = sfh_batched_launch(ctx, h.mb ? h.mb : m, h.plan, h.d_r, want_logd ? h.d_negL : nullptr,
                                h.d_G, h.eps_abs);
    if (rc) return rc;
    if (h.c.model == 0) {
        k_direct_grad<float><<<h.c.B, kT, 0, st>>>(h.s.theta, h.d_r, h.d_G, h.d_negL, h.c.D, h.s.g,
                                                   h.s.logd, want_logd ? 1 : 0);
    } else {
        const size_t sm = (size_t)(h.z.nages * 10 + 3) * sizeof(double);
        if (sm > 48 * 1024)
            SFH_CK(ctx, cudaFuncSetAttribute(k_mzr_grad<float>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_mzr_grad<float><<<h.c.B, 64, sm, st>>>(h.s.theta, h.d_r, h.d_G, h.d_negL, h.c, h.z,
                                                 h.s.g, h.s.logd, want_logd ? 1 : 0);
    }
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

int launch_trajectory(sfh_ctx *ctx, const sfh_models *m, HmcRun &h) {
    cudaStream_t st = ctx->stream;
    const int64_t n = (int64_t)h.c.B * h.c.D;
    const unsigned gb = (unsigned)((n + kT - 1) / kT);
    k_refresh<<<h.c.B, kT, 0, st>>>(h.s, h.c);
    SFH_LAUNCHED(ctx);
    for (int l = 0; l < h.c.nleap; ++l) {
        k_kick_drift<<<gb, kT, 0, st>>>(h.s, h.c, l == 0 ? 0.5 : 1.0, 1);
        SFH_LAUNCHED(ctx);
        int rc = launch_eval(ctx, m, h, l == h.c.nleap - 1);
        if (rc) return rc;
    }
    k_kick_drift<<<gb, kT, 0, st>>>(h.s, h.c, 0.5, 0);
    SFH_LAUNCHED(ctx);
    k_accept<<<h.c.B, kT, 0, st>>>(h.s, h.c);
    SFH_LAUNCHED(ctx);
    k_adapt_mass<<<(unsigned)((std::max(h.c.D, h.c.B) + kT - 1) / kT), kT, 0, st>>>(h.s, h.c);
    SFH_LAUNCHED(ctx);
    k_next_traj<<<1, 1, 0, st>>>(h.s);
    SFH_LAUNCHED(ctx);
    return SFH_OK;
}

__global__ void k_init_state(ChainState s, HmcConst c, double step0) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < (int64_t)c.B * c.D) {
        s.mean[k] = 0.0;
        s.m2[k] = 0.0;
    }
    if (k < c.D) s.minv[k] = 1.0;
    if (k < c.B) {
        s.eps[k] = step0;
        s.acc_sum[k] = 0.0;
        s.da[4 * k + 0] = log(10.0 * step0);
        s.da[4 * k + 1] = 0.0;
        s.da[4 * k + 2] = 0.0;
        s.da[4 * k + 3] = 0.0;
    }
    if (k == 0) *s.t = 0;
}

__global__ void k_finish(ChainState s, HmcConst c, double *mean, double *var, double *acc,
                         double *eps) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < (int64_t)c.B * c.D) {
        if (mean) mean[k] = s.mean[k];
        if (var) var[k] = c.nsamp > 1 ? s.m2[k] / (double)(c.nsamp - 1) : 0.0;
    }
    if (k < c.B) {
        if (acc) acc[k] = c.nsamp > 0 ? s.acc_sum[k] / (double)c.nsamp : 0.0;
        if (eps) eps[k] = s.eps[k];
    }
}


// Validates the configuration, allocates the run's device buffers (recorded in `owned`)
// and prepares the batched objective for nchains vectors.
// batched = false: one parameter vector for the single-vector objective of the device fit
// (any template storage; no sampler state, no batched plan).
int setup_run(sfh_ctx *ctx, const sfh_models *m, const double *d_data, const sfh_hmc_config *cfg,
              float *d_draws, HmcRun &h, std::vector<void *> &owned, bool batched = true) {
    if (!ctx || !m || !d_data || !cfg) return SFH_ERR_ARG;
    if (batched && m->storage != SFH_BF16X2)
        return sfh_set_error(ctx, SFH_ERR_ARG, "HMC needs models stored as SFH_BF16X2");
    if (batched && (cfg->nchains < 1 || cfg->nleap < 1 || cfg->ntraj < 0 || cfg->nwarmup < 0 ||
                    !(cfg->step0 > 0) || !(cfg->target_accept > 0 && cfg->target_accept < 1)))
        return sfh_set_error(ctx, SFH_ERR_ARG, "invalid HMC configuration");
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    HmcConst &c = h.c;
    c.B = batched ? cfg->nchains : 1;
    c.jac = 1;
    c.model = cfg->model;
    c.nwarm = cfg->nwarmup;
    c.nsamp = cfg->ntraj;
    c.nleap = cfg->nleap;
    c.target = cfg->target_accept;
    c.seed = cfg->seed;
    c.thin = cfg->thin > 0 ? cfg->thin : 1;
    c.ndraws = d_draws ? (cfg->ntraj + c.thin - 1) / c.thin : 0;
    h.eps_abs = 2.220446049250313e-16;
    const int nt = (int)m->nt;
    std::vector<int> jidx, age_off, age_tmpl, sorted, uni;
    if (c.model == SFH_HMC_DIRECT) {
        c.D = nt;
    } else if (c.model == SFH_HMC_MZR || c.model == SFH_HMC_LINEAR_AMR ||
               c.model == SFH_HMC_LOG_AMR) {
        if (cfg->nages < 1 || !cfg->h_age_index || !cfg->h_logAge || !cfg->h_MH ||
            !(cfg->alpha >= 0) || !(cfg->sigma > 0))
            return sfh_set_error(ctx, SFH_ERR_ARG, "invalid metallicity model description");
        if ((c.model == SFH_HMC_LINEAR_AMR || c.model == SFH_HMC_LOG_AMR) && !(cfg->T_max > 0))
            return sfh_set_error(ctx, SFH_ERR_ARG, "an AMR needs T_max > 0");  // amr.jl:188
        if (c.model == SFH_HMC_LOG_AMR && !(cfg->beta > 0))
            return sfh_set_error(ctx, SFH_ERR_ARG, "LogarithmicAMR needs β > 0");
        c.T_max = cfg->T_max;
        c.nages = cfg->nages;
        c.alpha_free = cfg->alpha_free ? 1 : 0;
        c.beta_free = cfg->beta_free ? 1 : 0;
        c.sigma_free = cfg->sigma_free ? 1 : 0;
        c.alpha = cfg->alpha;
        c.beta = cfg->beta;
        c.sigma = cfg->sigma;
        c.logM0 = cfg->logMstar0;
        c.D = c.nages + c.alpha_free + c.beta_free + c.sigma_free;
        jidx.assign(cfg->h_age_index, cfg->h_age_index + nt);
        age_off.assign(c.nages + 1, 0);
        for (int k = 0; k < nt; ++k) {
            if (jidx[k] < 0 || jidx[k] >= c.nages)
                return sfh_set_error(ctx, SFH_ERR_ARG, "age index out of range");
            age_off[jidx[k] + 1]++;
        }
        for (int j = 0; j < c.nages; ++j) age_off[j + 1] += age_off[j];
        age_tmpl.assign(nt, 0);
        std::vector<int> fill(age_off.begin(), age_off.end() - 1);
        for (int k = 0; k < nt; ++k) age_tmpl[fill[jidx[k]]++] = k;
        // each age's templates in ascending [M/H]; an age whose [M/H] are evenly spaced
        // (to 1e-9 of the step) takes the product recurrence in k_mzr_map
        uni.assign(c.nages, 0);
        for (int j = 0; j < c.nages; ++j) {
            int *b0 = age_tmpl.data() + age_off[j], *b1 = age_tmpl.data() + age_off[j + 1];
            std::stable_sort(b0, b1, [&](int a, int b) { return cfg->h_MH[a] < cfg->h_MH[b]; });
            const int n = (int)(b1 - b0);
            if (n < 3) continue;
            const double dl = (cfg->h_MH[b0[n - 1]] - cfg->h_MH[b0[0]]) / (n - 1);
            bool even = dl > 0.0;
            for (int k = 1; k < n && even; ++k)
                even = std::fabs(cfg->h_MH[b0[k]] - cfg->h_MH[b0[0]] - k * dl) <= 1e-9 * dl;
            uni[j] = even ? 1 : 0;
        }
        sorted.resize(c.nages);
        for (int j = 0; j < c.nages; ++j) sorted[j] = j;
        std::stable_sort(sorted.begin(), sorted.end(),
                         [&](int a, int b) { return cfg->h_logAge[a] > cfg->h_logAge[b]; });
    } else {
        return sfh_set_error(ctx, SFH_ERR_ARG, "unknown HMC model");
    }
    const int64_t BD = (int64_t)c.B * c.D;
    // ---- device buffers for the run (freed by the caller)
    auto alloc = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        owned.push_back(p);
        return p;
    };
    ChainState &s = h.s;
    s.theta = (double *)alloc(BD * 8);
    s.p = (double *)alloc(BD * 8);
    s.g = (double *)alloc(BD * 8);
    s.theta0 = (double *)alloc(BD * 8);
    s.g0 = (double *)alloc(BD * 8);
    s.mean = (double *)alloc(BD * 8);
    s.m2 = (double *)alloc(BD * 8);
    s.logd = (double *)alloc(c.B * 8);
    s.logd0 = (double *)alloc(c.B * 8);
    s.kin0 = (double *)alloc(c.B * 8);
    s.eps = (double *)alloc(c.B * 8);
    s.da = (double *)alloc(c.B * 4 * 8);
    s.acc_sum = (double *)alloc(c.B * 8);
    s.minv = (double *)alloc(c.D * 8);
    s.t = (int64_t *)alloc(8);
    s.draws = d_draws;
    h.d_r = (double *)alloc((size_t)c.B * nt * 8);
    h.d_negL = (double *)alloc(c.B * 8);
    h.d_G = (float *)alloc((size_t)c.B * nt * 4);
    if (c.model == SFH_HMC_MZR || c.model == SFH_HMC_LINEAR_AMR || c.model == SFH_HMC_LOG_AMR) {
        std::vector<double> tage(c.nages);
        for (int j = 0; j < c.nages; ++j) tage[j] = std::pow(10.0, cfg->h_logAge[j] - 9.0);
        double *dta = (double *)alloc(c.nages * 8);
        int *dj = (int *)alloc(nt * 4), *dao = (int *)alloc((c.nages + 1) * 4);
        int *dat = (int *)alloc(nt * 4), *dso = (int *)alloc(c.nages * 4);
        double *dmh = (double *)alloc(nt * 8);
        int *duni = (int *)alloc(c.nages * 4);
        h.z.aux = (double *)alloc((size_t)c.B * 4 * c.nages * 8);
        h.z.A = (double *)alloc((size_t)c.B * nt * 8);
        for (void *p : owned)
            if (!p) return sfh_set_error(ctx, SFH_ERR_NOMEM, "HMC buffers");
        cudaMemcpy(dj, jidx.data(), nt * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dao, age_off.data(), (c.nages + 1) * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dat, age_tmpl.data(), nt * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dso, sorted.data(), c.nages * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dmh, cfg->h_MH, nt * 8, cudaMemcpyHostToDevice);
        cudaMemcpy(dta, tage.data(), c.nages * 8, cudaMemcpyHostToDevice);
        cudaMemcpy(duni, uni.data(), c.nages * 4, cudaMemcpyHostToDevice);
        h.z.uni = duni;
        h.z.tage = dta;
        h.z.nt = nt;
        h.z.nages = c.nages;
        h.z.jidx = dj;
        h.z.age_off = dao;
        h.z.age_tmpl = dat;
        h.z.sorted = dso;
        h.z.MH = dmh;
    }
    for (void *p : owned)
        if (!p) return sfh_set_error(ctx, SFH_ERR_NOMEM, "HMC buffers");
    if (!batched) return SFH_OK;
    int rc;
    if (c.B == 1 && sfh_onepass_eligible(ctx, m)) {
        // one chain: the plain single-vector path (no batch to fill the tensor cores)
        h.single = true;
        h.d_data = d_data;
        h.d_Gd = (double *)alloc((size_t)nt * 8);
        h.d_comp = (double *)alloc((size_t)m->nbins * 8);
        if (!h.d_Gd || !h.d_comp) return sfh_set_error(ctx, SFH_ERR_NOMEM, "HMC buffers");
        return sfh_scratch_reserve(ctx, sfh_onepass_scratch(ctx, m));
    }
    // the occupied-bin plan's derived handle (the diagram is fixed for the whole run: its
    // counts are gathered and checked once here)
    const sfh_models *mb = m;
    const double *db = d_data;
    SfhOccPlan *occ = nullptr;
    if ((rc = sfh_occ_batched(ctx, const_cast<sfh_models *>(m), d_data, true, &mb, &db, &occ)))
        return rc;
    if (occ) {
        SFH_CK(ctx, cudaStreamSynchronize(ctx->stream));
        if (*occ->h_bviol) {
            sfh_occ_retire(occ);
            mb = m;
            db = d_data;
        }
    }
    h.mb = mb;
    if ((rc = sfh_batched_prepare(ctx, mb, c.B, db, nullptr, 0, &h.plan))) return rc;
    if ((rc = sfh_scratch_reserve(ctx, h.plan.scratch_bytes))) return rc;
    return sfh_batched_prepare(ctx, mb, c.B, db, ctx->scratch, ctx->scratch_bytes, &h.plan);
}

void free_run(sfh_ctx *ctx, std::vector<void *> &owned) {
    cudaStreamSynchronize(ctx->stream);
    for (void *p : owned) cudaFree(p);
    owned.clear();
}


// ---------------------------------------------------------------- NUTS
// No-U-Turn sampler with multinomial sampling (DynamicHMC's NUTS, the sampler of
// hmc_sample.jl:105-141 and sample_sfh): every chain runs its own trajectory state machine
// and advances by one leapfrog step per batched evaluation, so chains whose trees stop
// early start their next trajectory at once and no evaluation is wasted on a finished
// tree.  Per trajectory: momentum p0 ~ N(0, M), trees doubled in a random direction until
// the generalized no-U-turn criterion (p♯ = M⁻¹ p at either end against the momentum sum
// ρ: turning when p♯₋·ρ < 0 or p♯₊·ρ < 0) holds for the whole tree or for any subtree,
// the energy error exceeds 1000 (divergence), or the depth reaches max_depth.  States
// are weighted by exp(H0 - H): uniform progressive sampling inside a new subtree, biased
// progressive sampling when it joins the tree (Betancourt 2017).  Subtree checks run
// iteratively from O(max_depth) checkpoints of momenta and cumulative sums (the leaf
// index's bits name the subtrees a leaf closes).  Warmup: per-chain dual averaging of
// the step on the mean acceptance statistic of each tree (Hoffman & Gelman 2014), and a
// per-chain diagonal metric from the variance of the chain's own draws over the middle
// 70 % of warmup.
constexpr int kNutsMaxDepth = 12;
constexpr int kNutsMaxDense = 256;  // largest D for a dense metric
enum { NUTS_FRESH = 0, NUTS_RUN = 1 };

struct NutsState {
    double *thL, *pL, *gL, *sL, *thR, *pR, *gR, *sR;  // B x D trajectory ends (s: p♯ = M⁻¹ p)
    double *ths, *gs, *thu, *gu;            // B x D proposals: tree, subtree
    double *rho, *rhos;                     // B x D momentum sums: tree, subtree
    double *ckp, *ckr, *cks;                // B x maxdepth x D checkpoints: p, Σ p, p♯
    double *minv, *wm, *wm2;                // B x D diagonal metric and its Welford window
    double *q;                              // B x D scratch: M⁻¹ x, or the momentum draws
    const double *Md;                       // D x D dense M⁻¹ (row-major) or NULL: diagonal
    const double *Lt;                       // D x D: M⁻¹ = L Lᵀ, Lt = L⁻ᵀ (p = Lt z)
    double *logds, *logdu, *H0, *logW, *logWs, *accsum, *depth_sum;  // B
    int *depth, *dir, *leaf, *status, *nleaf, *ndiv, *div_now;       // B
    int64_t *tb, *tick, *nwin;              // B
    unsigned int *done;                     // chains that have all their draws
    int maxdepth;
};

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double logaddexp(double a, double b) {
    const double m = fmax(a, b);
    return m == -INFINITY ? -INFINITY : m + log(exp(a - m) + exp(b - m));
}
__device__ __forceinline__ double nuts_u01(const HmcConst &c, int b, int64_t tick, uint32_t stream) {
    const u4 r = philox(u4{0xFFFFFF00u + stream, (uint32_t)b, (uint32_t)tick, (uint32_t)(tick >> 32)},
                        (uint32_t)c.seed, (uint32_t)(c.seed >> 32));
    return u01(r.x, r.y);
}

// out = M⁻¹ x for chain b (a warp: lane l owns entries l, l + 32, ...; x is complete in
// memory before the call, out is complete after it).
__device__ __forceinline__ void nuts_sharp(const NutsState &n, int b, int D, const double *x,
                                           double *out, int lane) {
    __syncwarp();
    if (n.Md) {
        for (int d = lane; d < D; d += 32) {
            const double *row = n.Md + (int64_t)d * D;
            double a = 0.0;
            for (int j = 0; j < D; ++j) a = fma(row[j], x[j], a);
            out[d] = a;
        }
    } else {
        const double *mi = n.minv + (int64_t)b * D;
        for (int d = lane; d < D; d += 32) out[d] = mi[d] * x[d];
    }
    __syncwarp();
}

// One leapfrog step of chain b (warp) from the state in (th, p, g) in direction v: half
// kick, drift by M⁻¹ p; the evaluation supplies g at the new θ and the next tick the
// second kick.
__device__ __forceinline__ void nuts_leap(const NutsState &n, int b, double *th, double *p,
                                          const double *g, int D, double e, int v, int lane) {
    double *q = n.q + (int64_t)b * D;
    for (int d = lane; d < D; d += 32) p[d] += v * 0.5 * e * g[d];
    nuts_sharp(n, b, D, p, q, lane);
    for (int d = lane; d < D; d += 32) th[d] += v * e * q[d];
}

__device__ void nuts_start(ChainState &s, NutsState &n, const HmcConst &c, int b, int lane) {
    const int D = c.D;
    double *th = s.theta + (int64_t)b * D, *p = s.p + (int64_t)b * D, *g = s.g + (int64_t)b * D;
    double *q = n.q + (int64_t)b * D;
    const int64_t t = n.tb[b];
    // p ~ N(0, M): p = L⁻ᵀ z for a dense M⁻¹ = L Lᵀ, z / sqrt(minv) for a diagonal one;
    // either way ½ pᵀ M⁻¹ p = ½ |z|²
    double kin = 0.0;
    for (int d = lane; d < D; d += 32) {
        const double z = normal(c.seed, (uint32_t)d, (uint32_t)b, (uint32_t)t, 3u);
        q[d] = z;
        kin += 0.5 * z * z;
    }
    kin = warp_sum_d(kin);
    __syncwarp();
    if (n.Lt) {
        for (int d = lane; d < D; d += 32) {
            const double *row = n.Lt + (int64_t)d * D;
            double a = 0.0;
            for (int j = 0; j < D; ++j) a = fma(row[j], q[j], a);
            p[d] = a;
        }
    } else {
        const double *mi = n.minv + (int64_t)b * D;
        for (int d = lane; d < D; d += 32) p[d] = q[d] / sqrt(mi[d]);
    }
    nuts_sharp(n, b, D, p, q, lane);  // p♯ of the starting state
    for (int d = lane; d < D; d += 32) {
        const int64_t k = (int64_t)b * D + d;
        n.thL[k] = n.thR[k] = n.ths[k] = th[d];
        n.gL[k] = n.gR[k] = n.gs[k] = g[d];
        n.pL[k] = n.pR[k] = n.rho[k] = p[d];
        n.sL[k] = n.sR[k] = q[d];
    }
    const int64_t tk = n.tick[b];
    const int v = nuts_u01(c, b, tk, 0) < 0.5 ? -1 : 1;
    if (lane == 0) {
        n.H0[b] = -s.logd[b] + kin;
        n.logds[b] = s.logd[b];
        n.logW[b] = 0.0;
        n.depth[b] = 0;
        n.dir[b] = v;
        n.leaf[b] = 0;
        n.accsum[b] = 0.0;
        n.nleaf[b] = 0;
        n.div_now[b] = 0;
        n.status[b] = NUTS_RUN;
    }
    nuts_leap(n, b, th, p, g, D, s.eps[b], v, lane);
}

// The tree is finished: record its proposal, adapt during warmup, start the next tree.
__device__ void nuts_finish(ChainState &s, NutsState &n, const HmcConst &c, int b, int lane) {
    const int D = c.D;
    const int64_t t = n.tb[b];
    const double a = n.nleaf[b] > 0 ? n.accsum[b] / n.nleaf[b] : 0.0;
    double *th = s.theta + (int64_t)b * D, *g = s.g + (int64_t)b * D;
    for (int d = lane; d < D; d += 32) {  // the proposal becomes the chain's state
        const int64_t k = (int64_t)b * D + d;
        th[d] = n.ths[k];
        g[d] = n.gs[k];
    }
    const int64_t w0 = (int64_t)(0.15 * c.nwarm), w1 = (int64_t)(0.85 * c.nwarm);
    if (t < c.nwarm) {
        if (lane == 0) {
            dual_average(s.da + 4 * b, s.eps + b, a, c.target);
            if (t == c.nwarm - 1) s.eps[b] = exp(s.da[4 * b + 2]);
        }
        // the metric window (a diagonal metric only; a dense one is given and kept)
        if (!n.Md && t >= w0 && t < w1 && c.nwarm >= 20) {
            const double m1 = (double)(n.nwin[b] + 1);
            for (int d = lane; d < D; d += 32) {
                const int64_t k = (int64_t)b * D + d;
                const double x = th[d], dl = x - n.wm[k];
                n.wm[k] += dl / m1;
                n.wm2[k] += dl * (x - n.wm[k]);
            }
            __syncwarp();
            if (lane == 0) n.nwin[b] += 1;
            if (t == w1 - 1) {  // the diagonal metric from the window, regularised
                const double nw = m1;
                for (int d = lane; d < D; d += 32) {
                    const int64_t k = (int64_t)b * D + d;
                    const double var = nw > 1.0 ? n.wm2[k] / (nw - 1.0) : 1.0;
                    n.minv[k] = (nw / (nw + 5.0)) * var + 1e-3 * (5.0 / (nw + 5.0));
                }
                if (lane == 0) {  // restart the step adaptation around the current step
                    double *da = s.da + 4 * b;
                    da[0] = log(10.0 * s.eps[b]);
                    da[1] = da[2] = da[3] = 0.0;
                }
            }
        }
    } else if (t < c.nwarm + c.nsamp) {
        const int64_t ts = t - c.nwarm;
        for (int d = lane; d < D; d += 32) {
            const int64_t k = (int64_t)b * D + d;
            const double x = nat_param(c, th, d);
            const double n1 = (double)(ts + 1);
            const double delta = x - s.mean[k];
            s.mean[k] += delta / n1;
            s.m2[k] += delta * (x - s.mean[k]);
            if (s.draws && c.thin > 0 && ts % c.thin == 0 && ts / c.thin < c.ndraws)
                s.draws[((int64_t)b * c.ndraws + ts / c.thin) * D + d] = (float)x;
        }
        if (lane == 0) {
            s.acc_sum[b] += a;
            n.depth_sum[b] += n.depth[b];
            n.ndiv[b] += n.div_now[b];
        }
    }
    if (lane == 0) {
        s.logd[b] = n.logds[b];
        n.tb[b] = t + 1;
        if (t + 1 == c.nwarm + c.nsamp) atomicAdd(n.done, 1u);
    }
    __syncwarp();
    nuts_start(s, n, c, b, lane);
}

// One tick per chain (a warp each): the second half kick of the step just evaluated, the
// tree bookkeeping, and the next leapfrog step (whose position the next evaluation takes).
__global__ void k_nuts_tick(ChainState s, NutsState n, HmcConst c) {
    const int b = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (b >= c.B) return;
    const int D = c.D;
    if (n.status[b] == NUTS_FRESH) {  // the starting point was evaluated
        nuts_start(s, n, c, b, lane);
        if (lane == 0) n.tick[b] += 1;
        return;
    }
    double *th = s.theta + (int64_t)b * D, *p = s.p + (int64_t)b * D, *g = s.g + (int64_t)b * D;
    double *q = n.q + (int64_t)b * D;
    const double e = s.eps[b];
    const int v = n.dir[b], j = n.depth[b], leaf = n.leaf[b];
    const int64_t tk = n.tick[b];
    for (int d = lane; d < D; d += 32) p[d] += v * 0.5 * e * g[d];
    nuts_sharp(n, b, D, p, q, lane);  // p♯ of the new state
    double kin = 0.0;
    for (int d = lane; d < D; d += 32) kin += 0.5 * p[d] * q[d];
    kin = warp_sum_d(kin);
    const double logd = s.logd[b];
    const double delta = n.H0[b] - (-logd + kin);  // log weight of the new state
    const bool divergent = !(delta >= -1000.0);     // NaN counts as divergent
    if (lane == 0) {
        n.accsum[b] += divergent ? 0.0 : exp(fmin(0.0, delta));
        n.nleaf[b] += 1;
        n.tick[b] = tk + 1;
    }
    if (divergent) {
        if (lane == 0) n.div_now[b] = 1;
        __syncwarp();
        nuts_finish(s, n, c, b, lane);
        return;
    }
    // the subtree: progressive (uniform) sampling and the momentum sum
    const int64_t base = (int64_t)b * D;
    bool take;
    double lws;
    if (leaf == 0) {
        lws = delta;
        take = true;
    } else {
        lws = logaddexp(n.logWs[b], delta);
        take = nuts_u01(c, b, tk, 1) < exp(delta - lws);
    }
    for (int d = lane; d < D; d += 32) {
        const int64_t k = base + d;
        n.rhos[k] = (leaf == 0 ? 0.0 : n.rhos[k]) + p[d];
        if (take) {
            n.thu[k] = th[d];
            n.gu[k] = g[d];
        }
    }
    if (lane == 0) {
        n.logWs[b] = lws;
        if (take) n.logdu[b] = logd;
    }
    // checkpoints and the subtrees this leaf closes
    const int64_t ck = (int64_t)b * n.maxdepth * D;
    const int imax = __popc((unsigned)leaf >> 1);
    bool turning = false;
    if ((leaf & 1) == 0) {
        for (int d = lane; d < D; d += 32) {
            n.ckp[ck + (int64_t)imax * D + d] = p[d];
            n.ckr[ck + (int64_t)imax * D + d] = n.rhos[base + d];
            n.cks[ck + (int64_t)imax * D + d] = q[d];
        }
    } else {
        const int imin = imax - (__ffs(~(unsigned)leaf) - 1) + 1;  // trailing ones
        for (int i = imax; i >= imin && !turning; --i) {
            double a1 = 0.0, a2 = 0.0;
            for (int d = lane; d < D; d += 32) {
                const int64_t kc = ck + (int64_t)i * D + d;
                const double sr = n.rhos[base + d] - n.ckr[kc] + n.ckp[kc];
                a1 += n.cks[kc] * sr;
                a2 += q[d] * sr;
            }
            a1 = warp_sum_d(a1);
            a2 = warp_sum_d(a2);
            turning = a1 < 0.0 || a2 < 0.0;
        }
    }
    if (turning) {  // the subtree is dropped; the tree's proposal stands
        __syncwarp();
        nuts_finish(s, n, c, b, lane);
        return;
    }
    if (leaf + 1 < (1 << j)) {  // the subtree continues from this state
        if (lane == 0) n.leaf[b] = leaf + 1;
        nuts_leap(n, b, th, p, g, D, e, v, lane);
        return;
    }
    // the subtree is complete: join it (biased progressive sampling), check the whole tree
    const bool jump = nuts_u01(c, b, tk, 2) < exp(lws - n.logW[b]);
    double *eth = v > 0 ? n.thR : n.thL, *ep = v > 0 ? n.pR : n.pL, *eg = v > 0 ? n.gR : n.gL;
    double *es = v > 0 ? n.sR : n.sL;
    double t1 = 0.0, t2 = 0.0;
    for (int d = lane; d < D; d += 32) {
        const int64_t k = base + d;
        if (jump) {
            n.ths[k] = n.thu[k];
            n.gs[k] = n.gu[k];
        }
        eth[k] = th[d];
        ep[k] = p[d];
        eg[k] = g[d];
        es[k] = q[d];
        const double r = n.rho[k] + n.rhos[k];
        n.rho[k] = r;
        t1 += n.sL[k] * r;
        t2 += n.sR[k] * r;
    }
    t1 = warp_sum_d(t1);
    t2 = warp_sum_d(t2);
    if (lane == 0) {
        if (jump) n.logds[b] = n.logdu[b];
        n.logW[b] = logaddexp(n.logW[b], lws);
    }
    const int jn = j + 1;
    if (t1 < 0.0 || t2 < 0.0 || jn >= n.maxdepth) {
        if (lane == 0) n.depth[b] = jn;
        __syncwarp();
        nuts_finish(s, n, c, b, lane);
        return;
    }
    // double again from the end in a fresh direction
    const int vn = nuts_u01(c, b, tk, 3) < 0.5 ? -1 : 1;
    const double *sth = vn > 0 ? n.thR : n.thL, *sp = vn > 0 ? n.pR : n.pL, *sg = vn > 0 ? n.gR : n.gL;
    __syncwarp();
    for (int d = lane; d < D; d += 32) {
        th[d] = sth[base + d];
        p[d] = sp[base + d];
        g[d] = sg[base + d];
    }
    if (lane == 0) {
        n.depth[b] = jn;
        n.dir[b] = vn;
        n.leaf[b] = 0;
    }
    nuts_leap(n, b, th, p, g, D, e, vn, lane);
}

__global__ void k_nuts_init(NutsState n, HmcConst c, const double *minv0) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < (int64_t)c.B * c.D) {
        n.minv[k] = minv0 ? minv0[k % c.D] : 1.0;
        n.wm[k] = 0.0;
        n.wm2[k] = 0.0;
    }
    if (k < c.B) {
        n.status[k] = NUTS_FRESH;
        n.tb[k] = 0;
        n.tick[k] = 0;
        n.nwin[k] = 0;
        n.depth_sum[k] = 0.0;
        n.ndiv[k] = 0;
    }
}

__global__ void k_nuts_out(ChainState s, NutsState n, HmcConst c, double *depth, int64_t *ndiv) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < c.B) {
        if (depth) depth[k] = c.nsamp > 0 ? n.depth_sum[k] / (double)c.nsamp : 0.0;
        if (ndiv) ndiv[k] = n.ndiv[k];
    }
}

}  // namespace

extern "C" int sfh_logdensity_batched_dev(sfh_ctx *ctx, const sfh_models *m, const double *d_data,
                                          const sfh_hmc_config *cfg, const double *d_theta,
                                          double *d_logd, double *d_grad) {
    if (!ctx || !m || !d_data || !cfg || !d_theta || !d_logd || !d_grad) return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    HmcRun h{};
    std::vector<void *> owned;
    int rc = setup_run(ctx, m, d_data, cfg, nullptr, h, owned);
    if (!rc) {
        const int64_t BD = (int64_t)h.c.B * h.c.D;
        // evaluate into the run's state arrays, then copy out
        cudaMemcpyAsync(h.s.theta, d_theta, BD * 8, cudaMemcpyDeviceToDevice, ctx->stream);
        rc = launch_eval(ctx, m, h, true);
        if (!rc) rc = run_check(ctx, h);
        if (!rc) {
            cudaMemcpyAsync(d_logd, h.s.logd, (size_t)h.c.B * 8, cudaMemcpyDeviceToDevice, ctx->stream);
            cudaMemcpyAsync(d_grad, h.s.g, BD * 8, cudaMemcpyDeviceToDevice, ctx->stream);
        }
    }
    free_run(ctx, owned);
    return rc;
}

extern "C" int sfh_hmc_sample_dev(sfh_ctx *ctx, const sfh_models *m, const double *d_data,
                                  const sfh_hmc_config *cfg, const double *d_theta0,
                                  double *d_mean, double *d_var, double *d_accept,
                                  double *d_step, float *d_draws) {
    if (!ctx || !m || !d_data || !cfg || !d_theta0) return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    HmcRun h{};
    std::vector<void *> owned;
    auto cleanup = [&]() { free_run(ctx, owned); };
    int rc = setup_run(ctx, m, d_data, cfg, d_draws, h, owned);
    if (rc) { cleanup(); return rc; }
    HmcConst &c = h.c;
    ChainState &s = h.s;
    const int64_t BD = (int64_t)c.B * c.D;
    cudaStream_t st = ctx->stream;
    SFH_CK(ctx, cudaMemcpyAsync(s.theta, d_theta0, BD * 8, cudaMemcpyDeviceToDevice, st));
    k_init_state<<<(unsigned)((std::max(BD, (int64_t)std::max(c.B, c.D)) + kT - 1) / kT), kT, 0, st>>>(
        s, c, cfg->step0);
    SFH_LAUNCHED(ctx);
    if (cfg->d_minv0)  // a starting metric, e.g. the diagonal of a MAP fit's inverse Hessian
        SFH_CK(ctx, cudaMemcpyAsync(s.minv, cfg->d_minv0, (size_t)c.D * 8, cudaMemcpyDeviceToDevice, st));
    // gradient and log density at the starting points (eager: also warms every kernel)
    if ((rc = launch_eval(ctx, m, h, true))) { cleanup(); return rc; }
    if ((rc = run_check(ctx, h))) { cleanup(); return rc; }
    // capture one trajectory and replay it
    const int64_t ntot = c.nwarm + c.nsamp;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool use_graph = ntot > 1;
    if (use_graph) {
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) use_graph = false;
    }
    int64_t per_replay = 0;  // kernels in one replay (counted while capturing)
    if (use_graph) {
        const int64_t l0 = ctx->launches;
        ctx->internal_capture = true;  // the graph lives only inside this call
        rc = launch_trajectory(ctx, m, h);
        ctx->internal_capture = false;
        per_replay = ctx->launches - l0;
        ctx->launches = l0;
        cudaError_t e = cudaStreamEndCapture(st, &graph);
        if (rc || e != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            use_graph = false;
            exec = nullptr;
        }
    }
    for (int64_t t = 0; t < ntot; ++t) {
        if (use_graph) {
            if (cudaGraphLaunch(exec, st) != cudaSuccess) { rc = sfh_cuda_error(ctx, cudaGetLastError(), "graph launch"); break; }
            ctx->launches += per_replay;
        } else if ((rc = launch_trajectory(ctx, m, h))) {
            break;
        }
        if ((t & 63) == 63 && (rc = run_check(ctx, h))) break;
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (!rc) rc = run_check(ctx, h);
    if (!rc) {
        k_finish<<<(unsigned)((std::max(BD, (int64_t)c.B) + kT - 1) / kT), kT, 0, st>>>(
            s, c, d_mean, d_var, d_accept, d_step);
        cudaGetLastError();
    }
    cleanup();
    return rc;
}

extern "C" int sfh_nuts_sample_dev(sfh_ctx *ctx, const sfh_models *m, const double *d_data,
                                   const sfh_hmc_config *cfg, int max_depth,
                                   const double *d_minv_dense, const double *d_theta0,
                                   double *d_mean, double *d_var, double *d_accept,
                                   double *d_step, double *d_depth, int64_t *d_ndiv,
                                   float *d_draws) {
    if (!ctx || !m || !d_data || !cfg || !d_theta0) return SFH_ERR_ARG;
    if (max_depth < 1 || max_depth > kNutsMaxDepth)
        return sfh_set_error(ctx, SFH_ERR_ARG, "max_depth must be in 1..12");
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    HmcRun h{};
    std::vector<void *> owned;
    auto cleanup = [&]() { free_run(ctx, owned); };
    int rc = setup_run(ctx, m, d_data, cfg, d_draws, h, owned);
    if (rc) { cleanup(); return rc; }
    HmcConst &c = h.c;
    ChainState &s = h.s;
    const int64_t BD = (int64_t)c.B * c.D;
    cudaStream_t st = ctx->stream;
    NutsState n{};
    n.maxdepth = max_depth;
    if (d_minv_dense) {
        // a dense metric M⁻¹ (the reference's sample_sfh passes the MAP inverse Hessian,
        // generic_fitting.jl:484-490): its Cholesky factor L and Lt = L⁻ᵀ for the momenta
        const int D = c.D;
        if (D > kNutsMaxDense) {
            cleanup();
            return sfh_set_error(ctx, SFH_ERR_ARG, "a dense metric needs D <= 256");
        }
        std::vector<double> Mi((size_t)D * D), L((size_t)D * D, 0.0), Lt((size_t)D * D, 0.0);
        if (cudaMemcpy(Mi.data(), d_minv_dense, Mi.size() * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
            cleanup();
            return sfh_cuda_error(ctx, cudaGetLastError(), "dense metric copy");
        }
        for (int i = 0; i < D; ++i)
            for (int k = 0; k <= i; ++k) {
                double a = 0.5 * (Mi[(size_t)i * D + k] + Mi[(size_t)k * D + i]);
                for (int q = 0; q < k; ++q) a -= L[(size_t)i * D + q] * L[(size_t)k * D + q];
                if (i == k) {
                    if (!(a > 0.0)) {
                        cleanup();
                        return sfh_set_error(ctx, SFH_ERR_ARG, "the dense metric is not positive definite");
                    }
                    L[(size_t)i * D + i] = std::sqrt(a);
                } else {
                    L[(size_t)i * D + k] = a / L[(size_t)k * D + k];
                }
            }
        // X = L⁻¹ by forward substitution, then Lt = Xᵀ
        std::vector<double> X((size_t)D * D, 0.0);
        for (int col = 0; col < D; ++col)
            for (int i = col; i < D; ++i) {
                double a = i == col ? 1.0 : 0.0;
                for (int q = col; q < i; ++q) a -= L[(size_t)i * D + q] * X[(size_t)q * D + col];
                X[(size_t)i * D + col] = a / L[(size_t)i * D + i];
            }
        for (int i = 0; i < D; ++i)
            for (int k = 0; k < D; ++k) Lt[(size_t)i * D + k] = X[(size_t)k * D + i];
        // the symmetrised metric and Lt in one allocation
        double *dm = nullptr;
        if (cudaMalloc(&dm, Mi.size() * 16) != cudaSuccess) {
            cleanup();
            return sfh_set_error(ctx, SFH_ERR_NOMEM, "dense metric");
        }
        owned.push_back(dm);
        for (int i = 0; i < D; ++i)
            for (int k = 0; k < i; ++k)
                Mi[(size_t)i * D + k] = Mi[(size_t)k * D + i] =
                    0.5 * (Mi[(size_t)i * D + k] + Mi[(size_t)k * D + i]);
        if (cudaMemcpy(dm, Mi.data(), Mi.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dm + Mi.size(), Lt.data(), Lt.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
            cleanup();
            return sfh_cuda_error(ctx, cudaGetLastError(), "dense metric upload");
        }
        n.Md = dm;
        n.Lt = dm + Mi.size();
    }
    {
        double **vec[] = {&n.thL, &n.pL, &n.gL, &n.sL, &n.thR, &n.pR, &n.gR, &n.sR, &n.ths, &n.gs,
                          &n.thu, &n.gu, &n.rho, &n.rhos, &n.minv, &n.wm, &n.wm2, &n.q};
        double **sca[] = {&n.logds, &n.logdu, &n.H0, &n.logW, &n.logWs, &n.accsum, &n.depth_sum};
        int **isc[] = {&n.depth, &n.dir, &n.leaf, &n.status, &n.nleaf, &n.ndiv, &n.div_now};
        int64_t **lsc[] = {&n.tb, &n.tick, &n.nwin};
        auto get = [&](size_t bytes) -> void * {
            void *q = nullptr;
            if (cudaMalloc(&q, bytes) != cudaSuccess) return nullptr;
            owned.push_back(q);
            return q;
        };
        bool ok = true;
        for (auto v : vec) ok = ok && (*v = (double *)get((size_t)BD * 8));
        for (auto v : sca) ok = ok && (*v = (double *)get((size_t)c.B * 8));
        for (auto v : isc) ok = ok && (*v = (int *)get((size_t)c.B * 4));
        for (auto v : lsc) ok = ok && (*v = (int64_t *)get((size_t)c.B * 8));
        ok = ok && (n.ckp = (double *)get((size_t)BD * max_depth * 8));
        ok = ok && (n.ckr = (double *)get((size_t)BD * max_depth * 8));
        ok = ok && (n.cks = (double *)get((size_t)BD * max_depth * 8));
        if (!ok) {
            cleanup();
            return sfh_set_error(ctx, SFH_ERR_NOMEM, "NUTS state");
        }
    }
    unsigned int *h_done = nullptr, *d_done = nullptr;
    if (cudaHostAlloc((void **)&h_done, sizeof(unsigned int), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer((void **)&d_done, h_done, 0) != cudaSuccess) {
        if (h_done) cudaFreeHost(h_done);
        cleanup();
        return sfh_set_error(ctx, SFH_ERR_NOMEM, "NUTS completion flag");
    }
    *(volatile unsigned int *)h_done = 0u;
    n.done = d_done;
    auto done_call = [&](int r) {
        cudaStreamSynchronize(st);
        cudaFreeHost(h_done);
        cleanup();
        return r;
    };
    if (cudaMemcpyAsync(s.theta, d_theta0, BD * 8, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return done_call(sfh_cuda_error(ctx, cudaGetLastError(), "theta0 copy"));
    k_init_state<<<(unsigned)((std::max(BD, (int64_t)std::max(c.B, c.D)) + kT - 1) / kT), kT, 0, st>>>(
        s, c, cfg->step0);
    ctx->launches++;
    k_nuts_init<<<(unsigned)((std::max(BD, (int64_t)c.B) + kT - 1) / kT), kT, 0, st>>>(n, c, cfg->d_minv0);
    ctx->launches++;
    if ((rc = launch_eval(ctx, m, h, true))) return done_call(rc);
    if ((rc = run_check(ctx, h))) return done_call(rc);
    // K ticks per replay of a captured graph: a tick is the tree bookkeeping of every chain
    // and one batched evaluation at the positions it produced
    const int K = 16;
    const unsigned tb_grid = (unsigned)(((int64_t)c.B * 32 + kT - 1) / kT);
    auto tick = [&]() -> int {
        k_nuts_tick<<<tb_grid, kT, 0, st>>>(s, n, c);
        SFH_LAUNCHED(ctx);
        return launch_eval(ctx, m, h, true);
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t per_replay = 0;
    bool use_graph = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (use_graph) {
        const int64_t l0 = ctx->launches;
        ctx->internal_capture = true;
        for (int k = 0; k < K && !rc; ++k) rc = tick();
        ctx->internal_capture = false;
        cudaError_t e = cudaStreamEndCapture(st, &graph);
        per_replay = ctx->launches - l0;
        ctx->launches = l0;
        if (rc || e != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            graph = nullptr;
            exec = nullptr;
            cudaGetLastError();
            use_graph = false;
            rc = SFH_OK;
        }
    }
    // every chain needs nwarm + nsamp trees of at most 2^max_depth states each
    const int64_t ntot = c.nwarm + c.nsamp;
    const int64_t max_ticks = (ntot + 1) * ((int64_t)1 << max_depth) + 2 * K;
    for (int64_t t = 0; t < max_ticks && rc == SFH_OK; t += K) {
        if (use_graph) {
            if (cudaGraphLaunch(exec, st) != cudaSuccess) {
                rc = sfh_cuda_error(ctx, cudaGetLastError(), "graph launch");
                break;
            }
            ctx->launches += per_replay;
        } else {
            for (int k = 0; k < K && !rc; ++k) rc = tick();
            if (rc) break;
        }
        if ((t / K) % 8 == 7) {  // completion is read from mapped memory after a sync
            if ((rc = run_check(ctx, h))) break;
            if (*(volatile unsigned int *)h_done >= (unsigned)c.B) break;
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (!rc) rc = run_check(ctx, h);
    if (!rc && *(volatile unsigned int *)h_done < (unsigned)c.B)
        rc = sfh_set_error(ctx, SFH_ERR_TIMEOUT, "NUTS: chains did not finish within the tick bound");
    if (!rc) {
        k_finish<<<(unsigned)((std::max(BD, (int64_t)c.B) + kT - 1) / kT), kT, 0, st>>>(
            s, c, d_mean, d_var, d_accept, d_step);
        k_nuts_out<<<(unsigned)((c.B + kT - 1) / kT), kT, 0, st>>>(s, n, c, d_depth, d_ndiv);
        ctx->launches += 2;
        cudaGetLastError();
    }
    return done_call(rc);
}

// ---------------------------------------------------------------- device fit_sfh objective
namespace {
// f = -log p and ∇f = -∇ log p for the BFGS loop, from the model's log density.
__global__ void k_hier_out(const double *__restrict__ g, const double *__restrict__ logd, int D,
                           double *__restrict__ grad, double *__restrict__ f) {
    for (int k = threadIdx.x; k < D; k += blockDim.x) grad[k] = -g[k];
    if (threadIdx.x == 0) *f = -*logd;
}
}  // namespace

extern "C" int sfh_fit_sfh_dev(sfh_ctx *ctx, sfh_models *m, const double *d_data,
                               const sfh_hmc_config *cfg, const double *d_theta0, int map,
                               const sfh_fit_options *opt, double *d_theta_out, double *d_invH,
                               sfh_fit_result *res) {
    if (!ctx || !m || !d_data || !cfg || !d_theta0 || !opt || !d_theta_out || !res)
        return SFH_ERR_ARG;
    if (cfg->model != SFH_HMC_MZR && cfg->model != SFH_HMC_LINEAR_AMR &&
        cfg->model != SFH_HMC_LOG_AMR)
        return sfh_set_error(ctx, SFH_ERR_ARG, "fit_sfh needs a metallicity model");
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    HmcRun h{};
    std::vector<void *> owned;
    int rc = setup_run(ctx, m, d_data, cfg, nullptr, h, owned, false);
    if (rc) { free_run(ctx, owned); return rc; }
    h.c.jac = map ? 1 : 0;  // MAP: Jacobian terms of the transforms; MLE: logL only
    const HmcConst c = h.c;
    const MzrDev z = h.z;
    double *comp = nullptr, *Gr = nullptr, *gth = nullptr, *logd = nullptr;
    {
        void *p[4] = {nullptr, nullptr, nullptr, nullptr};
        const size_t bytes[4] = {(size_t)m->nbins * 8, (size_t)m->nt * 8, (size_t)c.D * 8, 8};
        for (int k = 0; k < 4; ++k) {
            if (cudaMalloc(&p[k], bytes[k]) != cudaSuccess) {
                free_run(ctx, owned);
                for (int q = 0; q < k; ++q) cudaFree(p[q]);
                return sfh_set_error(ctx, SFH_ERR_NOMEM, "fit_sfh buffers");
            }
            owned.push_back(p[k]);
        }
        comp = (double *)p[0];
        Gr = (double *)p[1];
        gth = (double *)p[2];
        logd = (double *)p[3];
    }
    double *r = h.d_r, *negL = h.d_negL;
    const size_t sm = (size_t)(c.nages * 10 + 3) * sizeof(double);
    if (sm > 48 * 1024)
        SFH_CK(ctx, cudaFuncSetAttribute(k_mzr_grad<double>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    cudaStream_t st = ctx->stream;
    FgArgs a{};
    a.data = d_data;
    a.composite = comp;
    a.coeffs = r;
    a.G = Gr;
    a.negLogL = negL;
    a.eps = opt->eps > 0.0 ? opt->eps : 2.220446049250313e-16;
    a.gsign = 1.0;
    a.mode = FG_MODE_FG;
    // θt -> r = calculate_coeffs (mzr.jl:50-79, amr.jl:50-72) -> fg!(r) -> chain rule
    // (mzr.jl:131-209, amr.jl:122-157) -> f = -log p, ∇f (generic_fitting.jl:90-199)
    SfhFitObjective obj = [&](const double *theta_t, double *, double *grad, double *f,
                              const int *skip) -> int {
        k_mzr_map<<<1, kT, 0, st>>>(theta_t, c, z, r);
        SFH_LAUNCHED(ctx);
        FgArgs b = a;
        b.skip = skip;
        int r2 = sfh_launch_fg(ctx, m, b);
        if (r2) return r2;
        k_mzr_grad<double><<<1, 64, sm, st>>>(theta_t, r, Gr, negL, c, z, gth, logd, 1);
        SFH_LAUNCHED(ctx);
        k_hier_out<<<1, 64, 0, st>>>(gth, logd, c.D, grad, f);
        SFH_LAUNCHED(ctx);
        return SFH_OK;
    };
    rc = sfh_bfgs_run(ctx, c.D, d_theta0, opt, SFH_FIT_OBJECTIVE, obj, d_theta_out, d_invH, res);
    free_run(ctx, owned);
    return rc;
}
