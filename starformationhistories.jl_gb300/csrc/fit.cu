// fit.cu -- device BFGS driver for fit_templates (src/fitting/solvers.jl:172-221) and
// fit_templates_fast (:238-275).
//
// The reference minimises fg! with Optim.BFGS (inverse-Hessian BFGS, H0 = I, update skipped
// when sᵀy <= 0, alphaguess InitialStatic(1.0, scaled=true): the first trial step of each
// line search is min(1, |d|) / |d|, line search HagerZhang) over a transformed vector θ:
//   log MAP: r = exp(θ), f = fg!(r) - Σθ, g = G r - 1   (:180-187)
//   log MLE: r = exp(θ), f = fg!(r),      g = G r       (:188-194)
//   sqrt:    r = θ²,     f = fg!(r),      g = 2 θ G     (:257-263)
// Here the whole optimisation stays on the GPU.  One evaluation slot is five launches on the
// context stream:
//   k_fit_trial   (1 CTA)  new direction bookkeeping, θt = θ + α d, r = transform(θt)
//   fg!                    the single-vector kernel (one-pass for FP32 storage)
//   k_fit_eval    (1 CTA)  transformed f, g; line-search test; accept (s, y) or backtrack
//   k_fit_hgemv   (grid)   H y and H g, one warp per row, after an accepted step
//   k_fit_hupdate (grid)   rank-two BFGS update of H and the next direction d = -H g
// The host captures a few slots into a CUDA graph and replays it, reading the state back
// once per replay; a finished state turns the queued slots into no-ops (the fg! kernel
// reads the same flag).  The line search accepts a trial step on sufficient decrease (or
// Hager-Zhang's approximate Wolfe conditions) together with the curvature condition; a
// step that decreases f while the slope is still steep is kept and the step expanded
// (secant of φ', 2x to 10x), and a failed step backtracks (secant / quadratic
// interpolation) or falls back to the kept point.  It is not HagerZhang's bracketing, so
// the iterates differ from the reference's while the optimum they converge to does not.
#include <algorithm>
#include <cmath>

#include "sfh_internal.cuh"

namespace {

constexpr int kVecThreads = 1024;
constexpr int kRowWarps = 8;
constexpr int kMaxBacktracks = 40;
constexpr int kMaxExpand = 10;
constexpr double kArmijo = 1e-4;
constexpr double kApproxEps = 1e-6, kSigma = 0.9, kDelta = 0.1;
// transform value of a general objective: it writes f(θt) to negLogL and ∇f(θt) to Graw
constexpr int kFitObjective = SFH_FIT_OBJECTIVE;

struct FitState {
    double f, f_prev, dg0, alpha, gnorm, xchange;
    double f_b, alpha_b;  // the last trial point that passed the decrease test while steep
    int64_t evals, iter;
    int backtracks, expansions, best_valid, status, done, first, accept, reset_h, newdir, skip;
};

struct FitVecs {
    double *theta, *g, *d, *theta_t, *r, *Graw, *s, *y, *Hy, *Hg, *negLogL, *theta_b, *g_b;
    double *H;  // nt x nt, symmetric
    int64_t nt;
    int transform;
    int max_iter;
    double g_abstol, f_reltol, x_abstol;
};

__device__ __forceinline__ double nanmax(double a, double b) {
    return (a != a || b != b) ? __longlong_as_double(0x7ff8000000000000LL) : fmax(a, b);
}

// Sum (or NaN-propagating max) over the block; every thread gets the result.
template <bool MAX>
__device__ double block_reduce(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_xor_sync(0xffffffffu, v, o);
        v = MAX ? nanmax(v, u) : v + u;
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double t = l < nw ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_xor_sync(0xffffffffu, t, o);
        t = MAX ? nanmax(t, u) : t + u;
    }
    return t;
}

__device__ __forceinline__ double to_coeff(int transform, double th) {
    return transform == SFH_FIT_SQRT ? th * th : exp(th);
}

__global__ void k_fit_init(FitState *S, FitVecs V) {
    const int64_t nt = V.nt, total = nt * nt;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total;
         k += (int64_t)gridDim.x * blockDim.x)
        V.H[k] = (k / nt == k % nt) ? 1.0 : 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *S = FitState{};
        S->status = -1;
        S->first = 1;
    }
}

__global__ void __launch_bounds__(kVecThreads) k_fit_trial(FitState *S, FitVecs V) {
    __shared__ double sh[32];
    const int64_t nt = V.nt;
    if (S->done) {
        if (threadIdx.x == 0) S->skip = 1;
        return;
    }
    const int first = S->first, accept = S->accept, newdir = S->newdir;
    int reset = accept ? 0 : S->reset_h;  // an accepted step consumed the pending reset
    double alpha = S->alpha;
    __syncthreads();
    if (first) {
        for (int64_t i = threadIdx.x; i < nt; i += blockDim.x) V.theta_t[i] = V.theta[i];
    } else {
        if (newdir) {
            double dg = 0.0, dd = 0.0;
            for (int64_t i = threadIdx.x; i < nt; i += blockDim.x) {
                dg += V.g[i] * V.d[i];
                dd += V.d[i] * V.d[i];
            }
            dg = block_reduce<false>(dg, sh);
            dd = block_reduce<false>(dd, sh);
            if (!(dg < 0.0)) {  // not a descent direction: steepest descent, H restarts at I
                double gg = 0.0;
                for (int64_t i = threadIdx.x; i < nt; i += blockDim.x) {
                    V.d[i] = -V.g[i];
                    gg += V.g[i] * V.g[i];
                }
                gg = block_reduce<false>(gg, sh);
                dg = -gg;
                dd = gg;
                reset = 1;
            }
            const double nd = sqrt(dd);
            alpha = nd > 0.0 ? fmin(1.0, nd) / nd : 1.0;  // InitialStatic(1.0, scaled=true)
            if (threadIdx.x == 0) {
                S->dg0 = dg;
                S->backtracks = 0;
                S->expansions = 0;
                S->best_valid = 0;
            }
        }
        for (int64_t i = threadIdx.x; i < nt; i += blockDim.x)
            V.theta_t[i] = V.theta[i] + alpha * V.d[i];
    }
    if (V.transform != kFitObjective)  // a general objective maps θ itself
        for (int64_t i = threadIdx.x; i < nt; i += blockDim.x)
            V.r[i] = to_coeff(V.transform, V.theta_t[i]);
    if (threadIdx.x == 0) {
        S->alpha = alpha;
        S->newdir = 0;
        S->accept = 0;
        S->reset_h = reset;
        S->skip = 0;
        S->evals += 1;
    }
}

__global__ void __launch_bounds__(kVecThreads) k_fit_eval(FitState *S, FitVecs V) {
    __shared__ double sh[32];
    const int64_t nt = V.nt;
    if (S->done) return;
    const int first = S->first, nexp = S->expansions, have_best = S->best_valid;
    const double f0 = S->f, alpha = S->alpha, dg0 = S->dg0, f_b = S->f_b, alpha_b = S->alpha_b;
    __syncthreads();
    // transformed gradient at θt, in place of the raw one, and the slope φ'(α) = gtᵀd
    double sumth = 0.0, dgt = 0.0;
    for (int64_t i = threadIdx.x; i < nt; i += blockDim.x) {
        const double th = V.theta_t[i], G = V.Graw[i];
        double gt;
        if (V.transform == kFitObjective) {
            gt = G;  // the objective wrote the gradient of f in θ
        } else if (V.transform == SFH_FIT_SQRT) {
            gt = G * 2.0 * th;
        } else {
            gt = V.transform == SFH_FIT_LOG_MAP ? G * V.r[i] - 1.0 : G * V.r[i];
            sumth += th;
        }
        V.Graw[i] = gt;
        if (!first) dgt += gt * V.d[i];
    }
    if (V.transform == SFH_FIT_LOG_MAP) sumth = block_reduce<false>(sumth, sh);
    const double ft = *V.negLogL - (V.transform == SFH_FIT_LOG_MAP ? sumth : 0.0);
    bool use_best = false;
    if (!first) {
        dgt = block_reduce<false>(dgt, sh);
        const bool finite = fabs(ft) < INFINITY && fabs(dgt) < INFINITY;
        // sufficient decrease, or Hager-Zhang's approximate Wolfe conditions (slope reduced
        // to within [σ φ'(0), (2δ - 1) φ'(0)], σ = 0.9, δ = 0.1, and f at most ε |f| higher,
        // ε = 1e-6), which keep making progress where f differences fall below rounding
        const bool armijo = finite && ft <= f0 + kArmijo * alpha * dg0;
        const bool approx = finite && ft <= f0 + kApproxEps * fabs(f0) && dgt >= kSigma * dg0 &&
                            dgt <= (2.0 * kDelta - 1.0) * dg0;
        const bool ok = armijo || approx;
        if (ok && dgt < kSigma * dg0 && nexp < kMaxExpand) {
            // decrease but the slope is still steep (curvature condition fails): keep this
            // point and try further along d, as HagerZhang's bracketing expands
            for (int64_t i = threadIdx.x; i < nt; i += blockDim.x) {
                V.theta_b[i] = V.theta_t[i];
                V.g_b[i] = V.Graw[i];
            }
            if (threadIdx.x == 0) {
                double a = dgt > dg0 ? alpha * dg0 / (dg0 - dgt) : 4.0 * alpha;  // secant of φ'
                a = fmin(fmax(a, 2.0 * alpha), 10.0 * alpha);
                S->f_b = ft;
                S->alpha_b = alpha;
                S->best_valid = 1;
                S->expansions = nexp + 1;
                S->alpha = a;
            }
            return;
        }
        use_best = !ok && have_best;  // the expansion overshot: take the kept point
        if (!ok && !use_best) {
            if (threadIdx.x == 0) {
                const int bt = S->backtracks + 1;
                S->backtracks = bt;
                double a = 0.5 * alpha;
                if (finite) {
                    // root of the secant of φ' when the slope turned positive, else the
                    // minimiser of the quadratic through φ(0), φ'(0), φ(α)
                    const double q = dgt > 0.0
                                         ? alpha * dg0 / (dg0 - dgt)
                                         : -dg0 * alpha * alpha / (2.0 * (ft - f0 - dg0 * alpha));
                    a = fmin(fmax(q, 0.1 * alpha), 0.5 * alpha);
                    if (!(a == a)) a = 0.5 * alpha;
                }
                S->alpha = a;
                if (bt >= kMaxBacktracks) {
                    S->status = SFH_FIT_LINESEARCH;
                    S->done = 1;
                }
            }
            return;
        }
    }
    const double *th_src = use_best ? V.theta_b : V.theta_t;
    const double *g_src = use_best ? V.g_b : V.Graw;
    const double a_acc = use_best ? alpha_b : alpha, f_acc = use_best ? f_b : ft;
    double gmax = 0.0, smax = 0.0;
    for (int64_t i = threadIdx.x; i < nt; i += blockDim.x) {
        const double gt = g_src[i];
        if (first) {
            V.d[i] = -gt;
        } else {
            const double s = a_acc * V.d[i];
            V.s[i] = s;
            V.y[i] = gt - V.g[i];
            smax = nanmax(smax, fabs(s));
        }
        V.theta[i] = th_src[i];
        V.g[i] = gt;
        gmax = nanmax(gmax, fabs(gt));
    }
    gmax = block_reduce<true>(gmax, sh);
    smax = block_reduce<true>(smax, sh);
    if (threadIdx.x == 0) {
        S->f_prev = first ? f_acc : f0;
        S->f = f_acc;
        S->gnorm = gmax;
        S->xchange = smax;
        S->newdir = 1;
        S->first = 0;
        int status = -1;
        if (!(fabs(f_acc) < INFINITY) || !(gmax < INFINITY)) {
            status = SFH_FIT_NONFINITE;
        } else if (gmax <= V.g_abstol) {
            status = SFH_FIT_CONVERGED_G;
        } else if (!first) {
            if (fabs(f0 - f_acc) <= V.f_reltol * fabs(f_acc)) status = SFH_FIT_CONVERGED_F;
            else if (smax <= V.x_abstol) status = SFH_FIT_CONVERGED_X;
        }
        if (!first) S->iter += 1;
        if (status < 0 && S->iter >= V.max_iter) status = SFH_FIT_MAXITER;
        // the inverse Hessian takes the accepted step even when it is the last one
        S->accept = (!first && status != SFH_FIT_NONFINITE) ? 1 : 0;
        if (status >= 0) {
            S->status = status;
            S->done = 1;
        }
    }
}

// Hy = H y, Hg = H g (H as I while a reset is pending), one warp per row.
__global__ void __launch_bounds__(kRowWarps * 32) k_fit_hgemv(const FitState *S, FitVecs V) {
    if (!S->accept) return;
    const int64_t nt = V.nt;
    const int64_t i = (int64_t)blockIdx.x * kRowWarps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= nt) return;
    if (S->reset_h) {
        if (lane == 0) {
            V.Hy[i] = V.y[i];
            V.Hg[i] = V.g[i];
        }
        return;
    }
    const double *row = V.H + i * nt;
    double a = 0.0, b = 0.0;
    for (int64_t j = lane; j < nt; j += 32) {
        const double h = row[j];
        a = fma(h, V.y[j], a);
        b = fma(h, V.g[j], b);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
        V.Hy[i] = a;
        V.Hg[i] = b;
    }
}

// H += c1 s sᵀ - c2 (Hy sᵀ + s Hyᵀ) with c1 = (sᵀy + yᵀHy) / (sᵀy)², c2 = 1 / sᵀy when
// sᵀy > 0 (Optim's BFGS update_h!), and d = -H_new g from the same vectors.  Every CTA
// forms the four dot products in the same order, so all see the same scalars.
__global__ void __launch_bounds__(kRowWarps * 32) k_fit_hupdate(const FitState *S, FitVecs V) {
    __shared__ double sh[32];
    if (!S->accept) return;
    const int64_t nt = V.nt;
    const int reset = S->reset_h;
    double sty = 0.0, yhy = 0.0, sg = 0.0, hyg = 0.0;
    for (int64_t j = threadIdx.x; j < nt; j += blockDim.x) {
        const double s = V.s[j], hy = V.Hy[j], g = V.g[j];
        sty += s * V.y[j];
        yhy += V.y[j] * hy;
        sg += s * g;
        hyg += hy * g;
    }
    sty = block_reduce<false>(sty, sh);
    yhy = block_reduce<false>(yhy, sh);
    sg = block_reduce<false>(sg, sh);
    hyg = block_reduce<false>(hyg, sh);
    const bool upd = sty > 0.0 && sty < INFINITY && fabs(yhy) < INFINITY;
    const double c1 = upd ? (sty + yhy) / (sty * sty) : 0.0, c2 = upd ? 1.0 / sty : 0.0;
    const int64_t i = (int64_t)blockIdx.x * kRowWarps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= nt) return;
    const double si = V.s[i], hyi = V.Hy[i];
    double *row = V.H + i * nt;
    if (upd || reset) {
        for (int64_t j = lane; j < nt; j += 32) {
            const double base = reset ? (j == i ? 1.0 : 0.0) : row[j];
            row[j] = base + c1 * si * V.s[j] - c2 * (hyi * V.s[j] + si * V.Hy[j]);
        }
    }
    if (lane == 0) V.d[i] = -(V.Hg[i] + c1 * si * sg - c2 * (hyi * sg + si * hyg));
}

}  // namespace

// The BFGS loop over an objective: `objective` enqueues the evaluation at θt (nvar) on
// the context stream.  For the transforms of fit_templates it receives r = transform(θt)
// and writes fg!'s -logL and raw gradient; for kFitObjective it writes f(θt) and ∇f(θt).
// The slots are captured in a CUDA graph when the objective is capturable.
int sfh_bfgs_run(sfh_ctx *ctx, int64_t nvar, const double *d_theta0, const sfh_fit_options *opt,
                 int transform, const SfhFitObjective &objective, double *d_theta_out,
                 double *d_invH, sfh_fit_result *res) {
    if (opt->max_iter < 0 || !(opt->g_abstol >= 0.0) || !(opt->f_reltol >= 0.0) ||
        !(opt->x_abstol >= 0.0) || opt->max_evals < 0 || opt->graph_slots < 0 ||
        opt->graph_slots > 64 || !(opt->eps >= 0.0))
        return sfh_set_error(ctx, SFH_ERR_ARG, "invalid fit options");
    *res = sfh_fit_result{};
    const int64_t nt = nvar;
    const size_t vec = sfh_align256((size_t)nt * 8);
    const size_t o_state = 0, o_vecs = 256, o_H = o_vecs + 13 * vec, total = o_H + (size_t)nt * nt * 8;
    char *buf = nullptr;
    SFH_CK(ctx, cudaMalloc(&buf, total));
    FitState *S = (FitState *)(buf + o_state);
    double *v[13];
    for (int k = 0; k < 13; ++k) v[k] = (double *)(buf + o_vecs + k * vec);
    FitVecs V{v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10], v[11], v[12],
              (double *)(buf + o_H), nt, transform, opt->max_iter, opt->g_abstol,
              opt->f_reltol, opt->x_abstol};
    cudaStream_t st = ctx->stream;
    int rc = SFH_OK;
    const int64_t max_evals = opt->max_evals > 0 ? opt->max_evals : 50 * ((int64_t)opt->max_iter + 1);
    const int K = opt->graph_slots > 0 ? opt->graph_slots : 8;
    const int hgrid = (int)((nt + kRowWarps - 1) / kRowWarps);
    auto slot = [&]() -> int {
        k_fit_trial<<<1, kVecThreads, 0, st>>>(S, V);
        SFH_LAUNCHED(ctx);
        int r = objective(V.theta_t, V.r, V.Graw, V.negLogL, &S->skip);
        if (r) return r;
        k_fit_eval<<<1, kVecThreads, 0, st>>>(S, V);
        SFH_LAUNCHED(ctx);
        k_fit_hgemv<<<hgrid, kRowWarps * 32, 0, st>>>(S, V);
        SFH_LAUNCHED(ctx);
        k_fit_hupdate<<<hgrid, kRowWarps * 32, 0, st>>>(S, V);
        SFH_LAUNCHED(ctx);
        return SFH_OK;
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    FitState h{};
    do {
        if ((rc = sfh_host_stage_reserve(ctx, sizeof(FitState)))) break;
        if (cudaMemcpyAsync(V.theta, d_theta0, nt * 8, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
            rc = sfh_cuda_error(ctx, cudaGetLastError(), "theta0 copy");
            break;
        }
        const int64_t ih = std::min<int64_t>((nt * nt + 255) / 256, 8 * (int64_t)ctx->sm_count);
        k_fit_init<<<(unsigned)std::max<int64_t>(ih, 1), 256, 0, st>>>(S, V);
        const cudaError_t e0 = cudaGetLastError();
        if (e0 != cudaSuccess) {
            rc = sfh_cuda_error(ctx, e0, "k_fit_init");
            break;
        }
        ctx->launches++;
        // the first evaluation runs eagerly (it also prepares the objective's plans and scratch)
        if ((rc = slot())) break;
        bool use_graph = true;
        int64_t per_replay = 0;  // kernels in one replay of the captured slots
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) use_graph = false;
        if (use_graph) {
            int r = SFH_OK;
            const int64_t l0 = ctx->launches;
            ctx->internal_capture = true;  // the graph lives only inside this call
            for (int k = 0; k < K && !r; ++k) r = slot();
            ctx->internal_capture = false;
            cudaError_t e = cudaStreamEndCapture(st, &graph);
            per_replay = ctx->launches - l0;
            ctx->launches = l0;  // captured, not launched: counted per replay below
            if (r || e != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                graph = nullptr;
                exec = nullptr;
                cudaGetLastError();
                use_graph = false;
            }
        }
        res->graph = use_graph ? 1 : 0;
        for (;;) {
            if (cudaMemcpyAsync(ctx->h_stage, S, sizeof(FitState), cudaMemcpyDeviceToHost, st) !=
                    cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess) {
                rc = sfh_cuda_error(ctx, cudaGetLastError(), "fit state readback");
                break;
            }
            h = *(const FitState *)ctx->h_stage;
            if (h.done || h.evals >= max_evals) break;
            if (use_graph) {
                if (cudaGraphLaunch(exec, st) != cudaSuccess) {
                    rc = sfh_cuda_error(ctx, cudaGetLastError(), "fit graph launch");
                    break;
                }
                ctx->launches += per_replay;
            } else {
                for (int k = 0; k < K && !rc; ++k) rc = slot();
                if (rc) break;
            }
        }
        if (rc) break;
        if ((rc = sfh_check_onepass(ctx))) break;
        if (cudaMemcpyAsync(d_theta_out, V.theta, nt * 8, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
            (d_invH && cudaMemcpyAsync(d_invH, V.H, (size_t)nt * nt * 8, cudaMemcpyDeviceToDevice,
                                       st) != cudaSuccess) ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            rc = sfh_cuda_error(ctx, cudaGetLastError(), "fit result copy");
            break;
        }
        res->f = h.f;
        res->g_norm = h.gnorm;
        res->iterations = h.iter;
        res->evaluations = h.evals;
        res->status = h.done ? h.status : SFH_FIT_MAXEVALS;
    } while (0);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamSynchronize(st);
    cudaFree(buf);
    return rc;
}

extern "C" int sfh_fit_bfgs_dev(sfh_ctx *ctx, sfh_models *m, const double *d_data,
                                const double *d_theta0, const sfh_fit_options *opt,
                                double *d_theta_out, double *d_invH, sfh_fit_result *res) {
    if (!ctx || !m || !d_data || !d_theta0 || !opt || !d_theta_out || !res) return SFH_ERR_ARG;
    if (opt->transform < SFH_FIT_LOG_MAP || opt->transform > SFH_FIT_SQRT)
        return sfh_set_error(ctx, SFH_ERR_ARG, "invalid fit options");
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    double *comp = nullptr;
    SFH_CK(ctx, cudaMalloc(&comp, (size_t)m->nbins * 8));
    FgArgs a{};
    a.data = d_data;
    a.composite = comp;
    a.eps = opt->eps > 0.0 ? opt->eps : 2.220446049250313e-16;
    a.gsign = 1.0;
    a.mode = FG_MODE_FG;
    // fg! at r = transform(θt): -logL and the raw gradient G (k_fit_eval transforms them)
    SfhFitObjective fg = [&](const double *, double *r, double *Graw, double *negLogL,
                             const int *skip) -> int {
        FgArgs b = a;
        b.coeffs = r;
        b.G = Graw;
        b.negLogL = negLogL;
        b.skip = skip;
        return sfh_launch_fg(ctx, m, b);
    };
    const int rc = sfh_bfgs_run(ctx, m->nt, d_theta0, opt, opt->transform, fg, d_theta_out, d_invH, res);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(comp);
    return rc;
}

// Host arrays: data (nbins), theta0 (nt) -> theta_out (nt), invH (nt x nt or NULL).
extern "C" int sfh_fit_bfgs(sfh_ctx *ctx, sfh_models *m, const double *data, const double *theta0,
                            const sfh_fit_options *opt, double *theta_out, double *invH,
                            sfh_fit_result *res) {
    if (!ctx || !m || !data || !theta0 || !opt || !theta_out || !res) return SFH_ERR_ARG;
    SFH_CK(ctx, cudaSetDevice(ctx->device));
    const int64_t nt = m->nt, nbins = m->nbins;
    const size_t o_th = sfh_align256((size_t)nbins * 8), o_out = o_th + sfh_align256((size_t)nt * 8),
                 o_H = o_out + sfh_align256((size_t)nt * 8),
                 total = o_H + (invH ? (size_t)nt * nt * 8 : 0);
    char *buf = nullptr;
    SFH_CK(ctx, cudaMalloc(&buf, total));
    cudaStream_t st = ctx->stream;
    int rc = SFH_OK;
    if (cudaMemcpyAsync(buf, data, nbins * 8, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(buf + o_th, theta0, nt * 8, cudaMemcpyHostToDevice, st) != cudaSuccess)
        rc = sfh_cuda_error(ctx, cudaGetLastError(), "fit input copy");
    if (!rc)
        rc = sfh_fit_bfgs_dev(ctx, m, (const double *)buf, (const double *)(buf + o_th), opt,
                              (double *)(buf + o_out), invH ? (double *)(buf + o_H) : nullptr, res);
    if (!rc && (cudaMemcpyAsync(theta_out, buf + o_out, nt * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                (invH && cudaMemcpyAsync(invH, buf + o_H, (size_t)nt * nt * 8, cudaMemcpyDeviceToHost,
                                         st) != cudaSuccess) ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = sfh_cuda_error(ctx, cudaGetLastError(), "fit output copy");
    cudaStreamSynchronize(st);
    cudaFree(buf);
    return rc;
}
