/*
 * sfhgpu.h -- C ABI of the GB300 (sm_103a) Hess-diagram library.
 *
 * This is the drop-in boundary for StarFormationHistories.jl v1.3.1's hot path:
 * a Julia wrapper `ccall`s these symbols in place of the Julia method bodies
 * named beside each declaration (file:line in the reference).  Every entry
 * point returns an int status (SFH_OK = 0); nothing traps, nothing is retained
 * after a call returns except objects owned by handles.
 *
 * Layout conventions (the reference's flattened layout, fitting_base.jl:34-65):
 *   - a Hess diagram is (nx, ny) column-major, colour (x) fastest;
 *   - the template matrix `models` is (nbins, ntempl) column-major, one
 *     template per contiguous column (stack_models, fitting/utilities.jl:12-13);
 *   - batched coefficient vectors are stored one vector per contiguous row:
 *     R[b * ntempl + j]; batched gradients G[b * ntempl + j].
 *
 * Threading: an sfh_ctx owns one CUDA stream and its scratch; use one context
 * per host thread.  sfh_models handles are read-only after upload and may be
 * shared by contexts on the same device.
 */
#ifndef SFHGPU_H
#define SFHGPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SFH_ABI_VERSION 1

enum sfh_status {
    SFH_OK = 0,
    SFH_ERR_ARG = 1,         /* invalid argument (NULL, negative size, bad enum) */
    SFH_ERR_SHAPE = 2,       /* shape mismatch: the reference's @argcheck -> ArgumentError */
    SFH_ERR_CUDA = 3,        /* CUDA runtime error (message in sfh_ctx_last_error) */
    SFH_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
    SFH_ERR_NOMEM = 5,       /* device allocation failed */
    SFH_ERR_UNSUPPORTED = 6, /* e.g. the device is not sm_103 */
    SFH_ERR_NUMERIC = 7      /* non-finite input where the reference would produce NaN */
};

/* Element types of host/device arrays and template storage formats. */
enum sfh_dtype {
    SFH_F64 = 0,    /* double */
    SFH_F32 = 1,    /* float */
    SFH_BF16X2 = 2  /* storage only: BF16 hi + BF16 lo planes (templates for the batched GEMMs) */
};

typedef struct sfh_ctx sfh_ctx;
typedef struct sfh_models sfh_models;

/* ---------------------------------------------------------------- context */
int sfh_abi_version(void);
const char *sfh_status_string(int status);
/* One context per host thread; binds `device` and creates a non-blocking stream. */
int sfh_ctx_create(int device, sfh_ctx **out);
int sfh_ctx_destroy(sfh_ctx *ctx);
const char *sfh_ctx_last_error(const sfh_ctx *ctx);
int sfh_ctx_synchronize(sfh_ctx *ctx);
/* The context's cudaStream_t, for callers that enqueue their own work around ours. */
int sfh_ctx_stream(sfh_ctx *ctx, void **stream_out);
/* Number of kernels this library has launched on this context (telemetry). */
int sfh_ctx_launch_count(const sfh_ctx *ctx, int64_t *count_out);
/* Budget of each bounded device-side wait of the single-vector fg! pipeline, in SM clock
   cycles (0 restores the default, 4e9 cycles, about 2 s at 2 GHz; minimum 1e5).  When a
   wait runs out the kernel stops at a tile boundary, drains its copies and the call
   returns SFH_ERR_TIMEOUT; the context stays usable.  No counterpart in the reference
   (Julia's fg! has no device waits). */
int sfh_ctx_set_wait_budget(sfh_ctx *ctx, int64_t cycles);
/* Back-to-back single-vector fg! launches on this context overlap: each one-pass launch is a
   programmatic dependent of the previous kernel in the stream, so its start-up and first
   template copies run while the previous launch finishes (its inputs and outputs are
   touched only after the previous kernel completes).  On by default; 0 turns it off.  No
   counterpart in the reference. */
int sfh_ctx_set_overlap(sfh_ctx *ctx, int on);
/* How the host-array entry point sfh_fg reaches the caller's arrays:
     SFH_HOST_ACCESS_STAGED  through the context's mapped pinned staging area (one host
                             copy in, one out);
     SFH_HOST_ACCESS_DIRECT  the kernels read r and n and write the composite and G in the
                             caller's arrays themselves (double arrays, 8-byte aligned,
                             composite given); needs a device that reads pageable host
                             memory through the host page tables (a coherent host link),
                             else SFH_ERR_UNSUPPORTED;
     SFH_HOST_ACCESS_AUTO    (default) DIRECT where the device supports it, else STAGED.
   Both give bit-identical results.  No counterpart in the reference (Julia's fg! runs on
   the host arrays). */
enum sfh_host_access {
    SFH_HOST_ACCESS_AUTO = -1,
    SFH_HOST_ACCESS_STAGED = 0,
    SFH_HOST_ACCESS_DIRECT = 1
};
int sfh_ctx_set_host_access(sfh_ctx *ctx, int mode);
/* The mode sfh_fg uses now (STAGED or DIRECT; AUTO resolved). */
int sfh_ctx_host_access(const sfh_ctx *ctx, int *mode_out);
/* One-shot failure injection for tests of the error paths (no counterpart in the
   reference); nothing here faults the GPU:
     SFH_INJECT_DROP_COPY   the next one-pass fg! launch skips its first bulk copy, so the
                            consumers' wait for that box runs out (SFH_ERR_TIMEOUT);
     SFH_INJECT_ALLOC_FAIL  the next device or pinned allocation of this context is
                            refused on the host (SFH_ERR_NOMEM). */
enum sfh_inject { SFH_INJECT_NONE = 0, SFH_INJECT_DROP_COPY = 1, SFH_INJECT_ALLOC_FAIL = 2 };
int sfh_ctx_inject_fault(sfh_ctx *ctx, int what);

/* ---------------------------------------------------------------- templates matrix */
/* Copies a host column-major (nbins, ntempl) matrix (src_dtype SFH_F64 or SFH_F32)
   to the device once, stored as `storage` (SFH_F64, SFH_F32 or SFH_BF16X2).
   Replaces the per-call reads of `models` by composite!/∇loglikelihood!
   (fitting_base.jl:55-65, :265-285); stack_models is fitting/utilities.jl:12-13. */
int sfh_models_upload(sfh_ctx *ctx, const void *host_models, int src_dtype, int64_t nbins,
                      int64_t ntempl, int storage, sfh_models **out);
/* Wraps device-resident FP32 templates (e.g. built by sfh_partial_cmd_smooth_batch_dev)
   into a handle, converting to `storage`; the source buffer is copied. */
int sfh_models_from_device(sfh_ctx *ctx, const float *dev_models_f32, int64_t nbins,
                           int64_t ntempl, int storage, sfh_models **out);
int sfh_models_free(sfh_models *models);
/* New matrix whose column g is Σ_q w_q M[:, cols_q] over q in [h_group_off[g],
   h_group_off[g+1]) (FP32 source storage; result stored as `storage`).  With one group per
   unique age and the relative weights of a fixed age-metallicity relation this is the
   expansion coeffs[idxs] = relweights[idxs] .* x[i] of fixed_amr
   (hierarchical/fixed_amr.jl:106-113), done once so every fg! reads n_ages columns. */
int sfh_models_combine(sfh_ctx *ctx, const sfh_models *models, int64_t ngroups,
                       const int64_t *h_group_off, const int32_t *h_cols,
                       const double *h_weights, int storage, sfh_models **out);
int sfh_models_info(const sfh_models *models, int64_t *nbins, int64_t *ntempl, int *storage);

/* ---------------------------------------------------------------- host-array drop-ins
 * `dtype` (SFH_F64 or SFH_F32) is the element type T of every host array passed;
 * eps(T) is the clamp used by the reference (fitting_base.jl:90,154,277).
 * Host arrays are copied in and out inside the call; the call returns after the
 * results are in host memory. */

/* composite!(composite, coeffs, models), fitting_base.jl:55-65 */
int sfh_composite(sfh_ctx *ctx, const sfh_models *models, int dtype, const void *coeffs,
                  void *composite_out);
/* loglikelihood(composite, data), fitting_base.jl:84-96 */
int sfh_loglikelihood(sfh_ctx *ctx, int dtype, const void *composite, const void *data,
                      int64_t nbins, double *out);
/* ∇loglikelihood!(G, composite, models, data), fitting_base.jl:265-285.
   Overwrites composite with 1 - data/max(composite, eps) exactly as the reference. */
int sfh_grad_loglikelihood(sfh_ctx *ctx, const sfh_models *models, int dtype,
                           void *composite_inout, const void *data, void *G);
/* fg!(F, G, coeffs, models, data, composite), solvers.jl:20-38.
   negLogL == NULL is the `F === nothing` branch, G == NULL the `G === nothing`
   branch.  composite receives what the reference leaves in it (the model when G
   is NULL, 1 - n/c otherwise); composite may be NULL to skip that copy-out.
   Non-finite coefficients: *negLogL and G are set to NaN (what the reference's
   arithmetic produces) and SFH_ERR_NUMERIC is returned without launching. */
int sfh_fg(sfh_ctx *ctx, const sfh_models *models, int dtype, const void *coeffs,
           const void *data, void *composite, void *G, double *negLogL);

/* ---------------------------------------------------------------- device-array forms
 * All pointers are device pointers; work is enqueued on the context stream and
 * the call returns without synchronising.  `eps` is eps(T) of the caller's type. */

/* fg! on device-resident arrays.  d_negLogL (1 double) and d_G (ntempl doubles)
   may be NULL.  d_composite (nbins doubles) receives the reference's contents. */
int sfh_fg_dev(sfh_ctx *ctx, const sfh_models *models, const double *d_coeffs,
               const double *d_data, double *d_composite, double *d_G, double *d_negLogL,
               double eps);

/* ---------------------------------------------------------------- device fit driver */
/* BFGS over fg! on the device, for fit_templates (src/fitting/solvers.jl:172-221: log
   transform, MAP with the Jacobian term -Σθ, then MLE) and fit_templates_fast (:238-275:
   coeffs = θ²).  As Optim.BFGS there: inverse-Hessian BFGS from H0 = I, the update skipped
   when sᵀy <= 0, first trial step min(1, |d|) / |d| (InitialStatic(1.0, scaled=true)),
   stops on |g|∞ <= g_abstol, |Δf| <= f_reltol |f|, |Δθ|∞ <= x_abstol or max_iter
   accepted steps.  The line search backtracks (Optim: HagerZhang), so iterates differ
   while the optimum does not.  The loop runs on the GPU (CUDA-graph replays of
   evaluation slots); the host reads a small state once per replay. */
enum sfh_fit_transform { SFH_FIT_LOG_MAP = 0, SFH_FIT_LOG_MLE = 1, SFH_FIT_SQRT = 2 };
enum sfh_fit_status {
    SFH_FIT_CONVERGED_G = 0, /* |g|∞ <= g_abstol */
    SFH_FIT_CONVERGED_F = 1, /* |Δf| <= f_reltol |f| */
    SFH_FIT_CONVERGED_X = 2, /* |Δθ|∞ <= x_abstol */
    SFH_FIT_MAXITER = 3,     /* max_iter accepted steps */
    SFH_FIT_LINESEARCH = 4,  /* no decrease along d after 40 backtracks (noise floor) */
    SFH_FIT_NONFINITE = 5,   /* f or g not finite at an accepted point */
    SFH_FIT_MAXEVALS = 6     /* max_evals fg! evaluations */
};
typedef struct sfh_fit_options {
    int transform;    /* sfh_fit_transform */
    int max_iter;     /* accepted steps (Optim's iterations; its default is 1000) */
    int max_evals;    /* fg! evaluations, 0 = 50 (max_iter + 1); checked between graph
                         replays, so a fit may run up to graph_slots - 1 more */
    int graph_slots;  /* evaluations per graph replay, 0 = 8 (at most 64) */
    double g_abstol;  /* Optim default 1e-8 */
    double f_reltol;  /* Optim default 0 (stops only on an unchanged f) */
    double x_abstol;  /* Optim default 0 */
    double eps;       /* composite floor of fg!, 0 = eps(Float64) */
} sfh_fit_options;
typedef struct sfh_fit_result {
    double f;            /* objective at theta_out (fg! value, minus Σθ for LOG_MAP) */
    double g_norm;       /* |g|∞ there */
    int64_t iterations;  /* accepted steps */
    int64_t evaluations; /* fg! evaluations */
    int status;          /* sfh_fit_status */
    int graph;           /* 1 when the slots ran as CUDA-graph replays */
} sfh_fit_result;
/* Device buffers: d_data (nbins), d_theta0 (nt, transformed start) -> d_theta_out (nt),
   d_invH (nt x nt, the final BFGS inverse Hessian in θ, or NULL).  Synchronous. */
int sfh_fit_bfgs_dev(sfh_ctx *ctx, sfh_models *models, const double *d_data,
                     const double *d_theta0, const sfh_fit_options *opt, double *d_theta_out,
                     double *d_invH, sfh_fit_result *res);
/* sfh_fit_bfgs_dev on host arrays. */
int sfh_fit_bfgs(sfh_ctx *ctx, sfh_models *models, const double *data, const double *theta0,
                 const sfh_fit_options *opt, double *theta_out, double *invH,
                 sfh_fit_result *res);

/* Telemetry: average device time (ms) of each of the four kernels of sfh_fg_dev over
   `iters` evaluations, timed with CUDA events on the context stream:
   ms_out[0] m = M r partials, [1] Poisson terms + w, [2] Mᵀ w partials, [3] G reduction.
   No reference counterpart; used to report the dominant kernel's roofline. */
int sfh_fg_kernel_times(sfh_ctx *ctx, const sfh_models *models, const double *d_coeffs,
                        const double *d_data, double *d_composite, double *d_G,
                        double *d_negLogL, double eps, int iters, double *ms_out);

/* Single-vector fg! paths for FP32 template storage (no reference counterpart; both
   compute fg!, src/fitting/solvers.jl:20-38, to the same tolerance):
     SFH_PATH_ONEPASS  one kernel keeps 16- or 32-bin tiles of every template in shared
                       memory (bulk-copy ring, one persistent CTA per SM) and forms the
                       composite, the Poisson terms, w and Mᵀ w from one read of the
                       matrix; needs nt <= 1536, and keeps a blocked copy of the FP32
                       templates (one more matrix of device memory, made on first use);
     SFH_PATH_TWOPASS  pass 1 (m = M r, terms, w) then pass 2 (G = Mᵀ w): two reads;
     SFH_PATH_AUTO     one-pass when the shape allows it (default).
   The path applies to calls that request G; composite-only calls read the matrix once
   either way. */
enum sfh_fg_path { SFH_PATH_AUTO = 0, SFH_PATH_ONEPASS = 1, SFH_PATH_TWOPASS = 2 };
/* Sets the path of later fg! calls on this handle (SFH_ERR_UNSUPPORTED when ONEPASS is
   asked for a shape it cannot take). */
int sfh_models_set_path(sfh_ctx *ctx, sfh_models *models, int path);
/* Tile width of the one-pass kernel: 16 or 32 bins per tile (default 16; the autotuner
   measures both; a shape whose tile does not fit the 32-bin ring takes 16). */
int sfh_models_set_onepass_tile(sfh_ctx *ctx, sfh_models *models, int bins);
/* CTAs per SM of the one-pass kernel: 1 (14 owner warps, the whole shared memory) or 2
   (6 owner warps each, 16-bin tiles, half the shared memory: the two CTAs' per-tile
   latencies overlap).  Default 1; the autotuner measures both; shapes that do not fit
   two CTAs per SM take one. */
int sfh_models_set_onepass_ctas(sfh_ctx *ctx, sfh_models *models, int ctas_per_sm);
/* Schedule of the one-pass kernel: 0 phased (per tile: phase A, finish, phase B), 1 skewed
   (phase B of a tile and phase A of the next in one barrier interval; 16-bin tiles, one CTA
   per SM, shapes whose ring holds two tiles, else phased).  Default 0; the autotuner
   measures both. */
int sfh_models_set_onepass_schedule(sfh_ctx *ctx, sfh_models *models, int skewed);
/* Boxes (64 templates x the tile's bins each) per bulk copy of the one-pass kernel: 1, 2 or
   4, or 0 for the default (4 for 16-bin tiles, 2 for 32-bin); fewer where the ring does not
   hold the runs. */
int sfh_models_set_onepass_run(sfh_ctx *ctx, sfh_models *models, int boxes);
/* The one-pass variant later calls launch: tile bins, CTAs per SM, skewed (0/1), boxes per
   bulk copy (SFH_ERR_UNSUPPORTED for a handle the one-pass kernel cannot take). */
int sfh_models_onepass_variant(sfh_ctx *ctx, const sfh_models *models, int *bins,
                               int *ctas_per_sm, int *skewed, int *run_boxes);
/* The path fg! calls with G take on this handle now (ONEPASS or TWOPASS), and the
   one-pass time measured by sfh_models_autotune (0 if not measured); either may be NULL. */
int sfh_models_path(sfh_ctx *ctx, const sfh_models *models, int *path_out, double *onepass_ms);

/* Occupied-bin restriction of the single-vector fg! with G (FP32 storage, one-pass path;
   no reference counterpart, same results as fitting_base.jl:84-96,265-285 and
   solvers.jl:20-38).  With G requested the composite matters only where n_i > 0: an
   empty bin has w_i = 1 exactly and adds -max(c_i, eps) to logL, so its terms reduce to
   the template column sums over the empty bins, E_j (kept in FP64):
     logL = Σ_{n_i > 0} (n_i - c_i - n_i log(n_i / c_i)) - Σ_j r_j E_j,
     G_j  = Σ_{n_i > 0} M_ij (1 - n_i / c_i) + E_j,
   and the composite output holds w, 1.0 in the empty bins, as fg! leaves it.  The only
   difference from the dense sum is -c_i for -max(c_i, eps) in empty bins whose model is
   below eps (at most eps per bin).  The handle keeps a plan per observed diagram (keyed by
   its data pointer, built on first use: the occupied bins, a blocked copy of their template
   rows, E_j; up to 4 diagrams per handle): the kernel then reads only the occupied rows.
   Every call checks that the plan's empty bins are still empty; a bin that is not is
   folded in exactly inside the same launch, and the next call builds a new plan.  Calls
   made during stream capture use an existing plan only.
     SFH_OCC_OFF    the dense kernel always;
     SFH_OCC_AUTO   (default) the plan when at most 60 % of the bins are occupied;
     SFH_OCC_ON     the plan whenever some bin is empty and some occupied. */
enum sfh_occ_mode { SFH_OCC_OFF = 0, SFH_OCC_AUTO = 1, SFH_OCC_ON = 2 };
int sfh_models_set_occupied(sfh_ctx *ctx, sfh_models *models, int mode);
/* Telemetry of the plan for d_data: occupied bins (or -1 when no plan exists), whether
   the restricted kernel serves it (0/1), and the host wall time of the last plan build
   (ms); any output may be NULL. */
int sfh_models_occupied_info(sfh_ctx *ctx, const sfh_models *models, const double *d_data,
                             int64_t *nocc_out, int *sparse_out, double *build_ms_out);

/* Autotuner (no reference counterpart): times candidate launch plans of the FP32
   single-vector fg! on this matrix with the caller's inputs (pass-1 template splits whose
   grids fill 1/2 to 4 whole waves of resident blocks; pass-2 row chunks of 1,024 / 2,048
   / 4,096 bins and column groups sized to 1, 2 or 4 waves; the one-pass kernel when the
   shape allows it), `iters` timed runs each, and stores the fastest in the handle; later
   fg! calls on it use that plan.  plan_out (3 ints: pass-1 template splits, pass-2 rows,
   pass-2 waves) and ms_out (2 doubles: pass-1 and pass-2 ms) may be NULL; the path chosen
   and the one-pass time are read back with sfh_models_path.  Call it before sharing the
   handle between contexts.  No-op for FP64 storage. */
int sfh_models_autotune(sfh_ctx *ctx, sfh_models *models, const double *d_coeffs,
                        const double *d_data, double eps, int iters, int *plan_out,
                        double *ms_out);

/* fg! for callers that cannot allocate device memory (no counterpart in the
   reference): graph-capture regions that must not allocate, plugins inside a host
   application that owns the device memory budget, allocation-free real-time loops.
   Same result as sfh_fg_dev on FP32 templates, computed by the two-pass FP32 plan
   (sfh_fg_dev prefers the one-pass kernel, whose blocked template copy is an
   allocation, so this entry is about 1.6x slower on large matrices).  All scratch
   lives in one fixed 11 MiB device array inside the library, so the call allocates
   nothing: the caller passes the (nbins, ntempl) column-major FP32 templates (any
   float-aligned address), every input and output, and the stream.  Limits:
   nbins <= 131072 and ntempl <= 4096 (SFH_ERR_SHAPE beyond).  The first call in each
   CUDA context looks up the array's device address in that context (the address is
   cached per context); make that first call before any stream capture.  All calls
   share the one array, so calls that overlap on the GPU (different streams, or
   different host threads) race: serialise them on one stream.  d_G and d_negLogL may
   be NULL as in sfh_fg_dev. */
int sfh_fg_dev_noalloc(void *stream, const float *d_models, int64_t nbins, int64_t ntempl,
                       const double *d_coeffs, const double *d_data, double *d_composite,
                       double *d_G, double *d_negLogL, double eps);

/* B coefficient vectors in one call (HMC chains, line-search probes):
   d_R[b*ntempl + j] -> d_negLogL[b] (may be NULL: gradient-only substeps skip the
   logarithms) and d_G[b*ntempl + j] = -∂logL/∂r (may be NULL).  Needs models
   stored as SFH_BF16X2 (tensor-core path).  With d_negLogL the composite is formed
   exactly on the stored FP32 templates from BF16 digit planes (ntempl <= 2304), so
   |ΔlogL| against FP64 stays below 1e-6 per 1e4 stars; the gradient accumulates BF16
   hi/lo products in FP32 (about 1e-5 of sum_i |M_ij w_i|).  Replaces fg! of
   src/fitting/solvers.jl:20-38 for every vector. */
int sfh_fg_batched_dev(sfh_ctx *ctx, const sfh_models *models, const double *d_R, int64_t B,
                       const double *d_data, double *d_negLogL, float *d_G, double eps);

/* ---------------------------------------------------------------- batched HMC */
enum sfh_hmc_model {
    SFH_HMC_DIRECT = 0, /* θ = log coeffs: hmc_sample's log density, hmc_sample.jl:24-37 */
    SFH_HMC_MZR = 1,    /* PowerLawMZR + GaussianDispersion: sample_sfh's log density,
                           generic_fitting.jl:90-199 with mzr.jl:50-215 */
    SFH_HMC_LINEAR_AMR = 2, /* LinearAMR + GaussianDispersion: generic_fitting.jl:90-199 with
                               amr.jl:50-160, 205-213 (μ_j = β + α (T_max - t_j)) */
    SFH_HMC_LOG_AMR = 3     /* LogarithmicAMR with the default MH_from_Z (utilities.jl:138-155)
                               + GaussianDispersion: amr.jl:278-290, θ = [log R, log α, log β,
                               log σ] (transforms (1, 1)) */
};
typedef struct {
    int32_t nchains;        /* chains advanced together (one batched gradient per step) */
    int32_t model;          /* enum sfh_hmc_model */
    int64_t ntraj;          /* trajectories kept after warmup */
    int64_t nwarmup;        /* warmup trajectories: step-size (dual averaging) and mass adaptation */
    int32_t nleap;          /* leapfrog steps per trajectory */
    int32_t thin;           /* keep every thin-th draw when draws are requested */
    double step0;           /* initial leapfrog step */
    double target_accept;   /* dual-averaging target acceptance (e.g. 0.8) */
    uint64_t seed;          /* Philox key */
    /* SFH_HMC_MZR and the AMR models: ages and metallicities of the templates */
    int32_t nages;
    const int32_t *h_age_index; /* per template: its age, 0..nages-1 */
    const double *h_logAge;     /* per age (any order) */
    const double *h_MH;         /* per template [M/H] */
    double logMstar0;           /* PowerLawMZR logMstar0 (fixed), mzr.jl:263-272 */
    int32_t alpha_free, beta_free, sigma_free;
    double alpha, beta, sigma;  /* values of parameters held fixed */
    double T_max;               /* the AMR models: earliest lookback time in Gyr */
    const double *d_minv0;      /* D starting diagonal inverse mass (device; NULL = ones), e.g.
                                   the diagonal of a MAP fit's inverse Hessian */
} sfh_hmc_config;

/* Batched HMC over all chains at once, every leapfrog step one sfh_fg_batched_dev-style
   evaluation on the tensor cores; replaces the per-chain DynamicHMC loop of hmc_sample
   (hmc_sample.jl:105-141) and sample_sfh (generic_fitting.jl:458-527).  Fixed-length
   trajectories, per-chain dual-averaging step size and a diagonal mass during warmup
   (pooled over chains with 16 or more; with fewer, each chain's own variance over the
   second quarter of warmup), Metropolis accept.  Device arrays: d_theta0 (nchains x D) starting points in
   the transformed space (D = ntempl for SFH_HMC_DIRECT; nages + free parameters, order
   [log R_j..., log α, β, log σ], for SFH_HMC_MZR).  Outputs (each may be NULL):
   d_mean / d_var (nchains x D) posterior mean and variance of the natural parameters
   (exp of the log-transformed ones), d_accept (nchains) mean acceptance, d_step
   (nchains) final step, d_draws (nchains x ceil(ntraj/thin) x D) FP32 natural draws.
   SFH_HMC_LINEAR_AMR uses the MZR layout with [log R_j..., log α, β, log σ] (amr.jl:212
   transforms (1, 0) for α, β).
   Models must be stored as SFH_BF16X2.  The call returns after the run completes. */
int sfh_hmc_sample_dev(sfh_ctx *ctx, const sfh_models *models, const double *d_data,
                       const sfh_hmc_config *cfg, const double *d_theta0, double *d_mean,
                       double *d_var, double *d_accept, double *d_step, float *d_draws);

/* The No-U-Turn sampler of DynamicHMC (the sampler of hmc_sample.jl:105-141 and
   sample_sfh, generic_fitting.jl:458-527) for all chains at once: multinomial sampling
   over each trajectory, trees doubled in a random direction until the generalized
   no-U-turn criterion holds for the tree or any subtree, an energy error above 1000
   (divergence) or max_depth doublings (1..12; DynamicHMC's default is 10).  Every chain
   runs its own tree and advances one leapfrog step per batched evaluation, so no
   evaluation waits for other chains' trees.  Warmup (nwarmup trees per chain): per-chain
   dual averaging of the step on each tree's mean acceptance statistic, and a per-chain
   diagonal metric from the chain's own draws over the middle 70 % of warmup (starting
   from cfg->d_minv0 or ones).  d_minv_dense (D x D, device, or NULL): a dense metric M⁻¹
   for all chains instead, kept through warmup; the reference's sample_sfh passes the
   MAP inverse Hessian and a fixed step with no warmup (generic_fitting.jl:458-490:
   GaussianKineticEnergy(MAP.invH), ϵ = 0.05), which nwarmup = 0 and step0 = 0.05
   reproduce (D <= 256).  cfg as sfh_hmc_sample_dev (nleap is ignored); outputs as there,
   plus d_depth (nchains) the mean tree depth and d_ndiv (nchains) the divergent
   trajectories after warmup; any output may be NULL.  Synchronous. */
int sfh_nuts_sample_dev(sfh_ctx *ctx, const sfh_models *models, const double *d_data,
                        const sfh_hmc_config *cfg, int max_depth,
                        const double *d_minv_dense, const double *d_theta0, double *d_mean,
                        double *d_var, double *d_accept, double *d_step, double *d_depth,
                        int64_t *d_ndiv, float *d_draws);

/* Log density and its gradient for B parameter vectors of the same model as
   sfh_hmc_sample_dev (logdensity_and_gradient of hmc_sample.jl:24-37 and
   generic_fitting.jl:90-199 with Jacobian terms), batched on the tensor cores:
   d_theta (B x D, B = cfg->nchains) -> d_logd (B), d_grad (B x D). */
int sfh_logdensity_batched_dev(sfh_ctx *ctx, const sfh_models *models, const double *d_data,
                               const sfh_hmc_config *cfg, const double *d_theta, double *d_logd,
                               double *d_grad);

/* fit_sfh's optimisations on the device (generic_fitting.jl:242-409): BFGS, as
   sfh_fit_bfgs_dev, over the hierarchical log density of cfg's metallicity model
   (SFH_HMC_MZR, SFH_HMC_LINEAR_AMR or SFH_HMC_LOG_AMR; the sampler fields of cfg are
   ignored) for one vector θ = [log R_j..., free model parameters in their transforms]
   (D = nages + free ones, the layout of sfh_hmc_sample_dev).  map = 1 minimises
   -(logL + Jacobian terms of the log transforms) (fg_map!, :324-334), map = 0 minimises
   -logL (fg_mle!, :335-345); opt->transform is ignored.  Each evaluation maps θ to the
   template coefficients (calculate_coeffs), runs the single-vector fg! (any template
   storage) and applies the chain rule, all on the device.  Device buffers: d_data
   (nbins), d_theta0 (D) -> d_theta_out (D), d_invH (D x D, the final BFGS inverse
   Hessian, or NULL).  Synchronous. */
int sfh_fit_sfh_dev(sfh_ctx *ctx, sfh_models *models, const double *d_data,
                    const sfh_hmc_config *cfg, const double *d_theta0, int map,
                    const sfh_fit_options *opt, double *d_theta_out, double *d_invH,
                    sfh_fit_result *res);

/* ---------------------------------------------------------------- mock observation */
/* model_cmd(mags, errfuncs, completefuncs, biasfuncs; rng, ret_idxs), src/simulate.jl:621-680:
   star i (of n) is kept when a uniform draw is <= detect_prob[i] (the product of its per-filter
   completeness values, evaluated by the caller as the reference evaluates its callables);
   a kept star's magnitudes become mags + z sigma + bias with standard normal z.  mags,
   sigma and bias (NULL = none) are n x nf row-major (star-major), nf <= 8.  out (n x nf
   capacity) and idx (n capacity, 0-based input indices) receive the kept stars in input
   order, *n_out their number.  Draws are Philox4x32-10 keyed by seed and counted by star
   and filter, so they do not depend on the launch or on which other stars are kept (the
   reference's draws come from Julia's RNG: the same distribution, not the same numbers).
   Host arrays; synchronous. */
int sfh_model_cmd(sfh_ctx *ctx, const double *mags, const double *sigma, const double *bias,
                  const double *detect_prob, int64_t n, int nf, uint64_t seed, double *out,
                  int64_t *idx, int64_t *n_out);
/* sfh_model_cmd on device buffers (synchronises to read *n_out). */
int sfh_model_cmd_dev(sfh_ctx *ctx, const double *d_mags, const double *d_sigma,
                      const double *d_bias, const double *d_detect_prob, int64_t n, int nf,
                      uint64_t seed, double *d_out, int64_t *d_idx, int64_t *n_out);

/* ---------------------------------------------------------------- template construction */
/* bin_cmd(colors, mags; weights, edges), StarFormationHistories.jl:544-553: the
   hard-binned Hess diagram, StatsBase fit(Histogram, (colors, mags), Weights(weights), edges;
   closed=:left).  Host arrays: colors, mags, weights (NULL = unit weights) of n points;
   xedges holds nx + 1 and yedges ny + 1 finite increasing values (the ranges' elements);
   bin (i, j) counts xedges[i] <= color < xedges[i+1] and yedges[j] <= mag < yedges[j+1].
   hist_out is host (nx, ny) column-major doubles, overwritten.  Synchronous. */
int sfh_bin_cmd(sfh_ctx *ctx, const double *colors, const double *mags, const double *weights,
                int64_t n, const double *xedges, int64_t nx, const double *yedges, int64_t ny,
                double *hist_out);
/* sfh_bin_cmd on device buffers, ordered on the context's stream (no synchronisation). */
int sfh_bin_cmd_dev(sfh_ctx *ctx, const double *d_colors, const double *d_mags,
                    const double *d_weights, int64_t n, const double *d_xedges, int64_t nx,
                    const double *d_yedges, int64_t ny, double *d_hist_out);

/* bin_cmd_smooth(colors, mags, color_err, mag_err, cov_mult; weights, edges),
   StarFormationHistories.jl:574-621 (kernels :191-340, addstar! :345-408).
   Host arrays of npts doubles; edges are ranges first + k*step (k = 0..n);
   hist_out is host (nx, ny) column-major doubles, overwritten. */
int sfh_bin_cmd_smooth(sfh_ctx *ctx, const double *colors, const double *mags,
                       const double *color_err, const double *mag_err, const double *weights,
                       int64_t npts, int cov_mult, double x_first, double x_step, int64_t nx,
                       double y_first, double y_step, int64_t ny, double *hist_out);

/* Device batch of bin_cmd_smooth calls sharing one grid: star lists of all
   templates concatenated (d_x..d_w, FP64), template t owns stars
   [d_offsets[t], d_offsets[t+1]); cov_mult per template.  Output d_models is
   (nx*ny, ntempl) column-major FP32, overwritten. */
int sfh_bin_cmd_smooth_batch_dev(sfh_ctx *ctx, const double *d_x, const double *d_y,
                                 const double *d_sx, const double *d_sy, const double *d_w,
                                 const int64_t *d_offsets, const int32_t *h_cov_mult,
                                 int64_t ntempl, double x_first, double x_step, int64_t nx,
                                 double y_first, double y_step, int64_t ny, float *d_models);

/* Closed-form stand-ins for partial_cmd_smooth's callables (a C ABI cannot carry
   Julia closures): */
typedef struct {
    /* exp_photerr(m, a, b, c, d) = a^(b(m-c)) + d, src/utilities.jl:218, capped at cap */
    double a, b, c, d, cap;
} sfh_err_model;
typedef struct {
    /* Martin2016_complete(m, A, m50, rho), src/utilities.jl:205 */
    double A, m50, rho;
} sfh_compl_model;
typedef struct {
    /* continuous broken power-law IMF on [mmin, mmax]; Kroupa2001(0.08, 100) is
       nseg = 2, breaks = {0.5}, alpha = {1.3, 2.3} */
    int32_t nseg;
    double mmin, mmax;
    double breaks[3];
    double alpha[4];
} sfh_imf;

/* Batched partial_cmd_smooth (single stars), StarFormationHistories.jl:829-888,
   fully on device: mini_spacing resampling (:110-148), interpolate_mini (:77-81),
   errors/completeness, calculate_weights (:765-776), bias, midpoints and the
   stamps.  Isochrone t has n_t = d_iso_len[t] points at d_iso_off[t] in d_m_ini
   (strictly increasing masses) and d_mags[f * total + d_iso_off[t] + i] for filter f.
   nf <= 8 filters; y_index/c1/c2 are 0-based; err/compl/bias have nf entries
   (bias: constant offsets, may be NULL).  d_dmod / d_norm are per template.
   Output d_models (nx*ny, ntempl) column-major FP32. */
int sfh_partial_cmd_smooth_batch_dev(sfh_ctx *ctx, const double *d_m_ini, const double *d_mags,
                                     int64_t total_points, const int64_t *h_iso_off,
                                     const int32_t *h_iso_len, int64_t ntempl, int nf,
                                     int y_index, int c1, int c2, const sfh_err_model *err,
                                     const sfh_compl_model *compl_, const double *bias,
                                     const sfh_imf *imf, double mean_mass, const double *h_dmod,
                                     const double *h_norm, double x_first, double x_step,
                                     int64_t nx, double y_first, double y_step, int64_t ny,
                                     float *d_models);

/* binary_hess(RandomBinaryPairs, m_ini, mags, ...) for a batch of templates,
   src/StarFormationHistories.jl:627-706 (the case y_index in color_indices, the only one the
   reference implements; SFH_ERR_UNSUPPORTED otherwise).  Template t's isochrone points
   (masses increasing, magnitudes with the distance modulus added; partial_cmd_smooth passes
   every fourth resampled point, :896) are [h_off[t], h_off[t] + h_len[t]) of d_m_ini and of
   each filter row of d_mags (row f at d_mags + f*total_points).  Every pair of interval
   left points is a binary (fluxes added, :656), weighted by the IMF and the colour filters'
   completeness, binned (left-closed), and the nonzero bins are smoothed as points at the
   bin centres by the bin_cmd_smooth stamps.  h_norm[t] is normalize_value.  Output
   (nx*ny, ntempl) column-major FP32, overwritten; edges must increase. */
int sfh_binary_hess_batch_dev(sfh_ctx *ctx, const double *d_m_ini, const double *d_mags,
                              int64_t total_points, const int64_t *h_off, const int32_t *h_len,
                              int64_t ntempl, int nf, int y_index, int c1, int c2,
                              const sfh_err_model *err, const sfh_compl_model *compl_,
                              const double *bias, const sfh_imf *imf, double mean_mass,
                              const double *h_norm, double x_first, double x_step, int64_t nx,
                              double y_first, double y_step, int64_t ny, float *d_models);
/* partial_cmd_smooth's single/binary mix (src/StarFormationHistories.jl:900-909):
   d_out[:, t] = (1 - bmf[t]) d_single[:, t] + bmf[t] d_binary[:, t], bmf[t] the binary mass
   fraction times trapz(new_mini, imf(new_mini)).  d_out may be d_single. */
int sfh_mix_binary_templates_dev(sfh_ctx *ctx, const float *d_single, const float *d_binary,
                                 const double *h_bmf, int64_t ntempl, int64_t nbins,
                                 float *d_out);

/* One template's Hess grid in a ragged batch: colour edges x_first + k x_step (k = 0..nx),
   magnitude edges y_first + k y_step (k = 0..ny); its (nx*ny) column-major histogram is
   written at d_models + out_offset. */
typedef struct {
    double x_first, x_step;
    int64_t nx;
    double y_first, y_step;
    int64_t ny;
    int64_t out_offset;
} sfh_hess_grid;

/* Ragged batch of partial_cmd_smooth calls (many galaxies with uneven Hess grids and
   isochrone lengths, StarFormationHistories.jl:829-888 per template): as
   sfh_partial_cmd_smooth_batch_dev, but template t is binned on h_grids[t] with its own
   mini_spacing step min(|x_step|, |y_step|) (:851).  d_models holds models_len floats;
   every template's histogram must lie inside it.  One launch per pass for the whole batch. */
int sfh_partial_cmd_smooth_ragged_dev(sfh_ctx *ctx, const double *d_m_ini, const double *d_mags,
                                      int64_t total_points, const int64_t *h_iso_off,
                                      const int32_t *h_iso_len, int64_t ntempl, int nf,
                                      int y_index, int c1, int c2, const sfh_err_model *err,
                                      const sfh_compl_model *compl_, const double *bias,
                                      const sfh_imf *imf, double mean_mass, const double *h_dmod,
                                      const double *h_norm, const sfh_hess_grid *h_grids,
                                      int64_t models_len, float *d_models);

/* ---------------------------------------------------------------- ragged galaxies (fg!) */
/* One galaxy of a ragged batch: its (nbins x ntempl) column-major FP32 templates start at
   d_models + model_offset; its data / composite bins at bin_offset and its coefficients /
   gradient at templ_offset of the packed arrays. */
typedef struct {
    int64_t model_offset;
    int64_t nbins, ntempl;
    int64_t bin_offset;
    int64_t templ_offset;
} sfh_galaxy;
typedef struct sfh_galaxies sfh_galaxies;

/* Builds the work lists of a ragged batch once (descriptors are copied; d_models is
   referenced, not copied, and must outlive the handle).  models_len: floats in d_models. */
int sfh_galaxies_create(sfh_ctx *ctx, const float *d_models, int64_t models_len,
                        const sfh_galaxy *h_galaxies, int64_t ngal, sfh_galaxies **out);
int sfh_galaxies_free(sfh_galaxies *galaxies);
int sfh_galaxies_info(const sfh_galaxies *galaxies, int64_t *ngal, int64_t *total_bins,
                      int64_t *total_templ);
/* fg! (solvers.jl:20-38) for every galaxy of the batch at once, device arrays packed by
   the descriptors: d_coeffs / d_G by templ_offset, d_data / d_composite by bin_offset,
   d_negLogL one value per galaxy.  d_G and d_negLogL may be NULL (the reference's
   `nothing` branches); d_composite receives what fg! leaves there (1 - n/c when G is
   requested, the model otherwise).  Enqueued on the context stream, no synchronisation. */
int sfh_fg_ragged_dev(sfh_ctx *ctx, const sfh_galaxies *galaxies, const double *d_coeffs,
                      const double *d_data, double *d_composite, double *d_G,
                      double *d_negLogL, double eps);

/* ---------------------------------------------------------------- learned template emulator */
/* No reference counterpart (new component).  An MLP in -> h1 -> h2 -> out (GELU after the
   hidden layers, FP32 master weights, BF16-rounded matmul operands with FP32
   accumulation) maps standardised (log age, [M/H], distance modulus) to scaled
   coefficients on a PCA basis of variance-stabilised templates; templates are rebuilt
   from the coefficients, and the exact partial_cmd_smooth template scores them by Poisson
   deviance per star and replaces any that fail.  All arrays are device FP32 and
   row-major.  Parameter block: W1 (h1 x in), b1, W2 (h2 x h1), b2, W3 (out x h2), b3. */
int sfh_mlp_param_count(int in, int h1, int h2, int out, int64_t *n);
/* d_Y (B x out) = MLP(d_X (B x in)). */
int sfh_mlp_forward(sfh_ctx *ctx, int in, int h1, int h2, int out, const float *d_params,
                    const float *d_X, int B, float *d_Y);
/* Mean-squared-error loss mean((Y - T)^2) over B x out and its gradient d_grad (same layout
   as the parameters); d_loss (one float) may be NULL. */
int sfh_mlp_loss_grad(sfh_ctx *ctx, int in, int h1, int h2, int out, const float *d_params,
                      const float *d_X, const float *d_T, int B, float *d_grad, float *d_loss);
/* nsteps Adam steps (beta 0.9 / 0.999, eps 1e-8, bias-corrected from step0 + 1) on
   minibatches of `batch` rows drawn with replacement (Philox keyed by seed and the step)
   from d_X (nsamples x in) / d_T (nsamples x out).  d_adam_m / d_adam_v hold the moment
   estimates (parameter layout, zero before the first call).  d_loss_trace (nsteps floats,
   may be NULL) receives each step's minibatch loss before its update. */
int sfh_mlp_train(sfh_ctx *ctx, int in, int h1, int h2, int out, float *d_params,
                  float *d_adam_m, float *d_adam_v, int64_t step0, const float *d_X,
                  const float *d_T, int64_t nsamples, int batch, int64_t nsteps, float lr,
                  uint64_t seed, float *d_loss_trace);
/* Local-basis emulator: ngroups independent MLPs (one per cell of the parameter space),
   parameter blocks back to back (d_params is ngroups x n).  Training draws batch_per_group
   rows per group and step from the group's samples [h_group_off[g], h_group_off[g+1]) of
   d_X / d_T (samples sorted by group; host offsets, every group non-empty); one Adam
   update covers all groups; d_loss_trace receives the loss averaged over groups. */
int sfh_mlp_train_grouped(sfh_ctx *ctx, int in, int h1, int h2, int out, int64_t ngroups,
                          float *d_params, float *d_adam_m, float *d_adam_v, int64_t step0,
                          const float *d_X, const float *d_T, const int64_t *h_group_off,
                          int batch_per_group, int64_t nsteps, float lr, uint64_t seed,
                          float *d_loss_trace);
/* d_Y (B x out): row b through the MLP of group d_group[b] (d_group may be NULL when
   ngroups == 1).  Same BF16-operand arithmetic as training.  Enqueued, not synchronised. */
int sfh_mlp_forward_rows(sfh_ctx *ctx, int in, int h1, int h2, int out, const float *d_params,
                         int64_t ngroups, const float *d_X, const int32_t *d_group, int64_t B,
                         float *d_Y);
/* As sfh_emu_reconstruct with one basis (ngroups x K x nbins) and offset (ngroups x nbins)
   per group; row b uses group d_group[b].  B <= 65535.  Enqueued, not synchronised. */
int sfh_emu_reconstruct_rows(sfh_ctx *ctx, const float *d_coef, const int32_t *d_group,
                             int64_t ngroups, const float *d_basis, const float *d_offset, int K,
                             int64_t nbins, int64_t B, int mode, float *d_out);
/* As sfh_emu_reconstruct_rows, one group's rows at a time: segment s (d_seg[3s..3s+2] =
   group, start, count; 1 <= count <= 16) builds rows d_rows[start .. start + count) from
   group `group`'s basis, read once for the whole segment.  d_rows holds row indices of d_out
   (0 <= row < B), normally sorted by group.  nseg <= 65535, K <= 1024.  A segment whose
   group, start or count is out of range writes NaN to the rows it can address; a row index
   outside [0, B) ends its segment there (the segment's later rows are not written).
   Enqueued, not synchronised. */
int sfh_emu_reconstruct_groups(sfh_ctx *ctx, const float *d_coef, const int32_t *d_rows,
                               const int32_t *d_seg, int64_t nseg, int64_t ngroups,
                               const float *d_basis, const float *d_offset, int K,
                               int64_t nbins, int64_t B, int mode, float *d_out);
/* d_C (M x N) = alpha op(A) op(B) (+ d_C when accum), FP32 accumulation, ta / tb select
   row-major A (M x K) / (K x M) and B (K x N) / (N x K); bf16 != 0 rounds the operands to
   BF16 first.  Used for the PCA basis (randomized range finder) and projections. */
int sfh_gemm_f32(sfh_ctx *ctx, const float *d_A, const float *d_B, float *d_C, int64_t M,
                 int64_t N, int64_t K, int ta, int tb, int accum, float alpha, int bf16);
/* In place on d_Y (rows templates x cols bins): transform (mode 1: sqrt; mode 0: none),
   column mean into d_mean (cols), then centre the rows on it. */
int sfh_emu_prepare(sfh_ctx *ctx, float *d_Y, int64_t rows, int64_t cols, int mode,
                    float *d_mean);
/* Templates from coefficients: d_out (B x nbins) = inverse transform of
   (d_offset + d_coef (B x K) d_basis (K x nbins)), clamped at 0 (mode 1 squares). */
int sfh_emu_reconstruct(sfh_ctx *ctx, const float *d_coef, const float *d_basis,
                        const float *d_offset, int K, int64_t nbins, int64_t B, int mode,
                        float *d_out);
/* Score: d_dev[t] = 2 sum_i (e - x + x log(x / e)) / sum_i x for exact x = d_exact[t, :],
   emulated e = d_emul[t, :] (floored at 1e-30), in FP64; B x nbins row-major inputs. */
int sfh_poisson_deviance(sfh_ctx *ctx, const float *d_exact, const float *d_emul,
                         int64_t nbins, int B, double *d_dev);

#ifdef __cplusplus
}
#endif
#endif
