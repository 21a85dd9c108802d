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
   is NULL, 1 - n/c otherwise); composite may be NULL to skip that copy-out. */
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

/* Telemetry: average device time (ms) of each of the four kernels of sfh_fg_dev over
   `iters` evaluations, timed with CUDA events on the context stream:
   ms_out[0] m = M r partials, [1] Poisson terms + w, [2] Mᵀ w partials, [3] G reduction.
   No reference counterpart; used to report the dominant kernel's roofline. */
int sfh_fg_kernel_times(sfh_ctx *ctx, const sfh_models *models, const double *d_coeffs,
                        const double *d_data, double *d_composite, double *d_G,
                        double *d_negLogL, double eps, int iters, double *ms_out);

/* fg! for callers that cannot allocate device memory (no counterpart in the
   reference): graph-capture regions that must not allocate, plugins inside a host
   application that owns the device memory budget, allocation-free real-time loops.
   Same result as sfh_fg_dev on FP32 templates, but all scratch lives in one fixed
   11 MiB device array inside the library, so the call allocates nothing: the caller
   passes the (nbins, ntempl) column-major FP32 templates, every input and output,
   and the stream.  Limits: nbins <= 131072 and ntempl <= 4096 (SFH_ERR_SHAPE beyond).
   The first call on each device looks up the array's device address; make that
   first call before any stream capture.  All calls share the one array, so calls
   that overlap on the GPU (different streams, or different host threads) race:
   serialise them on one stream.  d_G and d_negLogL may be NULL as in sfh_fg_dev. */
int sfh_fg_dev_noalloc(void *stream, const float *d_models, int64_t nbins, int64_t ntempl,
                       const double *d_coeffs, const double *d_data, double *d_composite,
                       double *d_G, double *d_negLogL, double eps);

/* B coefficient vectors in one call (HMC chains, line-search probes):
   d_R[b*ntempl + j] -> d_negLogL[b] (may be NULL: gradient-only substeps skip the
   logarithms) and d_G[b*ntempl + j] = -∂logL/∂r (may be NULL).  Needs models
   stored as SFH_BF16X2 (tensor-core path); |ΔlogL| against FP64 on the same stored
   templates is reported by the tests. */
int sfh_fg_batched_dev(sfh_ctx *ctx, const sfh_models *models, const double *d_R, int64_t B,
                       const double *d_data, double *d_negLogL, float *d_G, double eps);

/* ---------------------------------------------------------------- batched HMC */
enum sfh_hmc_model {
    SFH_HMC_DIRECT = 0, /* θ = log coeffs: hmc_sample's log density, hmc_sample.jl:24-37 */
    SFH_HMC_MZR = 1     /* PowerLawMZR + GaussianDispersion: sample_sfh's log density,
                           generic_fitting.jl:90-199 with mzr.jl:50-215 */
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
    /* SFH_HMC_MZR only: ages and metallicities of the templates */
    int32_t nages;
    const int32_t *h_age_index; /* per template: its age, 0..nages-1 */
    const double *h_logAge;     /* per age (any order) */
    const double *h_MH;         /* per template [M/H] */
    double logMstar0;           /* PowerLawMZR logMstar0 (fixed), mzr.jl:263-272 */
    int32_t alpha_free, beta_free, sigma_free;
    double alpha, beta, sigma;  /* values of parameters held fixed */
} sfh_hmc_config;

/* Batched HMC over all chains at once, every leapfrog step one sfh_fg_batched_dev-style
   evaluation on the tensor cores; replaces the per-chain DynamicHMC loop of hmc_sample
   (hmc_sample.jl:105-141) and sample_sfh (generic_fitting.jl:458-527).  Fixed-length
   trajectories, per-chain dual-averaging step size and a pooled diagonal mass during
   warmup, Metropolis accept.  Device arrays: d_theta0 (nchains x D) starting points in
   the transformed space (D = ntempl for SFH_HMC_DIRECT; nages + free parameters, order
   [log R_j..., log α, β, log σ], for SFH_HMC_MZR).  Outputs (each may be NULL):
   d_mean / d_var (nchains x D) posterior mean and variance of the natural parameters
   (exp of the log-transformed ones), d_accept (nchains) mean acceptance, d_step
   (nchains) final step, d_draws (nchains x ceil(ntraj/thin) x D) FP32 natural draws.
   Models must be stored as SFH_BF16X2.  The call returns after the run completes. */
int sfh_hmc_sample_dev(sfh_ctx *ctx, const sfh_models *models, const double *d_data,
                       const sfh_hmc_config *cfg, const double *d_theta0, double *d_mean,
                       double *d_var, double *d_accept, double *d_step, float *d_draws);

/* Log density and its gradient for B parameter vectors of the same model as
   sfh_hmc_sample_dev (logdensity_and_gradient of hmc_sample.jl:24-37 and
   generic_fitting.jl:90-199 with Jacobian terms), batched on the tensor cores:
   d_theta (B x D, B = cfg->nchains) -> d_logd (B), d_grad (B x D). */
int sfh_logdensity_batched_dev(sfh_ctx *ctx, const sfh_models *models, const double *d_data,
                               const sfh_hmc_config *cfg, const double *d_theta, double *d_logd,
                               double *d_grad);

/* ---------------------------------------------------------------- template construction */
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

#ifdef __cplusplus
}
#endif
#endif
