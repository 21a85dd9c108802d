/*
 * sfh_oracle.h -- FP64 CPU restatement of the StarFormationHistories.jl v1.3.1
 * Hess-diagram hot path.  TEST INFRASTRUCTURE ONLY: this library is the checker
 * that the CUDA library is compared against (tests/, __graft_entry__.smoke() and
 * the cpu_baseline leg of bench.py).  Nothing in the product links or calls it.
 *
 * Every function names the reference file:line it restates.  Arrays are
 * column-major like Julia; indices inside the template functions follow the
 * reference's 1-based pixel arithmetic so that rounding and window clipping
 * match it exactly.
 */
#ifndef SFH_ORACLE_H
#define SFH_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- fitting_base.jl / solvers.jl ---------------- */
/* composite!(composite, coeffs, models) flat form, src/fitting/fitting_base.jl:55-65 */
void sfho_composite(const double *M, int64_t nbins, int64_t nt, const double *r, double *out);
/* loglikelihood(composite, data), src/fitting/fitting_base.jl:84-96; eps = eps(T) */
double sfho_loglikelihood(const double *c, const double *n, int64_t nbins, double eps);
/* ∇loglikelihood(model, composite, data) single model, src/fitting/fitting_base.jl:144-160 */
double sfho_grad_single(const double *model, const double *c, const double *n, int64_t nbins, double eps);
/* ∇loglikelihood!(G, composite, models, data) flat form, src/fitting/fitting_base.jl:265-285.
   Overwrites c with 1 - n/max(c,eps). */
void sfho_grad_inplace(double *G, double *c, const double *M, const double *n,
                       int64_t nbins, int64_t nt, double eps);
/* fg!(F, G, coeffs, models, data, composite), src/fitting/solvers.jl:20-38.
   want_f/want_g select the F/G branches; returns -logL when want_f. */
double sfho_fg(int want_f, double *G, const double *r, const double *M, const double *n,
               double *c, int64_t nbins, int64_t nt, double eps);
/* Batched fg: B independent coefficient vectors R[b*nt + j]; negLogL[b], G[b*nt + j].
   OpenMP over vectors (used as the CPU baseline for the batched form). */
void sfho_fg_batched(const double *R, int64_t B, const double *M, const double *n,
                     int64_t nbins, int64_t nt, double eps, double *negLogL, double *G,
                     int nthreads);

/* ---------------- StarFormationHistories.jl templates ---------------- */
/* mini_spacing(m_ini, colors, mags, Δmag, true), src/StarFormationHistories.jl:110-148.
   Writes up to cap masses to out; returns the count (or -(needed) if cap too small). */
int64_t sfho_mini_spacing(const double *m_ini, const double *colors, const double *mags,
                          int64_t n, double dmag, double *out, int64_t cap);
/* interpolate_mini(m_ini, mags, new_mini), src/StarFormationHistories.jl:77-81
   (sort_ingested src/simulate.jl:54-63 + Gridded(Linear()) interpolation). */
void sfho_interpolate_mini(const double *m_ini, const double *mags, int64_t n,
                           const double *new_mini, int64_t nn, double *out);
/* midpoints(v), src/StarFormationHistories.jl:417-436 (element form). */
void sfho_midpoints(const double *v, int64_t n, double *out);
/* histogram_pix(d, edges::AbstractRange), src/StarFormationHistories.jl:502 */
double sfho_histogram_pix(double d, double first, double step);
/* gaussian_int_general (verf form), src/StarFormationHistories.jl:198-205 */
double sfho_gaussian_int_general(double dx, double dy, double hx, double hy,
                                 double sx, double sy, double A, double B);
/* gaussian_psf_covariant, src/StarFormationHistories.jl:315-334 */
double sfho_gaussian_psf_covariant(double x, double y, double hx, double hy, double x0,
                                   double y0, double sx, double sy, double cov, double A,
                                   double B);
/* addstar!(image, GaussianPSFAsymmetric, cutout), src/StarFormationHistories.jl:348-364 */
void sfho_addstar_asym(double *img, int64_t nx, int64_t ny, double x0, double y0,
                       double sx, double sy, double A, double B, int64_t cut_x,
                       int64_t cut_y);
/* addstar!(hist, GaussianPSFCovariant, cutout), src/StarFormationHistories.jl:366-408 */
void sfho_addstar_cov(double *img, int64_t nx, int64_t ny, double xfirst, double xstep,
                      double yfirst, double ystep, double x0, double y0, double sx,
                      double sy, double cov, double A, double cut_x, double cut_y);
/* bin_cmd_smooth(colors, mags, color_err, mag_err, cov_mult; weights, edges),
   src/StarFormationHistories.jl:574-621.  out is nx*ny, zeroed here. */
void sfho_bin_cmd_smooth(const double *x, const double *y, const double *sx,
                         const double *sy, const double *w, int64_t npts, int cov_mult,
                         double xfirst, double xstep, int64_t nx, double yfirst,
                         double ystep, int64_t ny, double *out);

/* Parametric callables for partial_cmd_smooth (the reference takes arbitrary
   Julia callables; the C boundary takes these closed forms instead). */
typedef struct {
    /* exp_photerr(m, a, b, c, d) = a^(b*(m-c)) + d, src/utilities.jl:218,
       optionally capped: min(., cap) as in test/templates/template_test.jl:75-77 */
    double a, b, c, d, cap;
} sfho_err_model;
typedef struct {
    /* Martin2016_complete(m, A, m50, rho) = A / (1 + exp((m-m50)/rho)), src/utilities.jl:205 */
    double A, m50, rho;
} sfho_compl_model;
typedef struct {
    /* Continuous broken power law dN/dm ∝ m^-alpha_k, normalised on [mmin, mmax].
       Kroupa (2001) with bounds (0.08, 100): nseg=2, breaks {0.5}, alpha {1.3, 2.3}. */
    int nseg;
    double mmin, mmax;
    double breaks[3];
    double alpha[4];
} sfho_imf;
double sfho_imf_pdf(const sfho_imf *imf, double m);
double sfho_imf_mean(const sfho_imf *imf);

/* calculate_weights, src/StarFormationHistories.jl:765-776 */
void sfho_calculate_weights(const double *mini, const double *completeness, int64_t n,
                            const sfho_imf *imf, double normalize_value, double mean_mass,
                            const double *spacing, double *out);

/* partial_cmd_smooth single-star branch, src/StarFormationHistories.jl:829-888.
   mags is nf*n (filter f at mags + f*n), y_index / c1 / c2 are 0-based, bias is a
   constant per filter (bias_funcs returning constants).  Returns the number of
   smoothed points used (N-1), or a negative value on error.  out is nx*ny. */
int64_t sfho_partial_cmd_smooth(const double *m_ini, const double *mags, int64_t n, int nf,
                                int y_index, int c1, int c2, const sfho_err_model *err,
                                const sfho_compl_model *compl_, const double *bias,
                                const sfho_imf *imf, double dmod, double normalize_value,
                                double mean_mass, double xfirst, double xstep, int64_t nx,
                                double yfirst, double ystep, int64_t ny, double *out);

/* bin_cmd, src/StarFormationHistories.jl:544-553 (StatsBase left-closed histogram on the
   stored edge values: xedges has nx + 1 increasing values, yedges ny + 1; w NULL means unit
   weights).  out is nx*ny. */
void sfho_bin_cmd(const double *x, const double *y, const double *w, int64_t n,
                  const double *xedges, int64_t nx, const double *yedges, int64_t ny,
                  double *out);
/* partial_cmd (error-free template), src/StarFormationHistories.jl:733-757. */
int sfho_partial_cmd(const double *m_ini, const double *colors, const double *mags, int64_t n,
                     const sfho_imf *imf, double dmod, double normalize_value, double mean_mass,
                     const double *xedges, int64_t nx, const double *yedges, int64_t ny,
                     double *out);

/* ---------------- binary-star templates ---------------- */
/* mag2flux / flux2mag with zero point 0, src/utilities.jl:57, 67 */
double sfho_mag2flux(double m);
double sfho_flux2mag(double f);
/* Trapz.jl trapz(x, y) (trapezoidal rule), used at StarFormationHistories.jl:642, 907 */
double sfho_trapz(const double *x, const double *y, int64_t n);
/* binary_hess(RandomBinaryPairs, m_ini, mags, ...), src/StarFormationHistories.jl:627-706,
   for y_index in color_indices (the only case the reference implements; -2 otherwise).
   mags is nf*n (filter f at mags + f*n, distance modulus already added), bias constant per
   filter, edges increasing.  out is nx*ny. */
int sfho_binary_hess(const double *m_ini, const double *mags, int64_t n, int nf, int y_index,
                     int c1, int c2, const sfho_err_model *err, const sfho_compl_model *compl_,
                     const double *bias, const sfho_imf *imf, double normalize_value,
                     double mean_mass, double xfirst, double xstep, int64_t nx, double yfirst,
                     double ystep, int64_t ny, double *out);
/* partial_cmd_smooth with binary_model = RandomBinaryPairs(binary_fraction),
   src/StarFormationHistories.jl:829-910. */
int sfho_partial_cmd_smooth_binary(const double *m_ini, const double *mags, int64_t n, int nf,
                                   int y_index, int c1, int c2, const sfho_err_model *err,
                                   const sfho_compl_model *compl_, const double *bias,
                                   const sfho_imf *imf, double dmod, double normalize_value,
                                   double mean_mass, double binary_fraction, double xfirst,
                                   double xstep, int64_t nx, double yfirst, double ystep,
                                   int64_t ny, double *out);

/* ---------------- hierarchical MZR (src/fitting/hierarchical) ---------------- */
/* PowerLawMZR(α, MH0, logMstar0)(Mstar), mzr.jl:275 */
double sfho_powerlaw_mzr(double alpha, double MH0, double logMstar0, double Mstar);
/* GaussianDispersion(σ)(x, μ), dispersion_models.jl:92 */
double sfho_gauss_disp(double sigma, double x, double mu);
/* calculate_coeffs(PowerLawMZR, GaussianDispersion, mstars, logAge, MH), mzr.jl:50-79 */
int sfho_mzr_calculate_coeffs(double alpha, double MH0, double logMstar0, double sigma,
                              const double *mstars, int64_t nages, const double *logAge,
                              const double *MH, int64_t nt, double *coeffs);
/* fg!(F, G, PowerLawMZR, GaussianDispersion, variables, ...), mzr.jl:84-215.
   variables = [R_1..R_nages, α, MH0, σ]; G has nages+3 entries (free params only
   are written; fixed ones are left 0).  Returns -logL. */
double sfho_mzr_fg(const double *variables, int64_t nages, double logMstar0,
                   int alpha_free, int MH0_free, int sigma_free, const double *M,
                   const double *n, int64_t nbins, int64_t nt, const double *logAge,
                   const double *MH, double eps, double *G);

/* LinearAMR(α, β, T_max)(logAge), amr.jl:205 */
double sfho_linear_amr(double alpha, double beta, double T_max, double logAge);
/* MH_from_Z / dMH_dZ with the package defaults, src/utilities.jl:117-155 */
double sfho_mh_from_z(double Z);
double sfho_dmh_dz(double Z);
/* fg! for an AMR + GaussianDispersion, amr.jl:78-160: kind 0 LinearAMR (amr.jl:205-213),
   kind 1 LogarithmicAMR with MH_from_Z (amr.jl:278-290).  variables = [R_1..R_nages, α, β,
   σ], ages in order of first appearance in logAge.  Returns -logL. */
double sfho_amr_fg(int kind, const double *variables, int64_t nages, double T_max,
                   int alpha_free, int beta_free, int sigma_free, const double *M,
                   const double *n, int64_t nbins, int64_t nt, const double *logAge,
                   const double *MH, double eps, double *G);

/* ---------------- learned template emulator (no reference counterpart) ---------------- */
/* MLP in -> h1 -> h2 -> out with GELU (erf form) after the two hidden layers.
   Parameter block (row-major): W1 (h1 x in), b1 (h1), W2 (h2 x h1), b2 (h2),
   W3 (out x h2), b3 (out).  Z1 = X W1^T + b1, A1 = gelu(Z1), ..., Y = A2 W3^T + b3.
   bf16 != 0 rounds every matmul operand to BF16 (round to nearest even, through
   FP32) before the FP64 products, as the device kernels do. */
int64_t sfho_mlp_param_count(int in, int h1, int h2, int out);
void sfho_mlp_forward(int in, int h1, int h2, int out, const double *params, const double *X,
                      int64_t B, int bf16, double *Y);
/* MSE loss mean((Y - T)^2) over B x out and its gradient w.r.t. params. */
double sfho_mlp_loss_grad(int in, int h1, int h2, int out, const double *params,
                          const double *X, const double *T, int64_t B, int bf16, double *grad);
/* Poisson deviance per star 2 sum(e - t + t log(t/e)) / sum(t), e floored at 1e-30. */
double sfho_poisson_deviance(const double *exact, const double *emul, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
