/*
 * sfh_oracle.c -- FP64 CPU restatement of the StarFormationHistories.jl v1.3.1
 * Hess-diagram hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / reference arm are the only callers.  The product
 * (the CUDA C-ABI library) never links or calls it.
 *
 * Parity pins: the known-answer values of test/fitting/fitting_core_test.jl:9-195,
 * the doctests of src/StarFormationHistories.jl:55-75 and :485-500,
 * src/fitting/hierarchical/dispersion_models.jl:63-67 and mzr.jl:245-249 and the
 * properties of test/templates/template_test.jl:10-33 are checked against this file
 * by tests/test_oracle_kats.py.  Template values themselves are not pinned by the
 * reference's tests (template_test.jl:55-108 is structural only), and the erf the
 * reference uses (SpecialFunctions.jl / VectorizationBase.verf, not vendored) is
 * replaced by C99 erf here.
 */
#include "sfh_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;
void sfho_set_threads(int n) { g_threads = n > 0 ? n : 1; }
int sfho_get_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ======================= fitting_base.jl ======================= */

/* composite! flat form: mul!(composite, models, coeffs), fitting_base.jl:55-65.
   Column-major gemv, bins split across threads. */
void sfho_composite(const double *M, int64_t nbins, int64_t nt, const double *r, double *out) {
    const int64_t chunk = 4096;
    const int64_t nchunks = (nbins + chunk - 1) / chunk;
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t c = 0; c < nchunks; ++c) {
        const int64_t i0 = c * chunk;
        const int64_t i1 = i0 + chunk < nbins ? i0 + chunk : nbins;
        for (int64_t i = i0; i < i1; ++i) out[i] = 0.0;
        for (int64_t j = 0; j < nt; ++j) {
            const double rj = r[j];
            const double *col = M + j * nbins;
            for (int64_t i = i0; i < i1; ++i) out[i] += col[i] * rj;
        }
    }
}

/* loglikelihood(composite, data), fitting_base.jl:84-96.
   ci = max(c, eps(T)); ni > 0 ? ni - ci - ni*log(ni/ci) : -ci; 0 -> -typemax(T). */
double sfho_loglikelihood(const double *c, const double *n, int64_t nbins, double eps) {
    double result = 0.0;
#pragma omp parallel for num_threads(g_threads) reduction(+ : result) schedule(static)
    for (int64_t i = 0; i < nbins; ++i) {
        const double ci = c[i] > eps ? c[i] : eps;
        const double ni = n[i];
        result += (ni > 0.0) ? (ni - ci - ni * log(ni / ci)) : -ci;
    }
    return result != 0.0 ? result : -INFINITY; /* -typemax(T) */
}

/* ∇loglikelihood(model, composite, data), fitting_base.jl:144-160 */
double sfho_grad_single(const double *model, const double *c, const double *n, int64_t nbins,
                        double eps) {
    double result = 0.0;
    for (int64_t i = 0; i < nbins; ++i) {
        const double ci = c[i] > eps ? c[i] : eps;
        result += -model[i] * (1.0 - n[i] / ci);
    }
    return result;
}

/* ∇loglikelihood! flat form, fitting_base.jl:265-285:
   composite .= 1 - n/max(c,eps); G = -Mᵀ composite. */
void sfho_grad_inplace(double *G, double *c, const double *M, const double *n, int64_t nbins,
                       int64_t nt, double eps) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t i = 0; i < nbins; ++i) {
        const double ci = c[i] > eps ? c[i] : eps;
        c[i] = 1.0 - n[i] / ci;
    }
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t j = 0; j < nt; ++j) {
        const double *col = M + j * nbins;
        double acc = 0.0;
        for (int64_t i = 0; i < nbins; ++i) acc += col[i] * c[i];
        G[j] = -acc;
    }
}

/* fg!(F, G, coeffs, models, data, composite), solvers.jl:20-38 */
double sfho_fg(int want_f, double *G, const double *r, const double *M, const double *n,
               double *c, int64_t nbins, int64_t nt, double eps) {
    sfho_composite(M, nbins, nt, r, c);
    double nlogl = 0.0;
    if (want_f) nlogl = -sfho_loglikelihood(c, n, nbins, eps);
    if (G) {
        sfho_grad_inplace(G, c, M, n, nbins, nt, eps);
        for (int64_t j = 0; j < nt; ++j) G[j] = -G[j];
    }
    return nlogl;
}

/* B independent fg! evaluations (the reference evaluates them one at a time from
   threads with task-local composite buffers, hmc_sample.jl:127).  OpenMP over
   vectors; each thread owns one composite buffer. */
void sfho_fg_batched(const double *R, int64_t B, const double *M, const double *n,
                     int64_t nbins, int64_t nt, double eps, double *negLogL, double *G,
                     int nthreads) {
    const int saved = g_threads;
    g_threads = 1;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        double *c = (double *)malloc(sizeof(double) * (size_t)nbins);
#pragma omp for schedule(dynamic, 1)
        for (int64_t b = 0; b < B; ++b)
            negLogL[b] = sfho_fg(1, G ? G + b * nt : NULL, R + b * nt, M, n, c, nbins, nt, eps);
        free(c);
    }
    g_threads = saved;
}

/* ======================= templates ======================= */

static int cmp_idx_by_key(const void *a, const void *b, void *ctx) {
    const double *key = (const double *)ctx;
    const int64_t ia = *(const int64_t *)a, ib = *(const int64_t *)b;
    if (key[ia] < key[ib]) return -1;
    if (key[ia] > key[ib]) return 1;
    return (ia > ib) - (ia < ib); /* stable */
}

/* Stable argsort (Julia's default sortperm is stable). Insertion sort keeps this
   dependency-free; isochrones are a few hundred points. */
static void stable_argsort(const double *key, int64_t n, int64_t *idx) {
    for (int64_t i = 0; i < n; ++i) idx[i] = i;
    for (int64_t i = 1; i < n; ++i) {
        const int64_t v = idx[i];
        int64_t j = i - 1;
        while (j >= 0 && cmp_idx_by_key(&idx[j], &v, (void *)key) > 0) {
            idx[j + 1] = idx[j];
            --j;
        }
        idx[j + 1] = v;
    }
}

/* mini_spacing, StarFormationHistories.jl:110-148.  new_mini starts with
   first(m_ini) of the *unsorted* input (:117), then walks the mass-sorted
   isochrone inserting ceil(d/Δmag) points per long CMD segment (:128-134), and
   finally keeps unique entries in first-appearance order (:141). */
int64_t sfho_mini_spacing(const double *m_ini, const double *colors, const double *mags,
                          int64_t n, double dmag, double *out, int64_t cap) {
    if (n <= 0) return 0;
    int64_t *idx = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    stable_argsort(m_ini, n, idx);
    /* first pass: count */
    int64_t count = 1;
    for (int64_t k = 0; k + 1 < n; ++k) {
        const int64_t i = idx[k], i1 = idx[k + 1];
        const double diffi = hypot(colors[i1] - colors[i], mags[i1] - mags[i]);
        count += (diffi > dmag) ? (int64_t)ceil(diffi / dmag) : 1;
    }
    double *tmp = (double *)malloc(sizeof(double) * (size_t)count);
    int64_t p = 0;
    tmp[p++] = m_ini[0];
    for (int64_t k = 0; k + 1 < n; ++k) {
        const int64_t i = idx[k], i1 = idx[k + 1];
        const double diffi = hypot(colors[i1] - colors[i], mags[i1] - mags[i]);
        if (diffi > dmag) {
            const int64_t npoints = (int64_t)ceil(diffi / dmag);
            const double mass_step = (m_ini[i1] - m_ini[i]) / (double)npoints;
            for (int64_t j = 1; j <= npoints; ++j) tmp[p++] = m_ini[i] + mass_step * (double)j;
        } else {
            tmp[p++] = m_ini[i1];
        }
    }
    free(idx);
    /* unique(): keep first appearance.  Values produced above are non-decreasing
       for sorted input, so a duplicate can only repeat an earlier value; a linear
       scan against all kept values keeps the general semantics. */
    int64_t u = 0;
    for (int64_t k = 0; k < p; ++k) {
        int dup = 0;
        for (int64_t q = u - 1; q >= 0; --q) {
            if (tmp[q] == tmp[k]) { dup = 1; break; }
            if (tmp[q] < tmp[k]) break; /* sorted prefix: no earlier equal value */
        }
        if (!dup) tmp[u++] = tmp[k];
    }
    if (u > cap) { free(tmp); return -u; }
    memcpy(out, tmp, sizeof(double) * (size_t)u);
    free(tmp);
    return u;
}

/* interpolate_mini, StarFormationHistories.jl:77-81.  sort_ingested
   (src/simulate.jl:54-63) sorts by mass and de-duplicates repeated knots
   (Interpolations.deduplicate_knots!: a repeated knot becomes nextfloat of the
   previous one), then Gridded(Linear()) evaluates inside the knot range. */
void sfho_interpolate_mini(const double *m_ini, const double *mags, int64_t n,
                           const double *new_mini, int64_t nn, double *out) {
    int64_t *idx = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    double *k = (double *)malloc(sizeof(double) * (size_t)n);
    double *v = (double *)malloc(sizeof(double) * (size_t)n);
    stable_argsort(m_ini, n, idx);
    for (int64_t i = 0; i < n; ++i) { k[i] = m_ini[idx[i]]; v[i] = mags[idx[i]]; }
    double last = k[0];
    for (int64_t i = 1; i < n; ++i) {
        if (k[i] == last) k[i] = nextafter(k[i - 1], INFINITY);
        else last = k[i];
    }
    for (int64_t q = 0; q < nn; ++q) {
        const double x = new_mini[q];
        /* searchsortedlast-style bracket */
        int64_t lo = 0, hi = n - 1;
        if (x <= k[0]) { out[q] = v[0]; continue; }
        if (x >= k[n - 1]) { out[q] = v[n - 1]; continue; }
        while (hi - lo > 1) {
            const int64_t mid = (lo + hi) / 2;
            if (k[mid] <= x) lo = mid; else hi = mid;
        }
        const double t = (x - k[lo]) / (k[hi] - k[lo]);
        out[q] = v[lo] * (1.0 - t) + v[hi] * t;
    }
    free(idx); free(k); free(v);
}

/* midpoints(v), StarFormationHistories.jl:417-436: v[i] + diff(v)[i]/2.  (The
   range form taken when all steps are isapprox-equal differs by rounding only.) */
void sfho_midpoints(const double *v, int64_t n, double *out) {
    for (int64_t i = 0; i + 1 < n; ++i) out[i] = v[i] + (v[i + 1] - v[i]) / 2.0;
}

/* histogram_pix(d, edges::AbstractRange), StarFormationHistories.jl:502 */
double sfho_histogram_pix(double d, double first, double step) { return (d - first) / step + 1.0; }

/* gaussian_int_general (verf method), StarFormationHistories.jl:198-205 */
double sfho_gaussian_int_general(double dx, double dy, double hx, double hy, double sx,
                                 double sy, double A, double B) {
    const double sqrt2 = sqrt(2.0);
    return A / 4.0 * (erf((dx - hx) / (sqrt2 * sx)) - erf((dx + hx) / (sqrt2 * sx))) *
               (erf((dy - hy) / (sqrt2 * sy)) - erf((dy + hy) / (sqrt2 * sy))) + B;
}

/* Gauss-Legendre 3-point nodes and weights, StarFormationHistories.jl:303-304 */
static const double GL_X[3] = {-0.7745966692414834, 0.0, 0.7745966692414834};
static const double GL_W[3] = {0.5555555555555556, 0.8888888888888888, 0.5555555555555556};

/* gaussian_psf_covariant, StarFormationHistories.jl:315-334 (B is not added by
   the reference). */
double sfho_gaussian_psf_covariant(double x, double y, double hx, double hy, double x0,
                                   double y0, double sx, double sy, double cov, double A,
                                   double B) {
    (void)B;
    const double dx = x - x0;
    const double prefac = A / 2.0 / sqrt(2.0 * M_PI) / sy;
    const double sqrt2 = sqrt(2.0);
    double result = 0.0;
    for (int k = 0; k < 3; ++k) {
        const double yv = GL_X[k] * hy + y;
        const double yw = GL_W[k] * hy;
        const double Dy = yv - y0;
        const double Dx = dx + Dy * cov;
        result += yw * exp(-(Dy / sy) * (Dy / sy) / 2.0) *
                  (erf((Dx + hx) / sqrt2 / sx) + erf((-Dx + hx) / sqrt2 / sx));
    }
    return result * prefac;
}

/* Julia round(Int, x) is RoundNearest with ties to even: rint() under the default
   FE_TONEAREST mode. */
static inline int64_t jround(double x) { return (int64_t)rint(x); }

/* addstar!(image, ::PixelSpaceKernel, cutout_size), StarFormationHistories.jl:348-364 */
void sfho_addstar_asym(double *img, int64_t nx, int64_t ny, double x0, double y0, double sx,
                       double sy, double A, double B, int64_t cut_x, int64_t cut_y) {
    const int64_t x = jround(x0), y = jround(y0);
    const int64_t xoff = (cut_x / 2) > 1 ? cut_x / 2 : 1;
    const int64_t yoff = (cut_y / 2) > 1 ? cut_y / 2 : 1;
    const int64_t xlo = x - xoff > 1 ? x - xoff : 1, xhi = x + xoff < nx ? x + xoff : nx;
    const int64_t ylo = y - yoff > 1 ? y - yoff : 1, yhi = y + yoff < ny ? y + yoff : ny;
    if (xhi - xlo + 1 > 1 && yhi - ylo + 1 > 1) {
        for (int64_t j = ylo; j <= yhi; ++j)
            for (int64_t i = xlo; i <= xhi; ++i)
                img[(i - 1) + (j - 1) * nx] += sfho_gaussian_int_general(
                    (double)i + 0.5 - x0, (double)j + 0.5 - y0, 0.5, 0.5, sx, sy, A, B);
    }
}

/* histogram_data(x, edges::AbstractRange), StarFormationHistories.jl:518 */
static inline double histogram_data(double x, double first, double step) {
    return (x - 1.0) * step + first;
}

/* addstar!(::Histogram, ::RealSpaceKernel, cutout_size), StarFormationHistories.jl:366-408 */
void sfho_addstar_cov(double *img, int64_t nx, int64_t ny, double xfirst, double xstep,
                      double yfirst, double ystep, double x0, double y0, double sx, double sy,
                      double cov, double A, double cut_x, double cut_y) {
    const int64_t xp = jround(sfho_histogram_pix(x0, xfirst, xstep));
    const int64_t yp = jround(sfho_histogram_pix(y0, yfirst, ystep));
    int64_t xoff = jround(cut_x / xstep / 2.0), yoff = jround(cut_y / ystep / 2.0);
    if (xoff < 1) xoff = 1;
    if (yoff < 1) yoff = 1;
    const int64_t xlo = xp - xoff > 1 ? xp - xoff : 1, xhi = xp + xoff < nx ? xp + xoff : nx;
    const int64_t ylo = yp - yoff > 1 ? yp - yoff : 1, yhi = yp + yoff < ny ? yp + yoff : ny;
    const int64_t lx = xhi - xlo + 1, ly = yhi - ylo + 1;
    if (!(lx > 1 && ly > 1)) return;
    /* range(histogram_data(first+1/2), histogram_data(last+1/2); length=len) */
    const double xr0 = histogram_data((double)xlo + 0.5, xfirst, xstep);
    const double xr1 = histogram_data((double)xhi + 0.5, xfirst, xstep);
    const double yr0 = histogram_data((double)ylo + 0.5, yfirst, ystep);
    const double yr1 = histogram_data((double)yhi + 0.5, yfirst, ystep);
    const double xrs = (xr1 - xr0) / (double)(lx - 1), yrs = (yr1 - yr0) / (double)(ly - 1);
    const double hx = xrs / 2.0, hy = yrs / 2.0;
    for (int64_t jj = 0; jj < ly; ++jj) {
        const double yreal = yr0 + (double)jj * yrs;
        for (int64_t ii = 0; ii < lx; ++ii) {
            const double xreal = xr0 + (double)ii * xrs;
            img[(xlo - 1 + ii) + (ylo - 1 + jj) * nx] +=
                sfho_gaussian_psf_covariant(xreal, yreal, hx, hy, x0, y0, sx, sy, cov, A, 0.0);
        }
    }
}

/* bin_cmd_smooth, StarFormationHistories.jl:574-621 */
void sfho_bin_cmd_smooth(const double *x, const double *y, const double *sx, const double *sy,
                         const double *w, int64_t npts, int cov_mult, double xfirst,
                         double xstep, int64_t nx, double yfirst, double ystep, int64_t ny,
                         double *out) {
    memset(out, 0, sizeof(double) * (size_t)(nx * ny));
    if (cov_mult == 0) {
        for (int64_t i = 0; i < npts; ++i) {
            const double x0 = sfho_histogram_pix(x[i], xfirst, xstep);
            const double y0 = sfho_histogram_pix(y[i], yfirst, ystep);
            const double ssx = sx[i] / xstep, ssy = sy[i] / ystep;
            /* size(GaussianPSFAsymmetric) = (ceil(Int, 10σx), ceil(Int, 10σy)), :247 */
            const int64_t cx = (int64_t)ceil(ssx * 10.0), cy = (int64_t)ceil(ssy * 10.0);
            sfho_addstar_asym(out, nx, ny, x0, y0, ssx, ssy, w[i], 0.0, cx, cy);
        }
    } else {
        for (int64_t i = 0; i < npts; ++i) {
            /* size(GaussianPSFCovariant) = (15σx, 10σy), :293 */
            sfho_addstar_cov(out, nx, ny, xfirst, xstep, yfirst, ystep, x[i], y[i], sx[i], sy[i],
                             (double)cov_mult, w[i], 15.0 * sx[i], 10.0 * sy[i]);
        }
    }
}

/* ---------------- IMF (InitialMassFunctions.Kroupa2001 stand-in) ---------------- */
/* Segment k covers [lo_k, hi_k); the unnormalised density m^-alpha_k is scaled so
   that it is continuous at the breaks. */
static void imf_segments(const sfho_imf *imf, double *lo, double *hi, double *scale) {
    double s = 1.0;
    for (int k = 0; k < imf->nseg; ++k) {
        lo[k] = (k == 0) ? imf->mmin : imf->breaks[k - 1];
        hi[k] = (k == imf->nseg - 1) ? imf->mmax : imf->breaks[k];
        if (k > 0) s *= pow(lo[k], imf->alpha[k] - imf->alpha[k - 1]);
        scale[k] = s;
    }
}
static double powint(double a, double b, double p) { /* ∫_a^b m^p dm */
    if (fabs(p + 1.0) < 1e-14) return log(b / a);
    return (pow(b, p + 1.0) - pow(a, p + 1.0)) / (p + 1.0);
}
static double imf_norm(const sfho_imf *imf, int moment) {
    double lo[4], hi[4], sc[4], tot = 0.0;
    imf_segments(imf, lo, hi, sc);
    for (int k = 0; k < imf->nseg; ++k) tot += sc[k] * powint(lo[k], hi[k], -imf->alpha[k] + moment);
    return tot;
}
double sfho_imf_pdf(const sfho_imf *imf, double m) {
    if (m < imf->mmin || m > imf->mmax) return 0.0;
    double lo[4], hi[4], sc[4];
    imf_segments(imf, lo, hi, sc);
    int k = 0;
    while (k < imf->nseg - 1 && m >= hi[k]) ++k;
    return sc[k] * pow(m, -imf->alpha[k]) / imf_norm(imf, 0);
}
double sfho_imf_mean(const sfho_imf *imf) { return imf_norm(imf, 1) / imf_norm(imf, 0); }

/* calculate_weights, StarFormationHistories.jl:765-776 */
void sfho_calculate_weights(const double *mini, const double *completeness, int64_t n,
                            const sfho_imf *imf, double normalize_value, double mean_mass,
                            const double *spacing, double *out) {
    for (int64_t i = 0; i + 1 < n; ++i) {
        out[i] = spacing[i] * (sfho_imf_pdf(imf, mini[i]) + sfho_imf_pdf(imf, mini[i + 1])) / 2.0;
        out[i] *= completeness[i] * normalize_value / mean_mass;
    }
}

static inline double err_eval(const sfho_err_model *e, double m) {
    double s = pow(e->a, e->b * (m - e->c)) + e->d; /* exp_photerr, src/utilities.jl:218 */
    return s < e->cap ? s : e->cap;
}
static inline double compl_eval(const sfho_compl_model *c, double m) {
    return c->A / (1.0 + exp((m - c->m50) / c->rho)); /* src/utilities.jl:205 */
}

/* partial_cmd_smooth, single-star branch, StarFormationHistories.jl:829-888 */
int64_t sfho_partial_cmd_smooth(const double *m_ini, const double *mags, int64_t n, int nf,
                                int y_index, int c1, int c2, const sfho_err_model *err,
                                const sfho_compl_model *compl_, const double *bias,
                                const sfho_imf *imf, double dmod, double normalize_value,
                                double mean_mass, double xfirst, double xstep, int64_t nx,
                                double yfirst, double ystep, int64_t ny, double *out) {
    if (nf < 2 || nf > 8 || y_index < 0 || y_index >= nf || c1 < 0 || c1 >= nf || c2 < 0 ||
        c2 >= nf || n < 2)
        return -1;
    /* :848-851 colors from the raw isochrone, Δmag = min bin step */
    double *colors = (double *)malloc(sizeof(double) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) colors[i] = mags[c1 * n + i] - mags[c2 * n + i];
    const double dmag = fabs(xstep) < fabs(ystep) ? fabs(xstep) : fabs(ystep);
    /* :852 */
    int64_t cap = 1024;
    double *new_mini = NULL;
    int64_t N;
    for (;;) {
        new_mini = (double *)realloc(new_mini, sizeof(double) * (size_t)cap);
        N = sfho_mini_spacing(m_ini, colors, mags + (int64_t)y_index * n, n, dmag, new_mini, cap);
        if (N >= 0) break;
        cap = -N;
    }
    free(colors);
    double *spacing = (double *)malloc(sizeof(double) * (size_t)N);
    for (int64_t i = 0; i + 1 < N; ++i) spacing[i] = new_mini[i + 1] - new_mini[i];
    /* :854-855 */
    double *imag = (double *)malloc(sizeof(double) * (size_t)(N * nf));
    double *merr = (double *)malloc(sizeof(double) * (size_t)(N * nf));
    for (int f = 0; f < nf; ++f) {
        sfho_interpolate_mini(m_ini, mags + (int64_t)f * n, n, new_mini, N, imag + (int64_t)f * N);
        for (int64_t i = 0; i < N; ++i) {
            imag[f * N + i] += dmod;
            merr[f * N + i] = err_eval(&err[f], imag[f * N + i]);
        }
    }
    double *cerr = (double *)malloc(sizeof(double) * (size_t)N);
    double *compl_v = (double *)malloc(sizeof(double) * (size_t)N);
    int cov_mult;
    if (y_index == c1 || y_index == c2) {
        /* :856-868 covariant case */
        const int xc = (c1 != y_index) ? c1 : c2;
        for (int64_t i = 0; i < N; ++i) {
            cerr[i] = merr[xc * N + i];
            compl_v[i] = compl_eval(&compl_[c1], imag[c1 * N + i]) *
                         compl_eval(&compl_[c2], imag[c2 * N + i]);
        }
        cov_mult = (y_index == c1) ? -1 : 1;
    } else {
        /* :869-881 separable case */
        for (int64_t i = 0; i < N; ++i) {
            const double e1 = merr[c1 * N + i], e2 = merr[c2 * N + i];
            cerr[i] = sqrt(e1 * e1 + e2 * e2);
            compl_v[i] = compl_eval(&compl_[c1], imag[c1 * N + i]) *
                         compl_eval(&compl_[c2], imag[c2 * N + i]) *
                         compl_eval(&compl_[y_index], imag[y_index * N + i]);
        }
        cov_mult = 0;
    }
    double *w = (double *)malloc(sizeof(double) * (size_t)N);
    sfho_calculate_weights(new_mini, compl_v, N, imf, normalize_value, mean_mass, spacing, w);
    /* :884-888 bias shift, midpoints, bin_cmd_smooth */
    double *bc = (double *)malloc(sizeof(double) * (size_t)N);
    double *by = (double *)malloc(sizeof(double) * (size_t)N);
    for (int64_t i = 0; i < N; ++i) {
        const double b1 = imag[c1 * N + i] + (bias ? bias[c1] : 0.0);
        const double b2 = imag[c2 * N + i] + (bias ? bias[c2] : 0.0);
        bc[i] = b1 - b2;
        by[i] = imag[y_index * N + i] + (bias ? bias[y_index] : 0.0);
    }
    const int64_t M1 = N - 1;
    double *mx = (double *)malloc(sizeof(double) * (size_t)(M1 > 0 ? M1 : 1));
    double *my = (double *)malloc(sizeof(double) * (size_t)(M1 > 0 ? M1 : 1));
    double *msx = (double *)malloc(sizeof(double) * (size_t)(M1 > 0 ? M1 : 1));
    double *msy = (double *)malloc(sizeof(double) * (size_t)(M1 > 0 ? M1 : 1));
    sfho_midpoints(bc, N, mx);
    sfho_midpoints(by, N, my);
    sfho_midpoints(cerr, N, msx);
    sfho_midpoints(merr + (int64_t)y_index * N, N, msy);
    sfho_bin_cmd_smooth(mx, my, msx, msy, w, M1, cov_mult, xfirst, xstep, nx, yfirst, ystep, ny,
                        out);
    free(new_mini); free(spacing); free(imag); free(merr); free(cerr); free(compl_v);
    free(w); free(bc); free(by); free(mx); free(my); free(msx); free(msy);
    return M1;
}

/* ======================= binary-star templates ======================= */

/* mag2flux(m, zpt = 0) = exp10(4 (zpt - m) / 10), src/utilities.jl:57 */
double sfho_mag2flux(double m) { return pow(10.0, 4.0 * (0.0 - m) / 10.0); }
/* flux2mag(f, zpt = 0) = zpt - 5 log10(f) / 2, src/utilities.jl:67 */
double sfho_flux2mag(double f) { return 0.0 - 5.0 * log10(f) / 2.0; }

/* Trapz.jl trapz(x, y): the trapezoidal rule Σ (x[i+1] - x[i]) (y[i] + y[i+1]) / 2. */
double sfho_trapz(const double *x, const double *y, int64_t n) {
    double s = 0.0;
    for (int64_t i = 0; i + 1 < n; ++i) s += (x[i + 1] - x[i]) * (y[i] + y[i + 1]) / 2.0;
    return s;
}

/* StatsBase fit(Histogram, ..., edges; closed=:left) on a range with step > 0: the bin k
   (0-based) with first + k step <= v < first + (k+1) step, -1 outside. */
static int64_t hist_bin(double v, double first, double step, int64_t n) {
    if (!(v >= first)) return -1;
    int64_t k = (int64_t)floor((v - first) / step);
    if (k > 0 && v < first + (double)k * step) --k;
    if (v >= first + (double)(k + 1) * step) ++k;
    return (k >= 0 && k < n) ? k : -1;
}

/* searchsortedlast(e, v) - 1 over the n + 1 increasing edge values e: the 0-based bin k with
   e[k] <= v < e[k+1], -1 outside or NaN (StatsBase's left-closed bin index on the stored
   range elements). */
static int64_t edge_bin(double v, const double *e, int64_t n) {
    if (!(v >= e[0]) || !(v < e[n])) return -1;
    int64_t lo = 0, hi = n; /* e[lo] <= v < e[hi] */
    while (hi - lo > 1) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (v >= e[mid]) lo = mid; else hi = mid;
    }
    return lo;
}

/* bin_cmd(colors, mags; weights, edges), src/StarFormationHistories.jl:544-553: StatsBase
   fit(Histogram, (x, y), Weights(w), edges; closed=:left) with xedges (nx + 1 values) and
   yedges (ny + 1).  w NULL means unit weights.  out is nx*ny (column-major), zeroed here. */
void sfho_bin_cmd(const double *x, const double *y, const double *w, int64_t n,
                  const double *xedges, int64_t nx, const double *yedges, int64_t ny,
                  double *out) {
    memset(out, 0, sizeof(double) * (size_t)(nx * ny));
    for (int64_t i = 0; i < n; ++i) {
        const int64_t ix = edge_bin(x[i], xedges, nx), iy = edge_bin(y[i], yedges, ny);
        if (ix >= 0 && iy >= 0) out[ix + nx * iy] += w ? w[i] : 1.0;
    }
}

/* partial_cmd(m_ini, colors, mags, imf; dmod, normalize_value, mean_mass, edges),
   src/StarFormationHistories.jl:733-757: mini_spacing with Δmag 0.01, interpolation,
   trapezoidal IMF weights times normalize_value / mean_mass, bin_cmd of the interval left
   points (magnitudes shifted by dmod).  out is nx*ny. */
int sfho_partial_cmd(const double *m_ini, const double *colors, const double *mags, int64_t n,
                     const sfho_imf *imf, double dmod, double normalize_value, double mean_mass,
                     const double *xedges, int64_t nx, const double *yedges, int64_t ny,
                     double *out) {
    if (n < 2) return -1;
    int64_t cap = 1024, N;
    double *new_mini = NULL;
    for (;;) {
        new_mini = (double *)realloc(new_mini, sizeof(double) * (size_t)cap);
        N = sfho_mini_spacing(m_ini, colors, mags, n, 0.01, new_mini, cap);
        if (N >= 0) break;
        cap = -N;
    }
    double *ic = (double *)malloc(sizeof(double) * (size_t)N);
    double *im = (double *)malloc(sizeof(double) * (size_t)N);
    double *w = (double *)malloc(sizeof(double) * (size_t)N);
    sfho_interpolate_mini(m_ini, colors, n, new_mini, N, ic);
    sfho_interpolate_mini(m_ini, mags, n, new_mini, N, im);
    for (int64_t i = 0; i + 1 < N; ++i) {
        w[i] = (new_mini[i + 1] - new_mini[i]) *
               (sfho_imf_pdf(imf, new_mini[i]) + sfho_imf_pdf(imf, new_mini[i + 1])) / 2.0;
        w[i] *= normalize_value / mean_mass;
        im[i] += dmod;
    }
    sfho_bin_cmd(ic, im, w, N - 1, xedges, nx, yedges, ny, out);
    free(new_mini); free(ic); free(im); free(w);
    return 0;
}

int sfho_binary_hess(const double *m_ini, const double *mags, int64_t n, int nf, int y_index,
                     int c1, int c2, const sfho_err_model *err, const sfho_compl_model *compl_,
                     const double *bias, const sfho_imf *imf, double normalize_value,
                     double mean_mass, double xfirst, double xstep, int64_t nx, double yfirst,
                     double ystep, int64_t ny, double *out) {
    if (nf < 2 || nf > 8 || n < 3 || !(xstep > 0) || !(ystep > 0)) return -1;
    if (!(y_index == c1 || y_index == c2)) return -2; /* :700, not implemented there either */
    /* :637-646 IMF values, pscale = trapz, prefactor, fluxes, mass spacing */
    double *imfv = (double *)malloc(sizeof(double) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) imfv[i] = sfho_imf_pdf(imf, m_ini[i]);
    const double pscale = sfho_trapz(m_ini, imfv, n);
    const double prefac = normalize_value / mean_mass / 4.0 / pscale;
    double *flux = (double *)malloc(sizeof(double) * (size_t)(n * nf));
    for (int64_t k = 0; k < n * nf; ++k) flux[k] = sfho_mag2flux(mags[k]);
    const int64_t ns = n - 1;
    double *hist = (double *)calloc((size_t)(nx * ny), sizeof(double));
    /* :648-664 pairs (i, j > i) of interval left points; :666-675 completeness (covariant
       case: the two colour filters); :677-680 bias, colour, the left-closed histogram */
    for (int64_t i = 0; i < ns; ++i) {
        const double dMp = m_ini[i + 1] - m_ini[i], Mpint = imfv[i] + imfv[i + 1];
        for (int64_t j = i + 1; j < ns; ++j) {
            const double bm1 = sfho_flux2mag(flux[c1 * n + i] + flux[c1 * n + j]);
            const double bm2 = sfho_flux2mag(flux[c2 * n + i] + flux[c2 * n + j]);
            const double bmy = sfho_flux2mag(flux[y_index * n + i] + flux[y_index * n + j]);
            double w = dMp * (m_ini[j + 1] - m_ini[j]) * Mpint * (imfv[j] + imfv[j + 1]) * prefac;
            w *= compl_eval(&compl_[c1], bm1) * compl_eval(&compl_[c2], bm2);
            const double b1 = bm1 + (bias ? bias[c1] : 0.0), b2 = bm2 + (bias ? bias[c2] : 0.0);
            const double by = bmy + (bias ? bias[y_index] : 0.0);
            const int64_t ix = hist_bin(b1 - b2, xfirst, xstep, nx);
            const int64_t iy = hist_bin(by, yfirst, ystep, ny);
            if (ix >= 0 && iy >= 0) hist[ix + nx * iy] += w;
        }
    }
    /* :684-697 nonzero bins as points at the bin centres, errors at the centres */
    int64_t ng = 0;
    for (int64_t k = 0; k < nx * ny; ++k) ng += hist[k] != 0.0;
    double *hx = (double *)malloc(sizeof(double) * (size_t)(ng + 1));
    double *hy = (double *)malloc(sizeof(double) * (size_t)(ng + 1));
    double *hsx = (double *)malloc(sizeof(double) * (size_t)(ng + 1));
    double *hsy = (double *)malloc(sizeof(double) * (size_t)(ng + 1));
    double *hw = (double *)malloc(sizeof(double) * (size_t)(ng + 1));
    const int xc = (c1 != y_index) ? c1 : c2;
    int64_t g = 0;
    for (int64_t k = 0; k < nx * ny; ++k) {
        if (hist[k] == 0.0) continue;
        const int64_t ix = k % nx, iy = k / nx;
        /* bin centres edges[k] + step / 2 with the edge correctly rounded (one fma), as the
           device computes them: a centre is a pixel-rounding tie in bin_cmd_smooth
           (x - first) / step + 1 = k + 1.5, so both must hold the same double */
        const double cx = fma((double)ix, xstep, xfirst) + xstep / 2.0;
        const double cy = fma((double)iy, ystep, yfirst) + ystep / 2.0;
        const double xmag = (y_index == c1) ? cy - cx : cy + cx;
        hx[g] = cx;
        hy[g] = cy;
        hsx[g] = err_eval(&err[xc], xmag);
        hsy[g] = err_eval(&err[y_index], cy);
        hw[g] = hist[k];
        ++g;
    }
    /* :702-704 */
    sfho_bin_cmd_smooth(hx, hy, hsx, hsy, hw, ng, (y_index == c1) ? -1 : 1, xfirst, xstep, nx,
                        yfirst, ystep, ny, out);
    free(imfv); free(flux); free(hist); free(hx); free(hy); free(hsx); free(hsy); free(hw);
    return 0;
}

int sfho_partial_cmd_smooth_binary(const double *m_ini, const double *mags, int64_t n, int nf,
                                   int y_index, int c1, int c2, const sfho_err_model *err,
                                   const sfho_compl_model *compl_, const double *bias,
                                   const sfho_imf *imf, double dmod, double normalize_value,
                                   double mean_mass, double binary_fraction, double xfirst,
                                   double xstep, int64_t nx, double yfirst, double ystep,
                                   int64_t ny, double *out) {
    /* :890-910: single stars, then for a binary fraction f > 0 the binary template of
       every fourth resampled isochrone point, mixed by the binary mass fraction
       2f / (1 + f) (simulate.jl:143, 190) times trapz(new_mini, imf(new_mini)) */
    if (!(binary_fraction >= 0.0 && binary_fraction <= 1.0)) return -1;
    if (sfho_partial_cmd_smooth(m_ini, mags, n, nf, y_index, c1, c2, err, compl_, bias, imf, dmod,
                                normalize_value, mean_mass, xfirst, xstep, nx, yfirst, ystep, ny,
                                out) < 0)
        return -1;
    if (binary_fraction == 0.0) return 0;
    double *colors = (double *)malloc(sizeof(double) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) colors[i] = mags[c1 * n + i] - mags[c2 * n + i];
    const double dmag = fabs(xstep) < fabs(ystep) ? fabs(xstep) : fabs(ystep);
    int64_t cap = 1024, N;
    double *new_mini = NULL;
    for (;;) {
        new_mini = (double *)realloc(new_mini, sizeof(double) * (size_t)cap);
        N = sfho_mini_spacing(m_ini, colors, mags + (int64_t)y_index * n, n, dmag, new_mini, cap);
        if (N >= 0) break;
        cap = -N;
    }
    free(colors);
    double *imag = (double *)malloc(sizeof(double) * (size_t)(N * nf));
    for (int f = 0; f < nf; ++f) {
        sfho_interpolate_mini(m_ini, mags + (int64_t)f * n, n, new_mini, N, imag + (int64_t)f * N);
        for (int64_t i = 0; i < N; ++i) imag[f * N + i] += dmod;
    }
    const int64_t nd = (N + 3) / 4;  /* new_mini[begin:4:end] */
    double *md = (double *)malloc(sizeof(double) * (size_t)nd);
    double *magd = (double *)malloc(sizeof(double) * (size_t)(nd * nf));
    for (int64_t i = 0; i < nd; ++i) {
        md[i] = new_mini[4 * i];
        for (int f = 0; f < nf; ++f) magd[f * nd + i] = imag[f * N + 4 * i];
    }
    double *bin = (double *)malloc(sizeof(double) * (size_t)(nx * ny));
    int rc = sfho_binary_hess(md, magd, nd, nf, y_index, c1, c2, err, compl_, bias, imf,
                              normalize_value, mean_mass, xfirst, xstep, nx, yfirst, ystep, ny, bin);
    if (rc == 0) {
        double *pv = (double *)malloc(sizeof(double) * (size_t)N);
        for (int64_t i = 0; i < N; ++i) pv[i] = sfho_imf_pdf(imf, new_mini[i]);
        const double bmf = 2.0 * binary_fraction / (1.0 + binary_fraction) * sfho_trapz(new_mini, pv, N);
        for (int64_t k = 0; k < nx * ny; ++k) out[k] = out[k] * (1.0 - bmf) + bmf * bin[k];
        free(pv);
    }
    free(new_mini); free(imag); free(md); free(magd); free(bin);
    return rc;
}

/* ======================= hierarchical MZR ======================= */

double sfho_powerlaw_mzr(double alpha, double MH0, double logMstar0, double Mstar) {
    return MH0 + alpha * (log10(Mstar) - logMstar0); /* mzr.jl:275 */
}
double sfho_gauss_disp(double sigma, double x, double mu) {
    const double t = (x - mu) / sigma;
    return exp(-t * t / 2.0); /* dispersion_models.jl:92 */
}

/* unique(logAge) in first-appearance order; jidx[k] = position of logAge[k]. */
static int64_t unique_ages(const double *logAge, int64_t nt, double *uniq, int64_t *jidx) {
    int64_t nu = 0;
    for (int64_t k = 0; k < nt; ++k) {
        int64_t f = -1;
        for (int64_t q = 0; q < nu; ++q)
            if (uniq[q] == logAge[k]) { f = q; break; }
        if (f < 0) { uniq[nu] = logAge[k]; f = nu++; }
        jidx[k] = f;
    }
    return nu;
}

/* sortperm(unique_logAge; rev=true), stable. */
static void argsort_desc(const double *v, int64_t n, int64_t *idx) {
    for (int64_t i = 0; i < n; ++i) idx[i] = i;
    for (int64_t i = 1; i < n; ++i) {
        const int64_t t = idx[i];
        int64_t j = i - 1;
        while (j >= 0 && v[idx[j]] < v[t]) { idx[j + 1] = idx[j]; --j; }
        idx[j + 1] = t;
    }
}

/* cumsum(x[s_idxs])[invperm(s_idxs)], mzr.jl:64 and :140 */
static void cum_mass(const double *x, const int64_t *s_idxs, int64_t n, double *out) {
    double acc = 0.0;
    for (int64_t p = 0; p < n; ++p) {
        acc += x[s_idxs[p]];
        out[s_idxs[p]] = acc;
    }
}

int sfho_mzr_calculate_coeffs(double alpha, double MH0, double logMstar0, double sigma,
                              const double *mstars, int64_t nages, const double *logAge,
                              const double *MH, int64_t nt, double *coeffs) {
    double *uniq = (double *)calloc((size_t)nt, sizeof(double));
    int64_t *jidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)nt);
    const int64_t nu = unique_ages(logAge, nt, uniq, jidx);
    if (nu != nages) { free(uniq); free(jidx); return -1; }
    int64_t *s = (int64_t *)malloc(sizeof(int64_t) * (size_t)nu);
    double *cm = (double *)malloc(sizeof(double) * (size_t)nu);
    double *Asum = (double *)calloc((size_t)nu, sizeof(double));
    argsort_desc(uniq, nu, s);
    cum_mass(mstars, s, nu, cm);
    for (int64_t k = 0; k < nt; ++k) {
        const double mu = sfho_powerlaw_mzr(alpha, MH0, logMstar0, cm[jidx[k]]);
        coeffs[k] = sfho_gauss_disp(sigma, MH[k], mu);
        Asum[jidx[k]] += coeffs[k];
    }
    for (int64_t k = 0; k < nt; ++k) coeffs[k] = coeffs[k] * mstars[jidx[k]] / Asum[jidx[k]];
    free(uniq); free(jidx); free(s); free(cm); free(Asum);
    return 0;
}

/* fg! for PowerLawMZR + GaussianDispersion, mzr.jl:84-215 */
double sfho_mzr_fg(const double *variables, int64_t nages, double logMstar0, int alpha_free,
                   int MH0_free, int sigma_free, const double *M, const double *n,
                   int64_t nbins, int64_t nt, const double *logAge, const double *MH,
                   double eps, double *G) {
    const double alpha = variables[nages], MH0 = variables[nages + 1], sigma = variables[nages + 2];
    double *coeffs = (double *)malloc(sizeof(double) * (size_t)nt);
    if (sfho_mzr_calculate_coeffs(alpha, MH0, logMstar0, sigma, variables, nages, logAge, MH, nt,
                                  coeffs) != 0) {
        free(coeffs);
        return NAN;
    }
    double *c = (double *)malloc(sizeof(double) * (size_t)nbins);
    sfho_composite(M, nbins, nt, coeffs, c);
    const double logL = sfho_loglikelihood(c, n, nbins, eps);
    if (G) {
        const int64_t NG = nages + 3;
        double *fullG = (double *)malloc(sizeof(double) * (size_t)nt);
        sfho_grad_inplace(fullG, c, M, n, nbins, nt, eps); /* ∂logL/∂r_{j,k} */
        double *uniq = (double *)malloc(sizeof(double) * (size_t)nt);
        int64_t *jidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)nt);
        unique_ages(logAge, nt, uniq, jidx);
        int64_t *s = (int64_t *)malloc(sizeof(int64_t) * (size_t)nages);
        double *cm = (double *)malloc(sizeof(double) * (size_t)nages);
        argsort_desc(uniq, nages, s);
        cum_mass(variables, s, nages, cm);
        double *mu = (double *)malloc(sizeof(double) * (size_t)nages);
        double *gmu_a = (double *)malloc(sizeof(double) * (size_t)nages);
        double *dmu_dR = (double *)malloc(sizeof(double) * (size_t)nages);
        for (int64_t j = 0; j < nages; ++j) {
            mu[j] = sfho_powerlaw_mzr(alpha, MH0, logMstar0, cm[j]);
            gmu_a[j] = log10(cm[j]) - logMstar0;          /* ∂μ/∂α */
            dmu_dR[j] = alpha / cm[j] / log(10.0);          /* ∂μ/∂M*, mzr.jl:279-281 */
        }
        double *Ajk = (double *)malloc(sizeof(double) * (size_t)nt);
        double *dA_dsig = (double *)malloc(sizeof(double) * (size_t)nt);
        double *dA_dmu = (double *)malloc(sizeof(double) * (size_t)nt);
        double *dA_dR = (double *)malloc(sizeof(double) * (size_t)nt);
        double *Avec = (double *)calloc((size_t)nages, sizeof(double));
        double *ks_dA_dR = (double *)calloc((size_t)nages, sizeof(double));
        for (int64_t k = 0; k < nt; ++k) {
            const int64_t j = jidx[k];
            const double d = MH[k] - mu[j];
            Ajk[k] = sfho_gauss_disp(sigma, MH[k], mu[j]);
            dA_dsig[k] = Ajk[k] * d * d / (sigma * sigma * sigma); /* dispersion_models.jl:97-101 */
            dA_dmu[k] = Ajk[k] * d / (sigma * sigma);
            dA_dR[k] = dA_dmu[k] * dmu_dR[j];
            Avec[j] += Ajk[k];
            ks_dA_dR[j] += dA_dR[k];
        }
        double *ks_drjk = (double *)calloc((size_t)nages, sizeof(double));
        for (int64_t k = 0; k < nt; ++k) {
            const int64_t j = jidx[k];
            const double drjk = fullG[k] * (variables[j] / Avec[j] *
                                            (dA_dR[k] - Ajk[k] * ks_dA_dR[j] / Avec[j]));
            ks_drjk[j] += drjk;
        }
        /* cum_drjk_dRj = reverse!(cumsum(reverse!(ksum[s_idxs]))), mzr.jl:179 */
        double *cumd = (double *)malloc(sizeof(double) * (size_t)nages);
        double acc = 0.0;
        for (int64_t p = nages - 1; p >= 0; --p) { acc += ks_drjk[s[p]]; cumd[p] = acc; }
        for (int64_t q = 0; q < NG; ++q) G[q] = 0.0;
        for (int64_t p = 1; p < nages; ++p) G[s[p - 1]] -= cumd[p]; /* mzr.jl:185-187 */
        for (int64_t j = 0; j < nages; ++j) {
            const double A = Avec[j], Rj = variables[j];
            double t1 = 0.0, ks_dmu = 0.0, ks_dsig = 0.0;
            for (int64_t k = 0; k < nt; ++k) {
                if (jidx[k] != j) continue;
                t1 += fullG[k] * (coeffs[k] / Rj + (dA_dR[k] - ks_dA_dR[j] * Ajk[k] / A) * Rj / A);
                ks_dmu += dA_dmu[k];
                ks_dsig += dA_dsig[k];
            }
            G[j] -= t1;
            double psum = 0.0, ssum = 0.0;
            for (int64_t k = 0; k < nt; ++k) {
                if (jidx[k] != j) continue;
                psum -= fullG[k] * Rj / A * (dA_dmu[k] - Ajk[k] / A * ks_dmu);
                ssum += fullG[k] * Rj / A * (dA_dsig[k] - Ajk[k] / A * ks_dsig);
            }
            if (alpha_free) G[nages] += psum * gmu_a[j];  /* mzr.jl:198-200 */
            if (MH0_free) G[nages + 1] += psum * 1.0;
            if (sigma_free) G[nages + 2] -= ssum;          /* mzr.jl:203-209 */
        }
        free(fullG); free(uniq); free(jidx); free(s); free(cm); free(mu); free(gmu_a);
        free(dmu_dR); free(Ajk); free(dA_dsig); free(dA_dmu); free(dA_dR); free(Avec);
        free(ks_dA_dR); free(ks_drjk); free(cumd);
    }
    free(coeffs);
    free(c);
    return -logL;
}

/* LinearAMR(α, β, T_max)(logAge) = β + α (T_max - 10^(logAge - 9)), amr.jl:205 */
double sfho_linear_amr(double alpha, double beta, double T_max, double logAge) {
    return beta + alpha * (T_max - pow(10.0, logAge - 9.0));
}

/* fg!(F, G, ::AbstractAMR, ::AbstractDispersionModel, variables, ...), amr.jl:78-160, for
   LinearAMR + GaussianDispersion: calculate_coeffs (amr.jl:50-72), composite, logL, then
   the chain rule to (R_j, α, β, σ) -- no cross-age terms, μ_j depends on age only. */
/* MH_from_Z(Z) and dMH_dZ(Z) with the defaults solZ = 0.01524, Y_p = 0.2485, γ = 1.78,
   src/utilities.jl:117-155 (X = 1 - (Y_p + γ Z + Z)). */
double sfho_mh_from_z(double Z) {
    const double Yp = 0.2485, g = 1.78, solZ = 0.01524;
    const double X = 1.0 - (Yp + g * Z + Z), Xsol = 1.0 - (Yp + g * solZ + solZ);
    return X > 0 ? log10(Z / (X * solZ) * Xsol) : NAN;
}
double sfho_dmh_dz(double Z) {
    const double Yp = 0.2485, g = 1.78;
    return (Yp - 1.0) / (log(10.0) * Z * (Yp + Z + g * Z - 1.0));
}

double sfho_amr_fg(int kind, const double *variables, int64_t nages, double T_max,
                   int alpha_free, int beta_free, int sigma_free, const double *M,
                   const double *n, int64_t nbins, int64_t nt, const double *logAge,
                   const double *MH, double eps, double *G) {
    const double alpha = variables[nages], beta = variables[nages + 1], sigma = variables[nages + 2];
    double *uniq = (double *)malloc(sizeof(double) * (size_t)nt);
    int64_t *jidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)nt);
    const int64_t nu = unique_ages(logAge, nt, uniq, jidx);
    if (nu != nages) {
        free(uniq);
        free(jidx);
        return NAN;
    }
    double *mu = (double *)malloc(sizeof(double) * (size_t)nages);
    double *Avec = (double *)calloc((size_t)nages, sizeof(double));
    double *Ajk = (double *)malloc(sizeof(double) * (size_t)nt);
    double *coeffs = (double *)malloc(sizeof(double) * (size_t)nt);
    for (int64_t j = 0; j < nages; ++j)
        mu[j] = kind == 1 ? sfho_mh_from_z(beta + alpha * (T_max - pow(10.0, uniq[j] - 9.0)))
                          : sfho_linear_amr(alpha, beta, T_max, uniq[j]);
    for (int64_t k = 0; k < nt; ++k) {
        Ajk[k] = sfho_gauss_disp(sigma, MH[k], mu[jidx[k]]);
        Avec[jidx[k]] += Ajk[k];
    }
    for (int64_t k = 0; k < nt; ++k) coeffs[k] = Ajk[k] * variables[jidx[k]] / Avec[jidx[k]];
    double *c = (double *)malloc(sizeof(double) * (size_t)nbins);
    sfho_composite(M, nbins, nt, coeffs, c);
    const double logL = sfho_loglikelihood(c, n, nbins, eps);
    if (G) {
        double *fullG = (double *)malloc(sizeof(double) * (size_t)nt);
        sfho_grad_inplace(fullG, c, M, n, nbins, nt, eps); /* ∂logL/∂r_{j,k} */
        for (int64_t q = 0; q < nages + 3; ++q) G[q] = 0.0;
        for (int64_t j = 0; j < nages; ++j) {
            const double Rj = variables[j], A = Avec[j];
            /* ∂μ/∂α, ∂μ/∂β: LinearAMR amr.jl:207-209; LogarithmicAMR amr.jl:280-288 */
            const double dt = T_max - pow(10.0, uniq[j] - 9.0);
            const double dz = kind == 1 ? sfho_dmh_dz(beta + alpha * dt) : 1.0;
            const double gmu_a = dz * dt, gmu_b = dz;
            double ks_dmu = 0.0, ks_dsig = 0.0;
            for (int64_t k = 0; k < nt; ++k) {
                if (jidx[k] != j) continue;
                const double d = MH[k] - mu[j];
                ks_dmu += Ajk[k] * d / (sigma * sigma);
                ks_dsig += Ajk[k] * d * d / (sigma * sigma * sigma);
            }
            double gR = 0.0, psum = 0.0, ssum = 0.0;
            for (int64_t k = 0; k < nt; ++k) {
                if (jidx[k] != j) continue;
                const double d = MH[k] - mu[j];
                const double dAmu = Ajk[k] * d / (sigma * sigma);
                const double dAs = Ajk[k] * d * d / (sigma * sigma * sigma);
                gR -= fullG[k] * coeffs[k] / Rj;                              /* amr.jl:133 */
                psum -= fullG[k] * Rj / A * (dAmu - Ajk[k] / A * ks_dmu);     /* :143-144 */
                ssum += fullG[k] * Rj / A * (dAs - Ajk[k] / A * ks_dsig);     /* :150-156 */
            }
            G[j] = gR;
            if (alpha_free) G[nages] += psum * gmu_a;
            if (beta_free) G[nages + 1] += psum * gmu_b;
            if (sigma_free) G[nages + 2] -= ssum;
        }
        free(fullG);
    }
    free(uniq); free(jidx); free(mu); free(Avec); free(Ajk); free(coeffs); free(c);
    return -logL;
}

/* ======================= learned template emulator (no reference counterpart) ====== */
/* A plain FP64 restatement of the device MLP: the forward pass, the backward pass of
   the mean-squared-error loss, and the Poisson deviance used as the score. */

static double bf16_round(double x) {
    float f = (float)x;
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) != 0x7F800000u) {
        u += 0x7FFFu + ((u >> 16) & 1u);
        u &= 0xFFFF0000u;
    }
    memcpy(&f, &u, 4);
    return (double)f;
}

static double gelu64(double z) { return 0.5 * z * (1.0 + erf(z / sqrt(2.0))); }
static double gelu64_grad(double z) {
    return 0.5 * (1.0 + erf(z / sqrt(2.0))) + z * exp(-0.5 * z * z) / sqrt(2.0 * M_PI);
}

int64_t sfho_mlp_param_count(int in, int h1, int h2, int out) {
    return (int64_t)h1 * in + h1 + (int64_t)h2 * h1 + h2 + (int64_t)out * h2 + out;
}

/* out (B x n) = rnd(A) (B x k) * rnd(W)^T (n x k) + b */
static void dense(const double *A, const double *W, const double *b, int64_t B, int k, int n,
                  int bf16, double *out) {
    for (int64_t r = 0; r < B; ++r)
        for (int j = 0; j < n; ++j) {
            double s = 0.0;
            for (int i = 0; i < k; ++i) {
                double a = A[r * k + i], w = W[(int64_t)j * k + i];
                if (bf16) { a = bf16_round(a); w = bf16_round(w); }
                s += a * w;
            }
            out[r * n + j] = s + b[j];
        }
}

void sfho_mlp_forward(int in, int h1, int h2, int out, const double *P, const double *X,
                      int64_t B, int bf16, double *Y) {
    const double *W1 = P, *b1 = W1 + (int64_t)h1 * in, *W2 = b1 + h1, *b2 = W2 + (int64_t)h2 * h1,
                 *W3 = b2 + h2, *b3 = W3 + (int64_t)out * h2;
    double *A1 = calloc((size_t)(B * h1), sizeof(double)), *A2 = calloc((size_t)(B * h2), sizeof(double));
    dense(X, W1, b1, B, in, h1, bf16, A1);
    for (int64_t k = 0; k < B * h1; ++k) A1[k] = gelu64(A1[k]);
    dense(A1, W2, b2, B, h1, h2, bf16, A2);
    for (int64_t k = 0; k < B * h2; ++k) A2[k] = gelu64(A2[k]);
    dense(A2, W3, b3, B, h2, out, bf16, Y);
    free(A1);
    free(A2);
}

/* dW (n x k) = rnd(dZ)^T (n x B) rnd(A) (B x k); db = column sums of dZ;
   dA (B x k) = rnd(dZ) (B x n) rnd(W) (n x k) when dA != NULL */
static void dense_back(const double *dZ, const double *A, const double *W, int64_t B, int k, int n,
                       int bf16, double *dW, double *db, double *dA) {
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < k; ++i) {
            double s = 0.0;
            for (int64_t r = 0; r < B; ++r) {
                double g = dZ[r * n + j], a = A[r * k + i];
                if (bf16) { g = bf16_round(g); a = bf16_round(a); }
                s += g * a;
            }
            dW[(int64_t)j * k + i] = s;
        }
    for (int j = 0; j < n; ++j) {
        double s = 0.0;
        for (int64_t r = 0; r < B; ++r) s += dZ[r * n + j];
        db[j] = s;
    }
    if (dA)
        for (int64_t r = 0; r < B; ++r)
            for (int i = 0; i < k; ++i) {
                double s = 0.0;
                for (int j = 0; j < n; ++j) {
                    double g = dZ[r * n + j], w = W[(int64_t)j * k + i];
                    if (bf16) { g = bf16_round(g); w = bf16_round(w); }
                    s += g * w;
                }
                dA[r * k + i] = s;
            }
}

double sfho_mlp_loss_grad(int in, int h1, int h2, int out, const double *P, const double *X,
                          const double *T, int64_t B, int bf16, double *grad) {
    const double *W1 = P, *b1 = W1 + (int64_t)h1 * in, *W2 = b1 + h1, *b2 = W2 + (int64_t)h2 * h1,
                 *W3 = b2 + h2, *b3 = W3 + (int64_t)out * h2;
    double *gW1 = grad, *gb1 = gW1 + (int64_t)h1 * in, *gW2 = gb1 + h1,
           *gb2 = gW2 + (int64_t)h2 * h1, *gW3 = gb2 + h2, *gb3 = gW3 + (int64_t)out * h2;
    double *Z1 = malloc(sizeof(double) * B * h1), *A1 = malloc(sizeof(double) * B * h1);
    double *Z2 = malloc(sizeof(double) * B * h2), *A2 = calloc((size_t)(B * h2), sizeof(double));
    double *Y = malloc(sizeof(double) * B * out), *dA2 = malloc(sizeof(double) * B * h2);
    double *dA1 = malloc(sizeof(double) * B * h1);
    dense(X, W1, b1, B, in, h1, bf16, Z1);
    for (int64_t k = 0; k < B * h1; ++k) A1[k] = gelu64(Z1[k]);
    dense(A1, W2, b2, B, h1, h2, bf16, Z2);
    for (int64_t k = 0; k < B * h2; ++k) A2[k] = gelu64(Z2[k]);
    dense(A2, W3, b3, B, h2, out, bf16, Y);
    const double scale = 1.0 / ((double)B * out);
    double loss = 0.0;
    for (int64_t k = 0; k < B * out; ++k) {
        const double d = Y[k] - T[k];
        loss += d * d * scale;
        Y[k] = 2.0 * d * scale; /* dY */
    }
    dense_back(Y, A2, W3, B, h2, out, bf16, gW3, gb3, dA2);
    for (int64_t k = 0; k < B * h2; ++k) dA2[k] *= gelu64_grad(Z2[k]);
    dense_back(dA2, A1, W2, B, h1, h2, bf16, gW2, gb2, dA1);
    for (int64_t k = 0; k < B * h1; ++k) dA1[k] *= gelu64_grad(Z1[k]);
    dense_back(dA1, X, W1, B, in, h1, bf16, gW1, gb1, NULL);
    free(Z1); free(A1); free(Z2); free(A2); free(Y); free(dA2); free(dA1);
    return loss;
}

double sfho_poisson_deviance(const double *exact, const double *emul, int64_t n) {
    double d = 0.0, tot = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double t = exact[i], e = emul[i] > 1e-30 ? emul[i] : 1e-30;
        d += e - t + (t > 0.0 ? t * log(t / e) : 0.0);
        tot += t;
    }
    return tot > 0.0 ? 2.0 * d / tot : 0.0;
}
