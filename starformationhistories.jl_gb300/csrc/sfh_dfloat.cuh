// sfh_dfloat.cuh -- double-float arithmetic (value = hi + lo, two FP32 numbers) for the
// per-bin Poisson terms, so that they run on the FP32 pipes.  GB300's FP64 rate is a small
// fraction of its FP32 rate; with these helpers a bin costs a handful of conversions on
// the FP64 pipe instead of an FP64 logarithm.
//
// Error-free transformations: two_sum (Knuth), fast_two_sum (Dekker), two_prod via FMA.
// Logarithm of a float: table-driven reduction (P. T. P. Tang, "Table-driven
// implementation of the logarithm function in IEEE floating-point arithmetic", ACM TOMS
// 16(4), 1990): x = 2^e m, m = F (1 + u) with F = 1 + j/128 nearest to m, |u| <= 2^-8,
// log x = e ln2 + log F + log1p(u), log F from a 129-entry table of float pairs and
// log1p(u) = u - u^2/2 + u^3 (1/3 - u/4 + u^2/5 - u^3/6 + u^4/7) (truncation < 2^-64).
// Host-compilable (the same header is exercised by a host check); additions and products
// use the round-to-nearest intrinsics on the device so no contraction can break the
// error-free transformations.
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>

#ifdef __CUDACC__
#define SFH_DF_HD __host__ __device__ __forceinline__
#else
#define SFH_DF_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define SFH_DF_ADD(a, b) __fadd_rn((a), (b))
#define SFH_DF_SUB(a, b) __fsub_rn((a), (b))
#define SFH_DF_MUL(a, b) __fmul_rn((a), (b))
#define SFH_DF_DIV(a, b) __fdiv_rn((a), (b))
#else
#define SFH_DF_ADD(a, b) ((a) + (b))
#define SFH_DF_SUB(a, b) ((a) - (b))
#define SFH_DF_MUL(a, b) ((a) * (b))
#define SFH_DF_DIV(a, b) ((a) / (b))
#endif

struct sfh_df {
    float h, l;
};

SFH_DF_HD sfh_df df_two_sum(float a, float b) {
    const float s = SFH_DF_ADD(a, b);
    const float bb = SFH_DF_SUB(s, a);
    const float e = SFH_DF_ADD(SFH_DF_SUB(a, SFH_DF_SUB(s, bb)), SFH_DF_SUB(b, bb));
    return sfh_df{s, e};
}
SFH_DF_HD sfh_df df_fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
    const float s = SFH_DF_ADD(a, b);
    return sfh_df{s, SFH_DF_SUB(b, SFH_DF_SUB(s, a))};
}
SFH_DF_HD sfh_df df_two_prod(float a, float b) {
    const float p = SFH_DF_MUL(a, b);
    return sfh_df{p, fmaf(a, b, -p)};
}
SFH_DF_HD sfh_df df_neg(sfh_df a) { return sfh_df{-a.h, -a.l}; }
SFH_DF_HD sfh_df df_add(sfh_df a, sfh_df b) {
    sfh_df s = df_two_sum(a.h, b.h);
    const sfh_df t = df_two_sum(a.l, b.l);
    s = df_fast_two_sum(s.h, SFH_DF_ADD(s.l, t.h));
    return df_fast_two_sum(s.h, SFH_DF_ADD(s.l, t.l));
}
// Sloppy double-float sum (one two_sum on the high parts, low parts added): relative
// error about 2^-44 (|a| + |b|) / |a + b|, so exact enough for sums of like-signed terms
// and for error budgets measured against the sum of magnitudes.
SFH_DF_HD sfh_df df_add_fast(sfh_df a, sfh_df b) {
    const sfh_df s = df_two_sum(a.h, b.h);
    return df_fast_two_sum(s.h, SFH_DF_ADD(s.l, SFH_DF_ADD(a.l, b.l)));
}
SFH_DF_HD sfh_df df_add_f(sfh_df a, float b) {
    const sfh_df s = df_two_sum(a.h, b);
    return df_fast_two_sum(s.h, SFH_DF_ADD(s.l, a.l));
}
SFH_DF_HD sfh_df df_mul(sfh_df a, sfh_df b) {
    const sfh_df p = df_two_prod(a.h, b.h);
    const float c = fmaf(a.h, b.l, SFH_DF_MUL(a.l, b.h));
    return df_fast_two_sum(p.h, SFH_DF_ADD(p.l, c));
}
SFH_DF_HD sfh_df df_mul_f(sfh_df a, float b) {
    const sfh_df p = df_two_prod(a.h, b);
    return df_fast_two_sum(p.h, fmaf(a.l, b, p.l));
}
SFH_DF_HD sfh_df df_div(sfh_df a, sfh_df b) {
    const float q0 = SFH_DF_DIV(a.h, b.h);
    const sfh_df r = df_add(a, df_neg(df_mul_f(b, q0)));
    const float q1 = SFH_DF_DIV(r.h, b.h);
    return df_fast_two_sum(q0, q1);
}

// ln 2 = LN2_HI + LN2_LO with LN2_HI holding 16 significant bits, so e * LN2_HI is exact
// for every float exponent e.
#define SFH_DF_LN2_HI 0.693145751953125f
#define SFH_DF_LN2_LO 1.428606765330187e-06f   // ln2 - LN2_HI rounded to float
#define SFH_DF_LN2_LO2 5.4979230187083712e-14f  // ln2 - LN2_HI - LN2_LO

SFH_DF_HD uint32_t df_bits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}
SFH_DF_HD float df_from_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, 4);
    return x;
#endif
}

// log(x) for a finite float x > 0 as a double-float.  tab holds log(1 + j/128) for
// j = 0..128 as (hi, lo) pairs (sfh_df_log_table fills it).
SFH_DF_HD sfh_df df_log_f(float x, const sfh_df *tab) {
    int e = 0;
    if (x < 1.1754943508e-38f) {  // subnormal: scale into the normal range
        x = SFH_DF_MUL(x, 16777216.0f);
        e = -24;
    }
    const uint32_t u = df_bits(x);
    e += (int)((u >> 23) & 0xffu) - 127;
    const uint32_t mant = u & 0x7fffffu;
    const int j = (int)((mant + (1u << 15)) >> 16);  // nearest j / 128, 0..128
    const float m = df_from_bits(mant | 0x3f800000u);  // [1, 2)
    // F = 1 + j/128 built from its bits (j = 128 gives 2.0): no integer-to-float conversion
    const float F = df_from_bits(0x3f800000u + ((uint32_t)j << 16));
    const float f = SFH_DF_SUB(m, F);                                   // exact, |f| <= 2^-8
    // u = f / F as a double-float
    const float uh = SFH_DF_DIV(f, F);
    const float ul = SFH_DF_DIV(fmaf(-uh, F, f), F);
    // log1p(u) = u - u^2/2 + u^3 (1/3 - u/4 + u^2/5 - u^3/6 + u^4/7)
    sfh_df u2 = df_two_prod(uh, uh);
    u2.l = fmaf(SFH_DF_ADD(uh, uh), ul, u2.l);
    float p = fmaf(uh, 1.0f / 7.0f, -1.0f / 6.0f);
    p = fmaf(uh, p, 0.2f);
    p = fmaf(uh, p, -0.25f);
    p = fmaf(uh, p, 1.0f / 3.0f);
    p = SFH_DF_MUL(SFH_DF_MUL(SFH_DF_MUL(uh, uh), uh), p);
    sfh_df s = df_two_sum(uh, SFH_DF_MUL(-0.5f, u2.h));
    s = df_fast_two_sum(s.h, SFH_DF_ADD(s.l, SFH_DF_ADD(SFH_DF_SUB(ul, SFH_DF_MUL(0.5f, u2.l)), p)));
    // (float)e exactly from bits: 1.5 * 2^23 + e (|e| < 2^22) minus 1.5 * 2^23
    const float fe = SFH_DF_SUB(df_from_bits(0x4b400000u + (uint32_t)e), 12582912.0f);
    sfh_df le = df_fast_two_sum(SFH_DF_MUL(fe, SFH_DF_LN2_HI),
                                fmaf(fe, SFH_DF_LN2_LO, SFH_DF_MUL(fe, SFH_DF_LN2_LO2)));
    return df_add(df_add(le, tab[j]), s);
}

#ifdef __CUDACC__
// log(x) for a finite float x >= 2^-126 as a double-float, the same reduction as df_log_f
// with fewer instructions: the quotient u = f / F from a fast approximate division whose
// residual f - u F is exact by FMA (so u_hi + u_lo keeps the double-float accuracy), and
// the final sum assembled from two error-free sums.  For kernels that take many
// logarithms per element (the batched epilogue).
__device__ __forceinline__ sfh_df df_log_f_fast(float x, const sfh_df *tab) {
    const uint32_t u = __float_as_uint(x);
    const int e = (int)((u >> 23) & 0xffu) - 127;
    const uint32_t mant = u & 0x7fffffu;
    const int j = (int)((mant + (1u << 15)) >> 16);
    const float m = __uint_as_float(mant | 0x3f800000u);
    const float F = __uint_as_float(0x3f800000u + ((uint32_t)j << 16));
    const float f = __fsub_rn(m, F);                         // exact, |f| <= 2^-8
    const float uh = __fdividef(f, F);
    const float ul = __fdividef(__fmaf_rn(-uh, F, f), F);    // residual exact, then divided
    // log1p(u) = u - u^2/2 + u^3 (1/3 - u/4 + u^2/5 - u^3/6 + u^4/7)
    sfh_df u2 = df_two_prod(uh, uh);
    u2.l = __fmaf_rn(__fadd_rn(uh, uh), ul, u2.l);
    float p = __fmaf_rn(uh, 1.0f / 7.0f, -1.0f / 6.0f);
    p = __fmaf_rn(uh, p, 0.2f);
    p = __fmaf_rn(uh, p, -0.25f);
    p = __fmaf_rn(uh, p, 1.0f / 3.0f);
    p = __fmul_rn(__fmul_rn(__fmul_rn(uh, uh), uh), p);
    const sfh_df lp = df_two_sum(uh, __fmul_rn(-0.5f, u2.h));
    const float lpl = __fadd_rn(lp.l, __fadd_rn(__fsub_rn(ul, __fmul_rn(0.5f, u2.l)), p));
    const float fe = __fsub_rn(__uint_as_float(0x4b400000u + (uint32_t)e), 12582912.0f);
    // e ln2 (hi exact) + log F + log1p(u): two error-free sums, the low parts added
    const sfh_df tj = tab[j];
    const sfh_df s1 = df_two_sum(__fmul_rn(fe, SFH_DF_LN2_HI), tj.h);
    const sfh_df s2 = df_two_sum(s1.h, lp.h);
    const float lo = __fadd_rn(__fadd_rn(s1.l, s2.l),
                               __fadd_rn(__fmaf_rn(fe, SFH_DF_LN2_LO, __fmul_rn(fe, SFH_DF_LN2_LO2)),
                                         __fadd_rn(tj.l, lpl)));
    return df_fast_two_sum(s2.h, lo);
}
#endif

// Poisson term of one bin, fitting_base.jl:93:  n - c - n log(n/c)  (n > 0),  -c  (n = 0),
// for c = ch + cl >= eps given as a double-float (compensated sum) and n = nh + nl, in a
// branch-free form (every lane of a warp takes the same path whatever its count):
//   t = n log c - c + (n - n log n),
// with n - n log n read from nlogn_tab for integer counts 0..255 (the usual case) and
// computed otherwise.  Only the absolute error enters a sum of terms: below
// 2e-12 (c + n) + 1e-13 n |log c| (checked against long double on 4e6 random bins).
SFH_DF_HD sfh_df df_poisson_term_bf(sfh_df c, float nh, float nl, const sfh_df *tab,
                                    const sfh_df *nlogn_tab) {
    sfh_df lc = df_log_f(c.h, tab);
    lc = df_add_f(lc, SFH_DF_DIV(c.l, c.h));  // log(ch + cl) = log ch + cl/ch
    sfh_df t = df_add(df_mul(lc, sfh_df{nh, nl}), df_neg(c));
    const bool small = (nl == 0.0f) && (nh >= 0.0f) && (nh < 256.0f) && (nh == floorf(nh));
    if (small) {
        t = df_add(t, nlogn_tab[(int)nh]);
    } else {  // n - n log n for other counts
        const sfh_df n{nh, nl};
        sfh_df ln = df_log_f(nh, tab);
        ln = df_add_f(ln, SFH_DF_DIV(nl, nh));
        t = df_add(t, df_add(n, df_neg(df_mul(ln, n))));
    }
    return t;
}

// Host-side table of n - n log n, n = 0..255, as double-float pairs (0 for n = 0).
static inline void sfh_df_nlogn_table(sfh_df *tab) {
    for (int n = 0; n < 256; ++n) {
        const double v = n > 0 ? (double)n - (double)n * log((double)n) : 0.0;
        const float h = (float)v;
        tab[n].h = h;
        tab[n].l = (float)(v - (double)h);
    }
}

// Entries of the device table: log(1 + j/128) (129), then n - n log n (256).
#define SFH_DF_TAB_LOG 129
#define SFH_DF_TAB_ALL (129 + 256)

// Host-side table of log(1 + j/128), j = 0..128, as double-float pairs.
static inline void sfh_df_log_table(sfh_df *tab) {
    for (int j = 0; j <= 128; ++j) {
        const double v = log1p((double)j / 128.0);
        const float h = (float)v;
        tab[j].h = h;
        tab[j].l = (float)(v - (double)h);
    }
}
