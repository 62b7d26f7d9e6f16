/*
 * Double-float arithmetic: a value is the unevaluated sum hi + lo of two
 * floats with |lo| <= ulp(hi) / 2, about 48 significant bits. Built only
 * from IEEE-rounded float operations and fused multiply-adds (the
 * error-free transformations of Knuth's two-sum, Dekker's fast two-sum
 * and the FMA two-product), so that it runs on the FP32 pipe: sm_103's
 * FP64 rate is 1/64 of its FP32 rate, and one double-float operation
 * costs 3-20 float instructions.
 *
 * The exact rounding of the denoise (denoise_round.cu) evaluates the
 * samples whose code its float decision stage cannot settle with these,
 * to about 1e-13 relative, so that they round as a double evaluation does.
 *
 * Every operation uses the explicitly rounded intrinsics, so no
 * contraction or reassociation by the compiler can change a result; the
 * same header compiles for the host (C++, -ffp-contract=off) so that a CPU
 * test can check the arithmetic against long double.
 */
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define DF_ADD(a, b) __fadd_rn((a), (b))
#define DF_SUB(a, b) __fsub_rn((a), (b))
#define DF_MUL(a, b) __fmul_rn((a), (b))
#define DF_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define DF_DIV(a, b) __fdiv_rn((a), (b))
#define DF_SQRT(a) __fsqrt_rn((a))
#define DF_RINT(a) rintf((a))
#else
#define DF_ADD(a, b) ((float)(a) + (float)(b))
#define DF_SUB(a, b) ((float)(a) - (float)(b))
#define DF_MUL(a, b) ((float)(a) * (float)(b))
#define DF_FMA(a, b, c) fmaf((a), (b), (c))
#define DF_DIV(a, b) ((float)(a) / (float)(b))
#define DF_SQRT(a) sqrtf((a))
#define DF_RINT(a) rintf((a))
#endif

struct dfl {
    float hi, lo;
};

DF_HD dfl df_make(float hi, float lo)
{
    dfl r;
    r.hi = hi;
    r.lo = lo;
    return r;
}

DF_HD dfl df_from(float a)
{
    return df_make(a, 0.0f);
}

/* a + b exactly, as s + e (Knuth). */
DF_HD dfl df_two_sum(float a, float b)
{
    const float s = DF_ADD(a, b);
    const float bb = DF_SUB(s, a);
    const float e = DF_ADD(DF_SUB(a, DF_SUB(s, bb)), DF_SUB(b, bb));
    return df_make(s, e);
}

/* a + b exactly when |a| >= |b| (Dekker). */
DF_HD dfl df_fast_two_sum(float a, float b)
{
    const float s = DF_ADD(a, b);
    return df_make(s, DF_SUB(b, DF_SUB(s, a)));
}

/* a * b exactly, as p + e. */
DF_HD dfl df_two_prod(float a, float b)
{
    const float p = DF_MUL(a, b);
    return df_make(p, DF_FMA(a, b, -p));
}

DF_HD dfl df_neg(dfl a)
{
    return df_make(-a.hi, -a.lo);
}

/* a + b, accurate under cancellation (both parts summed exactly). */
DF_HD dfl df_add(dfl a, dfl b)
{
    dfl s = df_two_sum(a.hi, b.hi);
    const dfl t = df_two_sum(a.lo, b.lo);
    s.lo = DF_ADD(s.lo, t.hi);
    s = df_fast_two_sum(s.hi, s.lo);
    s.lo = DF_ADD(s.lo, t.lo);
    return df_fast_two_sum(s.hi, s.lo);
}

DF_HD dfl df_sub(dfl a, dfl b)
{
    return df_add(a, df_neg(b));
}

/* a + b for operands of the same sign (no cancellation to guard). */
DF_HD dfl df_add_same(dfl a, dfl b)
{
    const dfl s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, DF_ADD(s.lo, DF_ADD(a.lo, b.lo)));
}

DF_HD dfl df_add_f(dfl a, float b)
{
    const dfl s = df_two_sum(a.hi, b);
    return df_fast_two_sum(s.hi, DF_ADD(s.lo, a.lo));
}

DF_HD dfl df_mul(dfl a, dfl b)
{
    const float p = DF_MUL(a.hi, b.hi);
    float e = DF_FMA(a.hi, b.hi, -p);
    e = DF_FMA(a.hi, b.lo, e);
    e = DF_FMA(a.lo, b.hi, e);
    return df_fast_two_sum(p, e);
}

DF_HD dfl df_mul_f(dfl a, float b)
{
    const float p = DF_MUL(a.hi, b);
    float e = DF_FMA(a.hi, b, -p);
    e = DF_FMA(a.lo, b, e);
    return df_fast_two_sum(p, e);
}

DF_HD dfl df_sqr(dfl a)
{
    const float p = DF_MUL(a.hi, a.hi);
    float e = DF_FMA(a.hi, a.hi, -p);
    e = DF_FMA(DF_ADD(a.hi, a.hi), a.lo, e);
    return df_fast_two_sum(p, e);
}

/* Multiplication by a power of two (exact unless it under/overflows). */
DF_HD dfl df_scale(dfl a, float p2)
{
    return df_make(DF_MUL(a.hi, p2), DF_MUL(a.lo, p2));
}

/* a / b: a float quotient and two corrections from the exact remainder. */
DF_HD dfl df_div(dfl a, dfl b)
{
    const float q1 = DF_DIV(a.hi, b.hi);
    dfl r = df_sub(a, df_mul_f(b, q1));
    const float q2 = DF_DIV(r.hi, b.hi);
    r = df_sub(r, df_mul_f(b, q2));
    const float q3 = DF_DIV(r.hi, b.hi);
    return df_add_f(df_fast_two_sum(q1, q2), q3);
}

/* sqrt(a) for a >= 0: the float root and one Newton correction computed
 * from the exact residual a - s^2. */
DF_HD dfl df_sqrt(dfl a)
{
    if (!(a.hi > 0.0f))
        return df_from(0.0f);
    const float s = DF_SQRT(a.hi);
    const dfl r = df_sub(a, df_two_prod(s, s));
    return df_fast_two_sum(s, DF_DIV(r.hi, DF_ADD(s, s)));
}

/* Signed comparison of two double-floats: <0, 0, >0. */
DF_HD int df_cmp(dfl a, dfl b)
{
    const dfl d = df_sub(a, b);
    return d.hi < 0.0f ? -1 : (d.hi > 0.0f ? 1 : (d.lo < 0.0f ? -1 : (d.lo > 0.0f ? 1 : 0)));
}

DF_HD dfl df_clamp01(dfl a)
{
    if (a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f))
        return df_from(0.0f);
    if (a.hi > 1.0f || (a.hi == 1.0f && a.lo > 0.0f))
        return df_from(1.0f);
    return a;
}

/* rint of a double-float (round half to even), as a float integer. */
DF_HD float df_rint(dfl a)
{
    const float n = DF_RINT(a.hi);
    /* a - n exactly: |a.hi - n| <= 1/2 is exact (Sterbenz). */
    const dfl f = df_add_f(df_from(DF_SUB(a.hi, n)), a.lo);
    if (f.hi > 0.5f || (f.hi == 0.5f && f.lo > 0.0f))
        return DF_ADD(n, 1.0f);
    if (f.hi < -0.5f || (f.hi == -0.5f && f.lo < 0.0f))
        return DF_SUB(n, 1.0f);
    if ((f.hi == 0.5f || f.hi == -0.5f) && f.lo == 0.0f) {
        /* An exact tie: to even. */
        const float m = f.hi > 0.0f ? DF_ADD(n, 1.0f) : DF_SUB(n, 1.0f);
        return fmodf(m, 2.0f) == 0.0f ? m : n;
    }
    return n;
}

/* Constants of the exponential: ln 2 as the sum of three floats (the
 * first with 16 significant bits, so that k * DF_LN2_HI is exact for
 * k < 2^8; together within 1.3e-21 of ln 2), and 1/24 and 1/6 as
 * double-floats. */
#define DF_LN2_HI 0.693145751953125f
#define DF_LN2_LO 1.4286068e-06f
#define DF_LN2_LO2 5.497923e-14f

/* exp(-y) for y >= 0, to about 1e-14 relative. Range reduction
 * y = k ln 2 + r with |r| <= ln2/2, then z = -r/8 and expm1(z) by its
 * Taylor series (the terms of order five and up in float, which is all
 * the precision they need at |z| <= 0.044), squared back three times as
 * e <- 2e + e^2, then 1 + e and the exact scaling by 2^-k.
 * 0 beyond y = 80 (below 2^-115). */
DF_HD dfl df_exp_neg(dfl y)
{
    if (y.hi > 80.0f)
        return df_from(0.0f);
    const float k = DF_RINT(DF_MUL(y.hi, 1.44269504f));
    dfl r = df_add_f(y, -DF_MUL(k, DF_LN2_HI));          /* exact product */
    r = df_sub(r, df_two_prod(k, DF_LN2_LO));
    r = df_add_f(r, -DF_MUL(k, DF_LN2_LO2));
    const dfl z = df_scale(df_neg(r), 0.125f);
    /* expm1(z) = z (1 + z (1/2 + z (1/6 + z (1/24 + z P)))),
     * P = 1/120 + z/720 + z^2/5040 + z^3/40320 in float. */
    const float zf = z.hi;
    float P = DF_FMA(zf, 1.0f / 40320.0f, 1.0f / 5040.0f);
    P = DF_FMA(zf, P, 1.0f / 720.0f);
    P = DF_FMA(zf, P, 1.0f / 120.0f);
    dfl a = df_add_f(df_make(0.041666668f, -1.2417635e-09f), DF_MUL(zf, P));
    a = df_add(df_make(0.16666667f, -4.967054e-09f), df_mul(z, a));
    a = df_add_f(df_mul(z, a), 0.5f);
    a = df_add_f(df_mul(z, a), 1.0f);
    dfl e = df_mul(z, a);
    for (int i = 0; i < 3; i++)
        e = df_add(df_scale(e, 2.0f), df_sqr(e));
    e = df_add_f(e, 1.0f);
    const int ki = (int)k;
#if defined(__CUDA_ARCH__)
    const float p2 = __int_as_float((127 - ki) << 23);
#else
    const float p2 = ldexpf(1.0f, -ki);
#endif
    return df_scale(e, p2);
}
