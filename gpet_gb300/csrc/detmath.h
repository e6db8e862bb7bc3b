/* detmath.h - deterministic single/double precision math for the random-number
 * transforms of the photon transport and the digitizer.
 *
 * Every function here is a fixed sequence of IEEE-754 operations that round the
 * same way on the GPU (sm_103a, compiled with -fmad=false; fused steps are
 * written as explicit fma) and on a CPU (gcc -ffp-contract=off): sqrt and
 * division are correctly rounded on both, fma is a single rounding on both.
 * The same source therefore yields bit-identical results in the CUDA kernels and
 * in the FP32 build of the CPU oracle, which is what lets the transport be
 * compared history by history.
 *
 * Methods (all from elementary series, coefficients are exact rationals):
 *   log  : x = m 2^e, m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s),
 *          s = (m-1)/(m+1), atanh series in s^2.
 *   exp  : x = k ln2 + r, |r| <= ln2/2, Taylor series of e^r, scale by 2^k.
 *   sin/cos of 2*pi*u : quadrant reduction on u (exact), Taylor series on
 *          |x| <= pi/4.
 * Accuracy is a few ulp, which the tests check against libm.
 *
 * This header is C99 and CUDA C++; it includes nothing from CUDA's math
 * library beyond the rounding intrinsics. */
#ifndef GPET_DETMATH_H
#define GPET_DETMATH_H

#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define DM_FN __host__ __device__ __forceinline__
#else
#define DM_FN static inline
#endif

DM_FN float dm_fma(float a, float b, float c)
{
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

DM_FN double dm_fmad(double a, double b, double c)
{
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return fma(a, b, c);
#endif
}

/* correctly rounded square root */
DM_FN float dm_sqrt(float x)
{
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(x);
#else
    return sqrtf(x);
#endif
}

DM_FN uint32_t dm_f2u(float x)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u; memcpy(&u, &x, 4); return u;
#endif
}

DM_FN float dm_u2f(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x; memcpy(&x, &u, 4); return x;
#endif
}

DM_FN uint64_t dm_d2u(double x)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u; memcpy(&u, &x, 8); return u;
#endif
}

DM_FN double dm_u2d(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x; memcpy(&x, &u, 8); return x;
#endif
}

/* ln 2 split so that e*DM_LN2_HI is exact for |e| < 2^9 */
#define DM_LN2_HI 0.693145751953125f
#define DM_LN2_LO 1.428606765330187e-06f
#define DM_INV_LN2 1.44269504088896341f
#define DM_TWO_PI 6.28318530717958648f

/* natural log of a positive normal float */
DM_FN float dm_logf(float x)
{
    uint32_t b = dm_f2u(x);
    int e = (int)((b >> 23) & 0xffu) - 127;
    uint32_t mb = (b & 0x7fffffu) | 0x3f800000u;      /* m in [1,2) */
    if (mb > 0x3fb504f3u) { mb -= 0x00800000u; e += 1; } /* m > sqrt(2): halve */
    float m = dm_u2f(mb);
    float s = (m - 1.0f) / (m + 1.0f);
    float z = s * s;
    /* 2 atanh(s) = s * (2 + z(2/3 + z(2/5 + z(2/7 + z 2/9)))) */
    float p = dm_fma(z, 0.222222222f, 0.285714298f);
    p = dm_fma(z, p, 0.400000006f);
    p = dm_fma(z, p, 0.666666687f);
    p = dm_fma(z, p, 2.0f);
    float lm = s * p;
    float fe = (float)e;
    return dm_fma(fe, DM_LN2_HI, dm_fma(fe, DM_LN2_LO, lm));
}

/* e^x for |x| < 87 */
DM_FN float dm_expf(float x)
{
    float kf = floorf(dm_fma(x, DM_INV_LN2, 0.5f));
    float r = dm_fma(-kf, DM_LN2_HI, x);
    r = dm_fma(-kf, DM_LN2_LO, r);
    /* Taylor to r^8, |r| <= 0.347 */
    float p = dm_fma(r, 2.48015873e-05f, 1.98412698e-04f);
    p = dm_fma(r, p, 1.38888889e-03f);
    p = dm_fma(r, p, 8.33333333e-03f);
    p = dm_fma(r, p, 4.16666667e-02f);
    p = dm_fma(r, p, 1.66666667e-01f);
    p = dm_fma(r, p, 0.5f);
    p = dm_fma(r, p, 1.0f);
    p = dm_fma(r, p, 1.0f);
    int k = (int)kf;
    return p * dm_u2f((uint32_t)(k + 127) << 23);
}

/* sin and cos of 2*pi*u for any finite u (turns) */
DM_FN void dm_sincos_turns(float u, float* s, float* c)
{
    float q = floorf(u * 4.0f + 0.5f);      /* nearest quarter turn */
    float r = u - q * 0.25f;                /* exact, |r| <= 1/8 */
    int qi = ((int)q) & 3;                  /* two's complement: mod 4 */
    float x = r * DM_TWO_PI;                /* |x| <= pi/4 */
    float z = x * x;
    float sp = dm_fma(z, 2.75573192e-06f, -1.98412698e-04f);
    sp = dm_fma(z, sp, 8.33333333e-03f);
    sp = dm_fma(z, sp, -1.66666667e-01f);
    float sn = dm_fma(x * z, sp, x);
    float cp = dm_fma(z, -2.75573192e-07f, 2.48015873e-05f);
    cp = dm_fma(z, cp, -1.38888889e-03f);
    cp = dm_fma(z, cp, 4.16666667e-02f);
    cp = dm_fma(z, cp, -0.5f);
    float cs = dm_fma(z, cp, 1.0f);
    switch (qi) {
    case 0: *s = sn;  *c = cs;  break;
    case 1: *s = cs;  *c = -sn; break;
    case 2: *s = -sn; *c = -cs; break;
    default: *s = -cs; *c = sn; break;
    }
}

/* cube root of u in (0, 1] */
DM_FN float dm_cbrtf(float u)
{
    float y = dm_expf(dm_logf(u) * 0.333333343f);
    /* one Newton step on y^3 = u */
    return y - (y * y * y - u) / (3.0f * y * y);
}

/* natural log of a positive normal double (decay-time sampling) */
DM_FN double dm_log(double x)
{
    uint64_t b = dm_d2u(x);
    int e = (int)((b >> 52) & 0x7ffu) - 1023;
    uint64_t mb = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;
    if (mb > 0x3ff6a09e667f3bcdull) { mb -= 0x0010000000000000ull; e += 1; }
    double m = dm_u2d(mb);
    double s = (m - 1.0) / (m + 1.0);
    double z = s * s;
    /* 2 atanh(s) series to s^23 */
    double p = 2.0 / 23.0;
    p = dm_fmad(z, p, 2.0 / 21.0);
    p = dm_fmad(z, p, 2.0 / 19.0);
    p = dm_fmad(z, p, 2.0 / 17.0);
    p = dm_fmad(z, p, 2.0 / 15.0);
    p = dm_fmad(z, p, 2.0 / 13.0);
    p = dm_fmad(z, p, 2.0 / 11.0);
    p = dm_fmad(z, p, 2.0 / 9.0);
    p = dm_fmad(z, p, 2.0 / 7.0);
    p = dm_fmad(z, p, 2.0 / 5.0);
    p = dm_fmad(z, p, 2.0 / 3.0);
    p = dm_fmad(z, p, 2.0);
    return dm_fmad((double)e, 0.69314718055994531, s * p);
}

/* log(1 + x) for |x| <= 2^-6 by its Taylor series x (1 - x/2 + ... - x^9/10)
 * (truncation below 2^-57 relative), no division: used for the decay-time
 * sampling of long-lived isotopes. Estrin's scheme: dependency depth 6
 * instead of 10 (FP64 latency is long on this GPU) */
DM_FN double dm_log1p_small(double x)
{
    const double x2 = x * x;
    const double x4 = x2 * x2;
    const double x8 = x4 * x4;
    const double p01 = dm_fmad(x, -0.5, 1.0);
    const double p23 = dm_fmad(x, -1.0 / 4.0, 1.0 / 3.0);
    const double p45 = dm_fmad(x, -1.0 / 6.0, 1.0 / 5.0);
    const double p67 = dm_fmad(x, -1.0 / 8.0, 1.0 / 7.0);
    const double p89 = dm_fmad(x, -1.0 / 10.0, 1.0 / 9.0);
    const double p03 = dm_fmad(x2, p23, p01);
    const double p47 = dm_fmad(x2, p67, p45);
    const double p07 = dm_fmad(x4, p47, p03);
    return x * dm_fmad(x8, p89, p07);
}

/* time per unit path, us/cm (1 / 29979.2458), for single-precision flight
 * times that are added to a double-precision time stamp once */
#define DM_INV_SPEED 3.3356409519815204e-05f

/* uniform (0,1) float from the top 23 random bits: (k + 1/2) 2^-23, exact
 * (k + 1/2 < 2^23 fits the 24-bit significand), so never 0 or 1: the values
 * run from 2^-24 to 1 - 2^-24. (With 24 bits, k + 1/2 would round to an even
 * integer for k >= 2^23 and k = 2^24 - 1 would give exactly 1.) */
DM_FN float dm_u01(uint32_t x)
{
    return ((float)(x >> 9) + 0.5f) * 1.1920928955078125e-07f;
}

/* uniform (0,1) double from 52 random bits: (k + 1/2) 2^-52, made as
 * (1 + k 2^-52) - (1 - 2^-53), one exact subtraction */
DM_FN double dm_u01d(uint32_t hi, uint32_t lo)
{
    const uint64_t k = ((uint64_t)(hi & 0xFFFFFu) << 32) | (uint64_t)lo;
    return dm_u2d(0x3FF0000000000000ull | k) - dm_u2d(0x3FEFFFFFFFFFFFFFull);
}

/* two independent standard normals from two uniforms (Box-Muller, both
 * branches) */
DM_FN void dm_normal2(float u1, float u2, float* n1, float* n2)
{
    float s, c;
    dm_sincos_turns(u2, &s, &c);
    const float R = dm_sqrt(-2.0f * dm_logf(u1));
    *n1 = R * c;
    *n2 = R * s;
}

/* standard normal from two uniforms (Box-Muller, cosine branch) */
DM_FN float dm_normal(float u1, float u2)
{
    float s, c;
    dm_sincos_turns(u2, &s, &c);
    return dm_sqrt(-2.0f * dm_logf(u1)) * c;
}

#endif /* GPET_DETMATH_H */
