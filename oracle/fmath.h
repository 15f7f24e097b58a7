/* oracle/fmath.h — portable float32 elementary functions for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links this file.
 *
 * The reference shader (src/shaders/path_trace.wgsl) calls the WGSL builtins
 * sin, cos, atan2, asin, pow, exp and normalize, whose precision WGSL leaves to
 * the backend (absolute error 2^-11 for sin/cos on [-pi, pi]).  To make the CPU
 * restatement and the CUDA kernels agree bit for bit, both sides evaluate these
 * functions with the same published methods, using only IEEE-754 correctly
 * rounded + - * / sqrt (no fused multiply-add: this file is compiled with
 * -ffp-contract=off):
 *
 *   sin/cos : Cody & Waite (1980) additive range reduction by pi/2 with a
 *             three-part split of pi/2 (12 + 12 + 24 significant bits, derived
 *             from pi at 200-bit precision), then the Taylor series of sin and
 *             cos on [-pi/4, pi/4] (coefficients 1/n!) in Horner form.
 *   atan    : argument reduction atan(x) = pi/2 - atan(1/x) for |x| > 1 and
 *             atan(x) = pi/6 + atan((x*sqrt3 - 1)/(x + sqrt3)) for
 *             x > tan(pi/12), then the Taylor series t - t^3/3 + ... (t^15).
 *   atan2   : quadrant selection on atan(y/x).
 *   asin    : asin(x) = atan2(x, sqrt((1-x)(1+x))).
 *   exp     : Cody & Waite reduction by ln2 (12-bit split), Taylor series to
 *             r^8, scaling by 2^k assembled from the exponent bits.
 *   log     : x = m * 2^e with m in [sqrt(1/2), sqrt(2)),
 *             log m = 2 atanh(s), s = (m-1)/(m+1), series to s^13.
 *   pow     : integer exponents |y| <= 32 by binary powering, otherwise
 *             exp(y * log x).
 *
 * Each function carries its own error bound test in tests/test_oracle_math.py.
 */
#ifndef MCRT_ORACLE_FMATH_H
#define MCRT_ORACLE_FMATH_H

#include <stdint.h>
#include <string.h>
#include <math.h>

static inline float of_bits(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint32_t of_u32(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

#define OF_PIO2_A 1.5703125f
#define OF_PIO2_B 0.0004837512969970703f
#define OF_PIO2_C 7.549790126404332e-08f
#define OF_TWO_OVER_PI 0.6366197466850281f

/* sin and cos of x via Cody-Waite reduction + Taylor polynomials. */
static inline void of_sincos(float x, float *s_out, float *c_out)
{
    float kf = floorf(x * OF_TWO_OVER_PI + 0.5f);
    float r = ((x - kf * OF_PIO2_A) - kf * OF_PIO2_B) - kf * OF_PIO2_C;
    int k = (int)kf;
    float r2 = r * r;
    /* sin r = r (1 - r^2/3! + r^4/5! - ... - r^10/11! + r^12/13!) */
    float ps = 1.6059043836821613e-10f;               /* 1/13! */
    ps = ps * r2 + -2.505210838544172e-08f;            /* -1/11! */
    ps = ps * r2 + 2.7557319223985893e-06f;            /* 1/9! */
    ps = ps * r2 + -0.0001984126984126984f;            /* -1/7! */
    ps = ps * r2 + 0.008333333333333333f;              /* 1/5! */
    ps = ps * r2 + -0.16666666666666666f;              /* -1/3! */
    float sn = r + r * (r2 * ps);
    /* cos r = 1 - r^2/2! + r^4/4! - ... + r^12/12! */
    float pc = 2.08767569878681e-09f;                  /* 1/12! */
    pc = pc * r2 + -2.755731922398589e-07f;            /* -1/10! */
    pc = pc * r2 + 2.48015873015873e-05f;              /* 1/8! */
    pc = pc * r2 + -0.001388888888888889f;             /* -1/6! */
    pc = pc * r2 + 0.041666666666666664f;              /* 1/4! */
    pc = pc * r2 + -0.5f;                              /* -1/2! */
    float cs = 1.0f + r2 * pc;
    switch (k & 3) {
    case 0: *s_out = sn;  *c_out = cs;  break;
    case 1: *s_out = cs;  *c_out = -sn; break;
    case 2: *s_out = -sn; *c_out = -cs; break;
    default: *s_out = -cs; *c_out = sn; break;
    }
}
static inline float of_sin(float x) { float s, c; of_sincos(x, &s, &c); return s; }
static inline float of_cos(float x) { float s, c; of_sincos(x, &s, &c); return c; }
static inline float of_tan(float x) { float s, c; of_sincos(x, &s, &c); return s / c; }

/* atan on [0, +inf) */
static inline float of_atan_pos(float x)
{
    float base = 0.0f;
    int inv = 0;
    if (x > 1.0f) { x = 1.0f / x; inv = 1; }
    if (x > 0.2679491937160492f) {                      /* tan(pi/12) */
        x = (x * 1.7320507764816284f - 1.0f) / (x + 1.7320507764816284f);
        base = 0.5235987901687622f;                     /* pi/6 */
    }
    float t2 = x * x;
    float p = 0.06666666666666667f;                     /* 1/15 */
    p = p * t2 + -0.07692307692307693f;                 /* -1/13 */
    p = p * t2 + 0.09090909090909091f;                  /* 1/11 */
    p = p * t2 + -0.1111111111111111f;                  /* -1/9 */
    p = p * t2 + 0.14285714285714285f;                  /* 1/7 */
    p = p * t2 + -0.2f;                                 /* -1/5 */
    p = p * t2 + 0.3333333333333333f;                   /* 1/3 */
    float a = base + (x - x * (t2 * p));
    if (inv) a = 1.5707963705062866f - a;
    return a;
}

static inline float of_atan2(float y, float x)
{
    if (isnan(x) || isnan(y)) return x + y;
    float ax = fabsf(x), ay = fabsf(y);
    float a;
    if (ax == 0.0f && ay == 0.0f) {
        a = 0.0f;
    } else if (ax >= ay) {
        a = of_atan_pos(ay / ax);
    } else {
        a = 1.5707963705062866f - of_atan_pos(ax / ay);
    }
    if (x < 0.0f || (x == 0.0f && signbit(x))) a = 3.1415927410125732f - a;
    return signbit(y) ? -a : a;
}

static inline float of_asin(float x)
{
    return of_atan2(x, sqrtf((1.0f - x) * (1.0f + x)));
}

static inline float of_ldexp(float p, int k)
{
    if (k > 127) { p = p * of_bits(0x7f000000u); k -= 127; if (k > 127) k = 127; }
    if (k < -126) { p = p * of_bits(0x0c800000u); k += 102; if (k < -126) k = -126; } /* 2^-102 */
    return p * of_bits((uint32_t)(k + 127) << 23);
}

static inline float of_exp(float x)
{
    if (isnan(x)) return x;
    if (x > 88.72283935546875f) return INFINITY;
    if (x < -103.97208404541016f) return 0.0f;
    float kf = floorf(x * 1.4426950216293335f + 0.5f);
    float r = (x - kf * 0.693115234375f) - kf * 3.194618329871446e-05f;
    float p = 2.48015873015873e-05f;                    /* 1/8! */
    p = p * r + 0.0001984126984126984f;                 /* 1/7! */
    p = p * r + 0.001388888888888889f;                  /* 1/6! */
    p = p * r + 0.008333333333333333f;                  /* 1/5! */
    p = p * r + 0.041666666666666664f;                  /* 1/4! */
    p = p * r + 0.16666666666666666f;                   /* 1/3! */
    p = p * r + 0.5f;                                   /* 1/2! */
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    return of_ldexp(p, (int)kf);
}

static inline float of_log(float x)
{
    if (isnan(x) || x < 0.0f) return NAN;
    if (x == 0.0f) return -INFINITY;
    if (isinf(x)) return x;
    int e = 0;
    uint32_t u = of_u32(x);
    if ((u >> 23) == 0) {                               /* subnormal */
        x = x * 16777216.0f; e = -24; u = of_u32(x);
    }
    e += (int)(u >> 23) - 127;
    float m = of_bits((u & 0x007fffffu) | 0x3f800000u); /* [1, 2) */
    if (m > 1.4142135381698608f) { m = m * 0.5f; e += 1; }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = 0.07692307692307693f;                     /* 1/13 */
    p = p * s2 + 0.09090909090909091f;                  /* 1/11 */
    p = p * s2 + 0.1111111111111111f;                   /* 1/9 */
    p = p * s2 + 0.14285714285714285f;                  /* 1/7 */
    p = p * s2 + 0.2f;                                  /* 1/5 */
    p = p * s2 + 0.3333333333333333f;                   /* 1/3 */
    float lm = 2.0f * s + 2.0f * s * (s2 * p);
    float ef = (float)e;
    return (ef * 0.693115234375f + lm) + ef * 3.194618329871446e-05f;
}

static inline float of_pow(float x, float y)
{
    if (y == 0.0f) return 1.0f;
    float yi = floorf(y);
    if (yi == y && fabsf(y) <= 32.0f) {
        int n = (int)fabsf(y);
        float base = x, acc = 1.0f;
        while (n) {
            if (n & 1) acc = acc * base;
            n >>= 1;
            if (n) base = base * base;
        }
        return y < 0.0f ? 1.0f / acc : acc;
    }
    if (x == 0.0f) return y > 0.0f ? 0.0f : INFINITY;
    if (x < 0.0f) return NAN;
    return of_exp(y * of_log(x));
}

/* WGSL f32 -> u32 conversion: truncation toward zero, saturating, NaN -> 0. */
static inline uint32_t of_f2u_sat(float f)
{
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)f;
}

#endif /* MCRT_ORACLE_FMATH_H */
