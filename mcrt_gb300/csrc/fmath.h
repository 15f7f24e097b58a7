// fmath.h — float32 elementary functions used by the kernels and by the host
// code of the library (camera basis, scene transforms, tone mapping), compiled
// for both sides so that the host and the device evaluate them identically.
//
// The reference calls the WGSL builtins sin, cos, atan2, asin, pow, exp
// (src/shaders/path_trace.wgsl) and Rust's f32 sin_cos/tan/powf on the host
// (src/scene.rs:387, src/camera.rs:89, src/headless.rs:96); WGSL leaves their
// precision to the backend.  Here they are evaluated with published methods
// using only IEEE-754 + - * / sqrt (callers compile without FMA contraction):
//   sin/cos : Cody & Waite (1980) additive range reduction by pi/2 with a
//             three-part split of pi/2 (12 + 12 + 24 significant bits), then
//             the Taylor series (coefficients 1/n!) on [-pi/4, pi/4];
//   atan    : atan(x) = pi/2 - atan(1/x) for x > 1 and
//             atan(x) = pi/6 + atan((x sqrt3 - 1)/(x + sqrt3)) for x > tan(pi/12),
//             then the Taylor series to t^15; atan2 by quadrant;
//   asin(x) = atan2(x, sqrt((1-x)(1+x)));
//   exp     : Cody & Waite reduction by ln 2, Taylor series to r^8, 2^k from
//             the exponent bits;
//   log     : log m = 2 atanh((m-1)/(m+1)) with m in [sqrt(1/2), sqrt(2));
//   pow     : binary powering for integer |y| <= 32, else exp(y log x).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define MCRT_HD __host__ __device__ __forceinline__
#else
#define MCRT_HD inline
#endif

namespace mcrt {

MCRT_HD float fm_bits(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
MCRT_HD uint32_t fm_u32(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
MCRT_HD float fm_inf() { return fm_bits(0x7f800000u); }
MCRT_HD float fm_nan() { return fm_bits(0x7fc00000u); }

MCRT_HD void fm_sincos(float x, float *s_out, float *c_out) {
    float kf = floorf(x * 0.6366197466850281f + 0.5f);
    float r = ((x - kf * 1.5703125f) - kf * 0.0004837512969970703f) - kf * 7.549790126404332e-08f;
    int k = (int)kf;
    float r2 = r * r;
    float ps = 1.6059043836821613e-10f;          // 1/13!
    ps = ps * r2 + -2.505210838544172e-08f;      // -1/11!
    ps = ps * r2 + 2.7557319223985893e-06f;      // 1/9!
    ps = ps * r2 + -0.0001984126984126984f;      // -1/7!
    ps = ps * r2 + 0.008333333333333333f;        // 1/5!
    ps = ps * r2 + -0.16666666666666666f;        // -1/3!
    float sn = r + r * (r2 * ps);
    float pc = 2.08767569878681e-09f;            // 1/12!
    pc = pc * r2 + -2.755731922398589e-07f;      // -1/10!
    pc = pc * r2 + 2.48015873015873e-05f;        // 1/8!
    pc = pc * r2 + -0.001388888888888889f;       // -1/6!
    pc = pc * r2 + 0.041666666666666664f;        // 1/4!
    pc = pc * r2 + -0.5f;                        // -1/2!
    float cs = 1.0f + r2 * pc;
    switch (k & 3) {
    case 0: *s_out = sn; *c_out = cs; break;
    case 1: *s_out = cs; *c_out = -sn; break;
    case 2: *s_out = -sn; *c_out = -cs; break;
    default: *s_out = -cs; *c_out = sn; break;
    }
}
MCRT_HD float fm_tan(float x) { float s, c; fm_sincos(x, &s, &c); return s / c; }

MCRT_HD float fm_atan_pos(float x) {
    float base = 0.0f;
    bool inv = false;
    if (x > 1.0f) { x = 1.0f / x; inv = true; }
    if (x > 0.2679491937160492f) {               // tan(pi/12)
        x = (x * 1.7320507764816284f - 1.0f) / (x + 1.7320507764816284f);
        base = 0.5235987901687622f;              // pi/6
    }
    float t2 = x * x;
    float p = 0.06666666666666667f;              // 1/15
    p = p * t2 + -0.07692307692307693f;          // -1/13
    p = p * t2 + 0.09090909090909091f;           // 1/11
    p = p * t2 + -0.1111111111111111f;           // -1/9
    p = p * t2 + 0.14285714285714285f;           // 1/7
    p = p * t2 + -0.2f;                          // -1/5
    p = p * t2 + 0.3333333333333333f;            // 1/3
    float a = base + (x - x * (t2 * p));
    if (inv) a = 1.5707963705062866f - a;
    return a;
}

MCRT_HD float fm_atan2(float y, float x) {
    if (x != x || y != y) return x + y;
    float ax = fabsf(x), ay = fabsf(y);
    float a;
    if (ax == 0.0f && ay == 0.0f) a = 0.0f;
    else if (ax >= ay) a = fm_atan_pos(ay / ax);
    else a = 1.5707963705062866f - fm_atan_pos(ax / ay);
    if (x < 0.0f || (x == 0.0f && (fm_u32(x) >> 31))) a = 3.1415927410125732f - a;
    return (fm_u32(y) >> 31) ? -a : a;
}

MCRT_HD float fm_asin(float x) { return fm_atan2(x, sqrtf((1.0f - x) * (1.0f + x))); }

MCRT_HD float fm_ldexp(float p, int k) {
    if (k > 127) { p = p * fm_bits(0x7f000000u); k -= 127; if (k > 127) k = 127; }
    if (k < -126) { p = p * fm_bits(0x0c800000u); k += 102; if (k < -126) k = -126; }
    return p * fm_bits((uint32_t)(k + 127) << 23);
}

MCRT_HD float fm_exp(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return fm_inf();
    if (x < -103.97208404541016f) return 0.0f;
    float kf = floorf(x * 1.4426950216293335f + 0.5f);
    float r = (x - kf * 0.693115234375f) - kf * 3.194618329871446e-05f;
    float p = 2.48015873015873e-05f;             // 1/8!
    p = p * r + 0.0001984126984126984f;          // 1/7!
    p = p * r + 0.001388888888888889f;           // 1/6!
    p = p * r + 0.008333333333333333f;           // 1/5!
    p = p * r + 0.041666666666666664f;           // 1/4!
    p = p * r + 0.16666666666666666f;            // 1/3!
    p = p * r + 0.5f;                            // 1/2!
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    return fm_ldexp(p, (int)kf);
}

MCRT_HD float fm_log(float x) {
    if (x != x || x < 0.0f) return fm_nan();
    if (x == 0.0f) return -fm_inf();
    if (x == fm_inf()) return x;
    int e = 0;
    uint32_t u = fm_u32(x);
    if ((u >> 23) == 0) { x = x * 16777216.0f; e = -24; u = fm_u32(x); }
    e += (int)(u >> 23) - 127;
    float m = fm_bits((u & 0x007fffffu) | 0x3f800000u);
    if (m > 1.4142135381698608f) { m = m * 0.5f; e += 1; }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = 0.07692307692307693f;              // 1/13
    p = p * s2 + 0.09090909090909091f;           // 1/11
    p = p * s2 + 0.1111111111111111f;            // 1/9
    p = p * s2 + 0.14285714285714285f;           // 1/7
    p = p * s2 + 0.2f;                           // 1/5
    p = p * s2 + 0.3333333333333333f;            // 1/3
    float lm = 2.0f * s + 2.0f * s * (s2 * p);
    float ef = (float)e;
    return (ef * 0.693115234375f + lm) + ef * 3.194618329871446e-05f;
}

MCRT_HD float fm_pow(float x, float y) {
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
    if (x == 0.0f) return y > 0.0f ? 0.0f : fm_inf();
    if (x < 0.0f) return fm_nan();
    return fm_exp(y * fm_log(x));
}

// WGSL / Rust `as` f32 -> u32: truncation toward zero, saturating, NaN -> 0.
MCRT_HD uint32_t fm_f2u_sat(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)f;
}

}  // namespace mcrt
