// obj.cu — Wavefront OBJ text parsed on the device into the reference's vertex
// and triangle records: load_obj (src/mesh.rs:474-642) followed by the mesh
// object's transform (src/scene.rs:829-879), appended to the context's device
// mesh.  The reference parses sequentially on the CPU; here every stage is a
// data-parallel pass over bytes, lines or face tokens:
//
//   k_obj_scan_text  16 bytes per thread: newlines per block, UTF-8 check
//   k_obj_lines      the newline positions (line boundaries)
//   k_obj_classify   per line: str::trim, the tag, the token count
//   (scans)          v / vn / vt slots, face-token and triangle offsets
//   k_obj_parse      per line: coordinates (correctly rounded binary32) and
//                    the face tokens' resolved (position, uv, normal) indices
//   k_obj_dedup      (position, uv, normal) key -> its first face token, in two
//                    open-addressing tables (the reference's HashMap cache)
//   k_obj_first      first occurrences (and their block sums)
//   k_obj_vertices   vertex numbers (scan) and the vertex records
//   k_obj_faces      fan triangles and the geometric-normal patch
//   k_obj_transform  scale -> rotate -> translate
//
// The sequential loop's results depend on order only through "first
// occurrence" and "last write", and both are fixed by token and triangle
// numbers here, so the output is the reference's, bit for bit.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "internal.h"

namespace mcrt {
namespace {

constexpr uint32_t kObjThreads = 256;
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr unsigned long long kEmptyKey = ~0ull;
enum : uint8_t { kLineNone = 0, kLineV = 1, kLineVN = 2, kLineVT = 3, kLineF = 4 };
// Face-token position word: index in bits 0-29, bit 30 "a position exists"
// (positions.get(pi) is Some), bit 31 "has_norm" (mesh.rs:585-589).
constexpr uint32_t kPosOk = 1u << 30, kHasNorm = 1u << 31, kPosMask = kPosOk - 1;

// ------------------------------------------------------------------ Rust str rules

__device__ __forceinline__ bool ascii_ws(uint8_t c) {          // u8::is_ascii_whitespace
    return c == ' ' || c == '\t' || c == '\n' || c == 0x0C || c == '\r';
}
__device__ __forceinline__ bool is_digit(uint8_t c) { return (uint8_t)(c - '0') < 10; }

// char::is_whitespace for the character that starts at p (text is valid
// UTF-8): its byte length, or 0.
__device__ int ws_forward(const uint8_t *p, const uint8_t *e) {
    const uint8_t c = p[0];
    if (c == ' ' || (c >= 0x09 && c <= 0x0D)) return 1;
    if (c == 0xC2 && e - p >= 2 && (p[1] == 0x85 || p[1] == 0xA0)) return 2;          // U+0085, U+00A0
    if (e - p >= 3) {
        if (c == 0xE1 && p[1] == 0x9A && p[2] == 0x80) return 3;                        // U+1680
        if (c == 0xE2 && p[1] == 0x80 &&
            (p[2] <= 0x8A || p[2] == 0xA8 || p[2] == 0xA9 || p[2] == 0xAF)) return 3;   // U+2000-200A, 2028, 2029, 202F
        if (c == 0xE2 && p[1] == 0x81 && p[2] == 0x9F) return 3;                        // U+205F
        if (c == 0xE3 && p[1] == 0x80 && p[2] == 0x80) return 3;                        // U+3000
    }
    return 0;
}
// The same for the character that ends at e (b: start of the line).
__device__ int ws_backward(const uint8_t *b, const uint8_t *e) {
    const uint8_t c = e[-1];
    if (c == ' ' || (c >= 0x09 && c <= 0x0D)) return 1;
    if (e - b >= 2 && e[-2] == 0xC2 && (c == 0x85 || c == 0xA0)) return 2;
    if (e - b >= 3 && ws_forward(e - 3, e) == 3) return 3;
    return 0;
}

// str::parse::<i64>: optional sign, one or more digits, no overflow.
__device__ bool parse_i64(const uint8_t *p, const uint8_t *e, long long *out) {
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) { neg = *p == '-'; ++p; }
    if (p == e) return false;
    unsigned long long v = 0;
    #pragma unroll 1
    for (int n = 0; p < e; ++p, ++n) {
        const uint32_t d = (uint32_t)*p - '0';
        if (d > 9) return false;
        // only a 19th digit (or later) can leave the range: 2^63 - 1 = 922337203685477580 * 10 + 7
        if (n >= 18 && (v > 922337203685477580ull || (v == 922337203685477580ull && d > (neg ? 8u : 7u))))
            return false;
        v = v * 10 + d;
    }
    *out = neg ? (long long)(0ull - v) : (long long)v;
    return true;
}

// resolve (mesh.rs:491-500): 1-based or negative (from the end) index into a
// list of n entries, of an already parsed integer.
__device__ __forceinline__ bool resolve_value(long long i, uint32_t n, uint32_t *out) {
    const long long idx = i < 0 ? (long long)n + i : i - 1;
    if (idx < 0 || idx >= (long long)n) return false;
    *out = (uint32_t)idx;
    return true;
}
__device__ bool resolve(const uint8_t *p, const uint8_t *e, uint32_t n, uint32_t *out) {
    long long i;
    if (!parse_i64(p, e, &i)) return false;
    const long long idx = i < 0 ? (long long)n + i : i - 1;
    if (idx < 0 || idx >= (long long)n) return false;
    *out = (uint32_t)idx;
    return true;
}

// Powers of ten exact in binary32 (5^10 < 2^24): Clinger's fast path.
__device__ const float kPow10f[11] = {1e0f, 1e1f, 1e2f, 1e3f, 1e4f, 1e5f, 1e6f, 1e7f, 1e8f, 1e9f, 1e10f};

// Correctly rounded powers of ten 1e-65 .. 1e39 (the compiler rounds each literal).
__device__ const double kPow10[105] = {
    1e-65, 1e-64, 1e-63, 1e-62, 1e-61, 1e-60, 1e-59, 1e-58, 1e-57, 1e-56, 1e-55, 1e-54, 1e-53, 1e-52, 1e-51,
    1e-50, 1e-49, 1e-48, 1e-47, 1e-46, 1e-45, 1e-44, 1e-43, 1e-42, 1e-41, 1e-40, 1e-39, 1e-38, 1e-37, 1e-36,
    1e-35, 1e-34, 1e-33, 1e-32, 1e-31, 1e-30, 1e-29, 1e-28, 1e-27, 1e-26, 1e-25, 1e-24, 1e-23, 1e-22, 1e-21,
    1e-20, 1e-19, 1e-18, 1e-17, 1e-16, 1e-15, 1e-14, 1e-13, 1e-12, 1e-11, 1e-10, 1e-9,  1e-8,  1e-7,  1e-6,
    1e-5,  1e-4,  1e-3,  1e-2,  1e-1,  1e0,   1e1,   1e2,   1e3,   1e4,   1e5,   1e6,   1e7,   1e8,   1e9,
    1e10,  1e11,  1e12,  1e13,  1e14,  1e15,  1e16,  1e17,  1e18,  1e19,  1e20,  1e21,  1e22,  1e23,  1e24,
    1e25,  1e26,  1e27,  1e28,  1e29,  1e30,  1e31,  1e32,  1e33,  1e34,  1e35,  1e36,  1e37,  1e38,  1e39};

// Arbitrary-precision non-negative integers for the exact comparison of a
// decimal with a binary32 rounding midpoint (at most ~700 bits are needed:
// 120 decimal digits times a power of two, or a 26-bit midpoint significand
// times 5^166 times a power of two).
constexpr int kBigWords = 26;
struct Big {
    uint32_t w[kBigWords];
    __device__ void set(unsigned long long v) {
        #pragma unroll 1
        for (int i = 0; i < kBigWords; ++i) w[i] = 0;
        w[0] = (uint32_t)v;
        w[1] = (uint32_t)(v >> 32);
    }
    __device__ void mul_add(uint32_t m, uint32_t a) {
        unsigned long long carry = a;
        #pragma unroll 1
        for (int i = 0; i < kBigWords; ++i) {
            unsigned long long t = (unsigned long long)w[i] * m + carry;
            w[i] = (uint32_t)t;
            carry = t >> 32;
        }
    }
    __device__ void mul_pow5(int k) {
        #pragma unroll 1
        while (k >= 13) { mul_add(1220703125u, 0); k -= 13; }     // 5^13
        uint32_t p = 1;
        #pragma unroll 1
        while (k-- > 0) p *= 5;
        mul_add(p, 0);
    }
    __device__ void shl(int bits) {
        const int ws = bits >> 5, bs = bits & 31;
        #pragma unroll 1
        for (int i = kBigWords - 1; i >= 0; --i) {
            uint32_t hi = i - ws >= 0 ? w[i - ws] : 0u;
            uint32_t lo = i - ws - 1 >= 0 ? w[i - ws - 1] : 0u;
            w[i] = bs ? (hi << bs) | (lo >> (32 - bs)) : hi;
        }
    }
};
__device__ int big_cmp(const Big &a, const Big &b) {
    #pragma unroll 1
    for (int i = kBigWords - 1; i >= 0; --i)
        if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
    return 0;
}

// Sign of (decimal value of the token [p, e)) - mid, exactly.  The first 120
// significant digits are kept and the rest reduce to a sticky bit: a binary32
// midpoint has at most 113 significant decimal digits, so no midpoint lies
// strictly inside the interval the dropped digits leave open.
__device__ __noinline__ int cmp_decimal_midpoint(const uint8_t *p, const uint8_t *e, double mid) {
    if (p < e && (*p == '+' || *p == '-')) ++p;
    Big D;
    D.set(0);
    int nd = 0;
    long long e10 = 0;
    bool sticky = false, nonzero = false;
    #pragma unroll 1
    for (; p < e && is_digit(*p); ++p) {
        const uint32_t d = *p - '0';
        if (nd < 120) {
            if (nonzero || d) { D.mul_add(10, d); ++nd; nonzero = true; }
        } else {
            ++e10;
            sticky |= d != 0;
        }
    }
    if (p < e && *p == '.') {
        #pragma unroll 1
        for (++p; p < e && is_digit(*p); ++p) {
            const uint32_t d = *p - '0';
            if (nd < 120) {
                if (nonzero || d) { D.mul_add(10, d); ++nd; nonzero = true; }
                --e10;
            } else {
                sticky |= d != 0;
            }
        }
    }
    long long ex = 0;
    if (p < e && (*p | 0x20) == 'e') {
        ++p;
        bool eneg = false;
        if (p < e && (*p == '+' || *p == '-')) { eneg = *p == '-'; ++p; }
        #pragma unroll 1
        for (; p < e && is_digit(*p); ++p)
            if (ex < 0x10000) ex = ex * 10 + (*p - '0');
        if (eneg) ex = -ex;
    }
    const int E = (int)(e10 + ex);        // in [-166, 39] for the values that reach here
    const unsigned long long bits = (unsigned long long)__double_as_longlong(mid);
    unsigned long long c = (bits & ((1ull << 52) - 1)) | (1ull << 52);
    int q = (int)((bits >> 52) & 0x7FF) - 1075;
    #pragma unroll 1
    while (!(c & 1)) { c >>= 1; ++q; }
    Big B;
    B.set(c);
    // D * 10^E against c * 2^q: D * 5^E * 2^E (E >= 0), or D * 2^E against c * 5^-E * 2^q.
    if (E >= 0) D.mul_pow5(E);
    else B.mul_pow5(-E);
    if (E > q) D.shl(E - q);
    else if (q > E) B.shl(q - E);
    int r = big_cmp(D, B);
    if (r == 0 && sticky) r = 1;
    return r;
}

__device__ __forceinline__ double f32_value(uint32_t b) {   // 0x7F800000 stands for 2^128
    return b >= 0x7F800000u ? 0x1p128 : (double)__uint_as_float(b);
}

// The binary32 nearest to m * 10^E (m < 10^19 the first significant digits,
// E in [-65, 39]); ties and near-ties are settled exactly against the token.
__device__ __noinline__ float round_decimal(unsigned long long m, int E, const uint8_t *tok, const uint8_t *tok_end) {
    const double d = __dmul_rn(__ull2double_rn(m), kPow10[E + 65]);   // relative error < 3.4e-16 (+1e-18 dropped digits)
    const float f = __double2float_rn(d);
    const uint32_t fb = __float_as_uint(f);
    const double tol = d * 0x1p-50;
    uint32_t lo = kNone, hi = kNone;
    double mid = 0.0;
    if (fb < 0x7F800000u) {
        const double m_hi = 0.5 * (f32_value(fb) + f32_value(fb + 1));
        if (fabs(d - m_hi) <= tol) { lo = fb; hi = fb + 1; mid = m_hi; }
    }
    if (lo == kNone && fb > 0) {
        const double m_lo = 0.5 * (f32_value(fb - 1) + f32_value(fb));
        if (fabs(d - m_lo) <= tol) { lo = fb - 1; hi = fb; mid = m_lo; }
    }
    if (lo == kNone) return f;
    const int c = cmp_decimal_midpoint(tok, tok_end, mid);
    const uint32_t r = c > 0 ? hi : c < 0 ? lo : ((lo & 1u) ? hi : lo);
    return __uint_as_float(r);
}

__device__ bool ieq3(const uint8_t *p, char a, char b, char c) {
    return (p[0] | 0x20) == a && (p[1] | 0x20) == b && (p[2] | 0x20) == c;
}

// str::parse::<f32> (core::num::dec2flt) of the token [p, e); false on a
// syntax error.  "inf", "infinity" and "nan" in any case, an optional sign,
// digits with an optional '.' fraction and exponent, at least one digit.
__device__ bool parse_f32(const uint8_t *p, const uint8_t *e, float *out) {
    const uint8_t *const tok = p;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) { neg = *p == '-'; ++p; }
    const long long n = e - p;
    if (n == 3 && ieq3(p, 'n', 'a', 'n')) { *out = __uint_as_float(neg ? 0xFFC00000u : 0x7FC00000u); return true; }
    if ((n == 3 || n == 8) && ieq3(p, 'i', 'n', 'f') &&
        (n == 3 || (ieq3(p + 3, 'i', 'n', 'i') && (p[6] | 0x20) == 't' && (p[7] | 0x20) == 'y'))) {
        *out = neg ? -INFINITY : INFINITY;
        return true;
    }
    unsigned long long m = 0;
    int nd = 0;
    long long e10 = 0;
    bool any = false;
    #pragma unroll 1
    for (; p < e && is_digit(*p); ++p) {
        any = true;
        const uint32_t d = *p - '0';
        if (nd < 19) {
            if (m || d) { m = m * 10 + d; ++nd; }
        } else {
            ++e10;
        }
    }
    if (p < e && *p == '.') {
        #pragma unroll 1
        for (++p; p < e && is_digit(*p); ++p) {
            any = true;
            const uint32_t d = *p - '0';
            if (nd < 19) {
                if (m || d) { m = m * 10 + d; ++nd; }
                --e10;
            }
        }
    }
    if (!any) return false;
    long long ex = 0;
    if (p < e && (*p | 0x20) == 'e') {
        ++p;
        bool eneg = false;
        if (p < e && (*p == '+' || *p == '-')) { eneg = *p == '-'; ++p; }
        if (p == e || !is_digit(*p)) return false;
        #pragma unroll 1
        for (; p < e && is_digit(*p); ++p)
            if (ex < 0x10000) ex = ex * 10 + (*p - '0');
        if (eneg) ex = -ex;
    }
    if (p != e) return false;
    float r = 0.0f;
    if (m != 0) {
        const long long E = e10 + ex;
        if (m <= (1u << 24) && E >= -10 && E <= 10) {  // both operands exact: one rounding (Clinger)
            const float fm = (float)(uint32_t)m;
            r = E < 0 ? __fdiv_rn(fm, kPow10f[-E]) : __fmul_rn(fm, kPow10f[E]);
        } else if (nd - 1 + E >= 39) {
            r = INFINITY;                              // >= 1e39: above the overflow threshold
        } else if (nd + E <= -46) {
            r = 0.0f;                                  // < 1e-46: below half the least subnormal
        } else {
            r = round_decimal(m, (int)E, tok, e);
        }
    }
    *out = neg ? -r : r;
    return true;
}

__device__ __forceinline__ float f32_or_zero(const uint8_t *p, const uint8_t *e) {   // .parse().unwrap_or(0.0)
    float v;
    return parse_f32(p, e, &v) ? v : 0.0f;
}

// Next ASCII-whitespace-separated token in [*p, e).
__device__ __forceinline__ bool next_token(const uint8_t *&p, const uint8_t *e, const uint8_t *&tb,
                                           const uint8_t *&te) {
    #pragma unroll 1
    while (p < e && ascii_ws(*p)) ++p;
    if (p == e) return false;
    tb = p;
    #pragma unroll 1
    while (p < e && !ascii_ws(*p)) ++p;
    te = p;
    return true;
}

// normalize3 (mesh.rs:663-670)
__device__ __forceinline__ float3 normalize3(float x, float y, float z) {
    const float len = sqrtf(x * x + y * y + z * z);
    if (len < 1e-8f) return make_float3(0.0f, 1.0f, 0.0f);
    return make_float3(x / len, y / len, z / len);
}

// ------------------------------------------------------------------ UTF-8 and lines

// A continuation byte must follow a lead byte of enough width with only
// continuation bytes between; a lead byte's sequence must be complete and in
// the ranges of core::str::run_utf8_validation.  The least failing position is
// the sequential validator's valid_up_to.
__device__ bool utf8_byte_ok(const uint8_t *t, unsigned long long len, unsigned long long i) {
    const uint8_t b = t[i];
    auto cont = [](uint8_t x) { return (x & 0xC0) == 0x80; };
    if (b < 0x80) return true;
    if (cont(b)) {
        for (int d = 1; d <= 3; ++d) {
            if (i < (unsigned long long)d) return false;
            const uint8_t c = t[i - d];
            if (cont(c)) continue;
            const int w = (c >= 0xC2 && c <= 0xDF) ? 2 : (c >= 0xE0 && c <= 0xEF) ? 3 : (c >= 0xF0 && c <= 0xF4) ? 4 : 0;
            return w > d;
        }
        return false;
    }
    int w = (b >= 0xC2 && b <= 0xDF) ? 2 : (b >= 0xE0 && b <= 0xEF) ? 3 : (b >= 0xF0 && b <= 0xF4) ? 4 : 0;
    if (w == 0 || i + (unsigned long long)w > len) return false;
    const uint8_t b1 = t[i + 1];
    bool ok;
    if (w == 2) ok = cont(b1);
    else if (w == 3)
        ok = (b == 0xE0 && b1 >= 0xA0 && b1 <= 0xBF) || (b >= 0xE1 && b <= 0xEC && cont(b1)) ||
             (b == 0xED && b1 >= 0x80 && b1 <= 0x9F) || (b >= 0xEE && cont(b1));
    else
        ok = (b == 0xF0 && b1 >= 0x90 && b1 <= 0xBF) || (b >= 0xF1 && b <= 0xF3 && cont(b1)) ||
             (b == 0xF4 && b1 >= 0x80 && b1 <= 0x8F);
    for (int k = 2; ok && k < w; ++k) ok = cont(t[i + k]);
    return ok;
}

// Newlines in a 32-bit word (exact zero-byte test on x ^ '\n'...).
__device__ __forceinline__ uint32_t nl_mask(uint32_t x) {
    const uint32_t y = x ^ 0x0A0A0A0Au;
    return ~(((y & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | y | 0x7F7F7F7Fu);   // 0x80 in each byte that was '\n'
}

// Block-wide exclusive scan of one value per thread (kObjThreads threads).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *total) {
    __shared__ uint32_t warp_sums[kObjThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < (int)(kObjThreads / 32) ? warp_sums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < (int)(kObjThreads / 32)) warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t before = warp ? warp_sums[warp - 1] : 0u;
    if (total) *total = warp_sums[kObjThreads / 32 - 1];
    __syncthreads();                      // warp_sums is reused by the next call
    return before + x - v;
}

// Block-wide exclusive scans of N values per thread at once (one set of barriers).
template <int N>
__device__ __forceinline__ void block_exclusive_scan_n(const uint32_t (&v)[N], uint32_t (&ex)[N]) {
    __shared__ uint32_t wsum[kObjThreads / 32][N];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x[N];
    for (int j = 0; j < N; ++j) x[j] = v[j];
    for (int o = 1; o < 32; o <<= 1)
        for (int j = 0; j < N; ++j) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x[j], o);
            if (lane >= o) x[j] += y;
        }
    if (lane == 31)
        for (int j = 0; j < N; ++j) wsum[warp][j] = x[j];
    __syncthreads();
    for (int j = 0; j < N; ++j) {
        uint32_t before = 0;
        for (int w = 0; w < warp; ++w) before += wsum[w][j];
        ex[j] = before + x[j] - v[j];
    }
    __syncthreads();
}

// Multi-field exclusive scans without waits between blocks: each block of
// kObjThreads elements writes its sums (sums[f * nb + block]); k_scan_top
// scans every field's block sums in place (one block; totals[f] = the field's
// total); the consumer kernels, launched over the same blocks, add a block
// scan of the elements to their block's prefix.

__global__ void __launch_bounds__(1024) k_scan_top(uint32_t *sums, uint32_t nb, int nf, uint32_t *totals) {
    constexpr uint32_t kItems = 8, kChunk = 1024 * kItems;
    __shared__ uint32_t stage[kChunk];
    __shared__ uint32_t ws[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int f = 0; f < nf; ++f) {
        uint32_t *a = sums + (size_t)f * nb;
        uint32_t carry = 0;
        for (uint32_t base = 0; base < nb; base += kChunk) {
            for (uint32_t j = threadIdx.x; j < kChunk; j += 1024)          // coalesced loads
                stage[j] = base + j < nb ? a[base + j] : 0u;
            __syncthreads();
            uint32_t v[kItems], sum = 0;
            for (uint32_t j = 0; j < kItems; ++j) {
                v[j] = stage[threadIdx.x * kItems + j];
                sum += v[j];
            }
            uint32_t x = sum;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) ws[warp] = x;
            __syncthreads();
            if (warp == 0) {
                uint32_t w = ws[lane];
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                    if (lane >= o) w += y;
                }
                ws[lane] = w;
            }
            __syncthreads();
            uint32_t run = carry + (warp ? ws[warp - 1] : 0u) + x - sum;
            for (uint32_t j = 0; j < kItems; ++j) {
                stage[threadIdx.x * kItems + j] = run;
                run += v[j];
            }
            carry += ws[31];
            __syncthreads();
            for (uint32_t j = threadIdx.x; j < kChunk; j += 1024)          // coalesced stores
                if (base + j < nb) a[base + j] = stage[j];
            __syncthreads();
        }
        if (threadIdx.x == 0) totals[f] = carry;
    }
}

// Bytes of 32-bit word j of 16-byte group i16 that lie in the text [off, end).
__device__ __forceinline__ uint32_t word_in_text(uint32_t i16, int j, uint32_t off, uint32_t end) {
    const uint32_t p0 = 16u * i16 + 4u * (uint32_t)j;
    if (p0 >= off && p0 + 4u <= end) return 0xFFFFFFFFu;
    uint32_t m = 0;
    for (uint32_t b = 0; b < 4; ++b)
        if (p0 + b >= off && p0 + b < end) m |= 0xFFu << (8 * b);
    return m;
}

// First pass over the text, 16 bytes per thread: src holds the text at byte
// offset off of 16-byte groups (the caller's host buffer read in place, its
// groups aligned down, or the device copy); dst (optional) receives the
// groups.  Newlines per block and the UTF-8 check, both over [off, off + len)
// only (an aligned group never crosses a page, so reading the groups that
// overlap the text reads mapped memory only).
__global__ void __launch_bounds__(kObjThreads) k_obj_scan_text(const uint4 *src16, uint4 *dst16, uint32_t off,
                                                               unsigned long long len, uint32_t n16,
                                                               uint32_t *block_nl, unsigned long long *first_bad) {
    const uint32_t i16 = blockIdx.x * kObjThreads + threadIdx.x;
    const uint32_t end = off + (uint32_t)len;
    uint32_t cnt = 0;
    if (i16 < n16) {
        const uint4 w = src16[i16];
        if (dst16) dst16[i16] = w;
        const uint32_t r[4] = {word_in_text(i16, 0, off, end), word_in_text(i16, 1, off, end),
                               word_in_text(i16, 2, off, end), word_in_text(i16, 3, off, end)};
        cnt = __popc(nl_mask(w.x) & r[0]) + __popc(nl_mask(w.y) & r[1]) + __popc(nl_mask(w.z) & r[2]) +
              __popc(nl_mask(w.w) & r[3]);
        if (((w.x & r[0]) | (w.y & r[1]) | (w.z & r[2]) | (w.w & r[3])) & 0x80808080u) {
            const uint8_t *t = reinterpret_cast<const uint8_t *>(src16) + off;     // the text itself
            for (int k = 0; k < 16; ++k) {
                const long long i = 16ll * i16 + k - off;
                if (i >= 0 && (unsigned long long)i < len && !utf8_byte_ok(t, len, (unsigned long long)i)) {
                    atomicMin(first_bad, (unsigned long long)i);
                    break;
                }
            }
        }
    }
    uint32_t total;
    block_exclusive_scan(cnt, &total);
    if (threadIdx.x == 0) block_nl[blockIdx.x] = total;
}

// Newline positions (in buffer coordinates) of the text [off, end).
__global__ void __launch_bounds__(kObjThreads) k_obj_lines(const uint4 *t16, uint32_t n16, uint32_t off, uint32_t end,
                                                           const uint32_t *block_off, uint32_t *nl_pos) {
    const uint32_t i16 = blockIdx.x * kObjThreads + threadIdx.x;
    uint4 w = make_uint4(0, 0, 0, 0);
    if (i16 < n16) w = t16[i16];
    const uint32_t m[4] = {nl_mask(w.x) & word_in_text(i16, 0, off, end), nl_mask(w.y) & word_in_text(i16, 1, off, end),
                           nl_mask(w.z) & word_in_text(i16, 2, off, end), nl_mask(w.w) & word_in_text(i16, 3, off, end)};
    const uint32_t cnt = __popc(m[0]) + __popc(m[1]) + __popc(m[2]) + __popc(m[3]);
    uint32_t at = block_off[blockIdx.x] + block_exclusive_scan(cnt, nullptr);
    for (int k = 0; k < 4; ++k)
        for (int b = 0; b < 4; ++b)
            if (m[k] & (0x80u << (8 * b))) nl_pos[at++] = 16u * i16 + 4u * k + b;
}
struct LineArrays {
    uint8_t *kind;
    uint32_t *rest_b, *rest_e;
    uint32_t *cnt[5];   // per line: v, vn, vt, face tokens, triangles (prefixes: line_offsets)
};

// Line k of the text [off, end) of the buffer.
__device__ __forceinline__ void line_bounds(uint32_t k, uint32_t n_nl, const uint32_t *nl_pos, uint32_t off,
                                            uint32_t end, uint32_t *b, uint32_t *e) {
    *b = k == 0 ? off : nl_pos[k - 1] + 1u;
    *e = k < n_nl ? nl_pos[k] : end;
}

// str::lines + str::trim + '#' + split_ascii_whitespace + the tag match of line k.
__device__ __forceinline__ void classify_line(const uint8_t *t, uint32_t off, uint32_t end, uint32_t n_nl,
                                              const uint32_t *nl_pos, uint32_t k, LineArrays A, uint32_t c[5]) {
    uint32_t b, e;
    line_bounds(k, n_nl, nl_pos, off, end, &b, &e);
    int n;
    #pragma unroll 1
    while (b < e && (n = ws_forward(t + b, t + e)) > 0) b += n;
    #pragma unroll 1
    while (e > b && (n = ws_backward(t + b, t + e)) > 0) e -= n;
    uint8_t kind = kLineNone;
    uint32_t ntok = 0, rest = e;
    if (b < e && t[b] != '#') {
        const uint8_t *p = t + b, *pe = t + e, *tb, *te;
        next_token(p, pe, tb, te);
        const long long tl = te - tb;
        const uint8_t *rb, *re;
        const uint8_t *q = p;
        #pragma unroll 1
        while (next_token(q, pe, rb, re)) {
            if (ntok == 0) rest = (uint32_t)(rb - t);
            ++ntok;
        }
        if (tl == 1 && tb[0] == 'v' && ntok >= 3) kind = kLineV;
        else if (tl == 2 && tb[0] == 'v' && tb[1] == 'n' && ntok >= 3) kind = kLineVN;
        else if (tl == 2 && tb[0] == 'v' && tb[1] == 't' && ntok >= 2) kind = kLineVT;
        else if (tl == 1 && tb[0] == 'f' && ntok >= 3) kind = kLineF;
    }
    A.kind[k] = kind;
    A.rest_b[k] = rest;
    A.rest_e[k] = e;
    c[0] = kind == kLineV;
    c[1] = kind == kLineVN;
    c[2] = kind == kLineVT;
    c[3] = kind == kLineF ? ntok : 0u;
    c[4] = kind == kLineF ? ntok - 2 : 0u;
    for (int j = 0; j < 5; ++j) A.cnt[j][k] = c[j];
}

// Per-line kind and counts (mesh.rs:502-521), and each block's sums of the counts.
__global__ void __launch_bounds__(kObjThreads) k_obj_classify(const uint8_t *t, uint32_t off, uint32_t end,
                                                              uint32_t n_nl, const uint32_t *nl_pos, uint32_t L,
                                                              LineArrays A, uint32_t *block_sums) {
    const uint32_t k = blockIdx.x * kObjThreads + threadIdx.x;
    uint32_t c[5] = {0, 0, 0, 0, 0}, ex[5];
    if (k < L) classify_line(t, off, end, n_nl, nl_pos, k, A, c);
    block_exclusive_scan_n<5>(c, ex);
    if (threadIdx.x == kObjThreads - 1)
        for (int j = 0; j < 5; ++j) block_sums[(size_t)j * gridDim.x + blockIdx.x] = ex[j] + c[j];
}

struct TokenArrays {
    uint32_t *pi, *ti, *ni, *slot, *first;   // first: first-occurrence flag, then the vertex number
};

// Coordinates of v / vn / vt lines (mesh.rs:514-531) and the resolved indices
// of every face token (mesh.rs:532-550).
// Exclusive prefixes of line k's counts of fields J0..J0+N-1: the block's
// prefix (scanned block sums) plus the block scan of the raw counts.  Every
// thread of the block must call it.
template <int J0, int N>
__device__ __forceinline__ void line_offsets(const LineArrays &A, const uint32_t *line_sums, uint32_t L, uint32_t k,
                                             uint32_t (&off)[N]) {
    uint32_t c[N];
    for (int j = 0; j < N; ++j) c[j] = k < L ? A.cnt[J0 + j][k] : 0u;
    block_exclusive_scan_n<N>(c, off);
    for (int j = 0; j < N; ++j) off[j] += line_sums[(size_t)(J0 + j) * gridDim.x + blockIdx.x];
}

__global__ void __launch_bounds__(kObjThreads) k_obj_parse(const uint8_t *t, uint32_t L, LineArrays A,
                                                           const uint32_t *line_sums, float *pos, float *nrm,
                                                           float *uv, TokenArrays T) {
    const uint32_t k = blockIdx.x * kObjThreads + threadIdx.x;
    uint32_t off[4];
    line_offsets<0, 4>(A, line_sums, L, k, off);
    const uint32_t nV = off[0], nVN = off[1], nVT = off[2];
    uint32_t s = off[3];
    if (k >= L) return;
    const uint8_t kind = A.kind[k];
    if (kind == kLineNone) return;
    const uint8_t *p = t + A.rest_b[k], *e = t + A.rest_e[k], *tb, *te;
    if (kind != kLineF) {
        float c[3];
        const int nc = kind == kLineVT ? 2 : 3;
        #pragma unroll 1
        for (int j = 0; j < nc; ++j) {
            next_token(p, e, tb, te);
            c[j] = f32_or_zero(tb, te);
        }
        if (kind == kLineV) {
            float *o = pos + 3ull * nV;
            o[0] = c[0]; o[1] = c[1]; o[2] = c[2];
        } else if (kind == kLineVN) {
            const float3 nn = normalize3(c[0], c[1], c[2]);
            float *o = nrm + 3ull * nVN;
            o[0] = nn.x; o[1] = nn.y; o[2] = nn.z;
        } else {
            float *o = uv + 2ull * nVT;
            o[0] = c[0]; o[1] = c[1];
        }
        return;
    }
    #pragma unroll 1
    while (next_token(p, e, tb, te)) {
        // token.split('/'): parts 0, 1, 2 (later parts are not read)
        const uint8_t *s1 = tb;
        #pragma unroll 1
        while (s1 < te && *s1 != '/') ++s1;
        uint32_t pi = 0, ti = kNone, ni = kNone, r;
        bool pres = resolve(tb, s1, nV, &r);
        if (pres) pi = r;
        bool has_norm = false;
        if (s1 < te) {
            const uint8_t *b1 = s1 + 1, *s2 = b1;
            #pragma unroll 1
            while (s2 < te && *s2 != '/') ++s2;
            if (s2 > b1 && resolve(b1, s2, nVT, &r)) ti = r;
            if (s2 < te) {
                const uint8_t *b2 = s2 + 1, *s3 = b2;
                #pragma unroll 1
                while (s3 < te && *s3 != '/') ++s3;
                long long iv;
                has_norm = parse_i64(b2, s3, &iv);        // an empty part does not parse
                if (has_norm && resolve_value(iv, nVN, &r)) ni = r;
            }
        }
        T.pi[s] = pi | ((pres || nV > 0) ? kPosOk : 0u) | (has_norm ? kHasNorm : 0u);
        T.ti[s] = ti;
        T.ni[s] = ni;
        ++s;
    }
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {   // SplitMix64 finaliser
    x ^= x >> 30; x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 27; x *= 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
// Open-addressing hash table entry: a 64-bit key and the least face token
// that carries it, in one 16-byte record (one sector per probe).
struct alignas(16) Slot {
    unsigned long long key;
    uint32_t min_tok;
    uint32_t pad;
};
// How (position, uv, normal) becomes a table key: one mixed-radix 64-bit key
// when the three index ranges fit (rp * rt * rn < 2^63), else two tables:
// (position, uv) -> slot of table A, then (slot A, normal).
struct KeyPack {
    int packed;
    unsigned long long rp, rt;
    uint32_t no_uv;            // uv index written as kNone -> rt - 1
};

// Slot of key (inserted if absent); kNone if the table is full, which the
// capacity (twice the face tokens) rules out.
__device__ uint32_t table_slot(Slot *tab, uint32_t mask, unsigned long long key) {
    uint32_t h = (uint32_t)mix64(key) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
        const unsigned long long cur = tab[h].key;
        if (cur == key) return h;
        if (cur == kEmptyKey) {
            const unsigned long long old = atomicCAS(&tab[h].key, kEmptyKey, key);
            if (old == kEmptyKey || old == key) return h;
        }
    }
    return kNone;
}

// vert_cache (mesh.rs:486-489, :556-575): tokens with a resolved normal share
// a vertex per (position, uv, normal); the vertex belongs to the key's first
// token (the least token number).
__global__ void __launch_bounds__(kObjThreads) k_obj_dedup(uint32_t n_tok, TokenArrays T, Slot *tab_a, Slot *tab_b,
                                                           uint32_t mask, KeyPack kp, uint32_t *err) {
    const uint32_t s = blockIdx.x * kObjThreads + threadIdx.x;
    if (s >= n_tok) return;
    const uint32_t ni = T.ni[s];
    if (ni == kNone) { T.slot[s] = kNone; return; }
    const uint32_t pi = T.pi[s] & kPosMask, ti = T.ti[s];
    uint32_t b;
    if (kp.packed) {
        const unsigned long long tt = ti == kNone ? kp.no_uv : ti;
        b = table_slot(tab_b, mask, pi + kp.rp * (tt + kp.rt * ni));
    } else {
        const uint32_t a = table_slot(tab_a, mask, (unsigned long long)pi | ((unsigned long long)ti << 32));
        b = a == kNone ? kNone : table_slot(tab_b, mask, (unsigned long long)a | ((unsigned long long)ni << 32));
    }
    if (b == kNone) { atomicExch(err, 1u); T.slot[s] = kNone; return; }
    atomicMin(&tab_b[b].min_tok, s);
    T.slot[s] = b;
}

// 1 for the token that creates a vertex: no resolved normal (always a fresh
// vertex, mesh.rs:576-591) or the first token of its key; block sums for the scan.
__global__ void __launch_bounds__(kObjThreads) k_obj_first(uint32_t n_tok, TokenArrays T, const Slot *tab,
                                                           uint32_t *block_sums) {
    const uint32_t s = blockIdx.x * kObjThreads + threadIdx.x;
    uint32_t f = 0;
    if (s < n_tok) {
        const uint32_t slot = T.slot[s];
        f = (slot == kNone || tab[slot].min_tok == s) ? 1u : 0u;
        T.first[s] = f;
    }
    uint32_t total;
    block_exclusive_scan(f, &total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// The records of the tokens that create vertices; their vertex numbers (the
// exclusive scan of the first-occurrence flags) replace the flags in T.first.
__global__ void __launch_bounds__(kObjThreads) k_obj_vertices(uint32_t n_tok, TokenArrays T, const uint32_t *tok_sums,
                                                              const float *pos, const float *nrm, const float *uv,
                                                              float4 *verts) {
    const uint32_t s = blockIdx.x * kObjThreads + threadIdx.x;
    const uint32_t f = s < n_tok ? T.first[s] : 0u;
    const uint32_t vid = tok_sums[blockIdx.x] + block_exclusive_scan(f, nullptr);
    if (!f) return;
    T.first[s] = vid;
    const uint32_t pw = T.pi[s], ti = T.ti[s], ni = T.ni[s];
    float4 P = make_float4(0.0f, 0.0f, 0.0f, 1.0f), N = make_float4(0.0f, 1.0f, 0.0f, 0.0f),
           U = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (pw & kPosOk) {
        const float *q = pos + 3ull * (pw & kPosMask);
        P.x = q[0]; P.y = q[1]; P.z = q[2];
    }
    if (ni != kNone) {
        const float *q = nrm + 3ull * ni;
        N.x = q[0]; N.y = q[1]; N.z = q[2];
    }
    if (ti != kNone) {
        const float *q = uv + 2ull * ti;
        U.x = q[0]; U.y = q[1];
    }
    float4 *o = verts + 3ull * vid;
    o[0] = P; o[1] = N; o[2] = U;
}

// Fan triangulation and the normal patch of tokens without has_norm
// (mesh.rs:593-630).  A token's vertex is patched by every triangle of its fan
// that contains it; the last one wins: triangle min(j, n-2) for token j >= 1,
// triangle n-2 for token 0.  Such tokens own fresh vertices, so no two threads
// write one vertex.
__device__ __forceinline__ uint32_t token_vertex(const TokenArrays &T, const Slot *tab, uint32_t x) {
    const uint32_t slot = T.slot[x];
    return T.first[slot == kNone ? x : tab[slot].min_tok];
}

__global__ void __launch_bounds__(kObjThreads) k_obj_faces(uint32_t L, LineArrays A, const uint32_t *line_sums,
                                                           TokenArrays T, const Slot *tab, float4 *verts,
                                                           uint32_t base_v, uint4 *tris, uint32_t mat_idx) {
    const uint32_t k = blockIdx.x * kObjThreads + threadIdx.x;
    uint32_t off[2];
    line_offsets<3, 2>(A, line_sums, L, k, off);
    const uint32_t s0 = off[0], t0 = off[1];
    if (k >= L || A.kind[k] != kLineF) return;
    const uint32_t n = A.cnt[3][k];
    const uint32_t v0 = token_vertex(T, tab, s0);
    uint32_t vb = token_vertex(T, tab, s0 + 1);
    for (uint32_t i = 1; i + 1 < n; ++i) {
        const uint32_t vc = token_vertex(T, tab, s0 + i + 1);
        tris[t0 + i - 1] = make_uint4(base_v + v0, base_v + vb, base_v + vc, mat_idx);
        vb = vc;
    }
    for (uint32_t j = 0; j < n; ++j) {
        if (T.pi[s0 + j] & kHasNorm) continue;
        const uint32_t i = j == 0 ? n - 2 : min(j, n - 2);
        const float4 p0 = verts[3ull * v0], p1 = verts[3ull * token_vertex(T, tab, s0 + i)],
                     p2 = verts[3ull * token_vertex(T, tab, s0 + i + 1)];
        const float e1x = p1.x - p0.x, e1y = p1.y - p0.y, e1z = p1.z - p0.z;
        const float e2x = p2.x - p0.x, e2y = p2.y - p0.y, e2z = p2.z - p0.z;
        const float3 g = normalize3(e1y * e2z - e1z * e2y, e1z * e2x - e1x * e2z, e1x * e2y - e1y * e2x);
        verts[3ull * token_vertex(T, tab, s0 + j) + 1] = make_float4(g.x, g.y, g.z, 0.0f);
    }
}

// Scale -> rotate -> translate of positions, rotate of normals (scene.rs:846-861, :473-494).
__global__ void __launch_bounds__(kObjThreads) k_obj_transform(float4 *verts, uint32_t nv, ObjTransform X) {
    const uint32_t i = blockIdx.x * kObjThreads + threadIdx.x;
    if (i >= nv) return;
    float4 P = verts[3ull * i], N = verts[3ull * i + 1];
    float q[3] = {P.x * X.s, P.y * X.s, P.z * X.s};
    float n[3] = {N.x, N.y, N.z};
    if (X.has_r) {
        float r[3], m[3];
        for (int a = 0; a < 3; ++a) {
            r[a] = X.m[3 * a] * q[0] + X.m[3 * a + 1] * q[1] + X.m[3 * a + 2] * q[2];
            m[a] = X.m[3 * a] * n[0] + X.m[3 * a + 1] * n[1] + X.m[3 * a + 2] * n[2];
        }
        for (int a = 0; a < 3; ++a) { q[a] = r[a]; n[a] = m[a]; }
    }
    verts[3ull * i] = make_float4(q[0] + X.t[0], q[1] + X.t[1], q[2] + X.t[2], P.w);
    verts[3ull * i + 1] = make_float4(n[0], n[1], n[2], N.w);
}

__global__ void k_rebase_tris(const uint4 *in, uint32_t n, uint32_t add, uint4 *out) {
    const uint32_t i = blockIdx.x * kObjThreads + threadIdx.x;
    if (i >= n) return;
    const uint4 t = in[i];
    out[i] = make_uint4(t.x + add, t.y + add, t.z + add, t.w);
}

uint32_t blocks_for(unsigned long long n) { return (uint32_t)((n + kObjThreads - 1) / kObjThreads); }

template <typename T> T *carve(char *&p, size_t n) {
    T *r = reinterpret_cast<T *>(p);
    p += (n * sizeof(T) + 255) & ~size_t(255);
    return r;
}
size_t carve_bytes(size_t n, size_t elem) { return (n * elem + 255) & ~size_t(255); }

#define OBJ_CK(x)                                  \
    do {                                           \
        cudaError_t e__ = (x);                     \
        if (e__ != cudaSuccess) return e__;        \
    } while (0)

}  // namespace

cudaError_t mesh_reserve(DeviceMesh &M, uint32_t add_v, uint32_t add_t, cudaStream_t st) {
    auto grow = [&](DBuf &b, size_t used, size_t need) -> cudaError_t {
        if (b.p && need <= b.cap) return cudaSuccess;
        size_t cap = std::max(need, b.cap + b.cap / 2);
        void *p = nullptr;
        OBJ_CK(cudaMalloc(&p, cap));
        if (used) {
            cudaError_t e = cudaMemcpyAsync(p, b.p, used, cudaMemcpyDeviceToDevice, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) { cudaFree(p); return e; }
        }
        if (b.p) cudaFree(b.p);
        b.p = p;
        b.cap = cap;
        return cudaSuccess;
    };
    OBJ_CK(grow(M.vertices, (size_t)M.nv * 48, ((size_t)M.nv + add_v) * 48));
    OBJ_CK(grow(M.triangles, (size_t)M.nt * 16, ((size_t)M.nt + add_t) * 16));
    return cudaSuccess;
}

cudaError_t mesh_append_host(DeviceMesh &M, const mcrt_gpu_vertex *v, uint32_t nv, const mcrt_gpu_triangle *t,
                             uint32_t nt, DBuf &staging, cudaStream_t st) {
    OBJ_CK(mesh_reserve(M, nv, nt, st));
    if (nv) OBJ_CK(cudaMemcpyAsync(M.vertices.as<char>() + (size_t)M.nv * 48, v, (size_t)nv * 48,
                                   cudaMemcpyHostToDevice, st));
    if (nt) {
        OBJ_CK(staging.ensure((size_t)nt * 16));
        OBJ_CK(cudaMemcpyAsync(staging.p, t, (size_t)nt * 16, cudaMemcpyHostToDevice, st));
        k_rebase_tris<<<blocks_for(nt), kObjThreads, 0, st>>>(staging.as<uint4>(), nt, M.nv,
                                                              M.triangles.as<uint4>() + M.nt);
        note_launch();
    }
    OBJ_CK(cudaStreamSynchronize(st));
    M.nv += nv;
    M.nt += nt;
    return cudaSuccess;
}

cudaError_t obj_append(const char *host_text, unsigned long long len, uint32_t mat_idx, const ObjTransform &X,
                       DeviceMesh &M, ObjScratch &S, cudaStream_t st, bool direct, ObjOutcome *out) {
    *out = ObjOutcome{};
    out->code = ObjOutcome::kNoGeometry;
    if (len == 0) return cudaSuccess;
    if (!S.ev[0])
        for (cudaEvent_t &e : S.ev) OBJ_CK(cudaEventCreate(&e));
    const unsigned long long launches0 = launch_count();
    if (len > 0xFFFFFF00ull - 16) return cudaErrorInvalidValue;  // byte offsets are 32-bit
    // ---- stage 1: text, newline counts per block, UTF-8 check.  direct: the
    // first pass reads the caller's buffer in place (pageable memory the GPU
    // reaches through the host page tables) and copies it as it scans; the
    // text then starts at byte `off` of its first 16-byte group.
    const uintptr_t hp = reinterpret_cast<uintptr_t>(host_text);
    const uint32_t off = direct ? (uint32_t)(hp & 15u) : 0u;
    const uint32_t end = off + (uint32_t)len;
    const uint32_t n16 = (uint32_t)((off + len + 15) / 16);
    const uint32_t nb = blocks_for(n16);
    {
        const size_t bytes = carve_bytes((size_t)n16 * 16 + 16, 1) + carve_bytes(nb, 4) + carve_bytes(16, 8);
        OBJ_CK(S.text.ensure(bytes));
    }
    char *p = S.text.as<char>();
    uint8_t *text = carve<uint8_t>(p, (size_t)n16 * 16 + 16);
    uint32_t *block_nl = carve<uint32_t>(p, nb);                      // newlines per block -> block offsets
    unsigned long long *small = carve<unsigned long long>(p, 16);     // [0] first bad byte, [1..] totals
    uint32_t *totals = reinterpret_cast<uint32_t *>(small + 2);       // [0] newlines, [1..5] line fields, [6] vertices
    OBJ_CK(cudaMemsetAsync(text + (size_t)n16 * 16 - 16, 0, 32, st));
    OBJ_CK(cudaMemsetAsync(small, 0xFF, 8, st));
    OBJ_CK(cudaEventRecord(S.ev[0], st));
    if (direct) {
        k_obj_scan_text<<<nb, kObjThreads, 0, st>>>(reinterpret_cast<const uint4 *>(hp - off),
                                                    reinterpret_cast<uint4 *>(text), off, len, n16, block_nl, small);
        note_launch();
        OBJ_CK(cudaEventRecord(S.ev[1], st));
    } else {
        OBJ_CK(cudaMemcpyAsync(text, host_text, len, cudaMemcpyHostToDevice, st));
        OBJ_CK(cudaEventRecord(S.ev[1], st));
        k_obj_scan_text<<<nb, kObjThreads, 0, st>>>(reinterpret_cast<const uint4 *>(text), nullptr, 0u, len, n16,
                                                    block_nl, small);
        note_launch();
    }
    k_scan_top<<<1, 1024, 0, st>>>(block_nl, nb, 1, totals);
    note_launch();
    OBJ_CK(cudaEventRecord(S.ev[2], st));
    unsigned long long first_bad = 0;
    uint32_t n_nl = 0;
    OBJ_CK(cudaMemcpyAsync(&first_bad, small, 8, cudaMemcpyDeviceToHost, st));
    OBJ_CK(cudaMemcpyAsync(&n_nl, totals, 4, cudaMemcpyDeviceToHost, st));
    OBJ_CK(cudaStreamSynchronize(st));
    if (first_bad < len) {
        out->code = ObjOutcome::kNotUtf8;
        out->valid_up_to = first_bad;
        return cudaSuccess;
    }
    const uint32_t L = n_nl + (host_text[len - 1] != '\n' ? 1u : 0u);
    if (L == 0) return cudaSuccess;
    // ---- stage 2: lines, classification, the five line scans
    const uint32_t nbl = blocks_for(L);
    {
        const size_t bytes = carve_bytes(std::max<uint32_t>(n_nl, 1), 4) + carve_bytes(L, 1) +
                             7 * carve_bytes(L, 4) + carve_bytes(5ull * nbl, 4);
        OBJ_CK(S.lines.ensure(bytes));
    }
    p = S.lines.as<char>();
    uint32_t *nl_pos = carve<uint32_t>(p, std::max<uint32_t>(n_nl, 1));
    LineArrays A;
    A.kind = carve<uint8_t>(p, L);
    A.rest_b = carve<uint32_t>(p, L);
    A.rest_e = carve<uint32_t>(p, L);
    for (int j = 0; j < 5; ++j) A.cnt[j] = carve<uint32_t>(p, L);
    uint32_t *line_sums = carve<uint32_t>(p, 5ull * nbl);
    OBJ_CK(cudaEventRecord(S.ev[3], st));
    k_obj_lines<<<nb, kObjThreads, 0, st>>>(reinterpret_cast<const uint4 *>(text), n16, off, end, block_nl, nl_pos);
    note_launch();
    k_obj_classify<<<nbl, kObjThreads, 0, st>>>(text, off, end, n_nl, nl_pos, L, A, line_sums);
    note_launch();
    k_scan_top<<<1, 1024, 0, st>>>(line_sums, nbl, 5, totals + 1);
    note_launch();
    OBJ_CK(cudaEventRecord(S.ev[4], st));
    uint32_t tot[5];
    OBJ_CK(cudaMemcpyAsync(tot, totals + 1, sizeof(tot), cudaMemcpyDeviceToHost, st));
    OBJ_CK(cudaStreamSynchronize(st));
    const uint32_t nV = tot[0], nVN = tot[1], nVT = tot[2], n_tok = tot[3], n_tri = tot[4];
    if (n_tri == 0) return cudaSuccess;           // no face line: no vertices and no triangles
    if (n_tok > (1u << 30)) return cudaErrorInvalidValue;
    // ---- stage 3: coordinates, face tokens, first occurrences
    uint32_t cap = 1024;
    while (cap < 2u * n_tok) cap <<= 1;
    KeyPack kp;
    kp.rp = std::max(nV, 1u);
    kp.rt = (unsigned long long)nVT + 1;
    kp.no_uv = nVT;
    const unsigned long long rn = std::max(nVN, 1u);
    kp.packed = kp.rp * kp.rt <= (1ull << 62) / rn;      // rp * rt * rn < 2^63: one table
    const uint32_t ntok_blocks = blocks_for(n_tok);
    {
        const size_t bytes = carve_bytes(3ull * std::max(nV, 1u), 4) + carve_bytes(3ull * std::max(nVN, 1u), 4) +
                             carve_bytes(2ull * std::max(nVT, 1u), 4) + 5 * carve_bytes(n_tok, 4) +
                             (kp.packed ? 1 : 2) * carve_bytes(cap, sizeof(Slot)) + carve_bytes(ntok_blocks, 4) +
                             carve_bytes(16, 4);
        OBJ_CK(S.tokens.ensure(bytes));
    }
    p = S.tokens.as<char>();
    float *pos = carve<float>(p, 3ull * std::max(nV, 1u));
    float *nrm = carve<float>(p, 3ull * std::max(nVN, 1u));
    float *uv = carve<float>(p, 2ull * std::max(nVT, 1u));
    TokenArrays T;
    T.pi = carve<uint32_t>(p, n_tok); T.ti = carve<uint32_t>(p, n_tok); T.ni = carve<uint32_t>(p, n_tok);
    T.slot = carve<uint32_t>(p, n_tok); T.first = carve<uint32_t>(p, n_tok);
    Slot *tab_b = carve<Slot>(p, cap);
    Slot *tab_a = kp.packed ? nullptr : carve<Slot>(p, cap);
    uint32_t *tok_sums = carve<uint32_t>(p, ntok_blocks);
    uint32_t *flags = carve<uint32_t>(p, 16);         // [0] table error
    OBJ_CK(cudaMemsetAsync(tab_b, 0xFF, (kp.packed ? 1 : 2) * carve_bytes(cap, sizeof(Slot)), st));   // empty keys
    OBJ_CK(cudaMemsetAsync(flags, 0, 64, st));
    OBJ_CK(cudaEventRecord(S.ev[5], st));
    k_obj_parse<<<nbl, kObjThreads, 0, st>>>(text, L, A, line_sums, pos, nrm, uv, T);
    note_launch();
    k_obj_dedup<<<ntok_blocks, kObjThreads, 0, st>>>(n_tok, T, tab_a, tab_b, cap - 1, kp, flags);
    note_launch();
    k_obj_first<<<ntok_blocks, kObjThreads, 0, st>>>(n_tok, T, tab_b, tok_sums);
    note_launch();
    k_scan_top<<<1, 1024, 0, st>>>(tok_sums, ntok_blocks, 1, totals + 6);
    note_launch();
    OBJ_CK(cudaEventRecord(S.ev[6], st));
    uint32_t table_err = 0, NV = 0;
    OBJ_CK(cudaMemcpyAsync(&table_err, flags, 4, cudaMemcpyDeviceToHost, st));
    OBJ_CK(cudaMemcpyAsync(&NV, totals + 6, 4, cudaMemcpyDeviceToHost, st));
    OBJ_CK(cudaStreamSynchronize(st));
    if (table_err) return cudaErrorUnknown;           // a full table: excluded by its capacity
    if ((unsigned long long)M.nv + NV >= (1ull << 31) || (unsigned long long)M.nt + n_tri >= (1ull << 27))
        return cudaErrorInvalidValue;
    // ---- stage 4: records, appended at the end of the device mesh
    OBJ_CK(mesh_reserve(M, NV, n_tri, st));
    float4 *verts = M.vertices.as<float4>() + 3ull * M.nv;
    OBJ_CK(cudaEventRecord(S.ev[7], st));
    k_obj_vertices<<<ntok_blocks, kObjThreads, 0, st>>>(n_tok, T, tok_sums, pos, nrm, uv, verts);
    note_launch();
    k_obj_faces<<<nbl, kObjThreads, 0, st>>>(L, A, line_sums, T, tab_b, verts, M.nv,
                                             M.triangles.as<uint4>() + M.nt, mat_idx);
    note_launch();
    if (!X.identity) {
        k_obj_transform<<<blocks_for(NV), kObjThreads, 0, st>>>(verts, NV, X);
        note_launch();
    }
    OBJ_CK(cudaGetLastError());
    OBJ_CK(cudaEventRecord(S.ev[8], st));
    OBJ_CK(cudaStreamSynchronize(st));
    float ms[5];
    OBJ_CK(cudaEventElapsedTime(&ms[0], S.ev[0], S.ev[1]));
    OBJ_CK(cudaEventElapsedTime(&ms[1], S.ev[1], S.ev[2]));
    OBJ_CK(cudaEventElapsedTime(&ms[2], S.ev[3], S.ev[4]));
    OBJ_CK(cudaEventElapsedTime(&ms[3], S.ev[5], S.ev[6]));
    OBJ_CK(cudaEventElapsedTime(&ms[4], S.ev[7], S.ev[8]));
    out->h2d_ms = ms[0];
    out->kernel_ms = ms[1] + ms[2] + ms[3] + ms[4];
    out->launches = launch_count() - launches0;
    M.nv += NV;
    M.nt += n_tri;
    out->code = ObjOutcome::kOk;
    out->n_vertices = NV;
    out->n_triangles = n_tri;
    out->n_lines = L;
    out->n_tokens = n_tok;
    return cudaSuccess;
}

}  // namespace mcrt
