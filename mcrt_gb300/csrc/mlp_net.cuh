// mlp_net.cuh — shape, parameter layout and input encoding of the radiance-cache
// MLP (shared by the cache kernels and the tracer that feeds them).
//
// Network: 96 encoded inputs -> 5 hidden layers of 64 ReLU units -> 3 outputs
// (the output layer is 16 wide for the tensor cores; rows 3..15 stay zero).
// Inputs of a query at a surface point: position p (world), the outgoing
// direction w_o (towards the previous path vertex), the shading normal n and
// the albedo a.  Encoding: u = clamp((p - lo) * inv_extent, 0, 1) per axis;
// features [0, 72): sin / cos of u * pi * 2^k for k = 0..11, axis-major;
// [72, 75) w_o, [75, 78) n, [78, 81) a, [81, 84) u, [84, 96) zero.
#pragma once

#include <cstdint>

#include "fmath.h"

namespace mcrt {
namespace mlp {

constexpr int kIn = 96, kHid = 64, kOutPad = 16, kOut = 3, kLayers = 6, kTile = 128;
constexpr int kBands = 12;

// fp32 parameter vector: W_l row-major [out][in] followed by b_l, layer by layer.
__host__ __device__ constexpr int in_of(int l) { return l == 0 ? kIn : kHid; }
__host__ __device__ constexpr int out_of(int l) { return l == kLayers - 1 ? kOutPad : kHid; }
__host__ __device__ constexpr int w_off(int l) {
    return l == 0 ? 0 : w_off(l - 1) + out_of(l - 1) * in_of(l - 1) + out_of(l - 1);
}
__host__ __device__ constexpr int b_off(int l) { return w_off(l) + out_of(l) * in_of(l); }
constexpr int kParams = b_off(kLayers - 1) + kOutPad;   // 23888
// bf16 weight image: layer l's matrix in the tensor-core operand layout
// (rows = out, K = in), layers back to back.
__host__ __device__ constexpr int img_off(int l) {
    return l == 0 ? 0 : img_off(l - 1) + out_of(l - 1) * in_of(l - 1) * 2;
}
constexpr int kImgBytes = img_off(kLayers);               // 47104
constexpr int kBiasFloats = kHid * (kLayers - 1) + kOutPad;  // 336
__host__ __device__ constexpr int bias_idx(int l) { return l * kHid; }

static_assert(kParams == 23888, "parameter count");
static_assert(kImgBytes == 47104, "weight image size");

// pi * 2^k rounded to float
__host__ __device__ inline float band_freq(int k) {
    constexpr float f[kBands] = {
        3.141592653589793f,  6.283185307179586f,  12.566370614359172f, 25.132741228718345f,
        50.26548245743669f,  100.53096491487338f, 201.06192982974676f, 402.1238596594935f,
        804.247719318987f,   1608.495438637974f,  3216.990877275948f,  6433.981754551896f};
    return f[k];
}

// The 96 features of a query (12 floats: p, w_o, n, a).  The bands come from
// one sine / cosine of pi * u per axis by the double-angle recurrence
// s' = (2 s) c, c' = c c - s s (each band doubles the frequency).
__host__ __device__ inline void encode(const float q[12], const float lo[3], const float inv_ext[3],
                                       float f[kIn]) {
    float u[3];
    for (int a = 0; a < 3; ++a) {
        float v = (q[a] - lo[a]) * inv_ext[a];
        u[a] = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
        float s, c;
        fm_sincos(u[a] * band_freq(0), &s, &c);
        for (int k = 0; k < kBands; ++k) {
            f[24 * a + 2 * k] = s;
            f[24 * a + 2 * k + 1] = c;
            const float s2 = (2.0f * s) * c, c2 = c * c - s * s;
            s = s2;
            c = c2;
        }
    }
    for (int k = 0; k < 9; ++k) f[72 + k] = q[3 + k];
    for (int a = 0; a < 3; ++a) f[81 + a] = u[a];
    for (int k = 84; k < kIn; ++k) f[k] = 0.0f;
}

}  // namespace mlp
}  // namespace mcrt
