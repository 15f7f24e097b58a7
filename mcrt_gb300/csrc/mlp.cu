// mlp.cu — the radiance-cache MLP on the tensor cores (tcgen05, BF16 operands,
// FP32 accumulators in tensor memory).
//
// This file starts with the probe of one tensor-core product, which pins the
// operand layouts and descriptors of tc.cuh against a CPU product.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"
#include "internal.h"
#include "mlp_net.cuh"
#include "tc.cuh"

namespace mcrt {

namespace {

constexpr uint32_t kProbeM = 128;
constexpr uint32_t kProbeARegion = 64 * 1024;   // operand regions sized so that any stride of the
constexpr uint32_t kProbeBRegion = 16 * 1024;   // descriptors stays inside them
constexpr uint32_t kPollLimit = 1u << 22;

// D[128 x N] = A[128 x K] * B[N x K]^T with A, B bf16 (row-major in global
// memory), staged in shared memory K-major or MN-major (flags bit 0: A, bit 1: B).
// status[0]: 0 ok, 1 the MMA did not complete within the poll limit.
__global__ void __launch_bounds__(128) k_gemm_probe(const uint16_t *A, const uint16_t *B, uint32_t K, uint32_t N,
                                                    uint32_t flags, float *D, uint32_t *status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sa = smem;
    uint8_t *sb = smem + kProbeARegion;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + kProbeARegion + kProbeBRegion);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 1);
    const bool a_mn = flags & 1u, b_mn = flags & 2u;
    const uint32_t t = threadIdx.x, warp = t >> 5;
    for (uint32_t i = t; i < kProbeARegion / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(sa)[i] = 0u;
    for (uint32_t i = t; i < kProbeBRegion / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(sb)[i] = 0u;
    __syncthreads();
    for (uint32_t i = t; i < kProbeM * K; i += blockDim.x) {
        uint32_t m = i / K, k = i - m * K;
        uint32_t off = a_mn ? tc::op_offset(k, m, K) : tc::op_offset(m, k, kProbeM);
        *reinterpret_cast<uint16_t *>(sa + off) = A[i];
    }
    for (uint32_t i = t; i < N * K; i += blockDim.x) {
        uint32_t n = i / K, k = i - n * K;
        uint32_t off = b_mn ? tc::op_offset(k, n, K) : tc::op_offset(n, k, N);
        *reinterpret_cast<uint16_t *>(sb + off) = B[i];
    }
    tc::fence_proxy_async();
    uint32_t ncols = 32;
    while (ncols < N) ncols <<= 1;
    if (warp == 0) tc::tmem_alloc(tslot, ncols);
    if (t == 0) tc::mbar_init(mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = *tslot;
    if (t == 0) {
        const uint32_t idesc = tc::idesc_bf16(kProbeM, N, a_mn, b_mn);
        const uint32_t a_lbo = a_mn ? 128u : (kProbeM / 8) * 128u, a_sbo = a_mn ? (K / 8) * 128u : 128u;
        const uint32_t b_lbo = b_mn ? 128u : (N / 8) * 128u, b_sbo = b_mn ? (K / 8) * 128u : 128u;
        for (uint32_t kk = 0; kk < K / 16; ++kk) {
            const uint32_t a_step = a_mn ? 256u : 2u * (kProbeM / 8) * 128u;
            const uint32_t b_step = b_mn ? 256u : 2u * (N / 8) * 128u;
            uint64_t ad = tc::make_desc(tc::smem_u32(sa) + kk * a_step, a_lbo, a_sbo);
            uint64_t bd = tc::make_desc(tc::smem_u32(sb) + kk * b_step, b_lbo, b_sbo);
            tc::mma_bf16(taddr, ad, bd, idesc, kk > 0 ? 1u : 0u);
        }
        tc::commit(mbar);
    }
    const bool ok = __syncthreads_and(tc::mbar_wait(mbar, 0, kPollLimit) ? 1 : 0) != 0;   // uniform
    tc::fence_after_sync();
    if (!ok) {
        if (t == 0) status[0] = 1u;
    } else {
        const uint32_t row = warp * 32 + (t & 31u);
        for (uint32_t c = 0; c < N; c += 16) {
            float v[16];
            tc::tmem_ld16(taddr + ((warp * 32u) << 16) + c, v);
            for (int j = 0; j < 16; ++j)
                if (c + j < N) D[(size_t)row * N + c + j] = v[j];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::tmem_dealloc(taddr, ncols);
        tc::tmem_relinquish();
    }
}

}  // namespace

// ============================================================================ radiance-cache MLP
namespace {

using namespace mlp;

// Device view of the network: bf16 weight image (operand layout, rows = out),
// fp32 biases (layer l at l * 64), encoding bounds.
struct NetDev {
    const uint8_t *img;
    const float *bias;
    float lo[3], inv_ext[3];
};

constexpr uint32_t kSmemImg = 0;
constexpr uint32_t kSmemBias = kSmemImg + kImgBytes;                       // 47104
constexpr uint32_t kSmemAct = kSmemBias + kBiasFloats * 4;                 // 48448
constexpr uint32_t kTileIn = kTile * kIn * 2;                              // 24576
constexpr uint32_t kTileHid = kTile * kHid * 2;                            // 16384
// inference: image | bias | one activation tile | mbarrier | TMEM slot
constexpr uint32_t kInferGroups = 7;                     // one CTA per SM (shared memory), 896 threads
constexpr uint32_t kInferSmem = kSmemAct + kInferGroups * kTileIn + 64;
constexpr uint32_t kInferTmemCols = 64 * kInferGroups <= 128 ? 128 : (64 * kInferGroups <= 256 ? 256 : 512);   // a power of 2
static_assert(64 * kInferGroups <= 512, "TMEM columns of the inference pipelines");
// training: image | bias | X0 | H1..H5 | G (128 x 128, upper half zero) | bias grads | misc
constexpr uint32_t kTrainX0 = kSmemAct;
constexpr uint32_t kTrainH = kTrainX0 + kTileIn;
constexpr uint32_t kTrainG = kTrainH + 5 * kTileHid;
constexpr uint32_t kTrainDb = kTrainG + 2 * kTileHid;
constexpr uint32_t kTrainMisc = kTrainDb + kBiasFloats * 4;
constexpr uint32_t kTrainSmem = kTrainMisc + 64;
static_assert(kTrainSmem <= 227 * 1024, "training kernel shared memory");
// TMEM columns of the training kernel: forward / backward-data accumulator at
// 0, weight-gradient accumulators of layer l at kDwCol[l] (in_of(l) columns)
__device__ constexpr uint32_t kDwCol[kLayers] = {64, 160, 224, 288, 352, 416};

__device__ __forceinline__ uint32_t bf16_bits(float x) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ float bf16_float(uint32_t b) { return __uint_as_float(b << 16); }
__device__ __forceinline__ uint32_t pack2(float a, float b) { return bf16_bits(a) | (bf16_bits(b) << 16); }
// bf16 pair of max(a, 0), max(b, 0) in one conversion: cvt.rn.relu.bf16x2.f32
// rounds both to bf16 and clamps negative results to +0 (rounding keeps the
// sign, so the order of the clamp and the rounding does not matter).
__device__ __forceinline__ uint32_t pack2_relu(float a, float b) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(b), "f"(a));
    return d;
}

// Stage the weight image and biases in shared memory (16-byte vector copies).
__device__ void load_net(const NetDev &net, uint8_t *smem) {
    const uint4 *src = reinterpret_cast<const uint4 *>(net.img);
    uint4 *dst = reinterpret_cast<uint4 *>(smem + kSmemImg);
    for (uint32_t i = threadIdx.x; i < kImgBytes / 16; i += blockDim.x) dst[i] = src[i];
    float *b = reinterpret_cast<float *>(smem + kSmemBias);
    for (uint32_t i = threadIdx.x; i < kBiasFloats; i += blockDim.x) b[i] = net.bias[i];
}

// Encode the query of this thread's row into the input tile (bf16, 12 chunks
// of 8): the features of mlp::encode (the same arithmetic), written 8 at a
// time as they are formed: one axis's 12 bands are three chunks
// of 4 (sin, cos) pairs, so at most 8 features are live (the register budget
// of the inference kernel's pipelines).
__device__ __forceinline__ void store_chunk(uint8_t *tile, uint32_t row, int c, const float f[8]) {
    *reinterpret_cast<uint4 *>(tile + tc::op_offset(row, 8 * c, kTile)) =
        make_uint4(pack2(f[0], f[1]), pack2(f[2], f[3]), pack2(f[4], f[5]), pack2(f[6], f[7]));
}
__device__ void encode_row_streamed(const NetDev &net, const float q[12], bool valid, uint8_t *tile, uint32_t row) {
    float u[3];
    for (int a = 0; a < 3; ++a) {
        float s = 0.0f, c = 0.0f;
        if (valid) {
            const float v = (q[a] - net.lo[a]) * net.inv_ext[a];
            u[a] = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
            fm_sincos(u[a] * band_freq(0), &s, &c);
        } else {
            u[a] = 0.0f;
        }
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            float f[8];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                f[2 * k] = valid ? s : 0.0f;
                f[2 * k + 1] = valid ? c : 0.0f;
                const float s2 = (2.0f * s) * c, c2 = c * c - s * s;
                s = s2;
                c = c2;
            }
            store_chunk(tile, row, 3 * a + ch, f);
        }
    }
    const float z = 0.0f;
    float f9[8] = {q[3], q[4], q[5], q[6], q[7], q[8], q[9], q[10]};
    float f10[8] = {q[11], u[0], u[1], u[2], z, z, z, z};
    if (!valid)
        for (int k = 0; k < 8; ++k) { f9[k] = 0.0f; f10[k] = 0.0f; }
    const float f11[8] = {z, z, z, z, z, z, z, z};
    store_chunk(tile, row, 9, f9);
    store_chunk(tile, row, 10, f10);
    store_chunk(tile, row, 11, f11);
}

// Issue D = A * B for a K-major activation tile A (128 rows) and the K-major
// weight tile of layer l (rows = out), then commit.  One thread.
__device__ __forceinline__ void issue_forward(uint32_t d_tmem, const uint8_t *act, const uint8_t *w, int l,
                                              uint64_t *mbar) {
    const uint32_t K = in_of(l), N = out_of(l);
    const uint32_t idesc = tc::idesc_bf16(kTile, N, false, false);
    for (uint32_t kk = 0; kk < K / 16; ++kk) {
        uint64_t ad = tc::make_desc(tc::smem_u32(act) + kk * 2u * (kTile / 8) * 128u, (kTile / 8) * 128u, 128u);
        uint64_t bd = tc::make_desc(tc::smem_u32(w) + kk * 2u * (N / 8) * 128u, (N / 8) * 128u, 128u);
        tc::mma_bf16(d_tmem, ad, bd, idesc, kk > 0 ? 1u : 0u);
    }
    tc::commit(mbar);
}

// Sync the CTA around shared-memory operand writes and TMEM traffic.
__device__ __forceinline__ void operand_sync() {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

struct InferIO {
    const float4 *q;          // 4 float4 per query: p | slot bits, w_o, n, a
    const uint32_t *count;    // device query count (tracer), or nullptr: n
    uint32_t n;
    float4 *L;                // tracer: L[slot] += thr[slot] * y
    const float4 *thr;
    float *out;               // host queries: out[3 i + c] = y_c
};

// Inference over tiles of 128 queries: the five hidden layers and the output
// layer as tensor-core products with the accumulator in TMEM; the epilogue
// (bias, ReLU, bf16) writes the next layer's operand in place.  A CTA runs
// kInferGroups independent tile pipelines (128 threads each, own operand tile,
// TMEM columns and mbarrier, synchronised by named barriers) over one copy of
// the weights, so one group's epilogue overlaps another's tensor-core work.
__device__ __forceinline__ void group_bar(uint32_t id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
__device__ __forceinline__ bool group_and(uint32_t id, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, %2, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"(v ? 1u : 0u), "r"(id)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ void group_operand_sync(uint32_t id) {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    group_bar(id);
    tc::fence_after_sync();
}

__global__ void __launch_bounds__(128 * kInferGroups) k_cache_infer(NetDev net, InferIO io, uint32_t *status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const uint32_t t = threadIdx.x, warp = t >> 5, g = t / 128u, row = t % 128u;
    uint8_t *act = smem + kSmemAct + g * kTileIn;
    uint8_t *misc = smem + kSmemAct + kInferGroups * kTileIn;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(misc) + g;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(misc + 8 * kInferGroups);
    const float *bias = reinterpret_cast<const float *>(smem + kSmemBias);
    const uint32_t bar_id = 1 + g;
    const uint32_t n = io.count ? min(*io.count, io.n) : io.n;
    load_net(net, smem);
    if (warp == 0) tc::tmem_alloc(tslot, kInferTmemCols);
    if (t == 0)
        for (uint32_t k = 0; k < kInferGroups; ++k) tc::mbar_init(reinterpret_cast<uint64_t *>(misc) + k, 1);
    operand_sync();
    const uint32_t taddr = *tslot + 64u * g;
    const uint32_t lane_base = ((warp & 3u) * 32u) << 16;
    uint32_t phase = 0;
    bool ok = true;
    for (uint32_t tile = blockIdx.x * kInferGroups + g; ok && tile * kTile < n; tile += gridDim.x * kInferGroups) {
        const uint32_t i = tile * kTile + row;
        const bool valid = i < n;
        float q[12];
        uint32_t slot = 0;
        if (valid) {
            float4 a = io.q[4 * (size_t)i], b = io.q[4 * (size_t)i + 1], c = io.q[4 * (size_t)i + 2],
                   d = io.q[4 * (size_t)i + 3];
            q[0] = a.x; q[1] = a.y; q[2] = a.z; slot = __float_as_uint(a.w);
            q[3] = b.x; q[4] = b.y; q[5] = b.z;
            q[6] = c.x; q[7] = c.y; q[8] = c.z;
            q[9] = d.x; q[10] = d.y; q[11] = d.z;
        }
        encode_row_streamed(net, q, valid, act, row);
        group_operand_sync(bar_id);
        for (int l = 0; l < kLayers; ++l) {
            if (row == 0) issue_forward(taddr, act, smem + kSmemImg + img_off(l), l, mbar);
            ok = group_and(bar_id, tc::mbar_wait(mbar, phase & 1u, kPollLimit));   // uniform in the group
            ++phase;
            tc::fence_after_sync();
            if (!ok) break;
            if (l < kLayers - 1) {
#pragma unroll
                for (uint32_t c = 0; c < (uint32_t)kHid; c += 32) {
                    float v[32];
                    tc::tmem_ld32(taddr + lane_base + c, v);
#pragma unroll
                    for (uint32_t k = 0; k < 32; k += 8) {
                        const float *bb = bias + bias_idx(l) + c + k;
                        *reinterpret_cast<uint4 *>(act + tc::op_offset(row, c + k, kTile)) = make_uint4(
                            pack2_relu(v[k] + bb[0], v[k + 1] + bb[1]),
                            pack2_relu(v[k + 2] + bb[2], v[k + 3] + bb[3]),
                            pack2_relu(v[k + 4] + bb[4], v[k + 5] + bb[5]),
                            pack2_relu(v[k + 6] + bb[6], v[k + 7] + bb[7]));
                    }
                }
                group_operand_sync(bar_id);
            } else {
                float v[16];
                tc::tmem_ld16(taddr + lane_base, v);
                const float y0 = v[0] + bias[bias_idx(l)], y1 = v[1] + bias[bias_idx(l) + 1],
                            y2 = v[2] + bias[bias_idx(l) + 2];
                if (valid) {
                    if (io.out) {
                        io.out[3 * (size_t)i] = y0;
                        io.out[3 * (size_t)i + 1] = y1;
                        io.out[3 * (size_t)i + 2] = y2;
                    } else {
                        const float4 th = io.thr[slot];
                        float4 L = io.L[slot];
                        io.L[slot] = make_float4(L.x + th.x * fmaxf(y0, 0.0f), L.y + th.y * fmaxf(y1, 0.0f),
                                                 L.z + th.z * fmaxf(y2, 0.0f), L.w);
                    }
                }
                tc::fence_before_sync();
                group_bar(bar_id);
                tc::fence_after_sync();
            }
        }
    }
    if (!ok && row == 0) atomicExch(status, 1u);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::tmem_dealloc(*tslot, kInferTmemCols);
        tc::tmem_relinquish();
    }
}

// Column sums over a warp's 32 rows: x[k] = the calling lane's value in column
// k.  A reduce-scatter butterfly (31 shuffles, each round's exchanges
// independent): after the round of distance h a lane keeps the half of its
// columns on its side of bit h, plus its partner's values of them; in the end
// lane c holds the sum of column c.  The order of additions is fixed.
__device__ __forceinline__ float warp_column_sums32(float x[32], uint32_t lane) {
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) {
        const bool upper = (lane & (uint32_t)h) != 0u;
#pragma unroll
        for (int k = 0; k < h; ++k) {
            const float send = upper ? x[k] : x[k + h];
            const float keep = upper ? x[k + h] : x[k];
            x[k] = keep + __shfl_xor_sync(0xffffffffu, send, h);
        }
    }
    return x[0];
}

__device__ __forceinline__ float warp_sum(float v) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

struct TrainIO {
    const float *samples;     // 16 floats per sample: query (12), target (3), weight (0 or 1)
    uint32_t n;
    float loss_scale;         // 1 / (3 * valid samples)
    float *partial;           // per CTA: kParams floats (weight and bias gradients)
    float *loss;              // per CTA: sum of the relative L2 terms
};

// One training step's gradients.  Per tile of 128 samples: forward with every
// layer's output kept in shared memory; relative L2 loss (y - t)^2 / (y^2 + 0.01)
// with y held fixed in the denominator; then per layer from the output down:
//   dW_l += G^T * H_l     (tensor cores; G and H_l read as MN-major operands,
//                          G's rows padded to 128 with zeros; the sums stay in
//                          TMEM across the CTA's tiles)
//   G    <- (G * W_l) .* [H_l > 0]    (tensor cores; W_l read MN-major)
// Bias gradients are column sums of G: per warp by warp_column_sums32, kept in
// registers across tiles (lane c: columns c and c + 32 of every layer), and
// combined over the warps in a fixed order at the end.  The CTA then writes
// its partial gradients; k_cache_reduce sums them in a fixed order.
__global__ void __launch_bounds__(128, 1) k_cache_train(NetDev net, TrainIO io, uint32_t *status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *x0 = smem + kTrainX0;
    uint8_t *G = smem + kTrainG;
    float *dbias = reinterpret_cast<float *>(smem + kTrainDb);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + kTrainMisc);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + kTrainMisc + 8);
    float *loss_acc = reinterpret_cast<float *>(smem + kTrainMisc + 16);
    const float *bias = reinterpret_cast<const float *>(smem + kSmemBias);
    auto H = [&](int l) { return smem + kTrainH + (uint32_t)(l - 1) * kTileHid; };   // input of layer l >= 1
    const uint32_t t = threadIdx.x, warp = t >> 5, row = t;
    load_net(net, smem);
    for (uint32_t k = t; k < 2 * kTileHid / 16; k += blockDim.x) reinterpret_cast<uint4 *>(G)[k] = make_uint4(0, 0, 0, 0);
    for (uint32_t k = t; k < (uint32_t)kBiasFloats; k += blockDim.x) dbias[k] = 0.0f;
    if (t == 0) *loss_acc = 0.0f;
    if (warp == 0) tc::tmem_alloc(tslot, 512);
    if (t == 0) tc::mbar_init(mbar, 1);
    operand_sync();
    const uint32_t taddr = *tslot;
    const uint32_t lane_base = (warp * 32u) << 16;
    const uint32_t lane = t & 31u;
    float db[kLayers - 1][2];                    // bias-gradient column sums of this warp's rows
    for (int l = 0; l < kLayers - 1; ++l) db[l][0] = db[l][1] = 0.0f;
    float db_out = 0.0f;                         // output layer: column = lane (lanes < 3)
    float loss_sum = 0.0f;                       // lane 0
    uint32_t phase = 0;
    bool ok = true, first = true;
    for (uint32_t tile = blockIdx.x; ok && tile * kTile < io.n; tile += gridDim.x) {
        const uint32_t i = tile * kTile + row;
        const float *s = io.samples + 16 * (size_t)min(i, io.n - 1);
        const float wgt = i < io.n ? s[15] : 0.0f;
        float q[12];
        for (int k = 0; k < 12; ++k) q[k] = s[k];
        const float tg0 = s[12], tg1 = s[13], tg2 = s[14];
        encode_row_streamed(net, q, wgt > 0.0f, x0, row);
        operand_sync();
        // ---- forward
        for (int l = 0; l < kLayers && ok; ++l) {
            const uint8_t *in = l == 0 ? x0 : H(l);
            if (t == 0) issue_forward(taddr, in, smem + kSmemImg + img_off(l), l, mbar);
            ok = __syncthreads_and(tc::mbar_wait(mbar, phase & 1u, kPollLimit) ? 1 : 0) != 0;   // uniform
            ++phase;
            tc::fence_after_sync();
            if (!ok) break;
            if (l < kLayers - 1) {
                uint8_t *out = H(l + 1);
#pragma unroll
                for (uint32_t c = 0; c < (uint32_t)kHid; c += 32) {
                    float v[32];
                    tc::tmem_ld32(taddr + lane_base + c, v);
#pragma unroll
                    for (uint32_t k = 0; k < 32; k += 8) {
                        const float *bb = bias + bias_idx(l) + c + k;
                        *reinterpret_cast<uint4 *>(out + tc::op_offset(row, c + k, kTile)) = make_uint4(
                            pack2_relu(v[k] + bb[0], v[k + 1] + bb[1]),
                            pack2_relu(v[k + 2] + bb[2], v[k + 3] + bb[3]),
                            pack2_relu(v[k + 4] + bb[4], v[k + 5] + bb[5]),
                            pack2_relu(v[k + 6] + bb[6], v[k + 7] + bb[7]));
                    }
                }
            } else {
                float v[16];
                tc::tmem_ld16(taddr + lane_base, v);
                const float y[3] = {v[0] + bias[bias_idx(l)], v[1] + bias[bias_idx(l) + 1],
                                    v[2] + bias[bias_idx(l) + 2]};
                const float tg[3] = {tg0, tg1, tg2};
                float g[3], lsum = 0.0f;
                for (int c = 0; c < 3; ++c) {
                    const float e = y[c] - tg[c], den = y[c] * y[c] + 0.01f;
                    lsum += wgt * ((e * e) / den);
                    g[c] = bf16_float(bf16_bits(wgt * (2.0f * e / den) * io.loss_scale));
                }
                lsum = warp_sum(lsum);
                if (lane == 0) loss_sum += lsum;
                for (int c = 0; c < 3; ++c) {
                    const float s = warp_sum(g[c]);
                    if (lane == (uint32_t)c) db_out += s;
                }
                *reinterpret_cast<uint4 *>(G + tc::op_offset(row, 0, kTile)) =
                    make_uint4(pack2(g[0], g[1]), pack2(g[2], 0.0f), 0u, 0u);
                for (uint32_t c = 8; c < (uint32_t)kHid; c += 8)
                    *reinterpret_cast<uint4 *>(G + tc::op_offset(row, c, kTile)) = make_uint4(0, 0, 0, 0);
            }
            operand_sync();
        }
        if (!ok) break;
        // ---- backward
        for (int l = kLayers - 1; l >= 0 && ok; --l) {
            const uint8_t *in = l == 0 ? x0 : H(l);
            if (t == 0) {
                // dW_l += G^T * H_l: M = 128 (out rows, zero beyond out_of(l)), N = in_of(l), K = 128 samples
                const uint32_t idw = tc::idesc_bf16(kTile, in_of(l), true, true);
                for (uint32_t ks = 0; ks < kTile / 16; ++ks) {
                    uint64_t ad = tc::make_desc(tc::smem_u32(G) + ks * 256u, 128u, (kTile / 8) * 128u);
                    uint64_t bd = tc::make_desc(tc::smem_u32(in) + ks * 256u, 128u, (kTile / 8) * 128u);
                    tc::mma_bf16(taddr + kDwCol[l], ad, bd, idw, (first && ks == 0) ? 0u : 1u);
                }
                if (l > 0) {
                    // G' = G * W_l: M = 128 samples, K = out_of(l), N = in_of(l) = 64
                    const uint32_t K = out_of(l);
                    const uint8_t *w = smem + kSmemImg + img_off(l);
                    const uint32_t idb = tc::idesc_bf16(kTile, kHid, false, true);
                    for (uint32_t kk = 0; kk < K / 16; ++kk) {
                        uint64_t ad = tc::make_desc(tc::smem_u32(G) + kk * 2u * (kTile / 8) * 128u,
                                                    (kTile / 8) * 128u, 128u);
                        uint64_t bd = tc::make_desc(tc::smem_u32(w) + kk * 256u, 128u, (K / 8) * 128u);
                        tc::mma_bf16(taddr, ad, bd, idb, kk > 0 ? 1u : 0u);
                    }
                }
                tc::commit(mbar);
            }
            ok = __syncthreads_and(tc::mbar_wait(mbar, phase & 1u, kPollLimit) ? 1 : 0) != 0;   // uniform
            ++phase;
            tc::fence_after_sync();
            if (!ok) break;
            if (l > 0) {
                const uint8_t *hl = H(l);
#pragma unroll
                for (uint32_t half = 0; half < 2; ++half) {
                    float g[32];
#pragma unroll
                    for (uint32_t q = 0; q < 2; ++q) {
                        const uint32_t c = half * 32u + q * 16u;
                        float v[16];
                        tc::tmem_ld16(taddr + lane_base + c, v);
                        const uint4 ha = *reinterpret_cast<const uint4 *>(hl + tc::op_offset(row, c, kTile));
                        const uint4 hb = *reinterpret_cast<const uint4 *>(hl + tc::op_offset(row, c + 8, kTile));
                        const uint32_t hw[8] = {ha.x, ha.y, ha.z, ha.w, hb.x, hb.y, hb.z, hb.w};
                        float *gq = g + q * 16u;
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            const uint32_t hbits = (hw[j >> 1] >> (16 * (j & 1))) & 0xffffu;
                            gq[j] = bf16_float(bf16_bits(hbits != 0u ? v[j] : 0.0f));   // ReLU output > 0 <=> bits != 0
                        }
                        *reinterpret_cast<uint4 *>(G + tc::op_offset(row, c, kTile)) =
                            make_uint4(pack2(gq[0], gq[1]), pack2(gq[2], gq[3]), pack2(gq[4], gq[5]), pack2(gq[6], gq[7]));
                        *reinterpret_cast<uint4 *>(G + tc::op_offset(row, c + 8, kTile)) =
                            make_uint4(pack2(gq[8], gq[9]), pack2(gq[10], gq[11]), pack2(gq[12], gq[13]),
                                       pack2(gq[14], gq[15]));
                    }
                    db[l - 1][half] += warp_column_sums32(g, lane);      // column half * 32 + lane
                }
                operand_sync();
            }
        }
        first = false;
    }
    if (!ok && t == 0) atomicExch(status, 1u);
    // the warps' bias-gradient sums and losses, added warp by warp (fixed order)
    for (uint32_t w = 0; w < 4u; ++w) {
        if (warp == w) {
            for (int l = 0; l < kLayers - 1; ++l) {
                dbias[bias_idx(l) + lane] += db[l][0];
                dbias[bias_idx(l) + 32u + lane] += db[l][1];
            }
            if (lane < 3u) dbias[bias_idx(kLayers - 1) + lane] += db_out;
            if (lane == 0) *loss_acc += loss_sum;
        }
        __syncthreads();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- partial gradients of this CTA
    float *part = io.partial + (size_t)blockIdx.x * kParams;
    for (int l = 0; l < kLayers; ++l) {
        const uint32_t nin = in_of(l), nout = out_of(l);
        if (warp * 32u < nout) {                      // TMEM lane = output row
            const uint32_t o = warp * 32u + (t & 31u);
            for (uint32_t c = 0; c < nin; c += 16) {
                float v[16];
                if (ok && !first) tc::tmem_ld16(taddr + lane_base + kDwCol[l] + c, v);
                else for (int j = 0; j < 16; ++j) v[j] = 0.0f;
                if (o < nout)
                    for (int j = 0; j < 16; ++j) part[w_off(l) + o * nin + c + j] = v[j];
            }
        }
        for (uint32_t o = t; o < nout; o += blockDim.x) part[b_off(l) + o] = dbias[bias_idx(l) + o];
    }
    if (t == 0) io.loss[blockIdx.x] = *loss_acc;
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::tmem_dealloc(taddr, 512);
        tc::tmem_relinquish();
    }
}

// grad[p] = sum over CTAs of partial[cta][p], in CTA order.
__global__ void k_cache_reduce(const float *partial, uint32_t n_cta, const float *loss_part, float *grad,
                               float *loss_out, uint32_t *adam_step) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < (uint32_t)kParams) {
        float s = 0.0f;
        for (uint32_t c = 0; c < n_cta; ++c) s += partial[(size_t)c * kParams + p];
        grad[p] = s;
    }
    if (p == 0) {
        float s = 0.0f;
        for (uint32_t c = 0; c < n_cta; ++c) s += loss_part[c];
        *loss_out = s;
        if (adam_step) *adam_step += 1u;           // the Adam step that follows (kept on the device)
    }
}

__device__ __forceinline__ void param_where(uint32_t p, int *layer, bool *is_bias, uint32_t *o, uint32_t *i) {
    int l = 0;
    while (l + 1 < kLayers && p >= (uint32_t)w_off(l + 1)) ++l;
    *layer = l;
    const uint32_t r = p - (uint32_t)w_off(l);
    const uint32_t nw = (uint32_t)(out_of(l) * in_of(l));
    *is_bias = r >= nw;
    if (*is_bias) { *o = r - nw; *i = 0; }
    else { *o = r / in_of(l); *i = r - *o * in_of(l); }
}

// Adam (Kingma & Ba 2015) on the fp32 parameters; refreshes the bf16 weight
// image and the bias copy the kernels read.
__global__ void k_cache_adam(float *params, float *m, float *v, const float *grad, float lr, float beta1, float beta2,
                             float eps, const uint32_t *adam_step, uint8_t *img, float *bias) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (uint32_t)kParams) return;
    const float t = (float)*adam_step;                 // bias corrections of step t
    const float bc1 = 1.0f - powf(beta1, t), bc2 = 1.0f - powf(beta2, t);
    const float g = grad[p];
    const float mi = beta1 * m[p] + (1.0f - beta1) * g;
    const float vi = beta2 * v[p] + (1.0f - beta2) * (g * g);
    m[p] = mi;
    v[p] = vi;
    const float w = params[p] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    params[p] = w;
    int l;
    bool is_bias;
    uint32_t o, i;
    param_where(p, &l, &is_bias, &o, &i);
    if (is_bias) bias[bias_idx(l) + o] = w;
    else *reinterpret_cast<uint16_t *>(img + img_off(l) + tc::op_offset(o, i, out_of(l))) = (uint16_t)bf16_bits(w);
}

// Weight image and bias copy from the fp32 parameters (after they are set).
__global__ void k_cache_refresh(const float *params, uint8_t *img, float *bias) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (uint32_t)kParams) return;
    int l;
    bool is_bias;
    uint32_t o, i;
    param_where(p, &l, &is_bias, &o, &i);
    if (is_bias) bias[bias_idx(l) + o] = params[p];
    else *reinterpret_cast<uint16_t *>(img + img_off(l) + tc::op_offset(o, i, out_of(l))) = (uint16_t)bf16_bits(params[p]);
}

// Training samples from the recorded vertices of the training paths: for
// recorded vertex j of training path t, query = (p, w_o, n, albedo) and target
// = (L_final - L_next) / thr_j, the radiance the path gathered after vertex j's
// light sample, per unit throughput: L_next is the radiance recorded at the
// path's next event (its next vertex, or the miss or emitter that ended it;
// the shadow ray of vertex j is resolved before that event is shaded), or
// L_final when the path ended at vertex j.  A path stopped into the cache at a
// vertex keeps that vertex's light sample, so this is what the cache stands
// for.  Appended (warp-aggregated) when finite.
__global__ void k_cache_targets(const float4 *rec, uint32_t n_train, uint32_t depth, uint32_t stride,
                                const float4 *L, float *samples, uint32_t *count) {
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u;
    bool ok = false;
    float s[16];
    if (idx < n_train * depth) {
        const float4 *r = rec + (size_t)idx * kTrainRecordFloat4;
        const float4 p = r[0];
        if (p.w > 0.0f) {
            const float4 wo = r[1], nn = r[2], al = r[3], th = r[4];
            const float4 lf = L[(size_t)(idx / depth) * stride];
            float4 ln = lf;
            if (idx % depth + 1 < depth && r[kTrainRecordFloat4].w != 0.0f) ln = r[kTrainRecordFloat4 + 5];
            const float tx = (lf.x - ln.x) / th.x, ty = (lf.y - ln.y) / th.y, tz = (lf.z - ln.z) / th.z;
            ok = th.x > 0.0f && th.y > 0.0f && th.z > 0.0f && isfinite(tx) && isfinite(ty) && isfinite(tz);
            s[0] = p.x; s[1] = p.y; s[2] = p.z; s[3] = wo.x; s[4] = wo.y; s[5] = wo.z;
            s[6] = nn.x; s[7] = nn.y; s[8] = nn.z; s[9] = al.x; s[10] = al.y; s[11] = al.z;
            s[12] = fmaxf(tx, 0.0f); s[13] = fmaxf(ty, 0.0f); s[14] = fmaxf(tz, 0.0f); s[15] = 1.0f;
        }
    }
    const unsigned mask = __ballot_sync(0xffffffffu, ok);
    if (!mask) return;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(count, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (ok) {
        float4 *dst = reinterpret_cast<float4 *>(samples + 16 * (size_t)(base + __popc(mask & ((1u << lane) - 1u))));
        dst[0] = make_float4(s[0], s[1], s[2], s[3]);
        dst[1] = make_float4(s[4], s[5], s[6], s[7]);
        dst[2] = make_float4(s[8], s[9], s[10], s[11]);
        dst[3] = make_float4(s[12], s[13], s[14], s[15]);
    }
}

// The batch of training step s of one pass, drawn from all n of the pass's
// samples: entry k takes stratum j = k * steps + s of steps * batch equal
// strata of [0, n), at a hashed offset inside the stratum.  The samples come in
// slot order (pixel-major), so neighbouring samples are neighbouring pixels:
// every step then sees the whole image, and successive passes (seeds) see
// different samples of each stratum.
__global__ void k_cache_gather(const float4 *src, const uint32_t *count, uint32_t steps, uint32_t s, uint32_t batch,
                               uint32_t seed, float4 *dst) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= batch) return;
    const uint32_t n = *count;
    if (n == 0) {                                                           // no sample: zero weights
        for (int c = 0; c < 4; ++c) dst[4 * (size_t)k + c] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const uint64_t total = (uint64_t)steps * batch;
    const uint64_t j = (uint64_t)k * steps + s;                             // < total
    const uint64_t r24 = pcg_hash(k ^ pcg_hash(seed + s)) >> 8;             // [0, 2^24)
    uint64_t idx = (j * n + ((r24 * n) >> 24)) / total;                     // < n
    if (idx >= n) idx = n - 1;
    const float4 *a = src + 4 * idx;
    float4 *d = dst + 4 * (size_t)k;
    d[0] = a[0]; d[1] = a[1]; d[2] = a[2]; d[3] = a[3];
}

// The bias judge: the training samples of a pass as inference queries (4
// float4 each: p | index, w_o, n, albedo), so the network can be compared with
// the radiance the full-length training paths actually gathered.
__global__ void k_cache_judge_queries(const float4 *s, const uint32_t *count, float4 *q) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *count) return;
    const float4 a = s[4 * (size_t)i], b = s[4 * (size_t)i + 1], c = s[4 * (size_t)i + 2];
    q[4 * (size_t)i] = make_float4(a.x, a.y, a.z, __uint_as_float(i));
    q[4 * (size_t)i + 1] = make_float4(a.w, b.x, b.y, 0.0f);
    q[4 * (size_t)i + 2] = make_float4(b.z, b.w, c.x, 0.0f);
    q[4 * (size_t)i + 3] = make_float4(c.y, c.z, c.w, 0.0f);
}

// acc[0..2] += sum of (max(y, 0) - target), acc[3..5] += sum of target, per
// channel over the weighted samples; acc[6] += their number.  Sums of
// differences, not of ratios: their quotient is the cache's relative bias on
// the radiance it stands for, and the per-sample noise of the targets averages
// out of the numerator.
__global__ void k_cache_judge(const float4 *s, const float *y, const uint32_t *count, double *acc) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *count;
    float v[7] = {0, 0, 0, 0, 0, 0, 0};
    if (i < n) {
        const float4 t = s[4 * (size_t)i + 3];
        if (t.w > 0.0f) {
            v[0] = fmaxf(y[3 * (size_t)i], 0.0f) - t.x;
            v[1] = fmaxf(y[3 * (size_t)i + 1], 0.0f) - t.y;
            v[2] = fmaxf(y[3 * (size_t)i + 2], 0.0f) - t.z;
            v[3] = t.x; v[4] = t.y; v[5] = t.z; v[6] = 1.0f;
        }
    }
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        const float w = warp_sum(v[k]);
        if ((threadIdx.x & 31u) == 0u && w != 0.0f) atomicAdd(acc + k, (double)w);
    }
}

// Synthetic queries (4 float4 each, slot = index) and training samples (16
// floats) inside the encoding bounds, for the throughput measurement.
__global__ void k_cache_synth(uint32_t n, NetDev net, float4 *q, float *samples) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t h = pcg_hash(i * 2654435761u + 17u);
    auto rnd = [&]() { h = pcg_hash(h); return (float)(h >> 8) * (1.0f / 16777216.0f); };
    float s[16];
    for (int a = 0; a < 3; ++a) s[a] = net.lo[a] + rnd() / fmaxf(net.inv_ext[a], 1e-30f);
    for (int k = 3; k < 9; ++k) s[k] = 2.0f * rnd() - 1.0f;
    for (int k = 9; k < 15; ++k) s[k] = rnd();
    s[15] = 1.0f;
    q[4 * (size_t)i] = make_float4(s[0], s[1], s[2], __uint_as_float(i));
    q[4 * (size_t)i + 1] = make_float4(s[3], s[4], s[5], 0.0f);
    q[4 * (size_t)i + 2] = make_float4(s[6], s[7], s[8], 0.0f);
    q[4 * (size_t)i + 3] = make_float4(s[9], s[10], s[11], 0.0f);
    float4 *d = reinterpret_cast<float4 *>(samples + 16 * (size_t)i);
    for (int k = 0; k < 4; ++k) d[k] = make_float4(s[4 * k], s[4 * k + 1], s[4 * k + 2], s[4 * k + 3]);
}

}  // namespace

// ---------------------------------------------------------------------------- cache state
struct CacheState {
    DBuf params, m, v, img, bias, grad, partial, loss_part, loss, samples, queries, status, batch, judge;
    DBuf adam_step;               // device Adam step counter (advanced by k_cache_reduce)
    uint32_t n_cta_partial = 0;
    uint32_t passes = 0;          // training passes from recorded paths (the batch draws' seed)
    float lo[3] = {0, 0, 0}, inv_ext[3] = {1, 1, 1};
    bool has_params = false;
    bool configured = false;
};

CacheState *cache_create() { return new CacheState(); }
void cache_destroy(CacheState *c) {
    if (!c) return;
    DBuf *bufs[] = {&c->params, &c->m, &c->v, &c->img, &c->bias, &c->grad, &c->partial, &c->loss_part,
                    &c->loss, &c->samples, &c->queries, &c->status, &c->batch, &c->judge,
                    &c->adam_step};
    for (DBuf *b : bufs) b->release();
    delete c;
}

void cache_set_bounds(CacheState *c, const float lo[3], const float hi[3]) {
    for (int a = 0; a < 3; ++a) {
        c->lo[a] = lo[a];
        const float ext = hi[a] - lo[a];
        c->inv_ext[a] = ext > 0.0f ? 1.0f / ext : 0.0f;
    }
}

static NetDev net_of(const CacheState *c) {
    NetDev n;
    n.img = c->img.as<uint8_t>();
    n.bias = c->bias.as<float>();
    for (int a = 0; a < 3; ++a) { n.lo[a] = c->lo[a]; n.inv_ext[a] = c->inv_ext[a]; }
    return n;
}

static cudaError_t ensure_net(CacheState *c) {
    cudaError_t e;
    if ((e = c->params.ensure(kParams * 4)) != cudaSuccess) return e;
    if ((e = c->m.ensure(kParams * 4)) != cudaSuccess) return e;
    if ((e = c->v.ensure(kParams * 4)) != cudaSuccess) return e;
    if ((e = c->grad.ensure(kParams * 4)) != cudaSuccess) return e;
    if ((e = c->img.ensure(kImgBytes)) != cudaSuccess) return e;
    if ((e = c->bias.ensure(kBiasFloats * 4)) != cudaSuccess) return e;
    if ((e = c->loss.ensure(16)) != cudaSuccess) return e;
    if ((e = c->status.ensure(16)) != cudaSuccess) return e;
    return cudaSuccess;
}

cudaError_t cache_set_params(CacheState *c, const float *host, cudaStream_t st) {
    cudaError_t e = ensure_net(c);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c->params.p, host, kParams * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(c->m.p, 0, kParams * 4, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(c->v.p, 0, kParams * 4, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(c->img.p, 0, kImgBytes, st)) != cudaSuccess) return e;
    k_cache_refresh<<<(kParams + 255) / 256, 256, 0, st>>>(c->params.as<float>(), c->img.as<uint8_t>(),
                                                          c->bias.as<float>());
    note_launch();
    if ((e = c->adam_step.ensure(16)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(c->adam_step.p, 0, 16, st)) != cudaSuccess) return e;
    c->has_params = true;
    return cudaGetLastError();
}

cudaError_t cache_get_params(CacheState *c, float *host, cudaStream_t st) {
    if (!c->has_params) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemcpyAsync(host, c->params.p, kParams * 4, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

static cudaError_t check_status(CacheState *c, cudaStream_t st, bool *timed_out) {
    uint32_t s = 0;
    cudaError_t e = cudaMemcpyAsync(&s, c->status.p, 4, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    *timed_out = s != 0;
    return cudaSuccess;
}

// Inference over device queries (4 float4 each); either out (host layout) or
// the tracer's L / thr.
// Shared-memory attributes of the two tensor-core kernels, set once (before
// any capture: cache_prepare sets them too).
static bool g_infer_attr = false, g_train_attr = false;

cudaError_t cache_infer_device(CacheState *c, const float4 *q, const uint32_t *d_count, uint32_t max_n, float *out,
                               float4 *L, const float4 *thr, cudaStream_t st) {
    if (!g_infer_attr) {
        cudaError_t e = cudaFuncSetAttribute(k_cache_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem);
        if (e != cudaSuccess) return e;
        g_infer_attr = true;
    }
    if (max_n == 0) return cudaSuccess;
    InferIO io{q, d_count, max_n, L, thr, out};
    const uint32_t tiles = (max_n + kTile - 1) / kTile;
    const uint32_t per_sm = std::max<uint32_t>(1u, (227u * 1024u) / kInferSmem);   // resident CTAs (shared memory)
    const int blocks = (int)std::max<uint32_t>(1u, std::min<uint32_t>((tiles + kInferGroups - 1) / kInferGroups,
                                                                      (uint32_t)sm_count() * per_sm));
    k_cache_infer<<<blocks, 128 * kInferGroups, kInferSmem, st>>>(net_of(c), io, c->status.as<uint32_t>());
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_infer_host(CacheState *c, const float *q12, uint32_t n, float *out3, cudaStream_t st,
                             bool *timed_out) {
    if (!c->has_params) return cudaErrorInvalidValue;
    cudaError_t e;
    if ((e = c->queries.ensure((size_t)n * 64 + (size_t)n * 12)) != cudaSuccess) return e;
    std::vector<float> q((size_t)n * 16, 0.0f);
    for (uint32_t i = 0; i < n; ++i) {
        for (int k = 0; k < 3; ++k) {
            q[16 * (size_t)i + k] = q12[12 * (size_t)i + k];
            q[16 * (size_t)i + 4 + k] = q12[12 * (size_t)i + 3 + k];
            q[16 * (size_t)i + 8 + k] = q12[12 * (size_t)i + 6 + k];
            q[16 * (size_t)i + 12 + k] = q12[12 * (size_t)i + 9 + k];
        }
    }
    float *d_out = reinterpret_cast<float *>(c->queries.as<char>() + (size_t)n * 64);
    if ((e = cudaMemcpyAsync(c->queries.p, q.data(), (size_t)n * 64, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(c->status.p, 0, 4, st)) != cudaSuccess) return e;
    if ((e = cache_infer_device(c, c->queries.as<float4>(), nullptr, n, d_out, nullptr, nullptr, st)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(out3, d_out, (size_t)n * 12, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    return check_status(c, st, timed_out);
}

// One optimisation step on n device samples (16 floats each): gradients into
// c->grad (and the loss into c->loss), then Adam when lr > 0.
cudaError_t cache_step_device(CacheState *c, const float *d_samples, uint32_t n, uint32_t n_valid, float lr,
                              cudaStream_t st) {
    cudaError_t e;
    if (!g_train_attr) {
        if ((e = cudaFuncSetAttribute(k_cache_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem)) !=
            cudaSuccess)
            return e;
        g_train_attr = true;
    }
    const uint32_t tiles = (n + kTile - 1) / kTile;
    const uint32_t blocks = std::max(1u, std::min<uint32_t>(tiles, (uint32_t)sm_count()));
    if ((e = c->partial.ensure((size_t)blocks * kParams * 4)) != cudaSuccess) return e;
    if ((e = c->loss_part.ensure((size_t)blocks * 4)) != cudaSuccess) return e;
    TrainIO io{d_samples, n, 1.0f / (3.0f * (float)std::max(n_valid, 1u)), c->partial.as<float>(),
               c->loss_part.as<float>()};
    k_cache_train<<<blocks, 128, kTrainSmem, st>>>(net_of(c), io, c->status.as<uint32_t>());
    note_launch();
    uint32_t *adam_step = lr > 0.0f ? c->adam_step.as<uint32_t>() : nullptr;
    k_cache_reduce<<<(kParams + 255) / 256, 256, 0, st>>>(c->partial.as<float>(), blocks, c->loss_part.as<float>(),
                                                          c->grad.as<float>(), c->loss.as<float>(), adam_step);
    note_launch();
    if (adam_step) {
        k_cache_adam<<<(kParams + 255) / 256, 256, 0, st>>>(c->params.as<float>(), c->m.as<float>(), c->v.as<float>(),
                                                            c->grad.as<float>(), lr, 0.9f, 0.99f, 1e-8f, adam_step,
                                                            c->img.as<uint8_t>(), c->bias.as<float>());
        note_launch();
    }
    return cudaGetLastError();
}

// Everything a render pass's training (cache_train_records) and inference
// allocate or configure, for up to `cap` samples and batches of `batch`: done
// before the passes, so that a pass allocates nothing and can be captured.
cudaError_t cache_prepare(CacheState *c, size_t cap, uint32_t batch) {
    if (!c->has_params) return cudaErrorInvalidValue;
    cudaError_t e;
    if (!g_infer_attr) {
        if ((e = cudaFuncSetAttribute(k_cache_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem)) !=
            cudaSuccess)
            return e;
        g_infer_attr = true;
    }
    if (!g_train_attr) {
        if ((e = cudaFuncSetAttribute(k_cache_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem)) !=
            cudaSuccess)
            return e;
        g_train_attr = true;
    }
    if ((e = c->samples.ensure(cap * 64 + 64)) != cudaSuccess) return e;
    if ((e = c->queries.ensure(cap * 64 + cap * 12)) != cudaSuccess) return e;
    const uint32_t b = batch ? (uint32_t)std::min<size_t>(batch, std::max<size_t>(cap, 1)) : (uint32_t)std::max<size_t>(cap, 1);
    if ((e = c->batch.ensure((size_t)b * 64)) != cudaSuccess) return e;
    const uint32_t blocks = std::max(1u, std::min<uint32_t>((b + kTile - 1) / kTile, (uint32_t)sm_count()));
    if ((e = c->partial.ensure((size_t)blocks * kParams * 4)) != cudaSuccess) return e;
    if ((e = c->loss_part.ensure((size_t)blocks * 4)) != cudaSuccess) return e;
    return c->judge.ensure(8 * sizeof(double));
}

// Device pointers of the cache's buffers (the identity of a captured pass).
void cache_buffer_ptrs(const CacheState *c, const void *out[12]) {
    const DBuf *b[12] = {&c->params, &c->m, &c->v, &c->img, &c->bias, &c->grad, &c->partial, &c->loss_part,
                         &c->samples, &c->queries, &c->batch, &c->judge};
    for (int k = 0; k < 12; ++k) out[k] = b[k]->p;
}

// One pass's training, with no host round trip: the sample count stays on the
// device (the judge, the batch draws and the inference read it there), so the
// pass can be replayed from a CUDA graph.  A batch of `batch` samples (0: the
// capacity) is drawn per step; with fewer samples than that, samples repeat.
cudaError_t cache_train_records(CacheState *c, const float4 *rec, uint32_t n_train, uint32_t depth, uint32_t stride,
                                const float4 *L, uint32_t steps, uint32_t batch, float lr, cudaStream_t st) {
    if (!c->has_params) return cudaErrorInvalidValue;
    const size_t cap = (size_t)n_train * depth;
    if (cap == 0) return cudaSuccess;
    if (cap > 0xffffffffu) return cudaErrorInvalidValue;
    cudaError_t e;
    if ((e = cache_prepare(c, cap, batch)) != cudaSuccess) return e;    // no-op when prepared
    uint32_t *count = reinterpret_cast<uint32_t *>(c->samples.as<char>() + cap * 64);
    if ((e = cudaMemsetAsync(count, 0, 4, st)) != cudaSuccess) return e;
    const uint32_t grid = (uint32_t)((cap + 255) / 256);
    k_cache_targets<<<grid, 256, 0, st>>>(rec, n_train, depth, stride, L, c->samples.as<float>(), count);
    note_launch();
    if (c->judge.p) {                              // judge the network on this pass's samples before training
        float4 *q = c->queries.as<float4>();
        float *y = reinterpret_cast<float *>(c->queries.as<char>() + cap * 64);
        k_cache_judge_queries<<<grid, 256, 0, st>>>(c->samples.as<float4>(), count, q);
        note_launch();
        if ((e = cache_infer_device(c, q, count, (uint32_t)cap, y, nullptr, nullptr, st)) != cudaSuccess) return e;
        k_cache_judge<<<grid, 256, 0, st>>>(c->samples.as<float4>(), y, count, c->judge.as<double>());
        note_launch();
    }
    if (steps == 0) return cudaSuccess;
    const uint32_t b = batch ? (uint32_t)std::min<size_t>(batch, cap) : (uint32_t)cap;
    const uint32_t seed = pcg_hash(++c->passes);
    for (uint32_t s = 0; s < steps; ++s) {       // each step's batch spread over all samples of the pass
        k_cache_gather<<<(b + 255) / 256, 256, 0, st>>>(c->samples.as<float4>(), count, steps, s, b, seed,
                                                        c->batch.as<float4>());
        note_launch();
        if ((e = cache_step_device(c, c->batch.as<float>(), b, b, lr, st)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

bool cache_ready(const CacheState *c) { return c && c->has_params; }

cudaError_t cache_judge_reset(CacheState *c, cudaStream_t st) {
    cudaError_t e = c->judge.ensure(8 * sizeof(double));
    if (e != cudaSuccess) return e;
    return cudaMemsetAsync(c->judge.p, 0, 8 * sizeof(double), st);
}

cudaError_t cache_judge_read(CacheState *c, double out[8], cudaStream_t st) {
    for (int k = 0; k < 8; ++k) out[k] = 0.0;
    if (!c->judge.p) return cudaSuccess;
    cudaError_t e = cudaMemcpyAsync(out, c->judge.p, 8 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

// Device time of inference over n synthetic queries and of one training step
// (gradients, reduction, Adam) on n synthetic samples, averaged over reps.
cudaError_t cache_bench(CacheState *c, uint32_t n, uint32_t reps, float *ms_infer, float *ms_train, cudaStream_t st) {
    if (!c->has_params) return cudaErrorInvalidValue;
    cudaError_t e;
    if ((e = c->queries.ensure((size_t)n * 64 + (size_t)n * 12)) != cudaSuccess) return e;
    if ((e = c->samples.ensure((size_t)n * 64 + 64)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(c->status.p, 0, 4, st)) != cudaSuccess) return e;
    k_cache_synth<<<(n + 255) / 256, 256, 0, st>>>(n, net_of(c), c->queries.as<float4>(), c->samples.as<float>());
    note_launch();
    float *out = reinterpret_cast<float *>(c->queries.as<char>() + (size_t)n * 64);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    auto timed = [&](auto fn, float *ms_out) -> cudaError_t {
        cudaError_t err = fn();                        // warm-up
        if (err != cudaSuccess) return err;
        cudaEventRecord(a, st);
        for (uint32_t r = 0; r < reps; ++r)
            if ((err = fn()) != cudaSuccess) return err;
        cudaEventRecord(b, st);
        if ((err = cudaEventSynchronize(b)) != cudaSuccess) return err;
        float t = 0.0f;
        cudaEventElapsedTime(&t, a, b);
        *ms_out = t / (float)std::max(reps, 1u);
        return cudaSuccess;
    };
    e = timed([&]() { return cache_infer_device(c, c->queries.as<float4>(), nullptr, n, out, nullptr, nullptr, st); },
              ms_infer);
    if (e == cudaSuccess)
        e = timed([&]() { return cache_step_device(c, c->samples.as<float>(), n, n, 1e-6f, st); }, ms_train);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return e;
}

cudaError_t cache_train_host(CacheState *c, const float *samples16, uint32_t n, uint32_t steps, uint32_t batch,
                             float lr, float *out_loss, float *out_grad, cudaStream_t st, bool *timed_out) {
    if (!c->has_params) return cudaErrorInvalidValue;
    cudaError_t e;
    if ((e = c->samples.ensure((size_t)n * 64)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c->samples.p, samples16, (size_t)n * 64, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(c->status.p, 0, 4, st)) != cudaSuccess) return e;
    if (batch == 0 || batch > n) batch = n;
    for (uint32_t s = 0; s < std::max(steps, 1u); ++s) {
        const uint32_t first = (uint32_t)(((uint64_t)s * batch) % n);
        const uint32_t cnt = std::min(batch, n - first);
        uint32_t valid = 0;
        for (uint32_t i = first; i < first + cnt; ++i) valid += samples16[16 * (size_t)i + 15] > 0.0f ? 1u : 0u;
        if ((e = cache_step_device(c, c->samples.as<float>() + 16 * (size_t)first, cnt, valid, steps ? lr : 0.0f,
                                   st)) != cudaSuccess)
            return e;
        if (out_loss && (e = cudaMemcpyAsync(out_loss + s, c->loss.p, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
            return e;
        if (s == 0 && out_grad &&
            (e = cudaMemcpyAsync(out_grad, c->grad.p, kParams * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
            return e;
    }
    return check_status(c, st, timed_out);
}

}  // namespace mcrt

extern "C" mcrt_status mcrt_mlp_gemm_probe(int device, const uint16_t *A, const uint16_t *B, uint32_t K, uint32_t N,
                                           uint32_t flags, float *D) {
    if (!A || !B || !D) { mcrt::set_global_error("NULL argument"); return MCRT_ERR_INVALID_ARG; }
    if (K == 0 || K % 16 || K > 64 || N < 16 || N > 64 || N % 16 || flags > 3) {
        mcrt::set_global_error("probe shape: K in 16..64 (multiple of 16), N in 16..64 (multiple of 16)");
        return MCRT_ERR_INVALID_ARG;
    }
    auto cuda_err = [](cudaError_t e, const char *what) {
        mcrt::set_global_error(std::string(what) + ": " + cudaGetErrorString(e));
        return MCRT_ERR_CUDA;
    };
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_err(e, "cudaSetDevice");
    const size_t na = (size_t)mcrt::kProbeM * K, nb = (size_t)N * K, nd = (size_t)mcrt::kProbeM * N;
    uint16_t *dA = nullptr, *dB = nullptr;
    float *dD = nullptr;
    uint32_t *dS = nullptr;
    mcrt_status rc = MCRT_OK;
    const size_t smem = mcrt::kProbeARegion + mcrt::kProbeBRegion + 64;
    if ((e = cudaMalloc(&dA, na * 2)) != cudaSuccess || (e = cudaMalloc(&dB, nb * 2)) != cudaSuccess ||
        (e = cudaMalloc(&dD, nd * 4)) != cudaSuccess || (e = cudaMalloc(&dS, 4)) != cudaSuccess) {
        rc = cuda_err(e, "allocate");
    } else if ((e = cudaMemcpy(dA, A, na * 2, cudaMemcpyHostToDevice)) != cudaSuccess ||
               (e = cudaMemcpy(dB, B, nb * 2, cudaMemcpyHostToDevice)) != cudaSuccess ||
               (e = cudaMemset(dD, 0, nd * 4)) != cudaSuccess || (e = cudaMemset(dS, 0, 4)) != cudaSuccess ||
               (e = cudaFuncSetAttribute(mcrt::k_gemm_probe, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem)) != cudaSuccess) {
        rc = cuda_err(e, "upload");
    } else {
        mcrt::k_gemm_probe<<<1, 128, smem>>>(dA, dB, K, N, flags, dD, dS);
        mcrt::note_launch();
        uint32_t st = 0;
        if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaDeviceSynchronize()) != cudaSuccess ||
            (e = cudaMemcpy(&st, dS, 4, cudaMemcpyDeviceToHost)) != cudaSuccess ||
            (e = cudaMemcpy(D, dD, nd * 4, cudaMemcpyDeviceToHost)) != cudaSuccess) {
            rc = cuda_err(e, "probe");
        } else if (st) {
            mcrt::set_global_error("tensor-core product did not complete");
            rc = MCRT_ERR_TIMEOUT;
        }
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dS);
    return rc;
}
