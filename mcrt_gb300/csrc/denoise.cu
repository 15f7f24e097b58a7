// denoise.cu — joint-bilateral denoiser (cs_denoise, src/shaders/denoise.wgsl:52-120),
// shared-memory tiled.
//
// A 16x16 block of output pixels stages its (16+2R)^2 input tile — radiance and
// G-buffer (normal, depth) — in shared memory once, with clamp-to-edge
// addressing (denoise.wgsl:77-79), and the spatial weights exp(-d^2/2s^2) in a
// (2R+1)^2 table, so each tap is served from shared memory instead of the
// reference's two texture loads.  The per-tap arithmetic is the reference's
// (same order of operations, denoise.wgsl:81-108).  Radii whose tile does not
// fit the shared-memory budget read the taps from global memory.
#include "common.cuh"
#include "internal.h"

namespace mcrt {

namespace {

constexpr int kTile = 16;
constexpr int kMaxSharedR = 8;   // (16 + 16)^2 * 32 B = 32 KB

template <bool kShared>
__global__ void __launch_bounds__(kTile *kTile) k_denoise(const float4 *__restrict__ in, const float4 *__restrict__ gb,
                                                         int W, int H, mcrt_denoise_params dp, float4 *out) {
    extern __shared__ float4 smem[];
    const int R = dp.radius;
    const int span = kTile + 2 * R;
    float4 *s_col = smem;
    float4 *s_g = smem + (kShared ? span * span : 0);
    float *s_w = reinterpret_cast<float *>(s_g + (kShared ? span * span : 0));
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = blockIdx.x * kTile - R, y0 = blockIdx.y * kTile - R;
    const float inv2ss = 1.0f / ((2.0f * dp.sigma_s) * dp.sigma_s);
    const float inv2ds = 1.0f / ((2.0f * dp.sigma_d) * dp.sigma_d);
    const int taps = 2 * R + 1;
    for (int k = ty * kTile + tx; k < taps * taps; k += kTile * kTile) {
        int dy = k / taps - R, dx = k % taps - R;
        s_w[k] = dm_exp(-(float)(dx * dx + dy * dy) * inv2ss);        // denoise.wgsl:90-91
    }
    if (kShared) {
        for (int k = ty * kTile + tx; k < span * span; k += kTile * kTile) {
            int qx = min(max(x0 + k % span, 0), W - 1);
            int qy = min(max(y0 + k / span, 0), H - 1);
            s_col[k] = __ldg(in + (size_t)qy * W + qx);
            s_g[k] = __ldg(gb + (size_t)qy * W + qx);
        }
    }
    __syncthreads();
    const int px = blockIdx.x * kTile + tx, py = blockIdx.y * kTile + ty;
    if (px >= W || py >= H) return;
    const float4 gp = kShared ? s_g[(ty + R) * span + tx + R] : __ldg(gb + (size_t)py * W + px);
    const f3 np = xyz(gp);
    const float d_p = gp.w;
    const bool on_sky = d_p < 0.0f;
    const float4 cp4 = kShared ? s_col[(ty + R) * span + tx + R] : __ldg(in + (size_t)py * W + px);
    const bool color_term = dp.sigma_color > 0.0f;
    const float inv2cs = color_term ? 1.0f / ((2.0f * dp.sigma_color) * dp.sigma_color) : 0.0f;
    const bool gauss_normal = dp.sigma_normal > 0.0f;
    const float inv2ns = gauss_normal ? 1.0f / ((2.0f * dp.sigma_normal) * dp.sigma_normal) : 0.0f;
    f3 acc = {0.0f, 0.0f, 0.0f};
    float wacc = 0.0f;
    for (int dy = -R; dy <= R; ++dy) {
        for (int dx = -R; dx <= R; ++dx) {
            float4 gq, cq;
            if (kShared) {
                int k = (ty + R + dy) * span + (tx + R + dx);
                gq = s_g[k];
                cq = s_col[k];
            } else {
                int qx = min(max(px + dx, 0), W - 1), qy = min(max(py + dy, 0), H - 1);
                gq = __ldg(gb + (size_t)qy * W + qx);
                cq = __ldg(in + (size_t)qy * W + qx);
            }
            const float d_q = gq.w;
            const bool q_sky = d_q < 0.0f;
            if (on_sky != q_sky) continue;                               // denoise.wgsl:85
            const float w_s = s_w[(dy + R) * taps + (dx + R)];
            float w_n = 1.0f;
            if (!on_sky) {
                float nd = dot(np, xyz(gq));
                if (gauss_normal) {
                    float e = 1.0f - nd;
                    w_n = dm_exp(-(e * e) * inv2ns);
                } else {
                    w_n = dm_pow(fmaxf(0.0f, nd), dp.normal_pow);      // :94-96
                }
            }
            float w_d = 1.0f;
            if (!on_sky) {
                float rel = (d_p - d_q) / fmaxf(d_p, 1e-4f);             // :101-104
                w_d = dm_exp(-(rel * rel) * inv2ds);
            }
            float w = (w_s * w_n) * w_d;
            if (color_term) {
                f3 dc = xyz(cq) - xyz(cp4);
                w = w * dm_exp(-dot(dc, dc) * inv2cs);
            }
            acc = acc + w * xyz(cq);
            wacc += w;
        }
    }
    f3 res = wacc > 0.0f ? acc / wacc : xyz(cp4);                         // :113-115
    out[(size_t)py * W + px] = make_float4(res.x, res.y, res.z, 1.0f);
}

}  // namespace

void launch_denoise(const float4 *in, const float4 *gbuf, uint32_t w, uint32_t h, const mcrt_denoise_params &p,
                    float4 *out, cudaStream_t st) {
    dim3 block(kTile, kTile);
    dim3 grid((w + kTile - 1) / kTile, (h + kTile - 1) / kTile);
    int R = p.radius < 0 ? 0 : p.radius;
    mcrt_denoise_params q = p;
    q.radius = R;
    size_t wbytes = (size_t)(2 * R + 1) * (2 * R + 1) * sizeof(float);
    if (R <= kMaxSharedR) {
        int span = kTile + 2 * R;
        size_t bytes = 2 * (size_t)span * span * sizeof(float4) + wbytes;
        k_denoise<true><<<grid, block, bytes, st>>>(in, gbuf, (int)w, (int)h, q, out); ::mcrt::note_launch();
    } else {
        static bool configured = false;
        if (!configured) {
            cudaFuncSetAttribute(k_denoise<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            configured = true;
        }
        k_denoise<false><<<grid, block, wbytes, st>>>(in, gbuf, (int)w, (int)h, q, out); ::mcrt::note_launch();
    }
}

}  // namespace mcrt
