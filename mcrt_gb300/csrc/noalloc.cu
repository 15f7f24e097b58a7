// noalloc.cu — mcrt_render_noalloc: the wavefront render of mcrt_render for
// callers that must not allocate GPU memory while they render.
//
// Who needs it: a host that reserves all of its GPU memory up front — a game
// engine or an interactive viewer with a fixed memory budget, or a renderer
// embedded in another application's frame loop — and treats any later
// allocation as an error, because cudaMalloc/cudaFree synchronise the device
// (a stall in the middle of a frame) and can fail with out-of-memory at a point
// where the frame cannot be abandoned.  mcrt_render sizes its path state per
// call and allocates when the image grows; this entry point instead keeps the
// per-path scratch (path state, ray queues, shadow queue, counters, f64 sums)
// in one statically sized device array that is part of the loaded library.
//
// Rules of use:
//  * The scratch is kNoAllocScratchBytes (64 MiB), a file-scope __device__
//    array: every GPU on which the library is loaded holds it until the
//    process exits.  Images larger than kNoAllocMaxPixels are rejected.
//  * All calls share the one array.  Calls that overlap on the GPU (several
//    threads or streams, several contexts on one device) race on it; issue
//    them one after another.
//  * The first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current and caches it; make that
//    first call before any stream capture is started on the device.
//  * The scene comes from an earlier mcrt_upload_scene on the context (that
//    set-up step allocates, as mcrt_upload_scene always does).
//  * The closest-hit kernel is the context's autotuned variant (or the one the
//    options name); a 4-wide variant whose quantised tree has not been built
//    since the last BVH build (building it allocates) traces with the binary
//    variant 0 instead, which gives the same image.
//  * The caller's current device is restored before the call returns.
#include <cstring>

#include "common.cuh"
#include "internal.h"

namespace {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;
constexpr uint32_t kNoAllocMaxPixels = 262144;          // e.g. 512 x 512
constexpr size_t kCounterBytes = 256;
// thr, L, q_o x2, q_d x2, hits, sh_o, sh_d, sh_c (16 B each) and the overflow list (4 B)
constexpr size_t kSlotBytes = 16 * 10 + 4;
constexpr size_t kSumBytesPerPixel = 24;                // f64 rgb

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
void *g_scratch_addr[kMaxDevices] = {};

}  // namespace

namespace mcrt {
void set_global_error(const std::string &msg);
// Scene of a context, and the closest-hit variant a render on it uses (api.cu).
bool context_scene(mcrt_ctx *ctx, DeviceScene *out, cudaStream_t *stream, int *device, std::string **err);
int context_variant(mcrt_ctx *ctx, const mcrt_render_opts &o);
}  // namespace mcrt

namespace {
// Puts the caller's current device back when the call returns.
struct DeviceRestore {
    int prev = -1;
    DeviceRestore() { if (cudaGetDevice(&prev) != cudaSuccess) prev = -1; }
    ~DeviceRestore() { if (prev >= 0) cudaSetDevice(prev); }
};
}  // namespace

extern "C" mcrt_status mcrt_render_noalloc(mcrt_ctx *ctx, const mcrt_camera_uniform *cam, uint32_t w, uint32_t h,
                                           uint32_t spp, uint32_t first_frame, const mcrt_render_opts *opts,
                                           float *d_out_rgba) {
    if (!ctx) { mcrt::set_global_error("ctx is NULL"); return MCRT_ERR_INVALID_ARG; }
    mcrt::DeviceScene S{};
    cudaStream_t st = nullptr;
    int device = 0;
    std::string *err = nullptr;
    if (!mcrt::context_scene(ctx, &S, &st, &device, &err)) return MCRT_ERR_NO_SCENE;
    auto fail = [&](mcrt_status code, const char *msg) { *err = msg; return code; };
    if (!cam || !d_out_rgba) return fail(MCRT_ERR_INVALID_ARG, "cam and d_out_rgba are required");
    if (w == 0 || h == 0 || spp == 0) return fail(MCRT_ERR_INVALID_ARG, "width, height and spp must be > 0");
    if ((uint64_t)w * h > kNoAllocMaxPixels)
        return fail(MCRT_ERR_INVALID_ARG, "mcrt_render_noalloc: image larger than 262144 pixels (the static scratch limit)");
    if (device < 0 || device >= kMaxDevices) return fail(MCRT_ERR_INVALID_ARG, "device index out of range");
    mcrt_render_opts o{};
    if (opts) o = *opts;
    if (o.flags & MCRT_RENDER_KEEP_ACCUM) return fail(MCRT_ERR_INVALID_ARG, "KEEP_ACCUM is not supported here");
    if (o.flags & MCRT_RENDER_CACHE)
        return fail(MCRT_ERR_INVALID_ARG, "the radiance cache is not supported here (its buffers are allocated)");
    if (o.flags & MCRT_RENDER_GBUFFER) return fail(MCRT_ERR_INVALID_ARG, "no G-buffer is produced here");
    const uint32_t depth = o.max_depth ? o.max_depth : mcrt::kDefaultBounces;
    if (depth > 1024) return fail(MCRT_ERR_INVALID_ARG, "max_depth too large");
    const int variant = mcrt::context_variant(ctx, o);
    if (variant < 0) return fail(MCRT_ERR_INVALID_ARG, "variant out of range");
    DeviceRestore restore;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(MCRT_ERR_CUDA, "cudaSetDevice failed");
    // once per device: the device address of the static array
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return fail(MCRT_ERR_CUDA, "cudaGetSymbolAddress of the no-alloc scratch failed");
        g_scratch_addr[device] = p;
    }
    unsigned char *base = static_cast<unsigned char *>(g_scratch_addr[device]);
    const uint32_t npix = w * h;
    // carve: counters | f64 sums | path state for n_slots = npix * spp_pass
    size_t sum_bytes = ((size_t)npix * kSumBytesPerPixel + 255) & ~(size_t)255;
    size_t avail = kNoAllocScratchBytes - kCounterBytes - sum_bytes;
    uint32_t spp_pass = (uint32_t)(avail / ((size_t)npix * kSlotBytes));
    if (spp_pass == 0) return fail(MCRT_ERR_INVALID_ARG, "image does not fit the static scratch");
    if (o.spp_per_pass) spp_pass = spp_pass < o.spp_per_pass ? spp_pass : o.spp_per_pass;
    if (spp_pass > spp) spp_pass = spp;
    const size_t n_slots = (size_t)npix * spp_pass;
    mcrt::PathBuffers B;
    unsigned char *p = base;
    B.counters = reinterpret_cast<uint32_t *>(p);
    B.stats = reinterpret_cast<unsigned long long *>(p + 128);
    p += kCounterBytes;
    double *sum = reinterpret_cast<double *>(p);
    p += sum_bytes;
    auto take = [&](size_t bytes) { unsigned char *r = p; p += bytes; return reinterpret_cast<float4 *>(r); };
    B.n_slots = (uint32_t)n_slots;
    B.thr = take(n_slots * 16);
    B.L = take(n_slots * 16);
    for (int k = 0; k < 2; ++k) {
        B.q_o[k] = take(n_slots * 16);
        B.q_d[k] = take(n_slots * 16);
    }
    B.hits = take(n_slots * 16);
    B.sh_o = take(n_slots * 16);
    B.sh_d = take(n_slots * 16);
    B.sh_c = take(n_slots * 16);
    B.ovf = reinterpret_cast<uint32_t *>(take(n_slots * 4));   // last: 4 B per slot
    // the array keeps the previous call's contents: clear the counters (the path
    // state and the sums are fully written by ray generation and the first resolve)
    e = cudaMemsetAsync(B.counters, 0, kCounterBytes, st);
    if (e != cudaSuccess) return fail(MCRT_ERR_CUDA, "clearing the no-alloc counters failed");
    const bool nee = (o.flags & MCRT_RENDER_NEE) != 0 && (S.n_lights > 0 || S.has_sun);
    uint32_t done = 0;
    while (done < spp) {
        mcrt::RenderParams P{};
        P.w = w; P.h = h; P.npix = npix;
        P.spp_pass = spp - done < spp_pass ? spp - done : spp_pass;
        P.frame0 = first_frame + done;
        P.max_depth = depth;
        P.flags = o.flags & ~(uint32_t)MCRT_RENDER_GRAPH;   // no capture here: the passes launch directly
        P.cam = *cam;
        P.gbuf_plane = -1;
        P.extend_variant = variant;
        mcrt::launch_raygen(S, P, B, st);
        int qi = 0;
        for (uint32_t b = 0; b < depth; ++b) {
            mcrt::launch_extend(S, P, B, qi, st, b == 0);
            mcrt::launch_shade(S, P, B, qi, b, nullptr, st);
            if (nee) mcrt::launch_shadow(S, P, B, st);
            qi ^= 1;
        }
        mcrt::launch_resolve(P, B, reinterpret_cast<float4 *>(d_out_rgba), sum, done > 0, st);
        done += P.spp_pass;
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(MCRT_ERR_CUDA, cudaGetErrorString(e));
    return MCRT_OK;
}
