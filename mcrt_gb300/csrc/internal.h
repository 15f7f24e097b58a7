// internal.h — declarations shared between the translation units of libmcrt_cuda.so.
#pragma once

#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "mcrt_cuda.h"

namespace mcrt {

// A growable device allocation.
struct DBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes == 0) bytes = 16;
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <typename T> T *as() const { return static_cast<T *>(p); }
};

// Process-wide count of kernel launches issued by this library (every launch
// site calls note_launch()); reported per call by mcrt_last_timings.
void note_launch();
unsigned long long launch_count();
// Streaming multiprocessors of the current device (cached).
int sm_count();
// Error message of calls that have no context (mcrt_last_error(NULL)).
void set_global_error(const std::string &msg);

struct DeviceScene;

// Path state for one render pass (structure of arrays, n_slots entries).
struct PathBuffers {
    uint32_t n_slots = 0;
    float4 *thr = nullptr;       // throughput rgb | previous-bounce BSDF pdf (< 0: no MIS)
    float4 *L = nullptr;         // radiance rgb | unused
    float4 *q_o[2] = {nullptr, nullptr};   // ray queues: origin | slot bits
    float4 *q_d[2] = {nullptr, nullptr};   // direction | unused
    float4 *hits = nullptr;      // t | prim bits | u | v, in queue order
    float4 *sh_o = nullptr;      // shadow queue: origin | slot bits
    float4 *sh_d = nullptr;      // direction | t_max
    float4 *sh_c = nullptr;      // contribution rgb | unused
    // [0],[1] ray queue sizes, [2] shadow queue size, [3] closest-hit overflow list size,
    // [4],[5] work counters of the closest-hit and any-hit launches, [6] cache queries,
    // [7] any-hit overflow list size
    uint32_t *counters = nullptr;
    unsigned long long *stats = nullptr;  // [0] rays traced, [1] shadow rays, [2] rays traced stackless
    uint32_t *ovf = nullptr;     // overflow list: queue entries whose traversal stack would overflow
    // adjoint replay only
    float4 *pend = nullptr;      // per slot: d log(BSDF weight) / d(albedo rgb | roughness) of the last vertex
    uint32_t *pend_mat = nullptr;  // per slot: (material + 1) << 8 of that term, 0: none
    float4 *sh_g = nullptr;      // per shadow ray: d log(NEE term) / d(albedo rgb | roughness)
};

// Adjoint (path-replay backpropagation) inputs of the replay kernels.
struct AdjointParams {
    const float4 *dimg = nullptr;   // dLoss / d(image), per pixel (rgb)
    float inv_spp = 0.0f;           // 1 / samples per pixel of the call
    double *grad = nullptr;         // 64 material slots x (albedo r, g, b, roughness)
    uint32_t planes = 1;            // sample planes of the pass: a slot's pixel is slot / planes
};

struct RenderParams {
    uint32_t w, h, npix;
    uint32_t spp_pass;       // sample planes in this pass
    uint32_t frame0;         // frame index of plane 0
    uint32_t max_depth;
    uint32_t flags;          // MCRT_RENDER_*
    int32_t gbuf_plane;      // plane whose primary hit is stored in the G-buffer (-1: none)
    int32_t extend_variant;  // closest-hit kernel variant (autotuned)
    mcrt_camera_uniform cam;
    // batched views (n_views > 0): pixel p of the concatenation belongs to view v
    // with view_px[v] <= p < view_px[v + 1]; its size and camera
    uint32_t n_views;
    const uint32_t *view_px;
    const uint2 *view_wh;
    const mcrt_camera_uniform *view_cam;
    // graph replay: [0] frame index of plane 0, [1] keep flag of the resolve,
    // read from device memory instead of frame0 / the launch argument
    const uint32_t *pass_state;
    // radiance cache (cache_query_vertex == 0: off): non-training paths stop at
    // that non-emissive vertex (1-based) and append a query; slots with
    // slot % train_stride == 0 are training paths recording their vertices
    uint32_t cache_query_vertex;
    uint32_t train_stride;
    float4 *cache_queries;      // 4 float4 per query: p | slot, w_o, n, albedo
    float4 *train_records;      // per training path and vertex: 6 float4 (p | valid, w_o, n, albedo, thr, L so far)
};

constexpr uint32_t kTrainRecordFloat4 = 6;
int extend_variant_count();
// (BVH width, block size, minimum resident blocks, stack depth, refill lanes,
// shared-memory top-tree records) of a variant.
void extend_variant_info(int v, int out[6]);
// Occupancy queries of every variant; call before capturing launches in a graph.
void prepare_extend_variants();

// Launchers (render.cu)
void launch_trace_closest(const DeviceScene &S, const mcrt_ray *rays, uint32_t n, mcrt_hit *hits, bool ref_layout,
                          cudaStream_t st);
// keep_radiance: replay of the same paths (the per-path radiance of the primal
// pass stays in B.L as the radiance still to be accounted for).
void launch_raygen(const DeviceScene &S, const RenderParams &P, PathBuffers &B, cudaStream_t st,
                   bool keep_radiance = false);
// primary: the queue holds the pass's camera rays in slot order (bounce 0).
void launch_extend(const DeviceScene &S, const RenderParams &P, PathBuffers &B, int qi, cudaStream_t st,
                   bool primary = false);
// adj non-null: the adjoint replay variants (same sampling, plus gradient accumulation).
void launch_shade(const DeviceScene &S, const RenderParams &P, PathBuffers &B, int qi, uint32_t bounce,
                  float4 *gbuf, cudaStream_t st, const AdjointParams *adj = nullptr);
void launch_shadow(const DeviceScene &S, const RenderParams &P, PathBuffers &B, cudaStream_t st,
                   const AdjointParams *adj = nullptr);
void launch_resolve(const RenderParams &P, const PathBuffers &B, float4 *mean, double *sum, bool keep,
                    cudaStream_t st);
void launch_tonemap(const float4 *mean, uint32_t npix, uint32_t mode, uchar4 *out, cudaStream_t st);

// BVH (bvh_build.cu)
struct BvhScratch;
// Build the reference-layout mesh BVH on the GPU (bvh.rs / mesh.rs algorithm).
cudaError_t gpu_build_mesh_bvh(const mcrt_gpu_vertex *d_verts, const mcrt_gpu_triangle *d_tris, uint32_t nt,
                               mcrt_gpu_bvh_node *d_nodes, uint32_t *d_order, uint32_t *n_nodes_out,
                               BvhScratch **scratch, cudaStream_t st, std::string *err);
void free_bvh_scratch(BvhScratch *s);
// Convert a reference-layout mesh BVH into the compact layout and the leaf-ordered triangle records.
cudaError_t gpu_make_compact(const mcrt_gpu_bvh_node *d_nodes, uint32_t n_nodes, const uint32_t *d_order,
                             const mcrt_gpu_vertex *d_verts, const mcrt_gpu_triangle *d_tris, uint32_t nt,
                             float4 **d_cnodes, uint32_t *n_cnodes, void *d_trirecs, uint32_t *d_tmp,
                             size_t tmp_words, cudaStream_t st);

// Shading records (3 float4 per triangle, DeviceScene::shade_recs) from the
// vertices and triangles in original order.
void launch_shade_recs(const mcrt_gpu_vertex *d_verts, const mcrt_gpu_triangle *d_tris, uint32_t nt, float4 *out,
                       cudaStream_t st);

// The compact tree's top levels in heap order (kTopNodes records of 64 B), see k_top_tree.
cudaError_t gpu_make_top(const float4 *d_cnodes, uint32_t n_cnodes, float4 *d_top, cudaStream_t st);

// Collapse into the quantised 4-wide layout (d_tmp: 2*n_nodes + 4 words).
cudaError_t gpu_make_wide4(const mcrt_gpu_bvh_node *d_nodes, uint32_t n_nodes, uint4 *d_wide, uint32_t *n_wide,
                           uint32_t *d_tmp, cudaStream_t st);

// Voxel world (world.cu)
struct WorldMeshBuffers {
    DBuf counts, vertices, triangles;
    uint32_t n_quads = 0;
};
void launch_world_generate(const mcrt_world_params &P, uint8_t *vox, cudaStream_t st);
// Mesh the device voxel grid (greedy: the reference's greedy mesher, else one
// quad per visible face) into M.vertices / M.triangles (4 and 2 per quad).
cudaError_t world_mesh(const uint8_t *d_vox, uint32_t nx, uint32_t ny, uint32_t nz, int32_t chunk_x0, int32_t chunk_z0,
                       bool greedy, const uint32_t *d_mat_of, float voxel, WorldMeshBuffers &M, cudaStream_t st);

// Scene ingestion on the device (obj.cu)
// The context's device mesh: vertex and triangle records in append order.
struct DeviceMesh {
    DBuf vertices, triangles;
    uint32_t nv = 0, nt = 0;
};
struct ObjScratch {
    DBuf text, lines, tokens, staging;
    cudaEvent_t ev[9] = {};   // copy and kernel stages of the last parse
};
// A mesh object's transform (scene.rs:438-495) as the kernel applies it:
// q = p * s, then m (row-major, has_r) applied to q, then + t.
struct ObjTransform {
    int identity;
    int has_r;
    float s;
    float m[9];
    float t[3];
};
struct ObjOutcome {
    enum { kOk = 0, kNotUtf8 = 1, kNoGeometry = 2 };
    int code = kNoGeometry;
    unsigned long long valid_up_to = 0;   // first invalid byte (kNotUtf8)
    uint32_t n_vertices = 0, n_triangles = 0, n_lines = 0, n_tokens = 0;
    float h2d_ms = 0.0f, kernel_ms = 0.0f;    // text to the device; the other stages (CUDA events, host waits excluded)
    unsigned long long launches = 0;
};
// Grow the mesh's buffers (keeping their records) for add_v / add_t more.
cudaError_t mesh_reserve(DeviceMesh &M, uint32_t add_v, uint32_t add_t, cudaStream_t st);
// Append host records; triangle indices are relative to this piece's first vertex.
cudaError_t mesh_append_host(DeviceMesh &M, const mcrt_gpu_vertex *v, uint32_t nv, const mcrt_gpu_triangle *t,
                             uint32_t nt, DBuf &staging, cudaStream_t st);
// load_obj (mesh.rs:474-642) of host OBJ text on the device, transformed and
// appended to M.  direct: the device reads the (pageable) host text in place
// in its first pass instead of a copy beforehand.  cudaErrorInvalidValue: text
// or mesh beyond the parser's limits.
cudaError_t obj_append(const char *host_text, unsigned long long len, uint32_t mat_idx, const ObjTransform &X,
                       DeviceMesh &M, ObjScratch &S, cudaStream_t st, bool direct, ObjOutcome *out);

// Radiance-cache MLP (mlp.cu)
struct CacheState;
CacheState *cache_create();
void cache_destroy(CacheState *c);
void cache_set_bounds(CacheState *c, const float lo[3], const float hi[3]);
cudaError_t cache_set_params(CacheState *c, const float *host_params, cudaStream_t st);
cudaError_t cache_get_params(CacheState *c, float *host_params, cudaStream_t st);
cudaError_t cache_infer_host(CacheState *c, const float *q12, uint32_t n, float *out3, cudaStream_t st,
                             bool *timed_out);
cudaError_t cache_train_host(CacheState *c, const float *samples16, uint32_t n, uint32_t steps, uint32_t batch,
                             float lr, float *out_loss, float *out_grad, cudaStream_t st, bool *timed_out);
cudaError_t cache_infer_device(CacheState *c, const float4 *q, const uint32_t *d_count, uint32_t max_n, float *out,
                               float4 *L, const float4 *thr, cudaStream_t st);
cudaError_t cache_step_device(CacheState *c, const float *d_samples, uint32_t n, uint32_t n_valid, float lr,
                              cudaStream_t st);
// Samples from the training paths' records (L: final path radiance per slot), the bias judge, then
// `steps` Adam steps; no host round trip (capturable once cache_prepare has run for the capacity).
cudaError_t cache_train_records(CacheState *c, const float4 *rec, uint32_t n_train, uint32_t depth, uint32_t stride,
                                const float4 *L, uint32_t steps, uint32_t batch, float lr, cudaStream_t st);
cudaError_t cache_prepare(CacheState *c, size_t cap, uint32_t batch);
void cache_buffer_ptrs(const CacheState *c, const void *out[12]);
bool cache_ready(const CacheState *c);
// Bias judge of the training passes (cache_train_records): clear the sums, and
// read them ([0..2] sum of prediction - target, [3..5] sum of target, [6] samples).
cudaError_t cache_judge_reset(CacheState *c, cudaStream_t st);
cudaError_t cache_judge_read(CacheState *c, double out[8], cudaStream_t st);
cudaError_t cache_bench(CacheState *c, uint32_t n, uint32_t reps, float *ms_infer, float *ms_train, cudaStream_t st);

// Denoiser (denoise.cu)
void launch_denoise(const float4 *in, const float4 *gbuf, uint32_t w, uint32_t h, const mcrt_denoise_params &p,
                    float4 *out, cudaStream_t st);

// scan utility (bvh_build.cu)
size_t scan_tmp_words(uint32_t n);
void exclusive_scan_u32(const uint32_t *d_in, uint32_t *d_out, uint32_t n, uint32_t *d_tmp, cudaStream_t st);

}  // namespace mcrt
