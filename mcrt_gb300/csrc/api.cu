// api.cu — the extern "C" entry points of libmcrt_cuda.so (include/mcrt_cuda.h):
// context, scene upload (with host-side validation of every index the kernels
// will dereference), closest-hit probe, render driver, denoiser.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "host/scene_internal.h"
#include "internal.h"
#include "mlp_net.cuh"

static_assert(sizeof(mcrt_gpu_sphere) == 32, "GpuSphere is 32 bytes (scene.rs:24-29)");
static_assert(sizeof(mcrt_gpu_bvh_node) == 48, "GpuBvhNode is 48 bytes (bvh.rs:56-68)");
static_assert(sizeof(mcrt_gpu_vertex) == 48, "GpuVertex is 48 bytes (mesh.rs:26-34)");
static_assert(sizeof(mcrt_gpu_triangle) == 16, "GpuTriangle is 16 bytes (mesh.rs:41-46)");
static_assert(sizeof(mcrt_gpu_material) == 48, "GpuMaterial is 48 bytes (material.rs:37-44)");
static_assert(sizeof(mcrt_gpu_material_data) == 3088, "GpuMaterialData is 3088 bytes (material.rs:56-63)");
static_assert(sizeof(mcrt_camera_uniform) == 112, "CameraUniform is 112 bytes (camera.rs:37-53)");
static_assert(sizeof(mcrt_ray) == 32 && sizeof(mcrt_hit) == 16, "ray/hit records");
static_assert(sizeof(mcrt_denoise_params) == 32, "denoise params");
static_assert(sizeof(mcrt::TriRec) == 48, "fast triangle record");

namespace mcrt {
void launch_light_cdf(const DeviceScene &S, float *d_cdf, float *d_total, cudaStream_t st);
cudaError_t gpu_build_sphere_bvh(const mcrt_gpu_sphere *d_spheres, uint32_t n, mcrt_gpu_bvh_node *d_nodes,
                                 uint32_t *d_order, uint32_t *n_nodes_out, BvhScratch **scratch, cudaStream_t st,
                                 std::string *err);
}  // namespace mcrt

namespace {

thread_local std::string g_error;   // errors of calls without a context

}  // namespace

namespace mcrt {
void set_global_error(const std::string &msg) { g_error = msg; }
static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }
}  // namespace mcrt

using mcrt::DBuf;

struct mcrt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    // scene
    bool has_scene = false;
    DBuf wnodes;
    uint32_t n_wnodes = 0;
    bool wide_valid = false;    // wnodes matches the current mesh BVH
    DBuf spheres, sphere_ids, sphere_nodes, vertices, triangles, mesh_nodes, tri_order, trirecs, cnodes, materials,
        env, lights, light_cdf, tmp, staging, albedo, shade_recs, top;
    uint32_t albedo_layers = 0, albedo_size = 0;
    size_t srgb_lut_offset = 0;
    uint32_t n_spheres = 0, n_sphere_nodes = 0, n_vertices = 0, n_triangles = 0, n_mesh_nodes = 0, n_cnodes = 0,
             n_lights = 0, env_w = 0, env_h = 0;
    float light_total = 0.0f;
    mcrt::BvhScratch *bvh_scratch = nullptr;
    // render state
    mcrt::PathBuffers pb;
    DBuf pbmem;
    DBuf mean, sum, gbuf;
    uint32_t acc_w = 0, acc_h = 0;
    bool acc_valid = false, gbuf_valid = false;
    // probe / denoise buffers
    DBuf io_a, io_b, io_c, counters;
    // timing
    std::vector<cudaEvent_t> ev_pool;
    float last_ms[6] = {0, 0, 0, 0, 0, 0};
    // rays, shadow rays, rays traced stackless, node and triangle records fetched (MCRT_RENDER_COUNT)
    unsigned long long last_counts[5] = {0, 0, 0, 0, 0};
    unsigned long long last_render_launches = 0, last_build_launches = 0, last_extend_launches = 0;
    float last_build_ms = 0.0f;
    int extend_variant = 0;   // chosen by mcrt_autotune
    // adjoint
    DBuf dimg, grad;
    mcrt_gpu_material_data host_materials{};
    // directional light
    float sun_dir[4] = {0, 1, 0, 0}, sun_E[4] = {0, 0, 0, 0};
    bool has_sun = false;
    // voxel world
    DBuf world_vox, world_matmap;
    uint32_t world_nx = 0, world_ny = 0, world_nz = 0;
    int32_t world_cx0 = 0, world_cz0 = 0;
    mcrt::WorldMeshBuffers wmesh;
    bool wmesh_valid = false;
    // device mesh assembled by mcrt_mesh_append / mcrt_mesh_append_obj
    mcrt::DeviceMesh dmesh;
    mcrt::ObjScratch obj;
    unsigned long long last_obj_counts[4] = {0, 0, 0, 0};   // bytes, lines, face tokens, kernel launches
    int pageable_access = -1;                                 // cudaDevAttrPageableMemoryAccess (-1: not read)
    float last_obj_ms[2] = {0.0f, 0.0f};                    // text copy, kernels
    // batched views and graph replay
    DBuf views, pass_state;
    std::vector<char> view_blob, graph_key;
    std::vector<uint32_t> view_px;
    cudaGraphExec_t graph_exec = nullptr;
    unsigned long long graph_captures = 0;
    // radiance cache
    mcrt::CacheState *cache = nullptr;
    mcrt_cache_params cache_cfg{};
    bool cache_cfg_set = false;
    // bias judge of the last cached render: relative bias rgb, samples, stopped
    double cache_stats[5] = {NAN, NAN, NAN, 0.0, 0.0};
    bool cache_fallback = false;   // the judge's last bias exceeds cache_cfg.max_bias
    DBuf cache_q, cache_rec;
    uint32_t last_train_samples = 0;
};

namespace {

mcrt_status fail(mcrt_ctx *c, mcrt_status code, const std::string &msg) {
    if (c) c->err = msg;
    else g_error = msg;
    return code;
}
mcrt_status cuda_fail(mcrt_ctx *c, cudaError_t e, const std::string &what) {
    std::string m = what + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return fail(c, MCRT_ERR_OOM, m);
    return fail(c, MCRT_ERR_CUDA, m);
}
#define CK(call, what)                                            \
    do {                                                          \
        cudaError_t e__ = (call);                                 \
        if (e__ != cudaSuccess) return cuda_fail(ctx, e__, what); \
    } while (0)

mcrt::DeviceScene device_scene(const mcrt_ctx *c) {
    mcrt::DeviceScene S{};
    S.spheres = c->spheres.as<mcrt_gpu_sphere>();
    S.n_spheres = c->n_spheres;
    S.sphere_ids = c->sphere_ids.as<uint32_t>();
    S.sphere_nodes = c->sphere_nodes.as<mcrt_gpu_bvh_node>();
    S.n_sphere_nodes = c->n_sphere_nodes;
    S.vertices = c->vertices.as<mcrt_gpu_vertex>();
    S.n_vertices = c->n_vertices;
    S.triangles = c->triangles.as<mcrt_gpu_triangle>();
    S.n_triangles = c->n_triangles;
    S.mesh_nodes = c->mesh_nodes.as<mcrt_gpu_bvh_node>();
    S.n_mesh_nodes = c->n_mesh_nodes;
    S.tri_ids = c->tri_order.as<uint32_t>();
    S.tris = c->trirecs.as<mcrt::TriRec>();
    S.shade_recs = c->shade_recs.as<float4>();
    S.cnodes = c->cnodes.as<float4>();
    S.n_cnodes = c->n_cnodes;
    S.top = c->top.as<float4>();
    S.wnodes = c->wnodes.as<uint4>();
    S.n_wnodes = c->n_wnodes;
    S.materials = c->materials.as<mcrt_gpu_material_data>();
    S.env = c->env.as<float4>();
    S.env_w = c->env_w;
    S.env_h = c->env_h;
    S.lights = c->lights.as<uint32_t>();
    S.n_lights = c->n_lights;
    S.light_cdf = c->light_cdf.as<float>();
    S.light_total = c->light_total;
    S.albedo = c->albedo.as<uchar4>();
    S.albedo_layers = c->albedo_layers;
    S.albedo_size = c->albedo_size;
    S.srgb_lut = reinterpret_cast<const float *>(c->albedo.as<char>() + c->srgb_lut_offset);
    S.has_sun = c->has_sun ? 1 : 0;
    S.sun_dir = make_float4(c->sun_dir[0], c->sun_dir[1], c->sun_dir[2], 0.0f);
    S.sun_E = make_float4(c->sun_E[0], c->sun_E[1], c->sun_E[2], 0.0f);
    return S;
}

// Host validation of a reference-layout BVH: pre-order children strictly after
// the parent (so every traversal terminates) and every index in range.
bool valid_bvh(const mcrt_gpu_bvh_node *nodes, uint32_t n_nodes, uint32_t n_prims, std::string *why) {
    for (uint32_t i = 0; i < n_nodes; ++i) {
        const mcrt_gpu_bvh_node &nd = nodes[i];
        if (nd.prim_count == 0) {
            if (i + 1 >= n_nodes || nd.right_or_offset <= i + 1 || nd.right_or_offset >= n_nodes) {
                *why = "internal node " + std::to_string(i) + " has an out-of-order or out-of-range child";
                return false;
            }
        } else if ((uint64_t)nd.right_or_offset + nd.prim_count > n_prims) {
            *why = "leaf " + std::to_string(i) + " references primitives beyond the primitive count";
            return false;
        }
    }
    return true;
}

bool valid_permutation(const uint32_t *order, uint32_t n) {
    std::vector<uint8_t> seen(n, 0);
    for (uint32_t i = 0; i < n; ++i) {
        if (order[i] >= n || seen[order[i]]) return false;
        seen[order[i]] = 1;
    }
    return true;
}

__global__ void k_scatter_tris(const mcrt_gpu_triangle *ordered, const uint32_t *order, uint32_t n,
                               mcrt_gpu_triangle *out) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) out[order[s]] = ordered[s];
}
__global__ void k_gather_spheres(const mcrt_gpu_sphere *orig, const uint32_t *order, uint32_t n,
                                 mcrt_gpu_sphere *out) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) out[s] = orig[order[s]];
}
__global__ void k_iota(uint32_t *p, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = i;
}
// Emissive-triangle list, ascending original id: flag, exclusive scan, scatter.
__global__ void k_emissive_flags(const mcrt_gpu_triangle *t, uint32_t n, const mcrt_gpu_material_data *m,
                                 uint32_t *flags) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    if (i == n) { flags[n] = 0u; return; }
    uint32_t mat = min(t[i].mat_idx & 0x7fffffffu, 63u);
    flags[i] = m->materials[mat].type_pad[0] == MCRT_MAT_EMISSIVE ? 1u : 0u;
}
__global__ void k_emissive_scatter(const uint32_t *flags, const uint32_t *pos, uint32_t n, uint32_t *out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flags[i]) out[pos[i]] = i;
}

cudaEvent_t ev(mcrt_ctx *ctx, size_t i) {
    while (ctx->ev_pool.size() <= i) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        ctx->ev_pool.push_back(e);
    }
    return ctx->ev_pool[i];
}

// Derived device structures of the mesh: compact nodes and triangle records.
mcrt_status finish_mesh(mcrt_ctx *ctx) {
    cudaStream_t st = ctx->stream;
    uint32_t nt = ctx->n_triangles, nn = ctx->n_mesh_nodes;
    CK(ctx->trirecs.ensure((size_t)std::max(nt, 1u) * sizeof(mcrt::TriRec)), "allocate triangle records");
    CK(ctx->shade_recs.ensure((size_t)std::max(nt, 1u) * 48), "allocate shading records");
    mcrt::launch_shade_recs(ctx->vertices.as<mcrt_gpu_vertex>(), ctx->triangles.as<mcrt_gpu_triangle>(), nt,
                            ctx->shade_recs.as<float4>(), st);
    CK(ctx->cnodes.ensure((size_t)(nn / 2 + 1) * 64), "allocate compact nodes");
    size_t tmp_words = 2 * (size_t)std::max(nn, 1u) + mcrt::scan_tmp_words(std::max(nn, 1u));
    CK(ctx->tmp.ensure(tmp_words * 4), "allocate scan scratch");
    float4 *cn = ctx->cnodes.as<float4>();
    uint32_t ncn = 0;
    CK(mcrt::gpu_make_compact(ctx->mesh_nodes.as<mcrt_gpu_bvh_node>(), nn, ctx->tri_order.as<uint32_t>(),
                              ctx->vertices.as<mcrt_gpu_vertex>(), ctx->triangles.as<mcrt_gpu_triangle>(), nt, &cn,
                              &ncn, ctx->trirecs.p, ctx->tmp.as<uint32_t>(), tmp_words, st),
       "compact BVH");
    ctx->n_cnodes = ncn;
    if (ncn >= mcrt::kTopBit) return fail(ctx, MCRT_ERR_INVALID_ARG, "mesh too large for the compact BVH codes");
    CK(ctx->top.ensure((size_t)mcrt::kTopNodes * 64), "allocate top tree");
    CK(mcrt::gpu_make_top(cn, ncn, ctx->top.as<float4>(), st), "top tree");
    ctx->wide_valid = false;                  // the 4-wide layout is built when a render first needs it
    ctx->n_wnodes = 0;
    return MCRT_OK;
}

// The quantised 4-wide BVH of the current mesh BVH, built on first use after
// each (re)build: only the 4-wide closest-hit variants read it.
mcrt_status ensure_wide(mcrt_ctx *ctx) {
    if (ctx->wide_valid) return MCRT_OK;
    const uint32_t nn = ctx->n_mesh_nodes;
    if (nn) {
        CK(ctx->wnodes.ensure((size_t)(nn / 2 + 1) * 64), "allocate wide nodes");
        uint32_t nw = 0;
        CK(mcrt::gpu_make_wide4(ctx->mesh_nodes.as<mcrt_gpu_bvh_node>(), nn, ctx->wnodes.as<uint4>(), &nw,
                                ctx->tmp.as<uint32_t>(), ctx->stream),
           "4-wide BVH");
        ctx->n_wnodes = nw;
    }
    ctx->wide_valid = true;
    return MCRT_OK;
}

// Closest-hit variant of a render (opts variant k + 1, else the context's),
// with the layout it reads made ready.
mcrt_status render_variant(mcrt_ctx *ctx, const mcrt_render_opts &o, int *variant) {
    const int v = o.variant ? (int)o.variant - 1 : ctx->extend_variant;
    if (v < 0 || v >= mcrt::extend_variant_count()) return fail(ctx, MCRT_ERR_INVALID_ARG, "variant out of range");
    int info[6];
    mcrt::extend_variant_info(v, info);
    if (info[0] == 4) {
        mcrt_status s = ensure_wide(ctx);
        if (s != MCRT_OK) return s;
    }
    *variant = v;
    return MCRT_OK;
}

// Light CDF over the light list (device), total weight read back.
mcrt_status finish_lights(mcrt_ctx *ctx) {
    ctx->light_total = 0.0f;
    if (ctx->n_lights == 0) return MCRT_OK;
    CK(ctx->light_cdf.ensure(((size_t)ctx->n_lights + 2) * sizeof(float)), "allocate light cdf");
    mcrt::DeviceScene S = device_scene(ctx);
    float *d_total = ctx->light_cdf.as<float>() + ctx->n_lights + 1;
    mcrt::launch_light_cdf(S, ctx->light_cdf.as<float>(), d_total, ctx->stream);
    float total = 0.0f;
    CK(cudaMemcpyAsync(&total, d_total, 4, cudaMemcpyDeviceToHost, ctx->stream), "read light total");
    CK(cudaStreamSynchronize(ctx->stream), "light cdf");
    ctx->light_total = total;
    if (!(total > 0.0f)) ctx->n_lights = 0;
    return MCRT_OK;
}

// Path state for n_slots concurrent samples (structure of arrays in one allocation).
mcrt_status ensure_path_buffers(mcrt_ctx *ctx, uint32_t n_slots) {
    if (ctx->pb.n_slots < n_slots) {
        // thr L, q_o q_d x2, hits, sh o d c, pend sh_g (16 B each), pend_mat and the overflow
        // list (4 B each, last: keeps the others aligned); a path's random state travels in its
        // ray's direction w
        size_t per = 16 * 2 + 16 * 4 + 16 + 16 * 3 + 16 * 2 + 4 + 4;
        CK(ctx->pbmem.ensure((size_t)n_slots * per + 256), "allocate path state");
        char *p = ctx->pbmem.as<char>();
        auto take = [&](size_t bytes) { char *r = p; p += bytes; return r; };
        ctx->pb.thr = reinterpret_cast<float4 *>(take((size_t)n_slots * 16));
        ctx->pb.L = reinterpret_cast<float4 *>(take((size_t)n_slots * 16));
        for (int k = 0; k < 2; ++k) {
            ctx->pb.q_o[k] = reinterpret_cast<float4 *>(take((size_t)n_slots * 16));
            ctx->pb.q_d[k] = reinterpret_cast<float4 *>(take((size_t)n_slots * 16));
        }
        ctx->pb.hits = reinterpret_cast<float4 *>(take((size_t)n_slots * 16));
        ctx->pb.sh_o = reinterpret_cast<float4 *>(take((size_t)n_slots * 16));
        ctx->pb.sh_d = reinterpret_cast<float4 *>(take((size_t)n_slots * 16));
        ctx->pb.sh_c = reinterpret_cast<float4 *>(take((size_t)n_slots * 16));
        ctx->pb.pend = reinterpret_cast<float4 *>(take((size_t)n_slots * 16));
        ctx->pb.sh_g = reinterpret_cast<float4 *>(take((size_t)n_slots * 16));
        ctx->pb.pend_mat = reinterpret_cast<uint32_t *>(take((size_t)n_slots * 4));
        ctx->pb.ovf = reinterpret_cast<uint32_t *>(take((size_t)n_slots * 4));
        ctx->pb.n_slots = n_slots;
    }
    CK(ctx->counters.ensure(256), "allocate counters");
    ctx->pb.counters = ctx->counters.as<uint32_t>();
    ctx->pb.stats = reinterpret_cast<unsigned long long *>(ctx->counters.as<char>() + 128);
    return MCRT_OK;
}

mcrt_status build_mesh_bvh_gpu(mcrt_ctx *ctx) {
    uint32_t nn = 0;
    std::string err;
    const unsigned long long l0 = mcrt::launch_count();
    cudaEvent_t a = ev(ctx, 0), b = ev(ctx, 1);
    cudaEventRecord(a, ctx->stream);
    cudaError_t e = mcrt::gpu_build_mesh_bvh(ctx->vertices.as<mcrt_gpu_vertex>(),
                                             ctx->triangles.as<mcrt_gpu_triangle>(), ctx->n_triangles,
                                             ctx->mesh_nodes.as<mcrt_gpu_bvh_node>(), ctx->tri_order.as<uint32_t>(),
                                             &nn, &ctx->bvh_scratch, ctx->stream, &err);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "mesh BVH build: " + err);
    ctx->n_mesh_nodes = nn;
    mcrt_status s = finish_mesh(ctx);
    if (s != MCRT_OK) return s;
    cudaEventRecord(b, ctx->stream);
    CK(cudaEventSynchronize(b), "BVH build");
    cudaEventElapsedTime(&ctx->last_build_ms, a, b);
    ctx->last_build_launches = mcrt::launch_count() - l0;
    return MCRT_OK;
}

}  // namespace

// ====================================================================== ABI

extern "C" {

const char *mcrt_version(void) { return "mcrt_gb300 1 (sm_103a)"; }

const char *mcrt_last_error(const mcrt_ctx *ctx) { return ctx ? ctx->err.c_str() : g_error.c_str(); }

mcrt_status mcrt_create(int device, void *stream, mcrt_ctx **out) {
    if (!out) return fail(nullptr, MCRT_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(nullptr, MCRT_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= ndev) return fail(nullptr, MCRT_ERR_INVALID_ARG, "device index out of range");
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(nullptr, MCRT_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    mcrt_ctx *c = new mcrt_ctx();
    c->device = device;
    if (stream) {
        c->stream = static_cast<cudaStream_t>(stream);
    } else {
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete c;
            return fail(nullptr, MCRT_ERR_CUDA, "cudaStreamCreate failed");
        }
        c->own_stream = true;
    }
    *out = c;
    return MCRT_OK;
}

void mcrt_destroy(mcrt_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    DBuf *bufs[] = {&ctx->spheres, &ctx->sphere_ids, &ctx->sphere_nodes, &ctx->vertices, &ctx->triangles,
                    &ctx->mesh_nodes, &ctx->tri_order, &ctx->trirecs, &ctx->cnodes, &ctx->top, &ctx->materials, &ctx->env,
                    &ctx->lights, &ctx->light_cdf, &ctx->tmp, &ctx->staging, &ctx->albedo, &ctx->wnodes, &ctx->pbmem, &ctx->mean,
                    &ctx->sum, &ctx->gbuf, &ctx->io_a, &ctx->io_b, &ctx->io_c, &ctx->counters, &ctx->dimg,
                    &ctx->grad, &ctx->world_vox, &ctx->world_matmap, &ctx->wmesh.counts, &ctx->wmesh.vertices,
                    &ctx->wmesh.triangles, &ctx->views, &ctx->pass_state, &ctx->cache_q, &ctx->cache_rec,
                    &ctx->shade_recs, &ctx->dmesh.vertices, &ctx->dmesh.triangles, &ctx->obj.text,
                    &ctx->obj.lines, &ctx->obj.tokens, &ctx->obj.staging};
    for (DBuf *b : bufs) b->release();
    for (cudaEvent_t e : ctx->obj.ev)
        if (e) cudaEventDestroy(e);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    mcrt::cache_destroy(ctx->cache);
    mcrt::free_bvh_scratch(ctx->bvh_scratch);
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

mcrt_status mcrt_upload_scene(mcrt_ctx *ctx, const mcrt_scene_desc *d) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!d) return fail(ctx, MCRT_ERR_INVALID_ARG, "desc is NULL");
    if (!d->materials) return fail(ctx, MCRT_ERR_INVALID_ARG, "materials is NULL");
    if (d->n_spheres && !d->spheres) return fail(ctx, MCRT_ERR_INVALID_ARG, "spheres is NULL");
    const bool world_mesh = (d->flags & MCRT_SCENE_WORLD_MESH) != 0;
    const bool device_mesh = (d->flags & MCRT_SCENE_DEVICE_MESH) != 0;
    if (world_mesh && device_mesh)
        return fail(ctx, MCRT_ERR_INVALID_ARG, "MCRT_SCENE_WORLD_MESH and MCRT_SCENE_DEVICE_MESH are exclusive");
    if (world_mesh || device_mesh) {
        if (d->vertices || d->triangles || d->n_vertices || d->n_triangles || d->mesh_bvh)
            return fail(ctx, MCRT_ERR_INVALID_ARG, "a device-resident mesh takes no host vertices, triangles or BVH");
        if (world_mesh && !ctx->wmesh_valid)
            return fail(ctx, MCRT_ERR_INVALID_ARG, "no world mesh (call mcrt_world_mesh first)");
    }
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(d->sun_dir[k]) || !std::isfinite(d->sun_irradiance[k]) || d->sun_irradiance[k] < 0.0f)
            return fail(ctx, MCRT_ERR_INVALID_ARG, "sun direction / irradiance must be finite, irradiance >= 0");
    if (d->n_triangles && (!d->triangles || !d->vertices))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "triangles or vertices is NULL");
    if (d->n_triangles >= (1u << 27) - 1) return fail(ctx, MCRT_ERR_INVALID_ARG, "too many triangles (max 2^27-2)");
    if (d->n_spheres >= (1u << 30)) return fail(ctx, MCRT_ERR_INVALID_ARG, "too many spheres");
    if ((d->env_w == 0) != (d->env_h == 0) || (d->env_w && !d->env_rgba))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "inconsistent environment map");
    if ((uint64_t)d->env_w * d->env_h > (1ull << 28)) return fail(ctx, MCRT_ERR_INVALID_ARG, "environment map too large");
    for (uint32_t i = 0; i < d->n_triangles; ++i)
        for (int k = 0; k < 3; ++k)
            if (d->triangles[i].v[k] >= d->n_vertices)
                return fail(ctx, MCRT_ERR_INVALID_ARG,
                            "triangle " + std::to_string(i) + " references a vertex beyond n_vertices");
    std::string why;
    if (d->mesh_bvh) {
        if (d->n_triangles == 0 || d->n_mesh_nodes == 0) return fail(ctx, MCRT_ERR_INVALID_ARG, "empty mesh BVH");
        if (!valid_bvh(d->mesh_bvh, d->n_mesh_nodes, d->n_triangles, &why))
            return fail(ctx, MCRT_ERR_INVALID_ARG, "mesh BVH: " + why);
        if (d->triangle_order && !valid_permutation(d->triangle_order, d->n_triangles))
            return fail(ctx, MCRT_ERR_INVALID_ARG, "triangle_order is not a permutation");
    }
    if (d->sphere_bvh) {
        if (d->n_spheres == 0 || d->n_sphere_nodes == 0) return fail(ctx, MCRT_ERR_INVALID_ARG, "empty sphere BVH");
        if (!valid_bvh(d->sphere_bvh, d->n_sphere_nodes, d->n_spheres, &why))
            return fail(ctx, MCRT_ERR_INVALID_ARG, "sphere BVH: " + why);
        if (d->sphere_order && !valid_permutation(d->sphere_order, d->n_spheres))
            return fail(ctx, MCRT_ERR_INVALID_ARG, "sphere_order is not a permutation");
    }
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    ctx->has_scene = false;
    ctx->acc_valid = false;
    const uint32_t ns = d->n_spheres;
    const uint32_t nv = world_mesh ? 4 * ctx->wmesh.n_quads : device_mesh ? ctx->dmesh.nv : d->n_vertices;
    const uint32_t nt = world_mesh ? 2 * ctx->wmesh.n_quads : device_mesh ? ctx->dmesh.nt : d->n_triangles;
    const void *dev_vertices = world_mesh ? ctx->wmesh.vertices.p : device_mesh ? ctx->dmesh.vertices.p : nullptr;
    const void *dev_triangles = world_mesh ? ctx->wmesh.triangles.p : device_mesh ? ctx->dmesh.triangles.p : nullptr;

    // ---- spheres, stored in BVH order, with their original ids
    CK(ctx->spheres.ensure((size_t)ns * 32), "allocate spheres");
    CK(ctx->sphere_ids.ensure((size_t)ns * 4), "allocate sphere ids");
    CK(ctx->sphere_nodes.ensure((size_t)2 * ns * 48), "allocate sphere nodes");
    ctx->n_spheres = ns;
    ctx->n_sphere_nodes = 0;
    if (ns) {
        if (d->sphere_bvh) {
            CK(cudaMemcpyAsync(ctx->spheres.p, d->spheres, (size_t)ns * 32, cudaMemcpyHostToDevice, st), "upload");
            CK(cudaMemcpyAsync(ctx->sphere_nodes.p, d->sphere_bvh, (size_t)d->n_sphere_nodes * 48,
                               cudaMemcpyHostToDevice, st), "upload");
            if (d->sphere_order)
                CK(cudaMemcpyAsync(ctx->sphere_ids.p, d->sphere_order, (size_t)ns * 4, cudaMemcpyHostToDevice, st),
                   "upload");
            else
                k_iota<<<(ns + 255) / 256, 256, 0, st>>>(ctx->sphere_ids.as<uint32_t>(), ns); ::mcrt::note_launch();
            ctx->n_sphere_nodes = d->n_sphere_nodes;
        } else {
            CK(ctx->staging.ensure((size_t)ns * 32), "allocate staging");
            CK(cudaMemcpyAsync(ctx->staging.p, d->spheres, (size_t)ns * 32, cudaMemcpyHostToDevice, st), "upload");
            uint32_t nn = 0;
            std::string err;
            cudaError_t e = mcrt::gpu_build_sphere_bvh(ctx->staging.as<mcrt_gpu_sphere>(), ns,
                                                       ctx->sphere_nodes.as<mcrt_gpu_bvh_node>(),
                                                       ctx->sphere_ids.as<uint32_t>(), &nn, &ctx->bvh_scratch, st,
                                                       &err);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "sphere BVH build: " + err);
            k_gather_spheres<<<(ns + 255) / 256, 256, 0, st>>>(ctx->staging.as<mcrt_gpu_sphere>(),
                                                               ctx->sphere_ids.as<uint32_t>(), ns,
                                                               ctx->spheres.as<mcrt_gpu_sphere>()); ::mcrt::note_launch();
            ctx->n_sphere_nodes = nn;
        }
    }
    // ---- vertices
    CK(ctx->vertices.ensure((size_t)nv * 48), "allocate vertices");
    if (nv)
        CK(cudaMemcpyAsync(ctx->vertices.p, dev_vertices ? dev_vertices : (const void *)d->vertices,
                           (size_t)nv * 48, dev_vertices ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st),
           "upload");
    ctx->n_vertices = nv;
    // ---- triangles (kept in original order on the device) and the mesh BVH
    CK(ctx->triangles.ensure((size_t)nt * 16), "allocate triangles");
    CK(ctx->tri_order.ensure((size_t)nt * 4), "allocate triangle order");
    CK(ctx->mesh_nodes.ensure((size_t)2 * nt * 48), "allocate mesh nodes");
    ctx->n_triangles = nt;
    ctx->n_mesh_nodes = 0;
    if (nt) {
        if (d->mesh_bvh) {
            CK(ctx->staging.ensure((size_t)nt * 16), "allocate staging");
            CK(cudaMemcpyAsync(ctx->staging.p, d->triangles, (size_t)nt * 16, cudaMemcpyHostToDevice, st), "upload");
            if (d->triangle_order)
                CK(cudaMemcpyAsync(ctx->tri_order.p, d->triangle_order, (size_t)nt * 4, cudaMemcpyHostToDevice, st),
                   "upload");
            else
                k_iota<<<(nt + 255) / 256, 256, 0, st>>>(ctx->tri_order.as<uint32_t>(), nt); ::mcrt::note_launch();
            k_scatter_tris<<<(nt + 255) / 256, 256, 0, st>>>(ctx->staging.as<mcrt_gpu_triangle>(),
                                                             ctx->tri_order.as<uint32_t>(), nt,
                                                             ctx->triangles.as<mcrt_gpu_triangle>()); ::mcrt::note_launch();
            CK(cudaMemcpyAsync(ctx->mesh_nodes.p, d->mesh_bvh, (size_t)d->n_mesh_nodes * 48, cudaMemcpyHostToDevice,
                               st), "upload");
            ctx->n_mesh_nodes = d->n_mesh_nodes;
            mcrt_status s = finish_mesh(ctx);
            if (s != MCRT_OK) return s;
        } else {
            CK(cudaMemcpyAsync(ctx->triangles.p, dev_triangles ? dev_triangles : (const void *)d->triangles,
                               (size_t)nt * 16, dev_triangles ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st),
               "upload");
            mcrt_status s = build_mesh_bvh_gpu(ctx);
            if (s != MCRT_OK) return s;
        }
    } else {
        ctx->n_cnodes = 0;
    }
    // ---- albedo texture array (binding 10)
    {
        uint32_t layers = d->albedo_rgba8 ? d->albedo_layers : MCRT_TEXTURE_LAYERS;
        uint32_t size = d->albedo_rgba8 ? d->albedo_size : MCRT_TEXTURE_SIZE;
        if (layers == 0 || size == 0 || (uint64_t)layers * size * size > (1ull << 28))
            return fail(ctx, MCRT_ERR_INVALID_ARG, "invalid albedo texture array size");
        size_t bytes = (size_t)layers * size * size * 4;
        CK(ctx->albedo.ensure(bytes + 1024), "allocate albedo array");
        std::vector<float> lut(256);
        for (int i = 0; i < 256; ++i) {
            double c = i / 255.0;
            lut[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
        }
        CK(cudaMemcpyAsync(ctx->albedo.as<char>() + bytes, lut.data(), 1024, cudaMemcpyHostToDevice, st), "upload");
        if (d->albedo_rgba8) {
            CK(cudaMemcpyAsync(ctx->albedo.p, d->albedo_rgba8, bytes, cudaMemcpyHostToDevice, st), "upload");
        } else {
            std::vector<uint8_t> def(bytes);
            mcrt_albedo_layers(def.data());
            CK(cudaMemcpyAsync(ctx->albedo.p, def.data(), bytes, cudaMemcpyHostToDevice, st), "upload");
        }
        CK(cudaStreamSynchronize(st), "upload");
        ctx->srgb_lut_offset = bytes;
        ctx->albedo_layers = layers;
        ctx->albedo_size = size;
    }
    // ---- materials, environment
    std::memcpy(&ctx->host_materials, d->materials, sizeof(mcrt_gpu_material_data));
    CK(ctx->materials.ensure(sizeof(mcrt_gpu_material_data)), "allocate materials");
    CK(cudaMemcpyAsync(ctx->materials.p, d->materials, sizeof(mcrt_gpu_material_data), cudaMemcpyHostToDevice, st),
       "upload");
    ctx->env_w = d->env_w;
    ctx->env_h = d->env_h;
    CK(ctx->env.ensure((size_t)d->env_w * d->env_h * 16), "allocate env map");
    if (d->env_w)
        CK(cudaMemcpyAsync(ctx->env.p, d->env_rgba, (size_t)d->env_w * d->env_h * 16, cudaMemcpyHostToDevice, st),
           "upload");
    // ---- lights: emissive triangles by original id (device flag + scan), then
    //      emissive spheres by ordered slot
    auto emissive = [&](uint32_t mat) {
        const mcrt_gpu_material &m = d->materials->materials[std::min(mat & 0x7fffffffu, 63u)];
        return m.type_pad[0] == MCRT_MAT_EMISSIVE;
    };
    std::vector<uint32_t> sphere_lights;
    if (ns) {
        std::vector<mcrt_gpu_sphere> ordered(ns);
        CK(cudaMemcpyAsync(ordered.data(), ctx->spheres.p, (size_t)ns * 32, cudaMemcpyDeviceToHost, st),
           "read spheres");
        CK(cudaStreamSynchronize(st), "sync");
        for (uint32_t s = 0; s < ns; ++s)
            if (emissive(ordered[s].mat_and_pad[0])) sphere_lights.push_back(s | MCRT_HIT_SPHERE);
    }
    uint32_t n_tri_lights = 0;
    uint32_t *lflags = nullptr, *lpos = nullptr;
    if (nt) {
        const size_t sw = mcrt::scan_tmp_words(nt + 1);
        CK(ctx->tmp.ensure((2 * ((size_t)nt + 1) + sw) * 4), "allocate scratch");
        lflags = ctx->tmp.as<uint32_t>();
        lpos = lflags + nt + 1;
        k_emissive_flags<<<(nt + 256) / 256, 256, 0, st>>>(ctx->triangles.as<mcrt_gpu_triangle>(), nt,
                                                          ctx->materials.as<mcrt_gpu_material_data>(), lflags);
        ::mcrt::note_launch();
        mcrt::exclusive_scan_u32(lflags, lpos, nt + 1, lpos + nt + 1, st);
        CK(cudaMemcpyAsync(&n_tri_lights, lpos + nt, 4, cudaMemcpyDeviceToHost, st), "count lights");
        CK(cudaStreamSynchronize(st), "count lights");
    }
    ctx->n_lights = n_tri_lights + (uint32_t)sphere_lights.size();
    CK(ctx->lights.ensure((size_t)ctx->n_lights * 4), "allocate lights");
    if (n_tri_lights) {
        k_emissive_scatter<<<(nt + 255) / 256, 256, 0, st>>>(lflags, lpos, nt, ctx->lights.as<uint32_t>());
        ::mcrt::note_launch();
    }
    if (!sphere_lights.empty())
        CK(cudaMemcpyAsync(ctx->lights.as<uint32_t>() + n_tri_lights, sphere_lights.data(), sphere_lights.size() * 4,
                           cudaMemcpyHostToDevice, st),
           "upload");
    // ---- directional light
    ctx->has_sun = d->sun_irradiance[0] > 0.0f || d->sun_irradiance[1] > 0.0f || d->sun_irradiance[2] > 0.0f;
    if (ctx->has_sun) {
        const double len = std::sqrt((double)d->sun_dir[0] * d->sun_dir[0] + (double)d->sun_dir[1] * d->sun_dir[1] +
                                     (double)d->sun_dir[2] * d->sun_dir[2]);
        if (!(len > 0.0)) return fail(ctx, MCRT_ERR_INVALID_ARG, "sun direction is zero");
        for (int k = 0; k < 3; ++k) {
            ctx->sun_dir[k] = (float)(d->sun_dir[k] / len);
            ctx->sun_E[k] = d->sun_irradiance[k];
        }
    }
    mcrt_status s = finish_lights(ctx);
    if (s != MCRT_OK) return s;
    CK(cudaStreamSynchronize(st), "scene upload");
    ctx->has_scene = true;
    return MCRT_OK;
}

mcrt_status mcrt_update_vertices(mcrt_ctx *ctx, const mcrt_gpu_vertex *vertices, uint32_t n_vertices) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!ctx->has_scene) return fail(ctx, MCRT_ERR_NO_SCENE, "no scene uploaded");
    if (n_vertices != ctx->n_vertices || (n_vertices && !vertices))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "vertex count differs from the uploaded scene");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    ctx->acc_valid = false;
    if (n_vertices)
        CK(cudaMemcpyAsync(ctx->vertices.p, vertices, (size_t)n_vertices * 48, cudaMemcpyHostToDevice, ctx->stream),
           "upload vertices");
    if (ctx->n_triangles) {
        mcrt_status s = build_mesh_bvh_gpu(ctx);
        if (s != MCRT_OK) return s;
    }
    return finish_lights(ctx);
}

mcrt_status mcrt_get_mesh_bvh(mcrt_ctx *ctx, mcrt_gpu_bvh_node *out_nodes, uint32_t capacity, uint32_t *out_n_nodes,
                              uint32_t *out_order) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!ctx->has_scene) return fail(ctx, MCRT_ERR_NO_SCENE, "no scene uploaded");
    if (out_n_nodes) *out_n_nodes = ctx->n_mesh_nodes;
    if (out_nodes) {
        if (capacity < ctx->n_mesh_nodes) return fail(ctx, MCRT_ERR_INVALID_ARG, "capacity too small");
        CK(cudaMemcpyAsync(out_nodes, ctx->mesh_nodes.p, (size_t)ctx->n_mesh_nodes * 48, cudaMemcpyDeviceToHost,
                           ctx->stream), "read nodes");
    }
    if (out_order && ctx->n_triangles)
        CK(cudaMemcpyAsync(out_order, ctx->tri_order.p, (size_t)ctx->n_triangles * 4, cudaMemcpyDeviceToHost,
                           ctx->stream), "read order");
    CK(cudaStreamSynchronize(ctx->stream), "read BVH");
    return MCRT_OK;
}

mcrt_status mcrt_trace_closest(mcrt_ctx *ctx, const mcrt_ray *rays, uint32_t n, mcrt_hit *hits, uint32_t flags) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!ctx->has_scene) return fail(ctx, MCRT_ERR_NO_SCENE, "no scene uploaded");
    if (n && (!rays || !hits)) return fail(ctx, MCRT_ERR_INVALID_ARG, "rays or hits is NULL");
    for (uint32_t i = 0; i < n; ++i)
        if (!(rays[i].tmin > 0.0f)) return fail(ctx, MCRT_ERR_INVALID_ARG, "ray.tmin must be > 0");
    if (n == 0) return MCRT_OK;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    CK(ctx->io_a.ensure((size_t)n * 32), "allocate rays");
    CK(ctx->io_b.ensure((size_t)n * 16), "allocate hits");
    CK(cudaMemcpyAsync(ctx->io_a.p, rays, (size_t)n * 32, cudaMemcpyHostToDevice, st), "upload rays");
    mcrt::DeviceScene S = device_scene(ctx);
    mcrt::launch_trace_closest(S, ctx->io_a.as<mcrt_ray>(), n, ctx->io_b.as<mcrt_hit>(),
                               (flags & MCRT_TRACE_REFERENCE_LAYOUT) != 0, st);
    CK(cudaGetLastError(), "trace launch");
    CK(cudaMemcpyAsync(hits, ctx->io_b.p, (size_t)n * 16, cudaMemcpyDeviceToHost, st), "read hits");
    CK(cudaStreamSynchronize(st), "trace");
    return MCRT_OK;
}

__global__ void k_pass_advance(uint32_t *pass_state, uint32_t spp_pass) {
    pass_state[0] += spp_pass;
    pass_state[1] = 1u;
}

// One render call: frames first_frame .. first_frame+spp-1 of a single w x h
// view (views == NULL) or of n_views views traced together, their pixels
// concatenated (the accumulation is then a flat row of all pixels).
static mcrt_status render_core(mcrt_ctx *ctx, const mcrt_camera_uniform *cam, uint32_t w, uint32_t h,
                               const mcrt_view *views, uint32_t n_views, uint32_t spp, uint32_t first_frame,
                               const mcrt_render_opts *opts) {
    if (!ctx->has_scene) return fail(ctx, MCRT_ERR_NO_SCENE, "no scene uploaded");
    if (spp == 0) return fail(ctx, MCRT_ERR_INVALID_ARG, "spp must be > 0");
    uint64_t total = 0;
    if (views) {
        if (n_views == 0 || n_views > 4096) return fail(ctx, MCRT_ERR_INVALID_ARG, "n_views must be in [1, 4096]");
        for (uint32_t v = 0; v < n_views; ++v) {
            if (views[v].width == 0 || views[v].height == 0)
                return fail(ctx, MCRT_ERR_INVALID_ARG, "view " + std::to_string(v) + " has a zero size");
            total += (uint64_t)views[v].width * views[v].height;
        }
    } else {
        if (!cam) return fail(ctx, MCRT_ERR_INVALID_ARG, "cam is NULL");
        if (w == 0 || h == 0) return fail(ctx, MCRT_ERR_INVALID_ARG, "width and height must be > 0");
        total = (uint64_t)w * h;
    }
    if (total > (1ull << 26)) return fail(ctx, MCRT_ERR_INVALID_ARG, "image too large (max 2^26 pixels)");
    mcrt_render_opts o{};
    if (opts) o = *opts;
    const uint32_t depth = o.max_depth ? o.max_depth : mcrt::kDefaultBounces;
    if (depth > 1024) return fail(ctx, MCRT_ERR_INVALID_ARG, "max_depth too large");
    const uint32_t npix = (uint32_t)total;
    if (views) {
        w = npix;
        h = 1;
    }
    const bool keep = (o.flags & MCRT_RENDER_KEEP_ACCUM) != 0;
    if (keep && (!ctx->acc_valid || ctx->acc_w != w || ctx->acc_h != h))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "KEEP_ACCUM needs a previous render of the same size");
    // samples traced at once: enough paths in flight that each closest-hit
    // launch's tail (the last, longest traversals, while most SMs idle) is a
    // small part of it — a 1080p frame of 16 spp traces 1.45x faster as one
    // pass of 16 sample planes than as 8 passes of 2, with the same result —
    // with bounded memory (196 B of path state per slot: 6.6 GB at 2^25 slots)
    const uint64_t kTargetSlots = 1ull << 25, kMaxSlots = 1ull << 25;
    uint32_t spp_pass = o.spp_per_pass;
    if (spp_pass == 0) spp_pass = (uint32_t)std::max<uint64_t>(1, (kTargetSlots + npix - 1) / npix);
    spp_pass = std::min(spp_pass, spp);
    spp_pass = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(spp_pass, kMaxSlots / npix));
    const uint32_t n_slots = npix * spp_pass;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    // ---- buffers
    {
        mcrt_status bs = ensure_path_buffers(ctx, n_slots);
        if (bs != MCRT_OK) return bs;
    }
    if (!keep || ctx->acc_w != w || ctx->acc_h != h) {
        CK(ctx->mean.ensure((size_t)npix * 16), "allocate accumulation");
        CK(ctx->sum.ensure((size_t)npix * 24), "allocate accumulation");
        CK(ctx->gbuf.ensure((size_t)npix * 16), "allocate G-buffer");
        ctx->acc_w = w;
        ctx->acc_h = h;
    }
    CK(cudaMemsetAsync(ctx->counters.p, 0, 256, st), "clear counters");
    int variant = 0;
    {
        mcrt_status vs = render_variant(ctx, o, &variant);
        if (vs != MCRT_OK) return vs;
    }
    mcrt::DeviceScene S = device_scene(ctx);
    const bool want_gbuf = true;
    // ---- view tables: pixel prefix sums, sizes, cameras
    if (views) {
        const size_t off_px = 0, off_wh = ((size_t)(n_views + 1) * 4 + 15) / 16 * 16,
                     off_cam = off_wh + ((size_t)n_views * 8 + 15) / 16 * 16;
        std::vector<char> blob(off_cam + (size_t)n_views * sizeof(mcrt_camera_uniform));
        uint32_t *px = reinterpret_cast<uint32_t *>(blob.data() + off_px);
        uint32_t acc = 0;
        for (uint32_t v = 0; v < n_views; ++v) {
            px[v] = acc;
            acc += views[v].width * views[v].height;
            reinterpret_cast<uint32_t *>(blob.data() + off_wh)[2 * v] = views[v].width;
            reinterpret_cast<uint32_t *>(blob.data() + off_wh)[2 * v + 1] = views[v].height;
            std::memcpy(blob.data() + off_cam + (size_t)v * sizeof(mcrt_camera_uniform), &views[v].cam,
                        sizeof(mcrt_camera_uniform));
        }
        px[n_views] = acc;
        if (ctx->view_blob != blob) {
            CK(ctx->views.ensure(blob.size()), "allocate view table");
            CK(cudaMemcpyAsync(ctx->views.p, blob.data(), blob.size(), cudaMemcpyHostToDevice, st), "upload views");
            CK(cudaStreamSynchronize(st), "upload views");
            ctx->view_blob = blob;
        }
        ctx->view_px.assign(px, px + n_views + 1);
    }
    // ---- passes
    const unsigned long long launches0 = mcrt::launch_count();
    unsigned long long extend_launches = 0;
    size_t evi = 2;
    std::vector<std::pair<size_t, int>> marks;   // (event index, category)
    cudaEvent_t e_begin = ev(ctx, evi++);
    cudaEventRecord(e_begin, st);
    const bool nee = (o.flags & MCRT_RENDER_NEE) != 0 && (ctx->n_lights > 0 || ctx->has_sun);
    const bool use_cache = (o.flags & MCRT_RENDER_CACHE) != 0;
    if (use_cache && !ctx->cache_cfg_set) return fail(ctx, MCRT_ERR_INVALID_ARG, "radiance cache not configured");
    const bool use_graph = (o.flags & MCRT_RENDER_GRAPH) != 0;
    const uint32_t train_stride = use_cache ? ctx->cache_cfg.train_stride : 1u;
    // fallback to the plain tracer while the judged bias is too large: no path
    // stops (no vertex index matches), the training paths still record
    const bool cache_stops = use_cache && !ctx->cache_fallback;
    if (use_cache) {
        const size_t n_train = (n_slots + train_stride - 1) / train_stride;
        CK(ctx->cache_q.ensure((size_t)n_slots * 64), "allocate cache queries");
        CK(ctx->cache_rec.ensure(n_train * depth * mcrt::kTrainRecordFloat4 * 16), "allocate training records");
        // every buffer of a pass's training is allocated here, not in the passes (which a graph may capture)
        CK(mcrt::cache_prepare(ctx->cache, n_train * depth, ctx->cache_cfg.train_batch), "cache buffers");
        CK(mcrt::cache_judge_reset(ctx->cache, st), "bias judge");
    }
    ctx->last_train_samples = 0;
    auto make_params = [&](uint32_t planes, uint32_t frame0) {
        mcrt::RenderParams P{};
        P.w = w; P.h = h; P.npix = npix;
        P.spp_pass = planes;
        P.frame0 = frame0;
        P.max_depth = depth;
        P.flags = o.flags;
        if (cam) P.cam = *cam;
        P.extend_variant = variant;
        if (views) {
            const size_t off_wh = ((size_t)(n_views + 1) * 4 + 15) / 16 * 16,
                         off_cam = off_wh + ((size_t)n_views * 8 + 15) / 16 * 16;
            P.n_views = n_views;
            P.view_px = ctx->views.as<uint32_t>();
            P.view_wh = reinterpret_cast<const uint2 *>(ctx->views.as<char>() + off_wh);
            P.view_cam = reinterpret_cast<const mcrt_camera_uniform *>(ctx->views.as<char>() + off_cam);
        }
        if (use_cache) {
            P.cache_query_vertex = cache_stops ? ctx->cache_cfg.query_vertex + 1 : 0xffffffffu;
            P.train_stride = train_stride;
            P.cache_queries = ctx->cache_q.as<float4>();
            P.train_records = ctx->cache_rec.as<float4>();
        }
        return P;
    };
    mcrt_status cache_status = MCRT_OK;
    // one pass: raygen, the bounces, resolve (into the accumulation)
    auto enqueue_pass = [&](const mcrt::RenderParams &P, bool keep_pass, bool timed) {
        mcrt::launch_raygen(S, P, ctx->pb, st);
        int qi = 0;
        for (uint32_t b = 0; b < depth; ++b) {
            size_t a0 = 0, a1 = 0, a2 = 0;
            if (timed) { a0 = evi++; cudaEventRecord(ev(ctx, a0), st); }
            mcrt::launch_extend(S, P, ctx->pb, qi, st, b == 0);
            ++extend_launches;
            if (timed) { a1 = evi++; cudaEventRecord(ev(ctx, a1), st); }
            mcrt::launch_shade(S, P, ctx->pb, qi, b, ctx->gbuf.as<float4>(), st);
            if (timed) {
                a2 = evi++;
                cudaEventRecord(ev(ctx, a2), st);
                marks.push_back({a0, 1});
                marks.push_back({a1, 2});
            }
            if (nee) {
                mcrt::launch_shadow(S, P, ctx->pb, st);
                if (timed) {
                    size_t a3 = evi++;
                    cudaEventRecord(ev(ctx, a3), st);
                    marks.push_back({a2, 3});
                }
            }
            qi ^= 1;
        }
        if (use_cache) {                              // the terminated paths take the cache's prediction
            cudaError_t e = mcrt::cache_infer_device(ctx->cache, ctx->cache_q.as<float4>(), ctx->pb.counters + 6,
                                                     P.npix * P.spp_pass, nullptr, ctx->pb.L, ctx->pb.thr, st);
            if (e != cudaSuccess) cache_status = cuda_fail(ctx, e, "cache inference");
        }
        size_t r0 = 0;
        if (timed) { r0 = evi++; cudaEventRecord(ev(ctx, r0), st); }
        mcrt::launch_resolve(P, ctx->pb, ctx->mean.as<float4>(), ctx->sum.as<double>(), keep_pass, st);
        if (timed) {
            cudaEventRecord(ev(ctx, evi++), st);
            marks.push_back({r0, 4});
        }
        if (use_cache && cache_status == MCRT_OK) {   // train on this pass's training paths
            const mcrt_cache_params &c = ctx->cache_cfg;
            const uint32_t n_train = (P.npix * P.spp_pass + train_stride - 1) / train_stride;
            cudaError_t e = mcrt::cache_train_records(ctx->cache, ctx->cache_rec.as<float4>(), n_train, depth,
                                                      train_stride, ctx->pb.L, c.train_steps, c.train_batch, c.lr,
                                                      st);
            if (e != cudaSuccess) cache_status = cuda_fail(ctx, e, "cache training");
        }
    };
    uint32_t done = 0;
    bool first_pass = true;
    // ---- CUDA-graph replay of the full passes: the pass is captured once (per
    //      configuration) with its frame index and keep flag in device memory;
    //      a last kernel of the graph advances them for the next replay.
    const uint32_t full_passes = use_graph ? spp / spp_pass : 0;
    if (full_passes > 0) {
        CK(ctx->pass_state.ensure(16), "allocate pass state");
        mcrt::RenderParams P = make_params(spp_pass, 0);
        P.gbuf_plane = want_gbuf ? (int)spp_pass - 1 : -1;
        P.pass_state = ctx->pass_state.as<uint32_t>();
        // configuration key: everything the captured launches bake in
        // (with the cache: its settings and buffers, which the captured training bakes in)
        const void *cbufs[12] = {};
        mcrt_cache_params ccfg{};
        if (use_cache) {
            mcrt::cache_buffer_ptrs(ctx->cache, cbufs);
            ccfg = ctx->cache_cfg;
        }
        std::vector<char> key(sizeof(S) + sizeof(P) + sizeof(mcrt::PathBuffers) + 3 * sizeof(void *) + 8 +
                              sizeof(cbufs) + sizeof(ccfg));
        {
            char *k = key.data();
            std::memcpy(k, &S, sizeof(S)); k += sizeof(S);
            std::memcpy(k, &P, sizeof(P)); k += sizeof(P);
            std::memcpy(k, &ctx->pb, sizeof(mcrt::PathBuffers)); k += sizeof(mcrt::PathBuffers);
            void *bufs[3] = {ctx->mean.p, ctx->sum.p, ctx->gbuf.p};
            std::memcpy(k, bufs, sizeof(bufs)); k += sizeof(bufs);
            uint32_t extra[2] = {depth, nee ? 1u : 0u};
            std::memcpy(k, extra, sizeof(extra)); k += sizeof(extra);
            std::memcpy(k, cbufs, sizeof(cbufs)); k += sizeof(cbufs);
            std::memcpy(k, &ccfg, sizeof(ccfg));
        }
        if (!ctx->graph_exec || ctx->graph_key != key) {
            if (ctx->graph_exec) { cudaGraphExecDestroy(ctx->graph_exec); ctx->graph_exec = nullptr; }
            mcrt::prepare_extend_variants();   // occupancy queries outside the capture
            cudaGraph_t graph = nullptr;
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
            enqueue_pass(P, false, false);
            k_pass_advance<<<1, 1, 0, st>>>(ctx->pass_state.as<uint32_t>(), spp_pass);
            ::mcrt::note_launch();
            cudaError_t ce = cudaStreamEndCapture(st, &graph);
            if (ce != cudaSuccess) return cuda_fail(ctx, ce, "capture render pass");
            ce = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
            cudaGraphDestroy(graph);
            if (ce != cudaSuccess) { ctx->graph_exec = nullptr; return cuda_fail(ctx, ce, "instantiate graph"); }
            ctx->graph_key = key;
            ++ctx->graph_captures;
        }
        const uint32_t init[2] = {first_frame, keep ? 1u : 0u};
        CK(cudaMemcpyAsync(ctx->pass_state.p, init, 8, cudaMemcpyHostToDevice, st), "pass state");
        for (uint32_t k = 0; k < full_passes; ++k) {
            CK(cudaGraphLaunch(ctx->graph_exec, st), "graph launch");
            ::mcrt::note_launch();
        }
        CK(cudaStreamSynchronize(st), "graph passes");   // the pass state copy above reads host memory
        done = full_passes * spp_pass;
        first_pass = false;
    }
    while (done < spp) {
        mcrt::RenderParams P = make_params(std::min(spp_pass, spp - done), first_frame + done);
        const bool last_pass = done + P.spp_pass >= spp;
        P.gbuf_plane = (want_gbuf && last_pass) ? (int)P.spp_pass - 1 : -1;
        enqueue_pass(P, keep || !first_pass, true);
        done += P.spp_pass;
        first_pass = false;
    }
    cudaEvent_t e_end = ev(ctx, evi++);
    cudaEventRecord(e_end, st);
    CK(cudaGetLastError(), "render launch");
    CK(cudaEventSynchronize(e_end), "render");
    if (cache_status != MCRT_OK) return cache_status;
    if (use_cache) {                               // the judge's verdict on this render's passes
        double j[8];
        CK(mcrt::cache_judge_read(ctx->cache, j, st), "bias judge");
        bool over = false;
        for (int c = 0; c < 3; ++c) {
            ctx->cache_stats[c] = j[3 + c] > 0.0 ? j[c] / j[3 + c] : NAN;
            over = over || !(std::fabs(ctx->cache_stats[c]) <= (double)ctx->cache_cfg.max_bias);
        }
        ctx->cache_stats[3] = j[6];
        ctx->cache_stats[4] = cache_stops ? 1.0 : 0.0;
        ctx->last_train_samples = (uint32_t)std::min(j[6], 4294967295.0);
        if (j[6] > 0.0) ctx->cache_fallback = ctx->cache_cfg.max_bias > 0.0f && over;
    }
    ctx->last_render_launches = mcrt::launch_count() - launches0;
    ctx->last_extend_launches = extend_launches;
    ctx->acc_valid = true;
    ctx->gbuf_valid = want_gbuf;
    // ---- timings
    float ms[6] = {0, 0, 0, 0, 0, ctx->last_build_ms};
    cudaEventElapsedTime(&ms[0], e_begin, e_end);
    for (auto &m : marks) {
        float t = 0.0f;
        cudaEventElapsedTime(&t, ev(ctx, m.first), ev(ctx, m.first + 1));
        ms[m.second] += t;
    }
    std::memcpy(ctx->last_ms, ms, sizeof(ms));
    CK(cudaMemcpy(ctx->last_counts, ctx->pb.stats, sizeof(ctx->last_counts), cudaMemcpyDeviceToHost),
       "read counters");
    return MCRT_OK;
}

mcrt_status mcrt_render(mcrt_ctx *ctx, const mcrt_camera_uniform *cam, uint32_t w, uint32_t h, uint32_t spp,
                        uint32_t first_frame, const mcrt_render_opts *opts, float *out_rgba, double *accum_rgb,
                        float *out_gbuf) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    mcrt_status s = render_core(ctx, cam, w, h, nullptr, 0, spp, first_frame, opts);
    if (s != MCRT_OK) return s;
    cudaStream_t st = ctx->stream;
    const uint32_t npix = w * h;
    // ---- outputs
    if (out_rgba)
        CK(cudaMemcpyAsync(out_rgba, ctx->mean.p, (size_t)npix * 16, cudaMemcpyDeviceToHost, st), "read image");
    if (accum_rgb) {
        std::vector<double> tmp((size_t)npix * 3);
        CK(cudaMemcpyAsync(tmp.data(), ctx->sum.p, (size_t)npix * 24, cudaMemcpyDeviceToHost, st), "read sums");
        CK(cudaStreamSynchronize(st), "read sums");
        for (size_t i = 0; i < tmp.size(); ++i) accum_rgb[i] += tmp[i];
    }
    if (out_gbuf)
        CK(cudaMemcpyAsync(out_gbuf, ctx->gbuf.p, (size_t)npix * 16, cudaMemcpyDeviceToHost, st), "read G-buffer");
    CK(cudaStreamSynchronize(st), "render outputs");
    return MCRT_OK;
}

mcrt_status mcrt_render_views(mcrt_ctx *ctx, const mcrt_view *views, uint32_t n_views, uint32_t spp,
                              uint32_t first_frame, const mcrt_render_opts *opts, float *const *out_rgba) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!views) return fail(ctx, MCRT_ERR_INVALID_ARG, "views is NULL");
    mcrt_status s = render_core(ctx, nullptr, 0, 0, views, n_views, spp, first_frame, opts);
    if (s != MCRT_OK) return s;
    if (out_rgba)
        for (uint32_t v = 0; v < n_views; ++v)
            if (out_rgba[v])
                CK(cudaMemcpyAsync(out_rgba[v], ctx->mean.as<float4>() + ctx->view_px[v],
                                   (size_t)views[v].width * views[v].height * 16, cudaMemcpyDeviceToHost, ctx->stream),
                   "read view");
    CK(cudaStreamSynchronize(ctx->stream), "render outputs");
    return MCRT_OK;
}

mcrt_status mcrt_update_materials(mcrt_ctx *ctx, const mcrt_gpu_material_data *materials) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!ctx->has_scene) return fail(ctx, MCRT_ERR_NO_SCENE, "no scene uploaded");
    if (!materials) return fail(ctx, MCRT_ERR_INVALID_ARG, "materials is NULL");
    for (int k = 0; k < 64; ++k) {
        const bool was = ctx->host_materials.materials[k].type_pad[0] == MCRT_MAT_EMISSIVE;
        const bool now = materials->materials[k].type_pad[0] == MCRT_MAT_EMISSIVE;
        if (was != now)
            return fail(ctx, MCRT_ERR_INVALID_ARG,
                        "material " + std::to_string(k) + " changes emissive type (upload the scene instead)");
    }
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    std::memcpy(&ctx->host_materials, materials, sizeof(mcrt_gpu_material_data));
    CK(cudaMemcpyAsync(ctx->materials.p, materials, sizeof(mcrt_gpu_material_data), cudaMemcpyHostToDevice,
                       ctx->stream),
       "upload materials");
    // light selection weights depend on the emitted radiance
    mcrt_status s = finish_lights(ctx);
    if (s != MCRT_OK) return s;
    CK(cudaStreamSynchronize(ctx->stream), "update materials");
    return MCRT_OK;
}

mcrt_status mcrt_adjoint(mcrt_ctx *ctx, const mcrt_camera_uniform *cam, uint32_t w, uint32_t h, uint32_t spp,
                         uint32_t first_frame, const mcrt_render_opts *opts, const float *d_image, double *grad,
                         float *out_rgba) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!ctx->has_scene) return fail(ctx, MCRT_ERR_NO_SCENE, "no scene uploaded");
    if (!cam || !d_image || !grad) return fail(ctx, MCRT_ERR_INVALID_ARG, "cam, d_image and grad are required");
    if (w == 0 || h == 0 || spp == 0) return fail(ctx, MCRT_ERR_INVALID_ARG, "width, height and spp must be > 0");
    if ((uint64_t)w * h > (1ull << 26)) return fail(ctx, MCRT_ERR_INVALID_ARG, "image too large (max 2^26 pixels)");
    mcrt_render_opts o{};
    if (opts) o = *opts;
    if (o.flags & MCRT_RENDER_KEEP_ACCUM) return fail(ctx, MCRT_ERR_INVALID_ARG, "KEEP_ACCUM is not supported");
    const uint32_t depth = o.max_depth ? o.max_depth : mcrt::kDefaultBounces;
    if (depth > 1024) return fail(ctx, MCRT_ERR_INVALID_ARG, "max_depth too large");
    const uint32_t npix = w * h;
    const uint64_t kTargetSlots = 1ull << 22, kMaxSlots = 1ull << 24;
    uint32_t spp_pass = o.spp_per_pass;
    if (spp_pass == 0) spp_pass = (uint32_t)std::max<uint64_t>(1, (kTargetSlots + npix - 1) / npix);
    spp_pass = std::min(spp_pass, spp);
    spp_pass = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(spp_pass, kMaxSlots / npix));
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    {
        mcrt_status bs = ensure_path_buffers(ctx, npix * spp_pass);
        if (bs != MCRT_OK) return bs;
    }
    CK(ctx->mean.ensure((size_t)npix * 16), "allocate accumulation");
    CK(ctx->sum.ensure((size_t)npix * 24), "allocate accumulation");
    CK(ctx->gbuf.ensure((size_t)npix * 16), "allocate G-buffer");
    ctx->acc_w = w;
    ctx->acc_h = h;
    CK(ctx->dimg.ensure((size_t)npix * 16), "allocate image gradient");
    CK(ctx->grad.ensure(256 * sizeof(double)), "allocate parameter gradient");
    CK(cudaMemcpyAsync(ctx->dimg.p, d_image, (size_t)npix * 16, cudaMemcpyHostToDevice, st), "upload d_image");
    CK(cudaMemsetAsync(ctx->grad.p, 0, 256 * sizeof(double), st), "clear gradient");
    CK(cudaMemsetAsync(ctx->counters.p, 0, 256, st), "clear counters");
    int variant = 0;
    {
        mcrt_status vs = render_variant(ctx, o, &variant);
        if (vs != MCRT_OK) return vs;
    }
    mcrt::DeviceScene S = device_scene(ctx);
    mcrt::AdjointParams A;
    A.dimg = ctx->dimg.as<float4>();
    A.inv_spp = 1.0f / (float)spp;
    A.grad = ctx->grad.as<double>();
    const bool nee = (o.flags & MCRT_RENDER_NEE) != 0 && (ctx->n_lights > 0 || ctx->has_sun);
    const unsigned long long launches0 = mcrt::launch_count();
    cudaEvent_t e_begin = ev(ctx, 2), e_end = ev(ctx, 3);
    cudaEventRecord(e_begin, st);
    uint32_t done = 0;
    while (done < spp) {
        mcrt::RenderParams P{};
        P.w = w; P.h = h; P.npix = npix;
        P.spp_pass = std::min(spp_pass, spp - done);
        P.frame0 = first_frame + done;
        P.max_depth = depth;
        P.flags = o.flags;
        P.cam = *cam;
        P.gbuf_plane = -1;
        P.extend_variant = variant;
        A.planes = P.spp_pass;
        // primal pass: the per-path radiance of these samples
        mcrt::launch_raygen(S, P, ctx->pb, st);
        int qi = 0;
        for (uint32_t b = 0; b < depth; ++b) {
            mcrt::launch_extend(S, P, ctx->pb, qi, st, b == 0);
            mcrt::launch_shade(S, P, ctx->pb, qi, b, nullptr, st);
            if (nee) mcrt::launch_shadow(S, P, ctx->pb, st);
            qi ^= 1;
        }
        mcrt::launch_resolve(P, ctx->pb, ctx->mean.as<float4>(), ctx->sum.as<double>(), done > 0, st);
        // adjoint pass: replay the same paths from their seeds
        mcrt::launch_raygen(S, P, ctx->pb, st, true);
        qi = 0;
        for (uint32_t b = 0; b < depth; ++b) {
            mcrt::launch_extend(S, P, ctx->pb, qi, st, b == 0);
            mcrt::launch_shade(S, P, ctx->pb, qi, b, nullptr, st, &A);
            if (nee) mcrt::launch_shadow(S, P, ctx->pb, st, &A);
            qi ^= 1;
        }
        done += P.spp_pass;
    }
    cudaEventRecord(e_end, st);
    CK(cudaGetLastError(), "adjoint launch");
    CK(cudaEventSynchronize(e_end), "adjoint");
    ctx->last_render_launches = mcrt::launch_count() - launches0;
    ctx->acc_valid = true;
    ctx->gbuf_valid = false;
    float ms[6] = {0, 0, 0, 0, 0, ctx->last_build_ms};
    cudaEventElapsedTime(&ms[0], e_begin, e_end);
    std::memcpy(ctx->last_ms, ms, sizeof(ms));
    CK(cudaMemcpy(ctx->last_counts, ctx->pb.stats, sizeof(ctx->last_counts), cudaMemcpyDeviceToHost),
       "read counters");
    CK(cudaMemcpy(grad, ctx->grad.p, 256 * sizeof(double), cudaMemcpyDeviceToHost), "read gradient");
    if (out_rgba)
        CK(cudaMemcpy(out_rgba, ctx->mean.p, (size_t)npix * 16, cudaMemcpyDeviceToHost), "read image");
    return MCRT_OK;
}

static mcrt_status check_world_dims(mcrt_ctx *ctx, uint32_t nx, uint32_t ny, uint32_t nz) {
    if (nx == 0 || nz == 0 || nx % 16 || nz % 16)
        return fail(ctx, MCRT_ERR_INVALID_ARG, "world nx and nz must be positive multiples of 16");
    if (ny < 2 || ny > 1024) return fail(ctx, MCRT_ERR_INVALID_ARG, "world ny must be in [2, 1024]");
    if ((uint64_t)nx * ny * nz > (1ull << 32)) return fail(ctx, MCRT_ERR_INVALID_ARG, "world grid too large");
    return MCRT_OK;
}

mcrt_status mcrt_world_generate(mcrt_ctx *ctx, const mcrt_world_params *p, uint8_t *out_voxels) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!p) return fail(ctx, MCRT_ERR_INVALID_ARG, "params is NULL");
    mcrt_status ds = check_world_dims(ctx, p->nx, p->ny, p->nz);
    if (ds != MCRT_OK) return ds;
    if (p->height_octaves == 0 || p->height_octaves > 16 || p->cave_octaves > 16)
        return fail(ctx, MCRT_ERR_INVALID_ARG, "octaves must be in [1, 16] (caves [0, 16])");
    const float fs[] = {p->height_base, p->height_amp, p->height_freq, p->lacunarity, p->gain, p->cave_freq,
                        p->cave_threshold, p->cave_contrast, p->sea_level, p->sand_line};
    for (float f : fs)
        if (!std::isfinite(f)) return fail(ctx, MCRT_ERR_INVALID_ARG, "world parameters must be finite");
    if (std::abs((int64_t)p->chunk_x0) > (1 << 22) || std::abs((int64_t)p->chunk_z0) > (1 << 22))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "chunk coordinates out of range");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t n = (size_t)p->nx * p->ny * p->nz;
    CK(ctx->world_vox.ensure(n), "allocate voxel grid");
    mcrt::launch_world_generate(*p, ctx->world_vox.as<uint8_t>(), ctx->stream);
    CK(cudaGetLastError(), "world generate");
    ctx->world_nx = p->nx; ctx->world_ny = p->ny; ctx->world_nz = p->nz;
    ctx->world_cx0 = p->chunk_x0; ctx->world_cz0 = p->chunk_z0;
    ctx->wmesh_valid = false;
    if (out_voxels) CK(cudaMemcpyAsync(out_voxels, ctx->world_vox.p, n, cudaMemcpyDeviceToHost, ctx->stream), "read");
    CK(cudaStreamSynchronize(ctx->stream), "world generate");
    return MCRT_OK;
}

mcrt_status mcrt_world_upload(mcrt_ctx *ctx, const uint8_t *voxels, uint32_t nx, uint32_t ny, uint32_t nz,
                              int32_t chunk_x0, int32_t chunk_z0) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!voxels) return fail(ctx, MCRT_ERR_INVALID_ARG, "voxels is NULL");
    mcrt_status ds = check_world_dims(ctx, nx, ny, nz);
    if (ds != MCRT_OK) return ds;
    if (std::abs((int64_t)chunk_x0) > (1 << 22) || std::abs((int64_t)chunk_z0) > (1 << 22))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "chunk coordinates out of range");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t n = (size_t)nx * ny * nz;
    CK(ctx->world_vox.ensure(n), "allocate voxel grid");
    CK(cudaMemcpyAsync(ctx->world_vox.p, voxels, n, cudaMemcpyHostToDevice, ctx->stream), "upload voxels");
    CK(cudaStreamSynchronize(ctx->stream), "upload voxels");
    ctx->world_nx = nx; ctx->world_ny = ny; ctx->world_nz = nz;
    ctx->world_cx0 = chunk_x0; ctx->world_cz0 = chunk_z0;
    ctx->wmesh_valid = false;
    return MCRT_OK;
}

mcrt_status mcrt_world_mesh(mcrt_ctx *ctx, uint32_t mode, const uint32_t *block_material, float voxel_size,
                            uint32_t *out_n_vertices, uint32_t *out_n_triangles) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!ctx->world_nx) return fail(ctx, MCRT_ERR_INVALID_ARG, "no voxel grid (generate or upload one first)");
    if (!block_material) return fail(ctx, MCRT_ERR_INVALID_ARG, "block_material is NULL");
    if (mode != MCRT_MESH_GREEDY && mode != MCRT_MESH_FACES) return fail(ctx, MCRT_ERR_INVALID_ARG, "unknown mode");
    if (!(voxel_size > 0.0f) || !std::isfinite(voxel_size))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "voxel_size must be positive");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    CK(ctx->world_matmap.ensure(256 * 4), "allocate material map");
    CK(cudaMemcpyAsync(ctx->world_matmap.p, block_material, 256 * 4, cudaMemcpyHostToDevice, st), "upload map");
    ctx->wmesh_valid = false;
    cudaError_t e = mcrt::world_mesh(ctx->world_vox.as<uint8_t>(), ctx->world_nx, ctx->world_ny, ctx->world_nz,
                                     ctx->world_cx0, ctx->world_cz0, mode == MCRT_MESH_GREEDY,
                                     ctx->world_matmap.as<uint32_t>(), voxel_size, ctx->wmesh, st);
    if (e == cudaErrorInvalidValue) return fail(ctx, MCRT_ERR_INVALID_ARG, "world mesh too large for the tracer");
    if (e != cudaSuccess) return cuda_fail(ctx, e, "world mesh");
    CK(cudaStreamSynchronize(st), "world mesh");
    ctx->wmesh_valid = true;
    if (out_n_vertices) *out_n_vertices = 4 * ctx->wmesh.n_quads;
    if (out_n_triangles) *out_n_triangles = 2 * ctx->wmesh.n_quads;
    return MCRT_OK;
}

mcrt_status mcrt_world_read_mesh(mcrt_ctx *ctx, mcrt_gpu_vertex *vertices, uint32_t vertex_capacity,
                                 mcrt_gpu_triangle *triangles, uint32_t triangle_capacity) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!ctx->wmesh_valid) return fail(ctx, MCRT_ERR_INVALID_ARG, "no world mesh");
    const uint32_t nv = 4 * ctx->wmesh.n_quads, nt = 2 * ctx->wmesh.n_quads;
    if ((vertices && vertex_capacity < nv) || (triangles && triangle_capacity < nt))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "capacity too small");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (vertices && nv)
        CK(cudaMemcpy(vertices, ctx->wmesh.vertices.p, (size_t)nv * sizeof(mcrt_gpu_vertex), cudaMemcpyDeviceToHost),
           "read vertices");
    if (triangles && nt)
        CK(cudaMemcpy(triangles, ctx->wmesh.triangles.p, (size_t)nt * sizeof(mcrt_gpu_triangle),
                      cudaMemcpyDeviceToHost),
           "read triangles");
    return MCRT_OK;
}

// ---------------------------------------------------------------- scene ingestion on the device

mcrt_status mcrt_mesh_reset(mcrt_ctx *ctx) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    ctx->dmesh.nv = ctx->dmesh.nt = 0;
    return MCRT_OK;
}

mcrt_status mcrt_mesh_append(mcrt_ctx *ctx, const mcrt_gpu_vertex *vertices, uint32_t n_vertices,
                             const mcrt_gpu_triangle *triangles, uint32_t n_triangles) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if ((n_vertices && !vertices) || (n_triangles && !triangles))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "vertices or triangles is NULL");
    for (uint32_t i = 0; i < n_triangles; ++i)
        for (int k = 0; k < 3; ++k)
            if (triangles[i].v[k] >= n_vertices)
                return fail(ctx, MCRT_ERR_INVALID_ARG,
                            "triangle " + std::to_string(i) + " references a vertex beyond n_vertices");
    if ((uint64_t)ctx->dmesh.nv + n_vertices >= (1ull << 31) || (uint64_t)ctx->dmesh.nt + n_triangles >= (1ull << 27))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "device mesh too large");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(mcrt::mesh_append_host(ctx->dmesh, vertices, n_vertices, triangles, n_triangles, ctx->obj.staging, ctx->stream),
       "append to the device mesh");
    return MCRT_OK;
}

namespace {
// Utf8Error::error_len of the invalid sequence at text[i] (core::str::run_utf8_validation):
// 1-3 bytes, or 0 when the text ends inside the sequence.
int utf8_error_len(const unsigned char *t, unsigned long long len, unsigned long long i) {
    const unsigned char b = t[i];
    auto cont = [](unsigned char x) { return (x & 0xC0) == 0x80; };
    const int w = (b >= 0xC2 && b <= 0xDF) ? 2 : (b >= 0xE0 && b <= 0xEF) ? 3 : (b >= 0xF0 && b <= 0xF4) ? 4 : 0;
    if (w == 0) return 1;
    if (i + 1 >= len) return 0;
    const unsigned char b1 = t[i + 1];
    bool ok = w == 2   ? cont(b1)
              : w == 3 ? (b == 0xE0 && b1 >= 0xA0 && b1 <= 0xBF) || (b >= 0xE1 && b <= 0xEC && cont(b1)) ||
                             (b == 0xED && b1 >= 0x80 && b1 <= 0x9F) || (b >= 0xEE && cont(b1))
                       : (b == 0xF0 && b1 >= 0x90 && b1 <= 0xBF) || (b >= 0xF1 && b <= 0xF3 && cont(b1)) ||
                             (b == 0xF4 && b1 >= 0x80 && b1 <= 0x8F);
    if (!ok) return 1;
    for (int k = 2; k < w; ++k) {
        if (i + k >= len) return 0;
        if (!cont(t[i + k])) return k;
    }
    return 1;   // not reached for a sequence the device check rejected
}
}  // namespace

mcrt_status mcrt_mesh_append_obj(mcrt_ctx *ctx, const char *text, uint64_t len, uint32_t mat_idx,
                                 const mcrt_mesh_transform *xf, const char *source, uint32_t *out_n_vertices,
                                 uint32_t *out_n_triangles) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (len && !text) return fail(ctx, MCRT_ERR_INVALID_ARG, "text is NULL");
    const std::string src = source ? source : "<obj>";
    mcrt::ObjTransform X{};
    X.identity = !xf || (!xf->has_translate && !xf->has_rotate && !xf->has_scale);
    X.s = xf && xf->has_scale ? xf->scale : 1.0f;
    X.has_r = xf && xf->has_rotate;
    for (int k = 0; k < 3; ++k) X.t[k] = xf && xf->has_translate ? xf->translate[k] : 0.0f;
    if (X.has_r) mcrt_host::rotation_matrix(xf->rotate_deg, X.m);
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (ctx->pageable_access < 0)
        CK(cudaDeviceGetAttribute(&ctx->pageable_access, cudaDevAttrPageableMemoryAccess, ctx->device), "attribute");
    // the device reads the host text in place where it can reach pageable
    // memory (coherent systems); MCRT_OBJ_COPY_TEXT=1 copies it first instead
    const char *copy_env = getenv("MCRT_OBJ_COPY_TEXT");
    const bool direct = ctx->pageable_access == 1 && !(copy_env && copy_env[0] == '1');
    const uint32_t nv0 = ctx->dmesh.nv, nt0 = ctx->dmesh.nt;
    mcrt::ObjOutcome r;
    cudaError_t e = mcrt::obj_append(text, len, mat_idx, X, ctx->dmesh, ctx->obj, ctx->stream, direct, &r);
    if (e == cudaErrorInvalidValue)
        return fail(ctx, MCRT_ERR_INVALID_ARG, "OBJ text '" + src + "' is beyond the device parser's limits");
    if (e != cudaSuccess) return cuda_fail(ctx, e, "OBJ parse");
    const std::string head = "mesh load error: failed to load mesh '" + src + "': '" + src + "'";   // scene.rs:835-837
    if (r.code == mcrt::ObjOutcome::kNotUtf8) {                                                        // mesh.rs:477-478
        const int el = utf8_error_len(reinterpret_cast<const unsigned char *>(text), len, r.valid_up_to);
        return fail(ctx, MCRT_ERR_MESH_LOAD,
                    head + " is not valid UTF-8: " +
                        (el ? "invalid utf-8 sequence of " + std::to_string(el) + " bytes from index "
                            : std::string("incomplete utf-8 byte sequence from index ")) +
                        std::to_string(r.valid_up_to));
    }
    if (r.code == mcrt::ObjOutcome::kNoGeometry)                                                       // mesh.rs:636-638
        return fail(ctx, MCRT_ERR_MESH_LOAD, head + ": no geometry found after parsing");
    if (!(X.s > 0.0f)) {                                           // scene.rs:842-847, checked after the load
        ctx->dmesh.nv = nv0;
        ctx->dmesh.nt = nt0;
        return fail(ctx, MCRT_ERR_INVALID_ARG, "mesh '" + src + "' transform.scale must be positive");
    }
    ctx->last_obj_counts[0] = len;
    ctx->last_obj_counts[1] = r.n_lines;
    ctx->last_obj_counts[2] = r.n_tokens;
    ctx->last_obj_counts[3] = r.launches;
    ctx->last_obj_ms[0] = r.h2d_ms;
    ctx->last_obj_ms[1] = r.kernel_ms;
    if (out_n_vertices) *out_n_vertices = r.n_vertices;
    if (out_n_triangles) *out_n_triangles = r.n_triangles;
    return MCRT_OK;
}

mcrt_status mcrt_mesh_obj_stats(mcrt_ctx *ctx, float *out_ms2, uint64_t *out_counts4) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (out_ms2) std::memcpy(out_ms2, ctx->last_obj_ms, sizeof(ctx->last_obj_ms));
    if (out_counts4)
        for (int k = 0; k < 4; ++k) out_counts4[k] = ctx->last_obj_counts[k];
    return MCRT_OK;
}

mcrt_status mcrt_mesh_read(mcrt_ctx *ctx, mcrt_gpu_vertex *vertices, uint32_t vertex_capacity,
                           mcrt_gpu_triangle *triangles, uint32_t triangle_capacity, uint32_t *out_n_vertices,
                           uint32_t *out_n_triangles) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    const uint32_t nv = ctx->dmesh.nv, nt = ctx->dmesh.nt;
    if (out_n_vertices) *out_n_vertices = nv;
    if (out_n_triangles) *out_n_triangles = nt;
    if ((vertices && vertex_capacity < nv) || (triangles && triangle_capacity < nt))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "capacity too small");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (vertices && nv)
        CK(cudaMemcpy(vertices, ctx->dmesh.vertices.p, (size_t)nv * 48, cudaMemcpyDeviceToHost), "read vertices");
    if (triangles && nt)
        CK(cudaMemcpy(triangles, ctx->dmesh.triangles.p, (size_t)nt * 16, cudaMemcpyDeviceToHost), "read triangles");
    return MCRT_OK;
}

mcrt_status mcrt_read_accum(mcrt_ctx *ctx, float *out_rgba, double *accum_rgb, float *out_gbuf) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!ctx->acc_valid) return fail(ctx, MCRT_ERR_INVALID_ARG, "no render to read");
    size_t npix = (size_t)ctx->acc_w * ctx->acc_h;
    cudaStream_t st = ctx->stream;
    if (out_rgba) CK(cudaMemcpyAsync(out_rgba, ctx->mean.p, npix * 16, cudaMemcpyDeviceToHost, st), "read image");
    if (accum_rgb) {
        std::vector<double> tmp(npix * 3);
        CK(cudaMemcpyAsync(tmp.data(), ctx->sum.p, npix * 24, cudaMemcpyDeviceToHost, st), "read sums");
        CK(cudaStreamSynchronize(st), "read sums");
        for (size_t i = 0; i < tmp.size(); ++i) accum_rgb[i] += tmp[i];
    }
    if (out_gbuf && ctx->gbuf_valid)
        CK(cudaMemcpyAsync(out_gbuf, ctx->gbuf.p, npix * 16, cudaMemcpyDeviceToHost, st), "read G-buffer");
    CK(cudaStreamSynchronize(st), "read accumulation");
    return MCRT_OK;
}

mcrt_status mcrt_variant_info(uint32_t variant, uint32_t *out6) {
    if (!out6 || variant >= (uint32_t)mcrt::extend_variant_count())
        return fail(nullptr, MCRT_ERR_INVALID_ARG, "variant out of range or out6 NULL");
    int info[6];
    mcrt::extend_variant_info((int)variant, info);
    for (int k = 0; k < 6; ++k) out6[k] = (uint32_t)info[k];
    return MCRT_OK;
}

mcrt_status mcrt_autotune(mcrt_ctx *ctx, const mcrt_camera_uniform *cam, uint32_t w, uint32_t h, uint32_t spp,
                          const mcrt_render_opts *opts, uint32_t *out_variant, float *out_ms) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    mcrt_render_opts o{};
    if (opts) o = *opts;
    o.flags &= ~(uint32_t)MCRT_RENDER_KEEP_ACCUM;
    const int nv = mcrt::extend_variant_count();
    float best = 0.0f;
    int best_v = -1;
    for (int v = 0; v < nv; ++v) {
        o.variant = (uint32_t)v + 1;
        float t = 0.0f;
        for (int rep = 0; rep < 2; ++rep) {           // the first run warms caches and occupancy queries
            mcrt_status s = mcrt_render(ctx, cam, w, h, spp, 0, &o, nullptr, nullptr, nullptr);
            if (s != MCRT_OK) return s;
            t = ctx->last_ms[1];                      // extend time, stackless retries of a short stack included
        }
        if (out_ms && v < 8) out_ms[v] = t;
        if (best_v < 0 || t < best) { best = t; best_v = v; }
    }
    ctx->extend_variant = best_v;
    if (out_variant) *out_variant = (uint32_t)best_v;
    return MCRT_OK;
}

mcrt_status mcrt_read_image_rgba8(mcrt_ctx *ctx, uint32_t mode, uint8_t *out) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!out) return fail(ctx, MCRT_ERR_INVALID_ARG, "out is NULL");
    if (mode > MCRT_TONEMAP_ACES_SRGB) return fail(ctx, MCRT_ERR_INVALID_ARG, "unknown tone-map mode");
    if (!ctx->acc_valid) return fail(ctx, MCRT_ERR_INVALID_ARG, "no render to read");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const uint32_t npix = ctx->acc_w * ctx->acc_h;
    CK(ctx->io_c.ensure((size_t)npix * 4), "allocate image");
    mcrt::launch_tonemap(ctx->mean.as<float4>(), npix, mode, ctx->io_c.as<uchar4>(), ctx->stream);
    CK(cudaGetLastError(), "tone-map launch");
    CK(cudaMemcpyAsync(out, ctx->io_c.p, (size_t)npix * 4, cudaMemcpyDeviceToHost, ctx->stream), "read image");
    CK(cudaStreamSynchronize(ctx->stream), "tone map");
    return MCRT_OK;
}

// A plain copy, float4 per thread and step, `reps` times in one launch (even
// repetitions a -> b, odd ones b -> a; each thread copies its own elements, so
// repetition r + 1 reads what the same thread wrote in r): the denominator of
// a roofline, with no launch gaps between repetitions.
__global__ void k_copy_float4(float4 *a, float4 *b, size_t n, uint32_t reps) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t r = 0; r < reps; ++r) {
        const float4 *src = (r & 1u) ? b : a;
        float4 *dst = (r & 1u) ? a : b;
        size_t i = i0;
        for (; i + 3 * stride < n; i += 4 * stride) {
            const float4 v0 = src[i], v1 = src[i + stride], v2 = src[i + 2 * stride], v3 = src[i + 3 * stride];
            dst[i] = v0; dst[i + stride] = v1; dst[i + 2 * stride] = v2; dst[i + 3 * stride] = v3;
        }
        for (; i < n; i += stride) dst[i] = src[i];
    }
}

mcrt_status mcrt_copy_bandwidth(mcrt_ctx *ctx, uint64_t bytes, uint32_t reps, float *out_gbs) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!out_gbs || bytes < 16 || reps == 0 || bytes > (1ull << 36))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "out_gbs required, 16 <= bytes <= 2^36, reps > 0");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t n = (size_t)(bytes / 16);
    void *src = nullptr, *dst = nullptr;
    CK(cudaMalloc(&src, n * 16), "allocate copy source");
    cudaError_t e = cudaMalloc(&dst, n * 16);
    if (e != cudaSuccess) { cudaFree(src); return cuda_fail(ctx, e, "allocate copy destination"); }
    cudaStream_t st = ctx->stream;
    cudaMemsetAsync(src, 0, n * 16, st);
    const int blocks = mcrt::sm_count() * 8;
    cudaEvent_t a = ev(ctx, 0), b = ev(ctx, 1);
    float4 *fa = static_cast<float4 *>(src), *fb = static_cast<float4 *>(dst);
    k_copy_float4<<<blocks, 256, 0, st>>>(fa, fb, n, 4);   // warm-up: the buffers resident where they fit
    ::mcrt::note_launch();
    cudaEventRecord(a, st);
    k_copy_float4<<<blocks, 256, 0, st>>>(fa, fb, n, reps);
    ::mcrt::note_launch();
    cudaEventRecord(b, st);
    e = cudaEventSynchronize(b);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    cudaFree(src);
    cudaFree(dst);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "copy bandwidth");
    *out_gbs = (float)(2.0 * (double)n * 16.0 * reps / (ms * 1e-3) / 1e9);
    return MCRT_OK;
}

mcrt_status mcrt_last_timings(mcrt_ctx *ctx, float *out_ms, uint64_t *out_counts) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (out_ms) {
        std::memcpy(out_ms, ctx->last_ms, sizeof(ctx->last_ms));
        out_ms[5] = ctx->last_build_ms;
    }
    if (out_counts) {
        out_counts[0] = ctx->last_counts[0];
        out_counts[1] = ctx->last_counts[1];
        out_counts[2] = ctx->last_render_launches;
        out_counts[3] = ctx->last_build_launches;
        out_counts[4] = ctx->last_extend_launches;
        out_counts[5] = ctx->last_counts[2];
        out_counts[6] = ctx->last_counts[3];
        out_counts[7] = ctx->last_counts[4];
    }
    return MCRT_OK;
}

mcrt_status mcrt_rebuild_bvh(mcrt_ctx *ctx) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!ctx->has_scene) return fail(ctx, MCRT_ERR_NO_SCENE, "no scene uploaded");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    ctx->acc_valid = false;
    if (ctx->n_triangles) {
        mcrt_status s = build_mesh_bvh_gpu(ctx);
        if (s != MCRT_OK) return s;
    }
    return finish_lights(ctx);
}

mcrt_status mcrt_denoise(mcrt_ctx *ctx, const float *in_rgba, const float *gbuf, uint32_t w, uint32_t h,
                         const mcrt_denoise_params *params, float *out_rgba) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!in_rgba || !gbuf || !out_rgba || !params) return fail(ctx, MCRT_ERR_INVALID_ARG, "NULL argument");
    if (w == 0 || h == 0 || (uint64_t)w * h > (1ull << 28)) return fail(ctx, MCRT_ERR_INVALID_ARG, "bad image size");
    if (params->radius < 0 || params->radius > 64) return fail(ctx, MCRT_ERR_INVALID_ARG, "radius must be in [0, 64]");
    if (!(params->sigma_s > 0.0f) || !(params->sigma_d > 0.0f))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "sigma_s and sigma_d must be > 0");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    size_t bytes = (size_t)w * h * 16;
    CK(ctx->io_a.ensure(bytes), "allocate");
    CK(ctx->io_b.ensure(bytes), "allocate");
    CK(ctx->io_c.ensure(bytes), "allocate");
    CK(cudaMemcpyAsync(ctx->io_a.p, in_rgba, bytes, cudaMemcpyHostToDevice, st), "upload");
    CK(cudaMemcpyAsync(ctx->io_b.p, gbuf, bytes, cudaMemcpyHostToDevice, st), "upload");
    cudaEvent_t a = ev(ctx, 0), b = ev(ctx, 1);
    cudaEventRecord(a, st);
    mcrt::launch_denoise(ctx->io_a.as<float4>(), ctx->io_b.as<float4>(), w, h, *params, ctx->io_c.as<float4>(), st);
    cudaEventRecord(b, st);
    CK(cudaGetLastError(), "denoise launch");
    CK(cudaMemcpyAsync(out_rgba, ctx->io_c.p, bytes, cudaMemcpyDeviceToHost, st), "read");
    CK(cudaStreamSynchronize(st), "denoise");
    float t = 0.0f;
    cudaEventElapsedTime(&t, a, b);
    ctx->last_ms[0] = t;
    return MCRT_OK;
}

// ------------------------------------------------------------------ radiance cache
uint32_t mcrt_cache_param_count(void) { return (uint32_t)mcrt::mlp::kParams; }

static mcrt::CacheState *cache_of(mcrt_ctx *ctx) {
    if (!ctx->cache) ctx->cache = mcrt::cache_create();
    return ctx->cache;
}

mcrt_status mcrt_cache_set_params(mcrt_ctx *ctx, const float *params) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!params) return fail(ctx, MCRT_ERR_INVALID_ARG, "params is NULL");
    for (int p = 0; p < mcrt::mlp::kParams; ++p)
        if (!std::isfinite(params[p])) return fail(ctx, MCRT_ERR_INVALID_ARG, "parameters must be finite");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(mcrt::cache_set_params(cache_of(ctx), params, ctx->stream), "cache parameters");
    CK(cudaStreamSynchronize(ctx->stream), "cache parameters");
    return MCRT_OK;
}

mcrt_status mcrt_cache_init(mcrt_ctx *ctx, uint32_t seed) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    // He-uniform weights U(-sqrt(6 / fan_in), +) from a PCG stream, zero biases,
    // output rows 3..15 zero
    std::vector<float> p(mcrt::mlp::kParams, 0.0f);
    uint32_t state = seed * 2654435761u + 12345u;
    for (int l = 0; l < mcrt::mlp::kLayers; ++l) {
        const int nin = mcrt::mlp::in_of(l), nout = mcrt::mlp::out_of(l);
        const double bound = std::sqrt(6.0 / (double)nin);
        for (int o = 0; o < nout; ++o)
            for (int i = 0; i < nin; ++i) {
                state = mcrt::pcg_hash(state);
                const double u = (double)(state >> 8) / 16777216.0;
                const bool live = l < mcrt::mlp::kLayers - 1 || o < mcrt::mlp::kOut;
                p[mcrt::mlp::w_off(l) + o * nin + i] = live ? (float)((2.0 * u - 1.0) * bound) : 0.0f;
            }
    }
    return mcrt_cache_set_params(ctx, p.data());
}

mcrt_status mcrt_cache_get_params(mcrt_ctx *ctx, float *out) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!out) return fail(ctx, MCRT_ERR_INVALID_ARG, "out is NULL");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaError_t e = mcrt::cache_get_params(cache_of(ctx), out, ctx->stream);
    if (e == cudaErrorInvalidValue) return fail(ctx, MCRT_ERR_INVALID_ARG, "cache parameters not set");
    CK(e, "cache parameters");
    return MCRT_OK;
}

mcrt_status mcrt_cache_set_bounds(mcrt_ctx *ctx, const float *lo3, const float *hi3) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!lo3 || !hi3) return fail(ctx, MCRT_ERR_INVALID_ARG, "bounds are NULL");
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(lo3[a]) || !std::isfinite(hi3[a]) || !(hi3[a] > lo3[a]))
            return fail(ctx, MCRT_ERR_INVALID_ARG, "bounds must be finite with hi > lo");
    mcrt::cache_set_bounds(cache_of(ctx), lo3, hi3);
    return MCRT_OK;
}

mcrt_status mcrt_cache_bench(mcrt_ctx *ctx, uint32_t n, uint32_t reps, float *out_ms) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!out_ms || n == 0 || n > (1u << 24) || reps == 0 || reps > 1000)
        return fail(ctx, MCRT_ERR_INVALID_ARG, "out_ms NULL, n out of [1, 2^24] or reps out of [1, 1000]");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    mcrt::CacheState *c = cache_of(ctx);
    if (!mcrt::cache_ready(c)) {
        mcrt_status s = mcrt_cache_init(ctx, 0);
        if (s != MCRT_OK) return s;
    }
    cudaError_t e = mcrt::cache_bench(c, n, reps, &out_ms[0], &out_ms[1], ctx->stream);
    CK(e, "cache benchmark");
    return MCRT_OK;
}

mcrt_status mcrt_cache_config(mcrt_ctx *ctx, const mcrt_cache_params *p) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!p) return fail(ctx, MCRT_ERR_INVALID_ARG, "params is NULL");
    if (p->train_stride == 0) return fail(ctx, MCRT_ERR_INVALID_ARG, "train_stride must be >= 1");
    if (!(p->lr >= 0.0f) || !std::isfinite(p->lr)) return fail(ctx, MCRT_ERR_INVALID_ARG, "lr must be >= 0");
    if (p->query_vertex > 1023) return fail(ctx, MCRT_ERR_INVALID_ARG, "query_vertex too large");
    if (!(p->max_bias >= 0.0f)) return fail(ctx, MCRT_ERR_INVALID_ARG, "max_bias must be >= 0");
    float lo[3], hi[3];
    bool given = true;
    for (int a = 0; a < 3; ++a) {
        if (!std::isfinite(p->lo[a]) || !std::isfinite(p->hi[a]))
            return fail(ctx, MCRT_ERR_INVALID_ARG, "bounds must be finite");
        lo[a] = p->lo[a];
        hi[a] = p->hi[a];
        given = given && hi[a] > lo[a];
    }
    if (!given) {                                  // the scene's bounding box (root nodes of the BVHs)
        if (!ctx->has_scene) return fail(ctx, MCRT_ERR_NO_SCENE, "no scene to take the bounds from");
        CK(cudaSetDevice(ctx->device), "cudaSetDevice");
        for (int a = 0; a < 3; ++a) { lo[a] = INFINITY; hi[a] = -INFINITY; }
        auto take = [&](const DBuf &nodes, uint32_t n) -> cudaError_t {
            if (n == 0) return cudaSuccess;
            mcrt_gpu_bvh_node root;
            cudaError_t e = cudaMemcpy(&root, nodes.p, sizeof(root), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return e;
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], root.aabb_min[a]);
                hi[a] = std::max(hi[a], root.aabb_max[a]);
            }
            return cudaSuccess;
        };
        CK(take(ctx->mesh_nodes, ctx->n_mesh_nodes), "read scene bounds");
        CK(take(ctx->sphere_nodes, ctx->n_sphere_nodes), "read scene bounds");
        for (int a = 0; a < 3; ++a)
            if (!(hi[a] > lo[a])) { lo[a] -= 0.5f; hi[a] += 0.5f; }
        if (!std::isfinite(lo[0])) return fail(ctx, MCRT_ERR_INVALID_ARG, "empty scene");
    }
    mcrt::cache_set_bounds(cache_of(ctx), lo, hi);
    ctx->cache_cfg = *p;
    for (int a = 0; a < 3; ++a) { ctx->cache_cfg.lo[a] = lo[a]; ctx->cache_cfg.hi[a] = hi[a]; }
    ctx->cache_cfg_set = true;
    ctx->cache_fallback = false;
    if (!mcrt::cache_ready(ctx->cache)) {
        mcrt_status s = mcrt_cache_init(ctx, 0);
        if (s != MCRT_OK) return s;
    }
    return MCRT_OK;
}

mcrt_status mcrt_cache_stats(mcrt_ctx *ctx, double *out5) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!out5) return fail(ctx, MCRT_ERR_INVALID_ARG, "out5 is NULL");
    for (int k = 0; k < 5; ++k) out5[k] = ctx->cache_stats[k];
    return MCRT_OK;
}

mcrt_status mcrt_cache_infer(mcrt_ctx *ctx, const float *queries, uint32_t n, float *out) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!queries || !out || n == 0 || n > (1u << 24))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "queries / out NULL or n out of [1, 2^24]");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    bool timed_out = false;
    cudaError_t e = mcrt::cache_infer_host(cache_of(ctx), queries, n, out, ctx->stream, &timed_out);
    if (e == cudaErrorInvalidValue) return fail(ctx, MCRT_ERR_INVALID_ARG, "cache parameters not set");
    CK(e, "cache inference");
    if (timed_out) return fail(ctx, MCRT_ERR_TIMEOUT, "tensor-core product did not complete");
    return MCRT_OK;
}

mcrt_status mcrt_cache_train(mcrt_ctx *ctx, const float *samples, uint32_t n, uint32_t steps, uint32_t batch,
                             float lr, float *out_loss, float *out_grad) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!samples || n == 0 || n > (1u << 24))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "samples NULL or n out of [1, 2^24]");
    if (!(lr >= 0.0f) || !std::isfinite(lr)) return fail(ctx, MCRT_ERR_INVALID_ARG, "lr must be >= 0");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    bool timed_out = false;
    cudaError_t e = mcrt::cache_train_host(cache_of(ctx), samples, n, steps, batch, lr, out_loss, out_grad,
                                           ctx->stream, &timed_out);
    if (e == cudaErrorInvalidValue) return fail(ctx, MCRT_ERR_INVALID_ARG, "cache parameters not set");
    CK(e, "cache training");
    if (timed_out) return fail(ctx, MCRT_ERR_TIMEOUT, "tensor-core product did not complete");
    return MCRT_OK;
}

mcrt_status mcrt_denoise_accum(mcrt_ctx *ctx, const mcrt_denoise_params *params, float *out_rgba) {
    if (!ctx) return fail(nullptr, MCRT_ERR_INVALID_ARG, "ctx is NULL");
    if (!params) return fail(ctx, MCRT_ERR_INVALID_ARG, "params is NULL");
    if (!ctx->acc_valid || !ctx->gbuf_valid)
        return fail(ctx, MCRT_ERR_INVALID_ARG, "no render with a G-buffer to denoise");
    if (params->radius < 0 || params->radius > 64) return fail(ctx, MCRT_ERR_INVALID_ARG, "radius must be in [0, 64]");
    if (!(params->sigma_s > 0.0f) || !(params->sigma_d > 0.0f))
        return fail(ctx, MCRT_ERR_INVALID_ARG, "sigma_s and sigma_d must be > 0");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    const uint32_t w = ctx->acc_w, h = ctx->acc_h;
    const size_t bytes = (size_t)w * h * 16;
    CK(ctx->io_c.ensure(bytes), "allocate");
    cudaEvent_t a = ev(ctx, 0), b = ev(ctx, 1);
    cudaEventRecord(a, st);
    mcrt::launch_denoise(ctx->mean.as<float4>(), ctx->gbuf.as<float4>(), w, h, *params, ctx->io_c.as<float4>(), st);
    cudaEventRecord(b, st);
    CK(cudaGetLastError(), "denoise launch");
    if (out_rgba) CK(cudaMemcpyAsync(out_rgba, ctx->io_c.p, bytes, cudaMemcpyDeviceToHost, st), "read");
    CK(cudaStreamSynchronize(st), "denoise");
    float t = 0.0f;
    cudaEventElapsedTime(&t, a, b);
    ctx->last_ms[0] = t;
    return MCRT_OK;
}

}  // extern "C"

namespace mcrt {
// The device scene and stream of a context, for entry points defined in other
// translation units.  *err receives the context's error string.
// The closest-hit variant of a render on ctx (opts variant k + 1, else the
// context's autotuned one) when the layout it reads is ready without
// allocating: a 4-wide variant whose quantised tree has not been built since
// the last BVH build gives the binary variant 0 (the same images).  -1: the
// requested variant is out of range.
int context_variant(mcrt_ctx *ctx, const mcrt_render_opts &o) {
    const int v = o.variant ? (int)o.variant - 1 : ctx->extend_variant;
    if (v < 0 || v >= extend_variant_count()) return -1;
    int info[6];
    extend_variant_info(v, info);
    if (info[0] == 4 && !(ctx->wide_valid && ctx->n_wnodes > 0)) return 0;
    return v;
}

bool context_scene(mcrt_ctx *ctx, DeviceScene *out, cudaStream_t *stream, int *device, std::string **err) {
    *err = &ctx->err;
    if (!ctx->has_scene) {
        ctx->err = "no scene uploaded";
        return false;
    }
    *out = device_scene(ctx);
    *stream = ctx->stream;
    *device = ctx->device;
    return true;
}
}  // namespace mcrt
