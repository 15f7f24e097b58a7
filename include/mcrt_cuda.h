/* mcrt_cuda.h — C ABI of libmcrt_cuda.so, the GB300-native path-tracing hot path.
 *
 * This ABI replaces the reference's wgpu "operator API" for the path tracer:
 * the 14-binding compute bind-group layout (src/gpu_layout.rs:78-234, slot
 * constants :28-54), the buffers built by build_scene_buffers
 * (src/gpu_layout.rs:259-390), the compute entry point cs_main
 * (src/shaders/path_trace.wgsl:626-662, created at src/gpu_layout.rs:484-502)
 * driven once per sample by headless::run (src/headless.rs:268-290), and the
 * denoiser cs_denoise (src/shaders/denoise.wgsl:52-120, dispatched at
 * src/gpu.rs:1155-1169).
 *
 * Conventions
 *  - Every call returns mcrt_status (0 = success, < 0 = error).  The message of
 *    the last failing call is available from mcrt_last_error(ctx) (or with a
 *    NULL ctx for calls that have no context) until the next call on the same
 *    context from the same thread.  No C++ exception crosses the ABI.
 *  - The caller owns every host pointer; the context owns all device memory.
 *  - Calls are synchronous on return unless documented otherwise.  A context is
 *    not thread-safe; separate contexts are independent.
 *  - Device loops are bounded; a bound that runs out is reported as a status,
 *    never as a hang.
 *  - Plain-old-data structs below are byte-identical to the reference's
 *    #[repr(C)] bytemuck types (sizes asserted in the implementation).
 */
#ifndef MCRT_CUDA_H
#define MCRT_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCRT_ABI_VERSION 1

typedef int32_t mcrt_status;
enum {
    MCRT_OK = 0,
    MCRT_ERR_INVALID_ARG = -1,
    MCRT_ERR_OOM = -2,
    MCRT_ERR_CUDA = -3,
    MCRT_ERR_TIMEOUT = -4,          /* a bounded device loop ran out */
    MCRT_ERR_STACK_OVERFLOW = -5,   /* reserved: no call returns it (a ray whose traversal stack would
                                       overflow is traced again without a stack) */
    MCRT_ERR_NO_SCENE = -6,
    MCRT_ERR_PARSE = -7,            /* SceneError::Parse, scene.rs:603 */
    MCRT_ERR_IO = -8,               /* SceneError::Io, scene.rs:601 */
    MCRT_ERR_UNKNOWN_MATERIAL = -9, /* SceneError::UnknownMaterial, scene.rs:605 */
    MCRT_ERR_MESH_LOAD = -10,       /* SceneError::MeshLoad, scene.rs:607 */
    MCRT_ERR_TOO_MANY_MATERIALS = -11, /* SceneError::TooManyMaterials, scene.rs:609 */
    MCRT_ERR_UNSUPPORTED = -12
};

/* ------------------------------------------------------------------ reference data types */

/* GpuSphere, src/scene.rs:24-29 (32 bytes). */
typedef struct { float center_r[4]; uint32_t mat_and_pad[4]; } mcrt_gpu_sphere;
/* GpuBvhNode, src/bvh.rs:56-68 (48 bytes). Pre-order; left = i+1. */
typedef struct {
    float aabb_min[4];
    float aabb_max[4];
    uint32_t right_or_offset;
    uint32_t prim_count;
    uint32_t _pad[2];
} mcrt_gpu_bvh_node;
/* GpuVertex, src/mesh.rs:26-34 (48 bytes). */
typedef struct { float position[4]; float normal[4]; float uv[4]; } mcrt_gpu_vertex;
/* GpuTriangle, src/mesh.rs:41-46 (16 bytes). mat_idx bit 31 = backface cull (scene.rs:709-718). */
typedef struct { uint32_t v[3]; uint32_t mat_idx; } mcrt_gpu_triangle;
/* GpuMaterial, src/material.rs:37-44 (48 bytes). */
typedef struct { uint32_t type_pad[4]; float albedo_fuzz[4]; float ior_pad[4]; } mcrt_gpu_material;
/* GpuMaterialData, src/material.rs:56-63 (3088 bytes). */
#define MCRT_MAX_MATERIALS 64
typedef struct {
    uint32_t mat_count;
    uint32_t n_emissive;
    uint32_t _pad[2];
    mcrt_gpu_material materials[MCRT_MAX_MATERIALS];
} mcrt_gpu_material_data;
/* CameraUniform, src/camera.rs:37-53 (112 bytes). */
typedef struct {
    float origin[4];
    float lower_left[4];
    float horizontal[4];
    float vertical[4];
    float defocus_u[4];
    float defocus_v[4];
    uint32_t frame_count;
    uint32_t _pad[3];
} mcrt_camera_uniform;

/* Material types: material.rs:70-75, plus GGX (an extension; the reference has
 * only fuzzy metal).  GGX: albedo_fuzz.xyz = F0 (Schlick), albedo_fuzz.w = roughness
 * (alpha = roughness^2), sampled by visible normals. */
enum { MCRT_MAT_LAMBERTIAN = 0, MCRT_MAT_METAL = 1, MCRT_MAT_DIELECTRIC = 2,
       MCRT_MAT_EMISSIVE = 3, MCRT_MAT_GGX = 4 };
#define MCRT_BACKFACE_CULL_FLAG 0x80000000u

/* ------------------------------------------------------------------ context */

typedef struct mcrt_ctx mcrt_ctx;

/* Create a context on CUDA device `device`.  stream: a cudaStream_t to issue
 * all work on, or NULL for a private non-blocking stream.  (No reference
 * counterpart: wgpu's Instance/Adapter/Device, headless.rs:135-148.) */
mcrt_status mcrt_create(int device, void *stream, mcrt_ctx **out);
void mcrt_destroy(mcrt_ctx *ctx);
const char *mcrt_last_error(const mcrt_ctx *ctx);
const char *mcrt_version(void);

/* ------------------------------------------------------------------ scene upload */

/* Scene buffers as the reference binds them (gpu_layout.rs:28-54):
 *   binding 2 spheres, 5 sphere_bvh, 6 vertices, 7 triangles, 8 mesh_bvh,
 *   4 materials, 11 env_map (RGBA32F), 12 emissive_spheres (derived here).
 * If sphere_bvh / mesh_bvh are given they are the outputs of the reference's
 * build_bvh / build_mesh_bvh (bvh.rs:239, mesh.rs:82) and spheres / triangles
 * are the matching ordered arrays; *_order then maps each ordered slot to its
 * original index (the id reported by hits; identity when NULL).
 * If a BVH pointer is NULL the BVH is built on the GPU by the binned SAH
 * builder (same algorithm as the reference: 8 bins, leaf <= 4, Ct=0/Ci=1). */
typedef struct {
    const mcrt_gpu_sphere *spheres; uint32_t n_spheres;
    const mcrt_gpu_bvh_node *sphere_bvh; uint32_t n_sphere_nodes;
    const uint32_t *sphere_order;
    const mcrt_gpu_vertex *vertices; uint32_t n_vertices;
    const mcrt_gpu_triangle *triangles; uint32_t n_triangles;
    const mcrt_gpu_bvh_node *mesh_bvh; uint32_t n_mesh_nodes;
    const uint32_t *triangle_order;
    const mcrt_gpu_material_data *materials;
    const float *env_rgba; uint32_t env_w; uint32_t env_h;
    /* binding 10: albedo texture array, RGBA8 sRGB, albedo_layers x size x size
     * (gpu_layout.rs:435-477; 4 x 512 x 512 in the reference).  NULL: the
     * reference's default layers (mcrt_albedo_layers). */
    const uint8_t *albedo_rgba8; uint32_t albedo_layers; uint32_t albedo_size;
    uint32_t flags; /* MCRT_SCENE_* */
    /* Directional light (an extension; the reference's sky is its environment
     * map alone): direction towards the light (normalised here) and the
     * irradiance it delivers at normal incidence (RGB).  All-zero irradiance:
     * no directional light.  Sampled by next-event estimation only (a delta
     * light: BSDF-sampled rays never reach it). */
    float sun_dir[4];
    float sun_irradiance[4];
} mcrt_scene_desc;

enum {
    /* take the triangle mesh from the context's last mcrt_world_mesh
     * (vertices / triangles must be NULL); the mesh BVH is built on the GPU */
    MCRT_SCENE_WORLD_MESH = 1u << 0,
    /* take the triangle mesh from the context's device mesh (mcrt_mesh_append,
     * mcrt_mesh_append_obj, mcrt_mesh_append_scene; vertices / triangles must
     * be NULL); the mesh BVH is built on the GPU */
    MCRT_SCENE_DEVICE_MESH = 1u << 1
};

/* Upload (or replace) the scene.  Replaces gpu_layout::build_scene_buffers
 * (gpu_layout.rs:259-390). */
mcrt_status mcrt_upload_scene(mcrt_ctx *ctx, const mcrt_scene_desc *desc);

/* Replace the vertex positions/normals/uvs of the current scene (same count and
 * topology) and rebuild the mesh BVH on the GPU (a per-frame rebuild). */
mcrt_status mcrt_update_vertices(mcrt_ctx *ctx, const mcrt_gpu_vertex *vertices, uint32_t n_vertices);

/* Rebuild the mesh BVH of the current scene on the GPU from the device-resident
 * vertices (the per-frame rebuild without a host upload). */
mcrt_status mcrt_rebuild_bvh(mcrt_ctx *ctx);

/* Copy the device-resident mesh BVH of the current scene (reference layout,
 * pre-order) back to the host.  out_nodes: capacity 2*n_triangles;
 * out_order: capacity n_triangles (original id per ordered slot).  */
mcrt_status mcrt_get_mesh_bvh(mcrt_ctx *ctx, mcrt_gpu_bvh_node *out_nodes, uint32_t capacity,
                              uint32_t *out_n_nodes, uint32_t *out_order);

/* ------------------------------------------------------------------ closest hit (parity probe) */

typedef struct { float org[3]; float tmin; float dir[3]; float tmax; } mcrt_ray;   /* 32 B */
typedef struct { float t; uint32_t prim; float u; float v; } mcrt_hit;             /* 16 B */
#define MCRT_HIT_MISS 0xFFFFFFFFu
#define MCRT_HIT_SPHERE 0x80000000u   /* prim = MCRT_HIT_SPHERE | sphere id, else triangle id */

enum {
    MCRT_TRACE_REFERENCE_LAYOUT = 1u << 0,  /* traverse the 48-byte reference nodes in
                                              the reference visit order (path_trace.wgsl:343-479) */
    MCRT_TRACE_STATS = 1u << 1              /* reserved */
};

/* world_hit (path_trace.wgsl:471-479) for n host rays.  Tie rule: smallest t,
 * then smallest original id; a sphere wins over a triangle at equal t.
 * Requires ray.tmin > 0.  miss: prim = MCRT_HIT_MISS, t = -1. */
mcrt_status mcrt_trace_closest(mcrt_ctx *ctx, const mcrt_ray *rays, uint32_t n, mcrt_hit *hits, uint32_t flags);

/* ------------------------------------------------------------------ render */

enum {
    MCRT_RENDER_NEE = 1u << 0,        /* next-event estimation + MIS (else the reference estimator) */
    MCRT_RENDER_GBUFFER = 1u << 1,    /* keep the primary-hit G-buffer (path_trace.wgsl:593-601) */
    MCRT_RENDER_KEEP_ACCUM = 1u << 2, /* continue the device running mean / f64 sum of the previous call */
    MCRT_RENDER_GRAPH = 1u << 3,      /* replay the passes as one captured CUDA graph (same results; no
                                         per-kernel timings for the replayed passes) */
    MCRT_RENDER_CACHE = 1u << 4,      /* terminate paths into the radiance cache and train it online
                                         (mcrt_cache_config); with MCRT_RENDER_GRAPH the cached passes,
                                         training included, are replayed as a graph too */
    MCRT_RENDER_COUNT = 1u << 5       /* the closest-hit kernels count their record fetches (internal
                                         nodes visited, triangles tested; counters [6], [7] of
                                         mcrt_last_timings): the bytes-per-ray model of the traversal;
                                         same image, slower kernels (not for timed runs) */
};

typedef struct {
    uint32_t max_depth;     /* bounces; 0 -> 8 = the reference's MAX_BOUNCES (path_trace.wgsl:61) */
    uint32_t flags;
    uint32_t spp_per_pass;  /* samples traced concurrently; 0 -> automatic */
    uint32_t variant;       /* closest-hit kernel variant: 0 = the context's (autotuned) choice, k = variant k-1 */
} mcrt_render_opts;

/* Autotuner (no reference counterpart): renders `spp` frames of w x h with each
 * closest-hit kernel variant — BVH width (compact binary / quantised 4-wide),
 * block size, register budget (minimum resident blocks), traversal stack
 * depth and shared-memory staging of the tree's top levels, see
 * mcrt_variant_info — keeps the fastest for this context and
 * reports it.  Every variant gives the same images: a ray whose stack would
 * overflow is traced again without a stack, which costs its variant time on
 * a deep tree but never a hit.  out_ms (optional) receives the extend time of
 * every variant; its capacity is 8 floats. */
/* out6: BVH width, block size, minimum resident blocks per SM, stack depth,
 * idle lanes at which a warp fetches new rays, records of the compact tree's
 * top levels staged in shared memory per block (0: none) */
mcrt_status mcrt_variant_info(uint32_t variant, uint32_t *out6);
mcrt_status mcrt_autotune(mcrt_ctx *ctx, const mcrt_camera_uniform *cam, uint32_t w, uint32_t h, uint32_t spp,
                          const mcrt_render_opts *opts, uint32_t *out_variant, float *out_ms);

/* Render frames first_frame .. first_frame+spp-1 of a w x h image
 * (headless.rs:249-290: one cs_main dispatch per frame, frame_count = index).
 * cam->frame_count is ignored.  Outputs (all optional, host memory):
 *   out_rgba  : the reference's accumulation texture after the last frame —
 *               the f32 running mean (path_trace.wgsl:656-661) with alpha 1
 *               (w*h*4 floats);
 *   accum_rgb : f64 sample sums per pixel, ADDED to the caller's values (w*h*3);
 *   out_gbuf  : primary-hit normal.xyz + depth of the last frame (w*h*4 floats).
 * With all outputs NULL the results stay on the device (see mcrt_read_accum). */
mcrt_status mcrt_render(mcrt_ctx *ctx, const mcrt_camera_uniform *cam, uint32_t w, uint32_t h,
                        uint32_t spp, uint32_t first_frame, const mcrt_render_opts *opts,
                        float *out_rgba, double *accum_rgb, float *out_gbuf);

/* Batched views (no reference counterpart; the reference renders one camera
 * per headless run): n_views cameras of uneven sizes traced together — every
 * bounce of every view is one launch of each wavefront kernel over the
 * concatenated pixels.  Pixel (x, y) of view v is seeded as in mcrt_render,
 * so each view's image equals mcrt_render of that view alone, bit for bit.
 * out_rgba (optional): n_views host pointers (each NULL or w*h*4 floats) that
 * receive the views' running means.  The device accumulation afterwards is the
 * flat concatenation of the views' pixels. */
typedef struct {
    mcrt_camera_uniform cam;
    uint32_t width, height;
    uint32_t _pad[2];
} mcrt_view;
mcrt_status mcrt_render_views(mcrt_ctx *ctx, const mcrt_view *views, uint32_t n_views, uint32_t spp,
                              uint32_t first_frame, const mcrt_render_opts *opts, float *const *out_rgba);

/* mcrt_render for callers that may not allocate GPU memory while rendering
 * (no counterpart in the reference).  Hosts that reserve their GPU memory up
 * front — an engine or viewer with a fixed memory budget, a renderer embedded
 * in another application's frame loop — cannot accept cudaMalloc/cudaFree in
 * the middle of a frame: those calls synchronise the device and can fail with
 * out-of-memory.  This call allocates nothing: its path state lives in a 64 MiB
 * statically sized device array that every GPU loading the library holds
 * until the process exits.
 *   - d_out_rgba: DEVICE memory owned by the caller, w*h*4 floats; receives the
 *     f32 running mean of frames first_frame .. first_frame+spp-1 (alpha 1), as
 *     out_rgba of mcrt_render.
 *   - w*h must not exceed 262144 pixels (MCRT_ERR_INVALID_ARG otherwise);
 *     KEEP_ACCUM, GBUFFER and CACHE are rejected (MCRT_ERR_INVALID_ARG);
 *     GRAPH is ignored (the passes launch directly, with the same result).
 *   - The closest-hit kernel is the context's autotuned variant (or
 *     opts->variant); a 4-wide variant whose quantised tree has not been built
 *     since the last BVH build (by an mcrt_render with a 4-wide variant) is
 *     replaced by the binary variant 0, with the same image.
 *   - The caller's current device is restored on return.
 *   - The scene is the one of an earlier mcrt_upload_scene on ctx.
 *   - All calls share the one array: calls that overlap on the GPU (other
 *     threads, streams or contexts on the same device) race; serialise them.
 *   - The first call on a device resolves the array's device address; make it
 *     before any stream capture begins on that device.
 * Synchronous on return. */
mcrt_status mcrt_render_noalloc(mcrt_ctx *ctx, const mcrt_camera_uniform *cam, uint32_t w, uint32_t h, uint32_t spp,
                                uint32_t first_frame, const mcrt_render_opts *opts, float *d_out_rgba);

/* ------------------------------------------------------------------ voxel world */

/* Seeded terrain generator (the reference's world/generator.rs:109-200 builds
 * its chunks on the host from the noise crate's Perlin / SuperSimplex fBm; this
 * generator is the project's own, on the GPU, with lattice value noise).
 * Column rule: limestone with gravel patches, 3 blocks of red soil, a grass top
 * (sand at and below sand_line), caves carved where the 3D fBm exceeds
 * cave_threshold (y >= cave_min_y), cave-glow flora on some cave floors, water
 * above the surface up to sea_level, shrubs on some grass tops — block ids of
 * the reference's registry (world/block.rs:14-24). */
typedef struct {
    uint32_t nx, ny, nz;             /* voxels; nx, nz multiples of 16, 2 <= ny <= 1024 */
    uint32_t seed;
    int32_t chunk_x0, chunk_z0;      /* chunk coordinates of the grid's first chunk column */
    float height_base, height_amp;   /* surface height = base + amp * (2 fbm - 1), in voxels */
    float height_freq;               /* first-octave frequency, cycles per voxel */
    uint32_t height_octaves;
    float lacunarity, gain;
    float cave_freq;
    uint32_t cave_octaves;
    float cave_threshold;
    float cave_contrast;             /* cave value = 0.5 + (fbm - 0.5) * contrast */
    uint32_t cave_min_y;
    float sea_level, sand_line;      /* in voxels */
} mcrt_world_params;

/* Generate the voxel grid on the device (kept in the context).  out_voxels
 * (optional, host, nx*ny*nz bytes): a copy, index (x*ny + y)*nz + z. */
mcrt_status mcrt_world_generate(mcrt_ctx *ctx, const mcrt_world_params *params, uint8_t *out_voxels);

/* Replace the context's voxel grid with a host one (same layout; block ids as
 * world/block.rs: 1..10 opaque, 0 and others air). */
mcrt_status mcrt_world_upload(mcrt_ctx *ctx, const uint8_t *voxels, uint32_t nx, uint32_t ny, uint32_t nz,
                              int32_t chunk_x0, int32_t chunk_z0);

enum { MCRT_MESH_GREEDY = 0, MCRT_MESH_FACES = 1 };

/* Mesh the context's voxel grid on the GPU, 16 x ny x 16 chunk by chunk.
 * MCRT_MESH_GREEDY restates mesh_chunk (world/mesher.rs:97-366) over every
 * chunk of the grid with its neighbours, concatenated as merge_chunk_meshes
 * (:377-400) in (chunk x outer, chunk z inner) order; MCRT_MESH_FACES emits one
 * quad per visible face in the same order.  4 vertices and 2 triangles per
 * quad; block_material[id] is the material slot of block id (256 entries);
 * voxel_size is VOXEL_SIZE (chunk.rs:20, 0.125).  The mesh stays on the device
 * (see MCRT_SCENE_WORLD_MESH and mcrt_world_read_mesh). */
mcrt_status mcrt_world_mesh(mcrt_ctx *ctx, uint32_t mode, const uint32_t *block_material, float voxel_size,
                            uint32_t *out_n_vertices, uint32_t *out_n_triangles);

/* Copy the last world mesh to the host (capacities in elements). */
mcrt_status mcrt_world_read_mesh(mcrt_ctx *ctx, mcrt_gpu_vertex *vertices, uint32_t vertex_capacity,
                                 mcrt_gpu_triangle *triangles, uint32_t triangle_capacity);

/* ------------------------------------------------------------------ scene ingestion on the device
 * The context's device mesh collects vertex and triangle records in call order,
 * as load_scene_from_str concatenates a scene's objects (scene.rs:687-899,
 * :865-878); mcrt_upload_scene takes it with MCRT_SCENE_DEVICE_MESH.  OBJ text
 * is parsed on the device (no host parse). */

/* Empty the device mesh (its memory is kept). */
mcrt_status mcrt_mesh_reset(mcrt_ctx *ctx);

/* Append host records; triangle vertex indices are relative to this call's
 * first vertex (the library adds the mesh's current vertex count). */
mcrt_status mcrt_mesh_append(mcrt_ctx *ctx, const mcrt_gpu_vertex *vertices, uint32_t n_vertices,
                             const mcrt_gpu_triangle *triangles, uint32_t n_triangles);

/* A mesh object's transform, TransformDesc (scene.rs:438-495): uniform scale,
 * then Euler rotation in degrees (euler_to_mat3, scene.rs:396-405), then the
 * translation; an absent part is skipped exactly as the reference skips it. */
typedef struct {
    uint32_t has_translate, has_rotate, has_scale;
    float translate[3];
    float rotate_deg[3];
    float scale;
} mcrt_mesh_transform;

/* Parse Wavefront OBJ text on the device and append it: load_obj
 * (mesh.rs:474-642) with every triangle's mat_idx, then the object's transform
 * (scene.rs:838-861; NULL = none).  Bit-identical to the reference's records:
 * UTF-8 check, str::lines / trim / split_ascii_whitespace, correctly rounded
 * f32 parsing, 1-based and negative indices, (position, uv, normal) vertex
 * sharing by first occurrence, fan triangulation and the geometric-normal
 * patch.  Errors (the device mesh is unchanged):
 *   MCRT_ERR_MESH_LOAD   not UTF-8, or no face (the reference's messages, with
 *                        source as the path);
 *   MCRT_ERR_INVALID_ARG scale not positive (checked after parsing, as the
 *                        reference asserts it), or text of 4 GiB or more.
 * out_n_vertices / out_n_triangles (optional): this call's counts. */
mcrt_status mcrt_mesh_append_obj(mcrt_ctx *ctx, const char *text, uint64_t len, uint32_t mat_idx,
                                 const mcrt_mesh_transform *xf, const char *source, uint32_t *out_n_vertices,
                                 uint32_t *out_n_triangles);

/* The last successful mcrt_mesh_append_obj: out_ms2 = [text to the device,
 * the other parse stages] (ms, CUDA events on the context stream, the parser's
 * host waits for sizes excluded); out_counts4 = [text bytes, lines, face
 * tokens, kernel launches].  On a device that reaches pageable host memory
 * (cudaDevAttrPageableMemoryAccess) the parser's first pass reads the text in
 * place and copies it as it counts the lines: out_ms2[0] is that pass; else it
 * is the copy (MCRT_OBJ_COPY_TEXT=1 in the environment forces the copy). */
mcrt_status mcrt_mesh_obj_stats(mcrt_ctx *ctx, float *out_ms2, uint64_t *out_counts4);

/* Copy the device mesh to the host (capacities in records; NULL arrays are
 * skipped); out_n_* receive the mesh's counts. */
mcrt_status mcrt_mesh_read(mcrt_ctx *ctx, mcrt_gpu_vertex *vertices, uint32_t vertex_capacity,
                           mcrt_gpu_triangle *triangles, uint32_t triangle_capacity, uint32_t *out_n_vertices,
                           uint32_t *out_n_triangles);

/* ------------------------------------------------------------------ radiance-cache MLP */

/* Probe of one tensor-core product (no reference counterpart; it pins the
 * operand layouts of the MLP kernels): D[128 x N] = A[128 x K] * B[N x K]^T with
 * A, B bf16 bit patterns in row-major host arrays and D f32, computed by
 * tcgen05.mma with the operands staged K-major or, with flags bit 0 / bit 1,
 * MN-major (as the backward pass reads its tiles).  K in {16, 32, 48, 64},
 * N in {16, 32, 48, 64}. */
mcrt_status mcrt_mlp_gemm_probe(int device, const uint16_t *A, const uint16_t *B, uint32_t K, uint32_t N,
                                uint32_t flags, float *D);

/* Radiance cache (no reference counterpart): a small MLP predicting the
 * radiance scattered from a surface point towards a direction.  Inputs per
 * query, 12 floats: position p, outgoing direction w_o (towards the previous
 * vertex), shading normal n, albedo a.  Encoding (96 features): u = clamp((p -
 * lo) / (hi - lo), 0, 1); sin and cos of u * pi * 2^k for k = 0..11 per axis
 * (from sin / cos of pi u by the double-angle recurrence s' = 2sc,
 * c' = c^2 - s^2); w_o, n, a, u; zeros.  Network: 5 hidden layers of 64 ReLU units, 3 linear
 * outputs; bf16 weights and activations on the tensor cores, fp32
 * accumulation, fp32 master parameters (mcrt_cache_param_count floats: W_l
 * row-major [out][in] then b_l per layer; the output layer is stored 16 wide,
 * rows 3..15 zero).  Training: relative L2 loss (y - t)^2 / (y^2 + 0.01) with y
 * held fixed in the denominator, averaged over samples and channels, Adam
 * (beta1 0.9, beta2 0.99, eps 1e-8). */
uint32_t mcrt_cache_param_count(void);

/* Rendering with the cache (MCRT_RENDER_CACHE).  In every pass, one path in
 * `train_stride` slots is a training path: it is traced to full depth and
 * records each non-emissive vertex (position, w_o, normal, albedo, throughput,
 * radiance gathered so far); every other path stops at its non-emissive
 * vertex number `query_vertex` (0 = the primary hit): it keeps that vertex's
 * next-event sample and adds throughput x the cache's prediction in place of
 * everything BSDF sampling would have gathered from there.  After the pass the
 * training paths' vertices become samples (target = radiance the path gathered
 * after that vertex's next-event sample / throughput at it) and `train_steps` Adam
 * steps of `train_batch` samples run; each step's batch is a stratified draw
 * over all of the pass's samples (so over the whole image), and a stride that
 * yields about train_steps x train_batch samples per pass wastes none.  lo / hi: the encoding bounds (hi <= lo
 * on every axis: the scene's bounding box). */
typedef struct {
    uint32_t query_vertex;
    uint32_t train_stride;
    uint32_t train_steps;
    uint32_t train_batch;
    float lr;
    float lo[3], hi[3];
    /* Fallback to the plain tracer: > 0 and the bias judge's last measurement
     * (mcrt_cache_stats) above it in any channel: the next render stops no
     * path into the cache (every path is traced in full, as without the cache)
     * while training goes on; 0: the cache is always used. */
    float max_bias;
} mcrt_cache_params;
mcrt_status mcrt_cache_config(mcrt_ctx *ctx, const mcrt_cache_params *params);

/* The bias judge of the last render with MCRT_RENDER_CACHE: before each
 * pass's training steps, the network (as that pass used it) is evaluated on
 * the pass's training samples, whose targets are what the full-length training
 * paths (the plain tracer) gathered.  out[0..2]: relative bias per channel,
 * sum(max(prediction, 0) - target) / sum(target) over those samples (NaN when
 * a sum of targets is 0); out[3]: samples judged; out[4]: 1 when that render
 * stopped paths into the cache, 0 when it ran as the plain tracer (max_bias
 * fallback).  No reference counterpart (the reference has no radiance cache). */
mcrt_status mcrt_cache_stats(mcrt_ctx *ctx, double *out5);

/* Device time (CUDA events) of cache inference over n synthetic queries and of
 * one training step on n synthetic samples, averaged over reps:
 * out_ms[0] inference, out_ms[1] training step.  Leaves the parameters
 * trained by reps + 1 tiny steps (learning rate 1e-6). */
mcrt_status mcrt_cache_bench(mcrt_ctx *ctx, uint32_t n, uint32_t reps, float *out_ms);
mcrt_status mcrt_cache_init(mcrt_ctx *ctx, uint32_t seed);              /* He-uniform weights, zero biases */
mcrt_status mcrt_cache_set_params(mcrt_ctx *ctx, const float *params);  /* also resets the Adam moments */
mcrt_status mcrt_cache_get_params(mcrt_ctx *ctx, float *out);
mcrt_status mcrt_cache_set_bounds(mcrt_ctx *ctx, const float *lo3, const float *hi3);
/* out: n x 3 predictions for n x 12 queries (host). */
mcrt_status mcrt_cache_infer(mcrt_ctx *ctx, const float *queries, uint32_t n, float *out);
/* samples: n x 16 (query 12, target 3, weight 0 or 1).  `steps` Adam steps on
 * consecutive batches of `batch` samples (wrapping); steps = 0 computes the
 * gradient of the first batch only.  out_loss (optional): the loss sum of each
 * step; out_grad (optional): the gradient of the first step. */
mcrt_status mcrt_cache_train(mcrt_ctx *ctx, const float *samples, uint32_t n, uint32_t steps, uint32_t batch,
                             float lr, float *out_loss, float *out_grad);

/* ------------------------------------------------------------------ differentiation */

/* Replace the material table of the uploaded scene (GpuMaterialData,
 * material.rs:56-63) without re-uploading geometry; the light-selection
 * weights are recomputed.  Which slots are emissive must not change
 * (MCRT_ERR_INVALID_ARG).  No counterpart in the reference, which rebuilds
 * its buffers (gpu_layout.rs:259-390). */
mcrt_status mcrt_update_materials(mcrt_ctx *ctx, const mcrt_gpu_material_data *materials);

/* Gradient of an image loss with respect to the material parameters by
 * path-replay backpropagation (no counterpart in the reference).  The call
 * renders frames first_frame .. first_frame+spp-1 as mcrt_render with the same
 * opts (the primal pass), then replays every path from its seed and
 * accumulates
 *   grad[4*m + k] = sum_pixels sum_c d_image[pixel].c / spp * d(mean of the
 *                   samples).c / d(param m,k)
 * for material slot m and k = albedo r, g, b (albedo_fuzz[0..2]) and
 * roughness (albedo_fuzz[3], GGX materials).  For emissive slots the albedo is
 * the radiance colour (radiance = ior_pad[0] * albedo).  BSDF sampling, light
 * choice and MIS weights are held fixed while differentiating (detached
 * sampling): the estimate is unbiased for the derivative of the expected image.
 * Metal fuzz, dielectric IOR and texture texels get no gradient.
 *   d_image : host, w*h*4 floats (alpha ignored) = dLoss/d(image)
 *   grad    : host, 256 doubles (overwritten)
 *   out_rgba: optional host w*h*4 floats, the primal running mean (as mcrt_render)
 * The device accumulation afterwards holds the primal render (mcrt_read_accum).
 * KEEP_ACCUM is not supported.  Synchronous on return. */
mcrt_status mcrt_adjoint(mcrt_ctx *ctx, const mcrt_camera_uniform *cam, uint32_t w, uint32_t h, uint32_t spp,
                         uint32_t first_frame, const mcrt_render_opts *opts, const float *d_image, double *grad,
                         float *out_rgba);

/* Copy the device accumulation of the last render to the host (any may be NULL). */
mcrt_status mcrt_read_accum(mcrt_ctx *ctx, float *out_rgba, double *accum_rgb, float *out_gbuf);

/* Tone-map the device accumulation of the last render on the GPU and copy the
 * RGBA8 result (w*h*4 bytes, alpha 255) to the host:
 *   MCRT_TONEMAP_REINHARD: non-finite -> 0, v/(v+1), gamma 1/2.2, +0.5 truncate
 *                          (tonemap_to_u8, headless.rs:93-98, :350-368);
 *   MCRT_TONEMAP_ACES_SRGB: ACES filmic (Narkowicz) then the sRGB transfer
 *                          (screenshot_to_u8, gpu.rs:1904-1939). */
enum { MCRT_TONEMAP_REINHARD = 0, MCRT_TONEMAP_ACES_SRGB = 1 };
mcrt_status mcrt_read_image_rgba8(mcrt_ctx *ctx, uint32_t mode, uint8_t *out);

/* Per-kernel device time of the last render, from CUDA events on the context
 * stream: [0] total, [1] trace (extend), [2] shade, [3] shadow rays, [4] resolve,
 * [5] BVH build (ms); counters: [0] rays traced, [1] shadow rays, [2] kernel
 * launches of the last render, [3] kernel launches of the last BVH build,
 * [4] extend launches of the last render, [5] rays of the last render traced
 * by the stackless walk because the traversal stack was too short for the
 * tree (included in [0] and [1]), [6] / [7] with MCRT_RENDER_COUNT: compact
 * BVH node records (64 B) and triangle records (48 B) the closest-hit kernels
 * fetched (the bounce-0 warp packets fetch one record per warp).
 * out_ms: 6 floats, out_counts: 8 uint64. */
mcrt_status mcrt_last_timings(mcrt_ctx *ctx, float *out_ms, uint64_t *out_counts);

/* Copy bandwidth of a plain float4 copy kernel over two `bytes`-sized device
 * buffers (a warm-up launch, then one launch that copies back and forth `reps`
 * times, timed on the context stream): out_gbs = 2 * bytes * reps / time
 * (read + write).  Buffers that fit the L2 give its bandwidth, buffers far
 * larger than it the HBM's: the measured denominators of the kernels'
 * rooflines.  Allocates and frees its buffers.  (No reference counterpart.) */
mcrt_status mcrt_copy_bandwidth(mcrt_ctx *ctx, uint64_t bytes, uint32_t reps, float *out_gbs);

/* ------------------------------------------------------------------ denoiser */

/* DenoiseParams, gpu.rs:166-185 (std140, 16 bytes) followed by extensions.
 * Defaults R=3, sigma_s=2, sigma_d=0.5, normal_pow=8.
 * Extensions (0 = the reference's filter):
 *   sigma_color  > 0: multiply by exp(-|c_p - c_q|^2 / (2 sigma_color^2));
 *   sigma_normal > 0: the normal term is exp(-(1 - n_p.n_q)^2 / (2 sigma_normal^2))
 *                     instead of max(0, n_p.n_q)^normal_pow. */
typedef struct {
    int32_t radius;
    float sigma_s;
    float sigma_d;
    float normal_pow;
    float sigma_color;
    float sigma_normal;
    uint32_t _pad[2];
} mcrt_denoise_params;

/* cs_denoise (denoise.wgsl:52-120) over host images (w*h*4 floats each). */
mcrt_status mcrt_denoise(mcrt_ctx *ctx, const float *in_rgba, const float *gbuf, uint32_t w, uint32_t h,
                         const mcrt_denoise_params *params, float *out_rgba);

/* cs_denoise of the device accumulation of the last mcrt_render with its
 * G-buffer (the reference's dispatch after the frame loop, gpu.rs:166-185), no
 * host copies in between; out_rgba (optional, host w*h*4 floats) receives the
 * result.  The filter's device time replaces timing [0] of mcrt_last_timings. */
mcrt_status mcrt_denoise_accum(mcrt_ctx *ctx, const mcrt_denoise_params *params, float *out_rgba);

/* ------------------------------------------------------------------ host-side scene API
 * (the reference's Scene/Material/Camera/YAML API, run on the CPU exactly as
 * the reference runs it). */

typedef struct mcrt_loaded_scene mcrt_loaded_scene;

/* load_scene_from_yaml / load_scene_from_str (scene.rs:640-999). */
mcrt_status mcrt_scene_load_yaml(const char *path, mcrt_loaded_scene **out);
mcrt_status mcrt_scene_load_yaml_str(const char *text, const char *source, mcrt_loaded_scene **out);
void mcrt_scene_free(mcrt_loaded_scene *scene);

enum {
    /* Read each mesh object's OBJ file but leave it unparsed: the scene's host
     * vertices / triangles then hold only the tessellated primitives, and
     * mcrt_mesh_append_scene parses the meshes on the device. */
    MCRT_LOAD_DEFER_MESHES = 1u << 0
};
mcrt_status mcrt_scene_load_yaml_ex(const char *path, uint32_t flags, mcrt_loaded_scene **out);
mcrt_status mcrt_scene_load_yaml_str_ex(const char *text, const char *source, uint32_t flags,
                                        mcrt_loaded_scene **out);
/* Append a loaded scene's triangle geometry to the context's device mesh in the
 * reference's object order: tessellated primitives from the host, mesh objects
 * (of a MCRT_LOAD_DEFER_MESHES load) through mcrt_mesh_append_obj, and the
 * reference's one-triangle stub when the scene has no geometry (scene.rs:887-899). */
mcrt_status mcrt_mesh_append_scene(mcrt_ctx *ctx, const mcrt_loaded_scene *scene);

typedef struct {
    const mcrt_gpu_sphere *spheres; uint32_t n_spheres;
    const mcrt_gpu_vertex *vertices; uint32_t n_vertices;
    const mcrt_gpu_triangle *triangles; uint32_t n_triangles;
    const mcrt_gpu_sphere *emissive_spheres; uint32_t n_emissive_spheres;
    const mcrt_gpu_material_data *materials;
    int32_t has_camera;
    float look_from[3]; float look_at[3]; float vfov; float aperture; float focus_dist;
    const char *env_map_path;   /* NULL when absent */
    uint32_t n_material_names;
} mcrt_scene_view;
mcrt_status mcrt_scene_view_get(const mcrt_loaded_scene *scene, mcrt_scene_view *out);
const char *mcrt_scene_material_name(const mcrt_loaded_scene *scene, uint32_t index);

/* compute_camera (camera.rs:76-127). */
mcrt_status mcrt_compute_camera(uint32_t width, uint32_t height, const float look_from[3], const float look_at[3],
                                float vfov_deg, float aperture, float focus_dist, mcrt_camera_uniform *out);

/* load_env_map_data (texture.rs:209-220): RGBA32F, 1024 x 512.  path may be NULL.
 * out must hold 1024*512*4 floats. */
#define MCRT_ENV_MAP_WIDTH 1024
#define MCRT_ENV_MAP_HEIGHT 512
mcrt_status mcrt_load_env_map(const char *path, float *out);
/* build_gradient_env_map (texture.rs:158-199). */
mcrt_status mcrt_gradient_env_map(float *out);

/* The reference's albedo texture array (load_all_textures, texture.rs:235-256):
 * 4 layers of 512 x 512 RGBA8 — layer 0 white, layer 1 the grey checker,
 * layers 2 and 3 the magenta "missing texture" checker (no texture files are
 * read; texture.rs:66-110 falls back to it when textures/earth.png is absent).
 * out must hold 4*512*512*4 bytes. */
#define MCRT_TEXTURE_SIZE 512
#define MCRT_TEXTURE_LAYERS 4
mcrt_status mcrt_albedo_layers(uint8_t *out);

/* tonemap_to_u8 over an RGBA32F image (headless.rs:93-98, :350-368): RGBA8, alpha 255. */
mcrt_status mcrt_tonemap_rgba8(const float *rgba, uint32_t n_pixels, uint8_t *out);
/* screenshot_to_u8 (ACES + sRGB, gpu.rs:1904-1939) over an RGBA32F image: RGBA8, alpha 255. */
mcrt_status mcrt_tonemap_aces_rgba8(const float *rgba, uint32_t n_pixels, uint8_t *out);
/* RGBA8 PNG writer (the image crate's save, headless.rs:380-382). */
mcrt_status mcrt_write_png(const char *path, const uint8_t *rgba, uint32_t w, uint32_t h);
/* Radiance RGBE (.hdr) writer of an RGBA32F image (alpha ignored): flat
 * scanlines, shared exponent from the largest channel, the encoding of the
 * reference's sky generator (tests/assets/gen_test_skymap.py:44-94); readable by
 * mcrt_load_env_map. */
mcrt_status mcrt_write_hdr(const char *path, const float *rgba, uint32_t w, uint32_t h);

/* headless::run (headless.rs:112-386): parameters CLI > sidecar [render] > 512/512/64.
 * width/height/spp = 0 means "not given".  opts may be NULL (reference estimator). */
mcrt_status mcrt_headless_run(const char *scene_path, const char *output_path, uint32_t width, uint32_t height,
                              uint32_t spp, const mcrt_render_opts *opts);

#ifdef __cplusplus
}
#endif
#endif /* MCRT_CUDA_H */
