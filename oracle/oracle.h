/* oracle/oracle.h — C interface of the CPU oracle (test infrastructure only).
 *
 * The oracle restates the reference's path-tracing hot path on the CPU:
 *   - BVH builders            src/bvh.rs:239-463, src/mesh.rs:82-291
 *   - closest-hit traversal   src/shaders/path_trace.wgsl:248-479
 *   - path_color / cs_main    src/shaders/path_trace.wgsl:194-242, :485-662
 *   - joint-bilateral denoise src/shaders/denoise.wgsl:52-120
 *   - image metrics           src/regression.rs:120-181
 *   - OBJ loader              src/mesh.rs:474-642
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 */
#ifndef MCRT_ORACLE_H
#define MCRT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float center_r[4]; uint32_t mat_and_pad[4]; } orc_sphere;                 /* scene.rs:24-29 */
typedef struct { float aabb_min[4]; float aabb_max[4]; uint32_t right_or_offset;
                 uint32_t prim_count; uint32_t pad[2]; } orc_node;                         /* bvh.rs:56-68 */
typedef struct { float position[4]; float normal[4]; float uv[4]; } orc_vertex;           /* mesh.rs:26-34 */
typedef struct { uint32_t v[3]; uint32_t mat_idx; } orc_triangle;                         /* mesh.rs:41-46 */
typedef struct { uint32_t type_pad[4]; float albedo_fuzz[4]; float ior_pad[4]; } orc_material; /* material.rs:37-44 */
typedef struct { uint32_t mat_count; uint32_t n_emissive; uint32_t pad[2];
                 orc_material materials[64]; } orc_material_data;                          /* material.rs:56-63 */
typedef struct { float origin[4]; float lower_left[4]; float horizontal[4]; float vertical[4];
                 float defocus_u[4]; float defocus_v[4]; uint32_t frame_count;
                 uint32_t pad[3]; } orc_camera;                                            /* camera.rs:37-53 */
typedef struct { float org[3]; float tmin; float dir[3]; float tmax; } orc_ray;
typedef struct { float t; uint32_t prim; float u; float v; } orc_hit;

/* A scene as the oracle traverses it: the reference's buffers after build_bvh /
 * build_mesh_bvh (ordered primitives + pre-order nodes) plus the original
 * primitive ids of the ordered slots. */
typedef struct {
    const orc_sphere *spheres; uint32_t n_spheres;          /* ordered */
    const uint32_t *sphere_ids;                             /* original index per ordered slot */
    const orc_node *sphere_nodes; uint32_t n_sphere_nodes;
    const orc_vertex *vertices; uint32_t n_vertices;
    const orc_triangle *triangles; uint32_t n_triangles;    /* ordered */
    const uint32_t *triangle_ids;
    const orc_node *mesh_nodes; uint32_t n_mesh_nodes;
    const orc_material_data *materials;
    const float *env_rgba; uint32_t env_w; uint32_t env_h;
    const uint8_t *albedo_rgba8; uint32_t albedo_layers; uint32_t albedo_size;  /* binding 10 (sRGB) */
    float sun_dir[4];          /* directional light (ORC_RENDER_NEE only): towards the light */
    float sun_irradiance[4];   /* all zero: none */
} orc_scene;

#define ORC_HIT_MISS 0xffffffffu
#define ORC_HIT_SPHERE 0x80000000u

/* Build the reference BVH.  out_nodes must hold 2*n entries; out_ordered and
 * out_ids n entries.  Returns the node count. */
uint32_t orc_build_sphere_bvh(const orc_sphere *spheres, uint32_t n,
                              orc_node *out_nodes, orc_sphere *out_ordered, uint32_t *out_ids);
uint32_t orc_build_mesh_bvh(const orc_vertex *verts, uint32_t nv,
                            const orc_triangle *tris, uint32_t nt,
                            orc_node *out_nodes, orc_triangle *out_ordered, uint32_t *out_ids);

/* compute_camera, camera.rs:76-127: the CameraUniform of a thin-lens camera. */
void orc_compute_camera(uint32_t width, uint32_t height, const float look_from[3], const float look_at[3],
                        float vfov_deg, float aperture, float focus_dist, orc_camera *out);

/* mode 0: reference traversal order with the tie rule; mode 1: brute force.
 * stats (optional, 2 entries per ray): nodes visited, primitives tested. */
void orc_trace(const orc_scene *scene, const orc_ray *rays, uint32_t n, orc_hit *hits,
               int mode, uint32_t *stats, int threads);

/* Render frames [first_frame, first_frame+spp) with the reference estimator.
 * out_mean_rgba : (optional) the reference's f32 running mean (path_trace.wgsl:656-661),
 *                 starting from zero, after the last frame.
 * out_sum_rgb   : (optional) += f64 sum of samples per pixel (3 doubles per pixel).
 * out_gbuf      : (optional) primary-hit normal.xyz + depth (path_trace.wgsl:593-601).
 * max_depth     : bounces (the reference's MAX_BOUNCES is 8). */
void orc_render(const orc_scene *scene, const orc_camera *cam, uint32_t w, uint32_t h,
                uint32_t spp, uint32_t first_frame, uint32_t max_depth,
                float *out_mean_rgba, double *out_sum_rgb, float *out_gbuf, int threads);

/* Render a sub-rectangle of pixels (x0,y0,cw,ch) of a w x h image; outputs are cw*ch sized. */
void orc_render_rect(const orc_scene *scene, const orc_camera *cam, uint32_t w, uint32_t h,
                     uint32_t x0, uint32_t y0, uint32_t cw, uint32_t ch,
                     uint32_t spp, uint32_t first_frame, uint32_t max_depth,
                     float *out_mean_rgba, double *out_sum_rgb, float *out_gbuf, int threads);

/* orc_render_rect that also returns traversal statistics of every closest-hit
 * query of the sampled paths: out_stats[0] rays, [1] BVH nodes visited (popped
 * and box-tested), [2] primitives tested — the per-ray figures of the
 * bytes-per-ray memory roofline. */
void orc_render_rect_stats(const orc_scene *scene, const orc_camera *cam, uint32_t w, uint32_t h,
                           uint32_t x0, uint32_t y0, uint32_t cw, uint32_t ch, uint32_t spp, uint32_t first_frame,
                           uint32_t max_depth, float *out_mean_rgba, double *out_sum_rgb, float *out_gbuf,
                           int threads, uint64_t *out_stats);

/* orc_render_rect_stats with render flags: ORC_RENDER_NEE adds next-event
 * estimation with power-heuristic MIS (an extension of the reference, which
 * has none), in the same order of operations as the kernels. */
#define ORC_RENDER_NEE 1u
void orc_render_ex(const orc_scene *scene, const orc_camera *cam, uint32_t w, uint32_t h,
                   uint32_t x0, uint32_t y0, uint32_t cw, uint32_t ch, uint32_t spp, uint32_t first_frame,
                   uint32_t max_depth, uint32_t flags, float *out_mean_rgba, double *out_sum_rgb, float *out_gbuf,
                   int threads, uint64_t *out_stats);

/* orc_render_ex with paths stopped into a radiance cache whose prediction is the
 * constant c3: frames are traced in passes of spp_pass (the last one shorter);
 * the sample of frame k, pixel p occupies slot p * planes + (k - pass start) of
 * its pass of `planes` frames; slots with slot % train_stride == 0 are traced in full,
 * the others, at their vertex number query_vertex (0 = primary hit) when it is
 * not emissive, keep that vertex's next-event sample, add throughput * max(c, 0)
 * and end. */
void orc_render_cache_const(const orc_scene *scene, const orc_camera *cam, uint32_t w, uint32_t h, uint32_t spp,
                            uint32_t first_frame, uint32_t max_depth, uint32_t flags, uint32_t spp_pass,
                            uint32_t train_stride, uint32_t query_vertex, const float *c3, float *out_mean_rgba,
                            double *out_sum_rgb, int threads);

/* The closest-hit queries of the sampled paths of a pixel rectangle (as
 * orc_render_ex samples them): for each pixel (row-major), frame and bounce
 * b < bmax, the ray (origin, direction, tmin = 1e-4, tmax = 1e9) and its hit by
 * the reference traversal; entries past a path's end hold tmax = -1.
 * out_rays / out_hits: cw*ch*spp*bmax entries. */
void orc_dump_rays(const orc_scene *scene, const orc_camera *cam, uint32_t w, uint32_t h, uint32_t x0, uint32_t y0,
                   uint32_t cw, uint32_t ch, uint32_t spp, uint32_t first_frame, uint32_t max_depth, uint32_t flags,
                   uint32_t bmax, orc_ray *out_rays, orc_hit *out_hits, int threads);

/* Brute-force gradient of an image loss with respect to the material
 * parameters, by forward-mode differentiation of every sampled path:
 *   grad[4*m + k] = sum_pixels sum_c d_image[pixel].c / spp * d(sample mean).c / d(param m,k)
 * with params (albedo r, albedo g, albedo b, roughness) of material slot m
 * (for emissive slots the albedo is the radiance colour, radiance = strength *
 * albedo).  BSDF sampling, light choice and MIS weights are held fixed
 * (detached sampling).  d_image: w*h RGBA floats (alpha ignored); grad: 256
 * doubles (out); out_sum_rgb: optional += f64 sums as orc_render. */
void orc_adjoint(const orc_scene *scene, const orc_camera *cam, uint32_t w, uint32_t h, uint32_t spp,
                 uint32_t first_frame, uint32_t max_depth, uint32_t flags, const float *d_image, double *grad,
                 double *out_sum_rgb, int threads);

/* Voxel world (world.cpp).  Parameters as mcrt_world_params. */
typedef struct {
    uint32_t nx, ny, nz;
    uint32_t seed;
    int32_t chunk_x0, chunk_z0;
    float height_base, height_amp;
    float height_freq;
    uint32_t height_octaves;
    float lacunarity, gain;
    float cave_freq;
    uint32_t cave_octaves;
    float cave_threshold;
    float cave_contrast;
    uint32_t cave_min_y;
    float sea_level, sand_line;
} orc_world_params;
void orc_world_generate(const orc_world_params *params, uint8_t *out_voxels);
/* The reference's greedy chunk mesher over the grid (greedy = 0: one quad per
 * visible face).  Returns the quad count; fills out_v / out_t (4 vertices and 2
 * triangles per quad) only when both are given and cap_quads suffices. */
uint64_t orc_world_mesh(const uint8_t *voxels, uint32_t nx, uint32_t ny, uint32_t nz, int32_t chunk_x0,
                        int32_t chunk_z0, int greedy, const uint32_t *block_material, float voxel_size,
                        orc_vertex *out_v, orc_triangle *out_t, uint64_t cap_quads);

/* Radiance-cache MLP (mlp.cpp): encoding, forward pass, and the gradient and
 * loss sum of one training step, with the kernels' bf16 rounding points. */
void orc_mlp_encode(const float *q12, const float *lo3, const float *inv3, float *out96);
void orc_mlp_forward(const float *params, const float *lo3, const float *inv3, const float *q12, uint32_t n,
                     float *out3);
void orc_mlp_grad(const float *params, const float *lo3, const float *inv3, const float *samples, uint32_t n,
                  double *grad, double *loss_out);

/* cs_denoise (denoise.wgsl:52-120). */
void orc_denoise(const float *accum_rgba, const float *gbuf, uint32_t w, uint32_t h,
                 int radius, float sigma_s, float sigma_d, float normal_pow, float *out_rgba);

/* cs_denoise with the library's extension terms (sigma_color, sigma_normal; 0 = off). */
void orc_denoise_ex(const float *accum_rgba, const float *gbuf, uint32_t w, uint32_t h, int radius, float sigma_s,
                    float sigma_d, float normal_pow, float sigma_color, float sigma_normal, float *out_rgba);

/* headless.rs:93-98 tonemap of an RGBA f32 image to RGBA8 (non-finite -> 0, alpha 255). */
void orc_tonemap_rgba8(const float *rgba, uint32_t n_pixels, uint8_t *out);

/* regression.rs:120-181 on RGBA8 images: out[0]=mse, out[1]=psnr, out[2]=max_delta. */
void orc_compare_images(const uint8_t *a, const uint8_t *b, uint32_t w, uint32_t h, double *out);

/* out[0] = d(D(m) G2(wo, wi))/d alpha and out[1] = D G2 of the GGX lobe (the
 * derivative the brute-force gradient uses; exposed for its finite-difference test). */
void orc_ggx_dg(double alpha, double mz, double cos_o, double cos_i, double *out);

/* Elementary functions (exposed for their error-bound tests). */
void orc_math_eval(int fn, const float *x, const float *y, float *out, uint32_t n);

uint32_t orc_pcg_hash(uint32_t v);

/* load_obj (mesh.rs:474-642) on the text of one OBJ file (obj.cpp).  Returns a
 * handle holding the vertices and triangles (NULL on error, with the text that
 * follows "'<path>' " / "'<path>': " in the reference's message in err). */
void *orc_obj_load(const char *text, uint64_t len, uint32_t mat_idx, uint32_t *n_vertices, uint32_t *n_triangles,
                   char *err, uint32_t err_cap);
void orc_obj_copy(void *handle, orc_vertex *vertices, orc_triangle *triangles);
void orc_obj_free(void *handle);
/* str::parse::<f32> of one token: 1 and the value, or 0 on a syntax error. */
int orc_parse_f32(const char *s, uint32_t len, float *out);

#ifdef __cplusplus
}
#endif
#endif
