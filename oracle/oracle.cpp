/* oracle/oracle.cpp — CPU restatement of the mcrt path-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it; the product
 * never links or calls it.
 *
 * Every function cites the reference file:line it restates.  Compiled with
 * -O2 -ffp-contract=off (no FMA contraction, no fast-math) so that the float
 * arithmetic is the IEEE sequence written here, identical on x86-64 and
 * aarch64.
 *
 * Deliberate, documented choices where the reference leaves freedom:
 *  - WGSL builtins sin/cos/atan2/asin/pow/exp/normalize: see fmath.h.
 *    normalize(v) = v * (1 / sqrt(dot(v, v))); dot(a,b) = (ax*bx + ay*by) + az*bz.
 *  - mix(a, b, t) = a*(1-t) + b*t (the WGSL specification's formula).
 *  - Tie rule for the closest hit: smallest t, then smallest original primitive
 *    id; a sphere wins over a triangle at equal t (path_trace.wgsl:471-479
 *    already gives spheres precedence).  To make ties reachable in any visit
 *    order the node cull is `tenter <= t_max` instead of `<` (path_trace.wgsl:255).
 *  - BVH build: the reference's sort_unstable_by on the centroid (bvh.rs:303,
 *    mesh.rs:153) is made deterministic by breaking ties on the original id.
 *    Binning is monotone in the centroid, so this changes only the order of
 *    primitives inside a leaf, never the tree.
 */
#include "oracle.h"
#include "fmath.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr float TAU = 6.283185307179586f;       /* path_trace.wgsl:36 */
constexpr float PI_F = 3.141592653589793f;      /* path_trace.wgsl:37 */
constexpr uint32_t MAX_MAT_IDX = 63u;           /* path_trace.wgsl:43 */
constexpr uint32_t MAT_METAL = 1u, MAT_DIELECTRIC = 2u, MAT_EMISSIVE = 3u; /* material.rs:70-75 */
constexpr uint32_t STACK_SIZE = 64u;            /* path_trace.wgsl:49 */
constexpr float T_MIN = 1e-4f;                  /* path_trace.wgsl:52 */
constexpr float T_MAX = 1e9f;                   /* path_trace.wgsl:55 */
constexpr uint32_t MAX_FRAME_COUNT = 65535u;    /* path_trace.wgsl:58 */
constexpr uint32_t BVH_LEAF_MAX = 4;            /* bvh.rs:32 */
constexpr int SAH_BINS = 8;                     /* bvh.rs:38 */

struct V3 { float x, y, z; };
inline V3 v3(float x, float y, float z) { return {x, y, z}; }
inline V3 ld3(const float *p) { return {p[0], p[1], p[2]}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 normalize(V3 a) { float inv = 1.0f / sqrtf(dot(a, a)); return {a.x * inv, a.y * inv, a.z * inv}; }

/* ------------------------------------------------------------------ RNG */
/* path_trace.wgsl:64-66, :194-204 */
inline uint32_t pcg_hash(uint32_t v) {
    uint32_t s = v * 747796405u + 2891336453u;
    uint32_t rot = s >> 28u;
    s = ((s >> (rot + 4u)) ^ s) * 277803737u;
    return (s >> 22u) ^ s;
}
inline float rand_f32(uint32_t &rng) {
    rng = pcg_hash(rng);
    return of_bits((rng >> 9u) | 0x3f800000u) - 1.0f;
}

/* path_trace.wgsl:210-227 */
inline V3 random_unit_sphere(uint32_t &rng) {
    float cos_phi = 1.0f - 2.0f * rand_f32(rng);
    float sin_phi = sqrtf(fmaxf(0.0f, 1.0f - cos_phi * cos_phi));
    float theta = TAU * rand_f32(rng);
    float s, c;
    of_sincos(theta, &s, &c);
    return {sin_phi * c, sin_phi * s, cos_phi};
}
inline V3 cosine_scatter(uint32_t &rng, V3 n) {
    V3 sc = n + random_unit_sphere(rng);
    if (dot(sc, sc) < 1e-6f) return n;
    return normalize(sc);
}

/* ------------------------------------------------------------------ env */
/* path_trace.wgsl:233-242 */
inline V3 sample_env(const orc_scene *sc, V3 dir) {
    if (sc->env_w == 0 || sc->env_h == 0) return {0, 0, 0};
    float phi = of_atan2(dir.z, dir.x);
    float theta = of_asin(fminf(fmaxf(dir.y, -1.0f), 1.0f));
    float u = phi / TAU + 0.5f;
    float v = 0.5f - theta / PI_F;
    uint32_t ix = of_f2u_sat(u * (float)sc->env_w) % sc->env_w;
    uint32_t iy = of_f2u_sat(v * (float)sc->env_h) % sc->env_h;
    const float *p = sc->env_rgba + 4ull * ((uint64_t)iy * sc->env_w + ix);
    return {p[0], p[1], p[2]};
}

/* ------------------------------------------------------------------ intersection */
struct Ray { V3 o, d; };

/* 1/d with the reference traversal test's clamp (bvh.rs:808-812, mesh.rs:950-954):
 * |d| < 1e-7 -> +-1e30.  WGSL's 1/0 = inf makes (min - o) * inf = 0 * inf = NaN
 * for a ray lying in a slab plane, whose min/max is backend-defined; with the
 * clamp such a ray counts as inside the slab and traversal equals brute force. */
inline float inv_dir(float d) { return fabsf(d) < 1e-7f ? (d >= 0.0f ? 1e30f : -1e30f) : 1.0f / d; }

/* The box test with a relative slack on both ends: a box is entered when
 * texit * CULL_SLACK > max(tenter, t_min) and tenter <= t_max * CULL_SLACK.
 * A hit on a shared edge or vertex lies on the boundary of its triangle's box,
 * and the Moller-Trumbore t can lie outside the box by its rounding (a few
 * ulps; hundreds for a grazing ray), so with the exact test such a box is
 * culled or not depending on which triangle the visit order found first: the
 * closest hit and the tie rule would depend on the order (about 1 in 200 rays
 * aimed at mesh vertices and edges).  With the slack (1 + 2^-12, about 2000
 * ulps) every box that can hold a hit at or before t is entered, so the
 * answer is the tie rule's over every triangle the test accepts, in any visit
 * order (no difference from brute force on 10^6 such rays). */
constexpr float CULL_SLACK = 1.000244140625f;
inline float cull_t(float t) { return t * CULL_SLACK; }

/* path_trace.wgsl:248-256, with the slack of CULL_SLACK on entry and exit */
inline bool ray_aabb_hit(const Ray &r, const orc_node &nd, float t_min, float t_max) {
    V3 inv = {inv_dir(r.d.x), inv_dir(r.d.y), inv_dir(r.d.z)};
    V3 t0 = (ld3(nd.aabb_min) - r.o) * inv;
    V3 t1 = (ld3(nd.aabb_max) - r.o) * inv;
    float tenter = fmaxf(fmaxf(fminf(t0.x, t1.x), fminf(t0.y, t1.y)), fminf(t0.z, t1.z));
    float texit = fminf(fminf(fmaxf(t0.x, t1.x), fmaxf(t0.y, t1.y)), fmaxf(t0.z, t1.z));
    return cull_t(texit) > fmaxf(tenter, t_min) && tenter <= cull_t(t_max);
}

/* path_trace.wgsl:262-281: candidate root with t > t_min (near first, then far),
 * independent of t_max; the caller applies t_max and the tie rule. */
inline bool sphere_t(const Ray &r, const orc_sphere &s, float t_min, float *t_out) {
    V3 c = ld3(s.center_r);
    float radius = s.center_r[3];
    V3 oc = r.o - c;
    float a = dot(r.d, r.d);
    float h = dot(oc, r.d);
    float cc = dot(oc, oc) - radius * radius;
    float disc = h * h - a * cc;
    if (disc < 0.0f) return false;
    float sq = sqrtf(disc);
    float t = (-h - sq) / a;
    if (t <= t_min) {
        t = (-h + sq) / a;
        if (t <= t_min) return false;
    }
    *t_out = t;
    return true;
}

/* path_trace.wgsl:300-317 (t_max applied by the caller) */
inline bool tri_uvt(const Ray &r, V3 v0, V3 v1, V3 v2, float t_min, float *t, float *uu, float *vv) {
    V3 e1 = v1 - v0;
    V3 e2 = v2 - v0;
    V3 h = cross(r.d, e2);
    float a = dot(e1, h);
    if (fabsf(a) < 1e-8f) return false;
    float f = 1.0f / a;
    V3 s = r.o - v0;
    float u = f * dot(s, h);
    if (u < 0.0f || u > 1.0f) return false;
    V3 q = cross(s, e1);
    float v = f * dot(r.d, q);
    if (v < 0.0f || u + v > 1.0f) return false;
    float tt = f * dot(e2, q);
    if (tt < t_min) return false;
    *t = tt; *uu = u; *vv = v;
    return true;
}

struct Closest {
    float t;
    uint32_t prim;   /* ORC_HIT_MISS, ORC_HIT_SPHERE|sphere_id, or triangle id */
    uint32_t slot;   /* ordered slot of the primitive */
    float u, v;
};

inline bool tie_better(float t, uint32_t id, const Closest &b) {
    if (t < b.t) return true;
    if (t == b.t && b.prim != ORC_HIT_MISS && !(b.prim & ORC_HIT_SPHERE) && id < b.prim) return true;
    return false;
}

/* Interpolated shading normal of an ordered triangle at (u, v) (path_trace.wgsl:448-450). */
inline V3 tri_normal(const orc_scene *sc, const orc_triangle &tri, float u, float v) {
    const orc_vertex &va = sc->vertices[tri.v[0]];
    const orc_vertex &vb = sc->vertices[tri.v[1]];
    const orc_vertex &vc = sc->vertices[tri.v[2]];
    float w = 1.0f - u - v;
    return normalize((w * ld3(va.normal) + u * ld3(vb.normal)) + v * ld3(vc.normal));
}

/* sphere_bvh_hit, path_trace.wgsl:343-364, :393-413 */
void sphere_bvh_hit(const orc_scene *sc, const Ray &r, float t_min, float t_max, Closest &best,
                    uint32_t *nodes_visited, uint32_t *prims_tested) {
    if (sc->n_sphere_nodes == 0) return;
    uint32_t stack[STACK_SIZE];
    uint32_t top = 0;
    stack[top++] = 0;
    best.t = t_max;
    while (top > 0) {
        uint32_t ni = stack[--top];
        const orc_node &nd = sc->sphere_nodes[ni];
        ++*nodes_visited;
        if (!ray_aabb_hit(r, nd, t_min, best.t)) continue;
        if (nd.prim_count > 0) {
            for (uint32_t j = 0; j < nd.prim_count; ++j) {
                uint32_t slot = nd.right_or_offset + j;
                ++*prims_tested;
                float t;
                if (!sphere_t(r, sc->spheres[slot], t_min, &t)) continue;
                if (!(t < t_max)) continue;
                uint32_t id = sc->sphere_ids ? sc->sphere_ids[slot] : slot;
                bool better = t < best.t ||
                              (t == best.t && best.prim != ORC_HIT_MISS && (id | ORC_HIT_SPHERE) < best.prim);
                if (better) { best.t = t; best.prim = id | ORC_HIT_SPHERE; best.slot = slot; best.u = 0; best.v = 0; }
            }
            continue;
        }
        if (top + 2u <= STACK_SIZE) {
            stack[top++] = nd.right_or_offset;
            stack[top++] = ni + 1u;
        }
    }
}

/* mesh_bvh_hit, path_trace.wgsl:368-387, :419-465 */
void mesh_bvh_hit(const orc_scene *sc, const Ray &r, float t_min, Closest &best,
                  uint32_t *nodes_visited, uint32_t *prims_tested) {
    if (sc->n_mesh_nodes == 0) return;
    uint32_t stack[STACK_SIZE];
    uint32_t top = 0;
    stack[top++] = 0;
    while (top > 0) {
        uint32_t ni = stack[--top];
        const orc_node &nd = sc->mesh_nodes[ni];
        ++*nodes_visited;
        if (!ray_aabb_hit(r, nd, t_min, best.t)) continue;
        if (nd.prim_count > 0) {
            for (uint32_t j = 0; j < nd.prim_count; ++j) {
                uint32_t slot = nd.right_or_offset + j;
                ++*prims_tested;
                const orc_triangle &tri = sc->triangles[slot];
                float t, u, v;
                if (!tri_uvt(r, ld3(sc->vertices[tri.v[0]].position), ld3(sc->vertices[tri.v[1]].position),
                             ld3(sc->vertices[tri.v[2]].position), t_min, &t, &u, &v))
                    continue;
                uint32_t id = sc->triangle_ids ? sc->triangle_ids[slot] : slot;
                if (!tie_better(t, id, best)) continue;
                if ((tri.mat_idx >> 31u) != 0u) {              /* backface cull, :438-452 */
                    V3 n = tri_normal(sc, tri, u, v);
                    if (!(dot(r.d, n) < 0.0f)) continue;
                }
                best.t = t; best.prim = id; best.slot = slot; best.u = u; best.v = v;
            }
            continue;
        }
        if (top + 2u <= STACK_SIZE) {
            stack[top++] = nd.right_or_offset;
            stack[top++] = ni + 1u;
        }
    }
}

/* world_hit, path_trace.wgsl:471-479 */
Closest world_hit(const orc_scene *sc, const Ray &r, float t_min, float t_max, uint32_t *nv, uint32_t *pt) {
    Closest best{t_max, ORC_HIT_MISS, 0, 0, 0};
    sphere_bvh_hit(sc, r, t_min, t_max, best, nv, pt);
    mesh_bvh_hit(sc, r, t_min, best, nv, pt);
    if (best.prim == ORC_HIT_MISS) best.t = -1.0f;
    return best;
}

Closest brute_hit(const orc_scene *sc, const Ray &r, float t_min, float t_max) {
    Closest best{t_max, ORC_HIT_MISS, 0, 0, 0};
    for (uint32_t slot = 0; slot < sc->n_spheres; ++slot) {
        float t;
        if (!sphere_t(r, sc->spheres[slot], t_min, &t) || !(t < t_max)) continue;
        uint32_t id = sc->sphere_ids ? sc->sphere_ids[slot] : slot;
        bool better = t < best.t || (t == best.t && best.prim != ORC_HIT_MISS && (id | ORC_HIT_SPHERE) < best.prim);
        if (better) { best.t = t; best.prim = id | ORC_HIT_SPHERE; best.slot = slot; best.u = best.v = 0; }
    }
    for (uint32_t slot = 0; slot < sc->n_triangles; ++slot) {
        const orc_triangle &tri = sc->triangles[slot];
        float t, u, v;
        if (!tri_uvt(r, ld3(sc->vertices[tri.v[0]].position), ld3(sc->vertices[tri.v[1]].position),
                     ld3(sc->vertices[tri.v[2]].position), t_min, &t, &u, &v))
            continue;
        uint32_t id = sc->triangle_ids ? sc->triangle_ids[slot] : slot;
        if (!tie_better(t, id, best)) continue;
        if ((tri.mat_idx >> 31u) != 0u) {
            V3 n = tri_normal(sc, tri, u, v);
            if (!(dot(r.d, n) < 0.0f)) continue;
        }
        best.t = t; best.prim = id; best.slot = slot; best.u = u; best.v = v;
    }
    if (best.prim == ORC_HIT_MISS) best.t = -1.0f;
    return best;
}

/* ------------------------------------------------------------------ shading */
struct HitRec { float t; V3 p; V3 n; bool front; uint32_t mat; };

inline HitRec make_hitrec(const orc_scene *sc, const Ray &r, const Closest &c) {
    HitRec h;
    h.t = c.t;
    h.p = r.o + c.t * r.d;                                       /* :283, :455 */
    if (c.prim & ORC_HIT_SPHERE) {                               /* :282-287 */
        const orc_sphere &s = sc->spheres[c.slot];
        V3 outn = (h.p - ld3(s.center_r)) / s.center_r[3];
        h.front = dot(r.d, outn) < 0.0f;
        h.n = h.front ? outn : -outn;
        h.mat = s.mat_and_pad[0];
    } else {                                                     /* :444-459 */
        const orc_triangle &tri = sc->triangles[c.slot];
        V3 n = tri_normal(sc, tri, c.u, c.v);
        h.front = dot(r.d, n) < 0.0f;
        h.n = h.front ? n : -n;
        h.mat = tri.mat_idx & 0x7fffffffu;
    }
    return h;
}

/* path_trace.wgsl:485-500 */
inline V3 reflect_vec(V3 v, V3 n) { return v - (2.0f * dot(v, n)) * n; }
inline V3 refract_vec(V3 v, V3 n, float eta) {
    float cos_theta = fminf(dot(-v, n), 1.0f);
    V3 r_perp = eta * (v + cos_theta * n);
    V3 r_para = (-sqrtf(fmaxf(0.0f, 1.0f - dot(r_perp, r_perp)))) * n;
    return r_perp + r_para;
}
inline float schlick(float cos_theta, float eta) {
    float r0 = (1.0f - eta) / (1.0f + eta);
    r0 = r0 * r0;
    return r0 + (1.0f - r0) * of_pow(1.0f - cos_theta, 5.0f);
}

/* uv of a hit: triangles interpolate vertex uvs (path_trace.wgsl:459); spheres
 * map the outward normal to longitude / latitude (:288-291). */
void hit_uv(const orc_scene *sc, const Closest &c, V3 p, float *uo, float *vo) {
    if (c.prim & ORC_HIT_SPHERE) {
        const orc_sphere &s = sc->spheres[c.slot];
        V3 outn = (p - ld3(s.center_r)) / s.center_r[3];
        float phi = of_atan2(outn.z, outn.x);
        float theta = of_asin(fminf(fmaxf(outn.y, -1.0f), 1.0f));
        *uo = phi / TAU + 0.5f;
        *vo = 0.5f - theta / PI_F;
        return;
    }
    const orc_triangle &tri = sc->triangles[c.slot];
    const float *ua = sc->vertices[tri.v[0]].uv, *ub = sc->vertices[tri.v[1]].uv, *uc = sc->vertices[tri.v[2]].uv;
    float u = c.u, v = c.v, w = 1.0f - u - v;
    *uo = (w * ua[0] + u * ub[0]) + v * uc[0];
    *vo = (w * ua[1] + u * ub[1]) + v * uc[1];
}

/* sRGB -> linear of an 8-bit channel (IEC 61966-2-1) in double, rounded to float */
const float *srgb_table() {
    static float t[256];
    static bool init = false;
    if (!init) {
        for (int i = 0; i < 256; ++i) {
            double c = i / 255.0;
            t[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
        }
        init = true;
    }
    return t;
}

/* textureSampleLevel of an Rgba8UnormSrgb array with a linear / repeat sampler
 * (gpu_layout.rs:435-477, headless.rs:184-191): texel centres at (i+0.5)/N,
 * decode then filter, weights (1-f, f). */
V3 sample_albedo(const orc_scene *sc, uint32_t layer, float u, float v) {
    const int N = (int)sc->albedo_size;
    const float *lut = srgb_table();
    float x = u * (float)N - 0.5f, y = v * (float)N - 0.5f;
    if (!(fabsf(x) < 1e8f)) x = 0.0f;
    if (!(fabsf(y) < 1e8f)) y = 0.0f;
    float x0 = floorf(x), y0 = floorf(y);
    float fx = x - x0, fy = y - y0;
    int ix = (int)x0 % N, iy = (int)y0 % N;
    if (ix < 0) ix += N;
    if (iy < 0) iy += N;
    int ix1 = ix + 1 == N ? 0 : ix + 1, iy1 = iy + 1 == N ? 0 : iy + 1;
    const uint8_t *base = sc->albedo_rgba8 + (size_t)layer * N * N * 4;
    auto texel = [&](int tx, int ty) {
        const uint8_t *t = base + 4 * ((size_t)ty * N + tx);
        return V3{lut[t[0]], lut[t[1]], lut[t[2]]};
    };
    V3 t00 = texel(ix, iy), t10 = texel(ix1, iy), t01 = texel(ix, iy1), t11 = texel(ix1, iy1);
    float gx = 1.0f - fx, gy = 1.0f - fy;
    V3 top = gx * t00 + fx * t10;
    V3 bot = gx * t01 + fx * t11;
    return gy * top + fy * bot;
}

/* material_albedo, path_trace.wgsl:506-515 */
V3 material_albedo(const orc_scene *sc, const orc_material &m, const Closest &c, V3 p) {
    V3 albedo = ld3(m.albedo_fuzz);
    uint32_t layer = m.type_pad[1];
    if (layer == 0u || sc->albedo_layers == 0u || !sc->albedo_rgba8) return albedo;
    uint32_t safe = std::min(layer, sc->albedo_layers - 1u);
    float u, v;
    hit_uv(sc, c, p, &u, &v);
    return sample_albedo(sc, safe, u, v) * albedo;
}

/* GGX conductor (an extension of the reference, material type 4): the same
 * Trowbridge-Reitz / Smith height-correlated / Schlick model and visible-normal
 * sampling (Heitz 2018) as the kernels, so the reference estimator with GGX is
 * reproduced sample for sample. */
constexpr uint32_t MAT_GGX = 4u;
inline void onb(V3 n, V3 *t, V3 *b) {   /* Duff et al. 2017 */
    float sign = n.z >= 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float bb = n.x * n.y * a;
    *t = {1.0f + sign * n.x * n.x * a, sign * bb, -sign * n.x};
    *b = {bb, sign + n.y * n.y * a, -n.y};
}
inline float ggx_lambda(float alpha, float cos_t) {
    float c2 = cos_t * cos_t;
    float t2 = fmaxf(0.0f, 1.0f - c2) / fmaxf(c2, 1e-12f);
    return 0.5f * (-1.0f + sqrtf(1.0f + alpha * alpha * t2));
}
inline float ggx_d(float alpha, float cos_h) {
    float a2 = alpha * alpha;
    float c2 = cos_h * cos_h;
    float den = c2 * (a2 - 1.0f) + 1.0f;
    return a2 / (PI_F * den * den);
}
struct GgxSample { V3 wi; V3 weight; float pdf; float mz; float fw; };
bool ggx_sample(V3 wo, float alpha, V3 f0, float r1, float r2, GgxSample *out) {
    V3 vh = normalize({alpha * wo.x, alpha * wo.y, wo.z});
    float lensq = vh.x * vh.x + vh.y * vh.y;
    V3 t1 = lensq > 0.0f ? V3{-vh.y, vh.x, 0.0f} / sqrtf(lensq) : V3{1.0f, 0.0f, 0.0f};
    V3 t2 = cross(vh, t1);
    float r = sqrtf(r1);
    float phi = 2.0f * PI_F * r2;
    float sp, cp;
    of_sincos(phi, &sp, &cp);
    float p1 = r * cp;
    float p2 = r * sp;
    float s = 0.5f * (1.0f + vh.z);
    p2 = (1.0f - s) * sqrtf(fmaxf(0.0f, 1.0f - p1 * p1)) + s * p2;
    V3 nh = (p1 * t1 + p2 * t2) + sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2)) * vh;
    V3 m = normalize({alpha * nh.x, alpha * nh.y, fmaxf(1e-6f, nh.z)});
    float wo_m = dot(wo, m);
    V3 wi = (2.0f * wo_m) * m - wo;
    if (wi.z <= 0.0f) return false;
    float l_o = ggx_lambda(alpha, wo.z), l_i = ggx_lambda(alpha, wi.z);
    float g1 = 1.0f / (1.0f + l_o);
    float g2 = 1.0f / ((1.0f + l_o) + l_i);
    float fw = of_pow(1.0f - fmaxf(0.0f, wo_m), 5.0f);
    V3 F = f0 + fw * (V3{1.0f, 1.0f, 1.0f} - f0);
    out->weight = (g2 / g1) * F;
    out->pdf = g1 * ggx_d(alpha, m.z) / (4.0f * wo.z);     /* D_v(m) / (4 wo.m) */
    out->wi = wi;
    out->mz = m.z;
    out->fw = fw;
    return true;
}

/* f(wo, wi) * cos(wi) and the visible-normal pdf of wi (zero below the surface). */
V3 ggx_eval(V3 wo, V3 wi, float alpha, V3 f0, float *pdf_out, float *mz_out, float *fw_out) {
    *pdf_out = 0.0f;
    if (wo.z <= 0.0f || wi.z <= 0.0f) return {0.0f, 0.0f, 0.0f};
    V3 m = normalize(wo + wi);
    float l_o = ggx_lambda(alpha, wo.z), l_i = ggx_lambda(alpha, wi.z);
    float g1 = 1.0f / (1.0f + l_o);
    float g2 = 1.0f / ((1.0f + l_o) + l_i);
    float D = ggx_d(alpha, m.z);
    float wo_m = dot(wo, m);
    float fw = of_pow(1.0f - fmaxf(0.0f, wo_m), 5.0f);
    V3 F = f0 + fw * (V3{1.0f, 1.0f, 1.0f} - f0);
    *pdf_out = g1 * D / (4.0f * wo.z);
    *mz_out = m.z;
    *fw_out = fw;
    return (D * g2 / (4.0f * wo.z)) * F;
}

/* Derivative with respect to alpha of D(m) * G2(wo, wi), in double precision,
 * by the product rule: dD/da = D (2/a - 4 a c^2 / (c^2 (a^2 - 1) + 1)),
 * dG2/da = -G2^2 (dL(wo)/da + dL(wi)/da), dL/da = a t^2 / (2 sqrt(1 + a^2 t^2)). */
void ggx_dg_dalpha(double alpha, double mz, double cos_o, double cos_i, double *dg_out, double *dgd_out) {
    double c2 = mz * mz;
    double den = c2 * (alpha * alpha - 1.0) + 1.0;
    double D = alpha * alpha / (3.141592653589793 * den * den);
    double dD = D * (2.0 / alpha - 4.0 * alpha * c2 / den);
    auto lam = [&](double c, double *dl) {
        double cc = c * c;
        double t2 = std::max(0.0, 1.0 - cc) / std::max(cc, 1e-12);
        double s = std::sqrt(1.0 + alpha * alpha * t2);
        *dl = 0.5 * alpha * t2 / s;
        return 0.5 * (-1.0 + s);
    };
    double dlo, dli;
    double lo = lam(cos_o, &dlo), li = lam(cos_i, &dli);
    double G2 = 1.0 / (1.0 + lo + li);
    double dG2 = -G2 * G2 * (dlo + dli);
    *dg_out = dD * G2 + D * dG2;   /* d(D G2)/da */
    *dgd_out = D * G2;
}

/* ------------------------------------------------------------------ next-event estimation
 * An extension of the reference, which reaches emitters only by hitting them.
 * The light list holds the emissive triangles (original ids, ascending) and then
 * the emissive spheres (ordered slots).  A light is picked with probability
 * proportional to area * luminance(emission) from a CDF summed in a fixed order:
 * 1024 contiguous chunks, then a sequential scan of the chunk sums.  Emitters
 * reached by BSDF sampling are weighted by the power heuristic.  The kernels do
 * exactly this, so renders with NEE are compared bit for bit. */
struct Lights {
    bool has_sun = false;            /* directional light: unit direction towards it, irradiance */
    V3 sun_dir = {0, 0, 0}, sun_E = {0, 0, 0};
    std::vector<uint32_t> codes;     /* triangle original id, or ORC_HIT_SPHERE | ordered sphere slot */
    std::vector<float> cdf;          /* n + 1 entries */
    std::vector<uint32_t> slot_of;   /* original triangle id -> ordered slot */
    float total = 0.0f;
    uint32_t n = 0;
};
inline float luminance(V3 c) { return (0.2126f * c.x + 0.7152f * c.y) + 0.0722f * c.z; }
inline bool is_emissive(const orc_scene *sc, uint32_t mat) {
    return sc->materials->materials[std::min(mat & 0x7fffffffu, MAX_MAT_IDX)].type_pad[0] == MAT_EMISSIVE;
}
inline V3 emission_of(const orc_scene *sc, uint32_t mat) {
    const orc_material &m = sc->materials->materials[std::min(mat, MAX_MAT_IDX)];
    if (m.type_pad[0] != MAT_EMISSIVE) return {0.0f, 0.0f, 0.0f};
    return m.ior_pad[0] * ld3(m.albedo_fuzz);
}
inline void tri_positions(const orc_scene *sc, const orc_triangle &tri, V3 *a, V3 *b, V3 *c) {
    *a = ld3(sc->vertices[tri.v[0]].position);
    *b = ld3(sc->vertices[tri.v[1]].position);
    *c = ld3(sc->vertices[tri.v[2]].position);
}
float light_weight(const orc_scene *sc, const Lights &L, uint32_t code) {
    if (code & ORC_HIT_SPHERE) {
        const orc_sphere &s = sc->spheres[code & ~ORC_HIT_SPHERE];
        float r = s.center_r[3];
        return ((4.0f * PI_F) * (r * r)) * luminance(emission_of(sc, s.mat_and_pad[0]));
    }
    const orc_triangle &tri = sc->triangles[L.slot_of[code]];
    V3 a, b, c;
    tri_positions(sc, tri, &a, &b, &c);
    V3 ng = cross(b - a, c - a);
    return (0.5f * sqrtf(dot(ng, ng))) * luminance(emission_of(sc, tri.mat_idx & 0x7fffffffu));
}
void make_lights(const orc_scene *sc, Lights &L) {
    L.has_sun = sc->sun_irradiance[0] > 0.0f || sc->sun_irradiance[1] > 0.0f || sc->sun_irradiance[2] > 0.0f;
    if (L.has_sun) {
        const double len = std::sqrt((double)sc->sun_dir[0] * sc->sun_dir[0] + (double)sc->sun_dir[1] * sc->sun_dir[1] +
                                     (double)sc->sun_dir[2] * sc->sun_dir[2]);
        L.sun_dir = {(float)(sc->sun_dir[0] / len), (float)(sc->sun_dir[1] / len), (float)(sc->sun_dir[2] / len)};
        L.sun_E = ld3(sc->sun_irradiance);
    }
    L.slot_of.assign(sc->n_triangles, 0u);
    std::vector<uint32_t> tris;
    for (uint32_t s = 0; s < sc->n_triangles; ++s) {
        uint32_t id = sc->triangle_ids ? sc->triangle_ids[s] : s;
        L.slot_of[id] = s;
        if (is_emissive(sc, sc->triangles[s].mat_idx)) tris.push_back(id);
    }
    std::sort(tris.begin(), tris.end());
    L.codes = tris;
    for (uint32_t s = 0; s < sc->n_spheres; ++s)
        if (is_emissive(sc, sc->spheres[s].mat_and_pad[0])) L.codes.push_back(s | ORC_HIT_SPHERE);
    const uint32_t n = (uint32_t)L.codes.size();
    L.n = n;
    L.cdf.assign(n + 1, 0.0f);
    if (n == 0) return;
    const uint32_t chunk = (n + 1023) / 1024;
    std::vector<float> part(1024, 0.0f);
    for (uint32_t t = 0; t < 1024; ++t) {
        float local = 0.0f;
        for (uint32_t k = t * chunk; k < std::min(t * chunk + chunk, n); ++k) local += light_weight(sc, L, L.codes[k]);
        part[t] = local;
    }
    float run = 0.0f;
    for (uint32_t k = 0; k < 1024; ++k) { float v = part[k]; part[k] = run; run += v; }
    const float total = run;
    for (uint32_t t = 0; t < 1024; ++t) {
        float r = part[t];
        for (uint32_t k = t * chunk; k < std::min(t * chunk + chunk, n); ++k) {
            L.cdf[k] = total > 0.0f ? r / total : 0.0f;
            r += light_weight(sc, L, L.codes[k]);
        }
    }
    L.cdf[0] = 0.0f;
    L.cdf[n] = 1.0f;
    L.total = total;
    if (!(total > 0.0f)) L.n = 0;
}
inline uint32_t pick_light(const Lights &L, float u) {       /* largest k with cdf[k] <= u */
    uint32_t lo = 0, hi = L.n;
    while (lo + 1 < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (L.cdf[mid] <= u) lo = mid; else hi = mid;
    }
    return lo;
}
struct LightSample { V3 dir; float dist; float pdf; V3 Le; uint32_t mat; bool ok; bool delta; };
/* With both a directional light and area lights, each kind is chosen with probability 1/2. */
inline float area_selection(const Lights &L) { return (L.has_sun && L.n > 0) ? 0.5f : 1.0f; }
/* A uniform point on an emissive triangle, or a direction in the cone of an
 * emissive sphere; pdf per unit solid angle at x, including the light choice. */
LightSample sample_light(const orc_scene *sc, const Lights &L, V3 x, uint32_t &rng) {
    LightSample ls{};
    ls.ok = false;
    ls.delta = false;
    const float sel = area_selection(L);
    if (L.has_sun && (L.n == 0 || rand_f32(rng) < 0.5f)) {     /* the directional (delta) light */
        ls.dir = L.sun_dir;
        ls.dist = T_MAX;
        ls.pdf = sel;
        ls.Le = L.sun_E;
        ls.mat = 0xffu;
        ls.ok = true;
        ls.delta = true;
        return ls;
    }
    uint32_t code = L.codes[pick_light(L, rand_f32(rng))];
    float prob = sel * (light_weight(sc, L, code) / L.total);
    float r1 = rand_f32(rng), r2 = rand_f32(rng);
    if (!(prob > 0.0f)) return ls;
    if (code & ORC_HIT_SPHERE) {
        const orc_sphere &s = sc->spheres[code & ~ORC_HIT_SPHERE];
        V3 wc = ld3(s.center_r) - x;
        float d2 = dot(wc, wc);
        float r2s = s.center_r[3] * s.center_r[3];
        if (d2 <= r2s) return ls;
        float dc = sqrtf(d2);
        V3 w = wc / dc;
        float cosmax = sqrtf(fmaxf(0.0f, 1.0f - r2s / d2));
        if (!(cosmax < 1.0f)) return ls;
        float cos_t = (1.0f - r1) + r1 * cosmax;
        float sin_t = sqrtf(fmaxf(0.0f, 1.0f - cos_t * cos_t));
        float sp, cp;
        of_sincos(TAU * r2, &sp, &cp);
        V3 t, b;
        onb(w, &t, &b);
        V3 dir = normalize(((sin_t * cp) * t + (sin_t * sp) * b) + cos_t * w);
        float proj = dot(wc, dir);
        float disc = r2s - (d2 - proj * proj);
        float dist = proj - sqrtf(fmaxf(0.0f, disc));
        ls.dir = dir;
        ls.dist = dist;
        ls.pdf = prob / (TAU * (1.0f - cosmax));
        ls.mat = std::min(s.mat_and_pad[0], MAX_MAT_IDX);
        ls.Le = emission_of(sc, s.mat_and_pad[0]);
        ls.ok = dist > 0.0f;
        return ls;
    }
    const orc_triangle &tri = sc->triangles[L.slot_of[code]];
    V3 a, bq, cq;
    tri_positions(sc, tri, &a, &bq, &cq);
    float su = sqrtf(r1);
    float b0 = 1.0f - su, b1 = r2 * su, b2 = (1.0f - b0) - b1;
    V3 y = (b0 * a + b1 * bq) + b2 * cq;
    V3 ng = cross(bq - a, cq - a);
    float area2 = sqrtf(dot(ng, ng));
    if (!(area2 > 0.0f)) return ls;
    V3 wv = y - x;
    float dist2 = dot(wv, wv);
    float dist = sqrtf(dist2);
    if (!(dist > 0.0f)) return ls;
    V3 dir = wv / dist;
    float cos_l = fabsf(dot(ng, dir)) / area2;
    if (!(cos_l > 1e-7f)) return ls;
    if (tri.mat_idx & 0x80000000u) {                  /* invisible from behind (path_trace.wgsl:452) */
        V3 ns = tri_normal(sc, tri, b1, b2);
        if (!(dot(dir, ns) < 0.0f)) return ls;
    }
    ls.dir = dir;
    ls.dist = dist;
    ls.pdf = prob * dist2 / (cos_l * (0.5f * area2));
    ls.mat = std::min(tri.mat_idx & 0x7fffffffu, MAX_MAT_IDX);
    ls.Le = emission_of(sc, tri.mat_idx & 0x7fffffffu);
    ls.ok = true;
    return ls;
}
/* Solid-angle pdf at o with which sample_light produces the emitter hit c along d. */
float light_pdf_of_hit(const orc_scene *sc, const Lights &L, const Closest &c, V3 o, V3 d) {
    if (c.prim & ORC_HIT_SPHERE) {
        float prob = area_selection(L) * (light_weight(sc, L, c.slot | ORC_HIT_SPHERE) / L.total);
        const orc_sphere &s = sc->spheres[c.slot];
        V3 wc = ld3(s.center_r) - o;
        float d2 = dot(wc, wc);
        float r2s = s.center_r[3] * s.center_r[3];
        if (d2 <= r2s) return 0.0f;
        float cosmax = sqrtf(fmaxf(0.0f, 1.0f - r2s / d2));
        if (!(cosmax < 1.0f)) return 0.0f;
        return prob / (TAU * (1.0f - cosmax));
    }
    float prob = area_selection(L) * (light_weight(sc, L, c.prim) / L.total);
    V3 a, bq, cq;
    tri_positions(sc, sc->triangles[c.slot], &a, &bq, &cq);
    V3 ng = cross(bq - a, cq - a);
    float area2 = sqrtf(dot(ng, ng));
    if (!(area2 > 0.0f)) return 0.0f;
    float cos_l = fabsf(dot(ng, d)) / area2;
    if (!(cos_l > 1e-7f)) return 0.0f;
    return prob * (c.t * c.t) / (cos_l * (0.5f * area2));
}

/* Texture factor of a material at a hit: material_albedo = factor * albedo. */
V3 material_tex(const orc_scene *sc, const orc_material &m, const Closest &c, V3 p) {
    uint32_t layer = m.type_pad[1];
    if (layer == 0u || sc->albedo_layers == 0u || !sc->albedo_rgba8) return {1.0f, 1.0f, 1.0f};
    float u, v;
    hit_uv(sc, c, p, &u, &v);
    return sample_albedo(sc, std::min(layer, sc->albedo_layers - 1u), u, v);
}

/* Forward-mode derivatives of one path's radiance with respect to the material
 * parameters (4 per material slot: albedo r, g, b and roughness), carried in
 * double precision alongside the float path: dthr = d(throughput)/dparam,
 * dL = d(radiance)/dparam.  This is the brute-force counterpart of the
 * kernels' path-replay adjoint: same estimator (BSDF sampling, light choice and
 * MIS weights held fixed), derivatives propagated forward instead of replayed
 * backward. */
struct Deriv {
    uint32_t np = 0;
    std::vector<double> dthr, dL;   /* np x 3 */
};

/* path_color, path_trace.wgsl:583-620 (+ G-buffer :592-602).
 * stats (optional): [0] rays traced, [1] nodes visited, [2] primitives tested.
 * lights: next-event estimation with MIS when non-null.  D: derivatives when non-null. */
/* A path stopped into a radiance cache whose prediction is the constant c: at
 * its non-emissive vertex number `bounce` it keeps that vertex's light sample
 * (next-event estimation), then adds thr * max(c, 0) and ends. */
struct CacheStop { uint32_t bounce; V3 c; };
/* The closest-hit queries of one path: ray and hit of bounces 0 .. bmax-1. */
struct PathLog { orc_ray *rays; orc_hit *hits; uint32_t bmax; };

V3 path_color(const orc_scene *sc, Ray ray, uint32_t &rng, uint32_t max_depth, float *gbuf, uint64_t *stats,
              const Lights *lights, Deriv *D, const CacheStop *stop = nullptr, PathLog *log = nullptr) {
    const bool nee = lights && (lights->n > 0 || lights->has_sun);
    V3 thr = {1.0f, 1.0f, 1.0f};
    V3 Lacc = {0.0f, 0.0f, 0.0f};
    float prev_pdf = -1.0f;
    bool first = true;
    const uint32_t np = D ? D->np : 0;
    if (D) {
        std::fill(D->dthr.begin(), D->dthr.end(), 0.0);
        std::fill(D->dL.begin(), D->dL.end(), 0.0);
    }
    auto dthr = [&](uint32_t p, int c) -> double & { return D->dthr[3 * p + c]; };
    auto dL = [&](uint32_t p, int c) -> double & { return D->dL[3 * p + c]; };
    auto comp = [](V3 v, int c) { return c == 0 ? v.x : (c == 1 ? v.y : v.z); };
    for (uint32_t bounce = 0; bounce < max_depth; ++bounce) {
        uint32_t nv = 0, pt = 0;
        Closest c = world_hit(sc, ray, T_MIN, T_MAX, &nv, &pt);
        if (stats) { stats[0] += 1; stats[1] += nv; stats[2] += pt; }
        if (log && bounce < log->bmax) {
            orc_ray &lr = log->rays[bounce];
            lr.org[0] = ray.o.x; lr.org[1] = ray.o.y; lr.org[2] = ray.o.z; lr.tmin = T_MIN;
            lr.dir[0] = ray.d.x; lr.dir[1] = ray.d.y; lr.dir[2] = ray.d.z; lr.tmax = T_MAX;
            log->hits[bounce] = orc_hit{c.t, c.prim, c.u, c.v};
        }
        if (c.t < 0.0f) {
            if (first && gbuf) { gbuf[0] = 0; gbuf[1] = 0; gbuf[2] = 0; gbuf[3] = T_MAX; }
            V3 e = thr * sample_env(sc, ray.d);
            if (D)
                for (uint32_t p = 0; p < np; ++p)
                    for (int k = 0; k < 3; ++k) dL(p, k) += dthr(p, k) * (double)comp(sample_env(sc, ray.d), k);
            return nee ? Lacc + e : e;
        }
        HitRec h = make_hitrec(sc, ray, c);
        if (first) {
            if (gbuf) { gbuf[0] = h.n.x; gbuf[1] = h.n.y; gbuf[2] = h.n.z; gbuf[3] = h.t; }
            first = false;
        }
        uint32_t mi = std::min(h.mat, MAX_MAT_IDX);
        const orc_material &m = sc->materials->materials[mi];
        V3 albedo = ld3(m.albedo_fuzz);
        if (m.type_pad[0] == MAT_EMISSIVE) {                                   /* :608-610 */
            V3 e = m.ior_pad[0] * (thr * albedo);
            float wmis = 1.0f;
            if (nee && prev_pdf > 0.0f && lights->n > 0) {
                float pl = light_pdf_of_hit(sc, *lights, c, ray.o, ray.d);
                wmis = (prev_pdf * prev_pdf) / (prev_pdf * prev_pdf + pl * pl);
            }
            if (D) {
                const double s = (double)wmis * (double)m.ior_pad[0];
                for (uint32_t p = 0; p < np; ++p)
                    for (int k = 0; k < 3; ++k) dL(p, k) += s * (double)comp(albedo, k) * dthr(p, k);
                if (4 * mi + 3 < np)
                    for (int k = 0; k < 3; ++k) dL(4 * mi + k, k) += s * (double)comp(thr, k);
            }
            return nee ? Lacc + wmis * e : e;
        }
        albedo = material_albedo(sc, m, c, h.p);                               /* :506-515 */
        const V3 tex = D ? material_tex(sc, m, c, h.p) : V3{1.0f, 1.0f, 1.0f};
        const bool own = D && 4 * mi + 3 < np;
        V3 dir = {0, 0, 0}, atten = {0, 0, 0};
        bool absorbed = false;
        float pdf = -1.0f;
        /* local derivatives of this vertex's throughput factor: d atten_k / d param */
        double datt_alb[3] = {0, 0, 0}, datt_rough[3] = {0, 0, 0};
        bool have_shadow = false;
        V3 sc_c = {0, 0, 0}, sh_o = {0, 0, 0}, sh_d = {0, 0, 0};
        float sh_max = 0.0f;
        double dsc_alb[3] = {0, 0, 0}, dsc_rough[3] = {0, 0, 0}, dsc_light[3] = {0, 0, 0}, sc_scale = 0.0;
        V3 sc_f = {0, 0, 0};   /* the per-channel factor multiplying thr in the NEE term */
        uint32_t sc_lmat = 0;
        if (m.type_pad[0] == MAT_GGX) {
            V3 t, b;
            onb(h.n, &t, &b);
            V3 wo = {-dot(ray.d, t), -dot(ray.d, b), -dot(ray.d, h.n)};
            float rough = m.albedo_fuzz[3];
            float alpha = fmaxf(rough * rough, 1e-4f);
            const double dadr = rough * rough > 1e-4f ? 2.0 * (double)rough : 0.0;
            float r1 = rand_f32(rng), r2 = rand_f32(rng);
            GgxSample gs;
            if (wo.z > 0.0f && ggx_sample(wo, alpha, albedo, r1, r2, &gs)) {
                dir = normalize((gs.wi.x * t + gs.wi.y * b) + gs.wi.z * h.n);
                atten = gs.weight;
                pdf = gs.pdf;
                if (own) {
                    double dg, dgd;
                    ggx_dg_dalpha(alpha, gs.mz, wo.z, gs.wi.z, &dg, &dgd);
                    for (int k = 0; k < 3; ++k) {
                        double f0 = comp(albedo, k);
                        double F = f0 + (double)gs.fw * (1.0 - f0);
                        /* weight = D G2 F / (4 cos_o) / pdf, the sampling pdf held fixed */
                        datt_alb[k] = (dgd * 0.25 / (double)wo.z) / (double)gs.pdf * (1.0 - gs.fw) * comp(tex, k);
                        datt_rough[k] = F * dg * 0.25 / (double)wo.z / (double)gs.pdf * dadr;
                    }
                }
                if (nee) {
                    LightSample ls = sample_light(sc, *lights, h.p, rng);
                    if (ls.ok) {
                        V3 wl = {dot(ls.dir, t), dot(ls.dir, b), dot(ls.dir, h.n)};
                        float bp, mz, fw;
                        V3 fc = ggx_eval(wo, wl, alpha, albedo, &bp, &mz, &fw);
                        if (wl.z > 0.0f && (fc.x > 0.0f || fc.y > 0.0f || fc.z > 0.0f)) {
                            float wmis = ls.delta ? 1.0f : (ls.pdf * ls.pdf) / (ls.pdf * ls.pdf + bp * bp);
                            sc_c = (wmis / ls.pdf) * (thr * (fc * ls.Le));
                            sh_o = h.p; sh_d = ls.dir; sh_max = ls.dist * (1.0f - 1e-4f);
                            have_shadow = true;
                            if (D) {
                                sc_scale = (double)(wmis / ls.pdf);
                                sc_f = fc * ls.Le;
                                sc_lmat = ls.mat;
                                double dg, dgd;
                                ggx_dg_dalpha(alpha, mz, wo.z, wl.z, &dg, &dgd);
                                const double lstrength = ls.mat <= MAX_MAT_IDX ? (double)sc->materials->materials[ls.mat].ior_pad[0] : 0.0;
                                for (int k = 0; k < 3; ++k) {
                                    double f0 = comp(albedo, k);
                                    double F = f0 + (double)fw * (1.0 - f0);
                                    dsc_alb[k] = sc_scale * comp(thr, k) * comp(ls.Le, k) *
                                                 (dgd * 0.25 / (double)wo.z) * (1.0 - fw) * comp(tex, k);
                                    dsc_rough[k] = sc_scale * comp(thr, k) * comp(ls.Le, k) * F * dg * 0.25 /
                                                   (double)wo.z * dadr;
                                    dsc_light[k] = sc_scale * comp(thr, k) * comp(fc, k) * lstrength;
                                }
                            }
                        }
                    }
                }
            } else {
                absorbed = true;
            }
        } else if (m.type_pad[0] == MAT_METAL) {                               /* :530-541 */
            float fuzz = m.albedo_fuzz[3];
            V3 refl = reflect_vec(normalize(ray.d), h.n);
            V3 pert = refl + fuzz * random_unit_sphere(rng);
            dir = normalize(dot(pert, pert) >= 1e-6f ? pert : refl);
            atten = albedo;
            absorbed = dot(dir, h.n) <= 0.0f;
            for (int k = 0; k < 3; ++k) datt_alb[k] = comp(tex, k);
        } else if (m.type_pad[0] == MAT_DIELECTRIC) {                          /* :543-564 */
            atten = {1.0f, 1.0f, 1.0f};
            float ior = m.ior_pad[0];
            float eta = h.front ? 1.0f / ior : ior;
            float cos_t = fminf(dot(-ray.d, h.n), 1.0f);
            float sin_t = sqrtf(fmaxf(0.0f, 1.0f - cos_t * cos_t));
            bool cannot = eta * sin_t > 1.0f;
            float scos = (!h.front && !cannot)
                             ? sqrtf(fmaxf(0.0f, 1.0f - (eta * eta) * (1.0f - cos_t * cos_t)))
                             : cos_t;
            float refl = schlick(scos, eta);
            if (cannot || refl > rand_f32(rng))
                dir = reflect_vec(ray.d, h.n);
            else
                dir = normalize(refract_vec(ray.d, h.n, eta));
        } else {                                                               /* :521-528 */
            if (nee) {
                LightSample ls = sample_light(sc, *lights, h.p, rng);
                float cs = dot(ls.dir, h.n);
                if (ls.ok && cs > 0.0f) {
                    float bp = cs / PI_F;
                    float wmis = ls.delta ? 1.0f : (ls.pdf * ls.pdf) / (ls.pdf * ls.pdf + bp * bp);
                    sc_c = (wmis * bp / ls.pdf) * (thr * (albedo * ls.Le));
                    sh_o = h.p; sh_d = ls.dir; sh_max = ls.dist * (1.0f - 1e-4f);
                    have_shadow = true;
                    if (D) {
                        sc_scale = (double)(wmis * bp / ls.pdf);
                        sc_f = albedo * ls.Le;
                        sc_lmat = ls.mat;
                        const double lstrength = ls.mat <= MAX_MAT_IDX ? (double)sc->materials->materials[ls.mat].ior_pad[0] : 0.0;
                        for (int k = 0; k < 3; ++k) {
                            dsc_alb[k] = sc_scale * comp(thr, k) * comp(tex, k) * comp(ls.Le, k);
                            dsc_light[k] = sc_scale * comp(thr, k) * comp(albedo, k) * lstrength;
                        }
                    }
                }
            }
            dir = cosine_scatter(rng, h.n);
            atten = albedo;
            pdf = fmaxf(dot(dir, h.n), 0.0f) / PI_F;
            for (int k = 0; k < 3; ++k) datt_alb[k] = comp(tex, k);
        }
        if (have_shadow) {
            uint32_t snv = 0, spt = 0;
            Closest occ = world_hit(sc, Ray{sh_o, sh_d}, T_MIN, sh_max, &snv, &spt);
            if (occ.prim == ORC_HIT_MISS) {
                Lacc = Lacc + sc_c;
                if (D) {
                    for (uint32_t p = 0; p < np; ++p)
                        for (int k = 0; k < 3; ++k) dL(p, k) += sc_scale * dthr(p, k) * (double)comp(sc_f, k);
                    if (own)
                        for (int k = 0; k < 3; ++k) {
                            dL(4 * mi + k, k) += dsc_alb[k];
                            dL(4 * mi + 3, k) += dsc_rough[k];
                        }
                    if (4 * sc_lmat + 3 < np)
                        for (int k = 0; k < 3; ++k) dL(4 * sc_lmat + k, k) += dsc_light[k];
                }
            }
        }
        if (stop && bounce == stop->bounce)
            return Lacc + V3{thr.x * fmaxf(stop->c.x, 0.0f), thr.y * fmaxf(stop->c.y, 0.0f),
                             thr.z * fmaxf(stop->c.z, 0.0f)};
        if (absorbed) return Lacc;
        if (D) {
            for (uint32_t p = 0; p < np; ++p)
                for (int k = 0; k < 3; ++k) dthr(p, k) *= (double)comp(atten, k);
            if (own)
                for (int k = 0; k < 3; ++k) {
                    dthr(4 * mi + k, k) += (double)comp(thr, k) * datt_alb[k];
                    dthr(4 * mi + 3, k) += (double)comp(thr, k) * datt_rough[k];
                }
        }
        thr = thr * atten;
        prev_pdf = pdf;
        ray = {h.p, dir};
    }
    return Lacc;
}

/* cs_main raygen, path_trace.wgsl:626-652 */
inline Ray camera_ray(const orc_camera *cam, uint32_t x, uint32_t y, uint32_t w, uint32_t h, uint32_t &rng) {
    float u = ((float)x + rand_f32(rng)) / (float)w;
    float v = 1.0f - ((float)y + rand_f32(rng)) / (float)h;
    V3 focal = (ld3(cam->lower_left) + u * ld3(cam->horizontal)) + v * ld3(cam->vertical);
    float r = sqrtf(rand_f32(rng));
    float theta = TAU * rand_f32(rng);
    float s, c;
    of_sincos(theta, &s, &c);
    float lx = r * c, ly = r * s;
    V3 lens = lx * ld3(cam->defocus_u) + ly * ld3(cam->defocus_v);
    V3 o = ld3(cam->origin) + lens;
    return {o, normalize(focal - o)};
}

/* ------------------------------------------------------------------ BVH build */
struct Aabb { float mn[3], mx[3]; };
inline Aabb aabb_empty() { return {{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}}; }
inline Aabb aabb_union(const Aabb &a, const Aabb &b) {
    Aabb r;
    for (int i = 0; i < 3; ++i) { r.mn[i] = fminf(a.mn[i], b.mn[i]); r.mx[i] = fmaxf(a.mx[i], b.mx[i]); }
    return r;
}
inline float half_area(const Aabb &a) {                       /* bvh.rs:168-175 */
    float d0 = a.mx[0] - a.mn[0], d1 = a.mx[1] - a.mn[1], d2 = a.mx[2] - a.mn[2];
    return d0 * d1 + d1 * d2 + d0 * d2;
}
inline void centroid(const Aabb &a, float c[3]) {            /* bvh.rs:179-185 */
    for (int i = 0; i < 3; ++i) c[i] = (a.mn[i] + a.mx[i]) * 0.5f;
}
inline Aabb padded(const Aabb &a) {                          /* bvh.rs:194-207 */
    const float EPS = 1e-4f;
    Aabb r;
    for (int i = 0; i < 3; ++i) { r.mn[i] = fminf(a.mn[i], a.mx[i] - EPS); r.mx[i] = fmaxf(a.mx[i], a.mn[i] + EPS); }
    return r;
}

struct Prim { Aabb b; float c[3]; uint32_t id; };

/* find_best_split, bvh.rs:388-463 (identical in mesh.rs:206-275) */
bool find_best_split(const Prim *p, size_t n, const Aabb &cb, const Aabb &nb, int *axis_out, size_t *split_out) {
    float parent = fmaxf(half_area(nb), 1e-8f);
    float best_cost = (float)n;
    int best_axis = 0;
    size_t best_split = 0;
    bool found = false;
    for (int axis = 0; axis < 3; ++axis) {
        float len = cb.mx[axis] - cb.mn[axis];
        if (len < 1e-8f) continue;
        Aabb bb[SAH_BINS];
        uint32_t bc[SAH_BINS];
        for (int i = 0; i < SAH_BINS; ++i) { bb[i] = aabb_empty(); bc[i] = 0; }
        for (size_t k = 0; k < n; ++k) {
            float t = (p[k].c[axis] - cb.mn[axis]) / len;
            uint32_t b = of_f2u_sat(t * (float)SAH_BINS);
            if (b > SAH_BINS - 1) b = SAH_BINS - 1;
            bb[b] = aabb_union(bb[b], p[k].b);
            bc[b] += 1;
        }
        Aabb lb[SAH_BINS];
        uint32_t lc[SAH_BINS];
        lb[0] = bb[0]; lc[0] = bc[0];
        for (int i = 1; i < SAH_BINS; ++i) { lb[i] = aabb_union(lb[i - 1], bb[i]); lc[i] = lc[i - 1] + bc[i]; }
        Aabb rb = aabb_empty();
        uint32_t rc = 0;
        for (int s = SAH_BINS - 2; s >= 0; --s) {
            rb = aabb_union(rb, bb[s + 1]);
            rc += bc[s + 1];
            uint32_t l = lc[s];
            if (l == 0 || rc == 0) continue;
            float cost = (half_area(lb[s]) * (float)l + half_area(rb) * (float)rc) / parent;
            if (cost < best_cost) { best_cost = cost; best_axis = axis; best_split = l; found = true; }
        }
    }
    if (found && best_split > 0 && best_split < n) { *axis_out = best_axis; *split_out = best_split; return true; }
    return false;
}

/* build_recursive, bvh.rs:285-349 / mesh.rs:129-183; make_leaf bvh.rs:352-370 */
uint32_t build_recursive(Prim *p, size_t n, std::vector<orc_node> &nodes, std::vector<uint32_t> &order) {
    uint32_t idx = (uint32_t)nodes.size();
    nodes.push_back(orc_node{});
    Aabb b = aabb_empty();
    for (size_t k = 0; k < n; ++k) b = aabb_union(b, p[k].b);
    auto make_leaf = [&]() {
        orc_node nd{};
        for (int i = 0; i < 3; ++i) { nd.aabb_min[i] = b.mn[i]; nd.aabb_max[i] = b.mx[i]; }
        nd.right_or_offset = (uint32_t)order.size();
        nd.prim_count = (uint32_t)n;
        for (size_t k = 0; k < n; ++k) order.push_back(p[k].id);
        nodes[idx] = nd;
    };
    if (n <= BVH_LEAF_MAX) { make_leaf(); return idx; }
    Aabb cb = aabb_empty();
    for (size_t k = 0; k < n; ++k) {
        Aabb pt;
        for (int i = 0; i < 3; ++i) { pt.mn[i] = p[k].c[i]; pt.mx[i] = p[k].c[i]; }
        cb = aabb_union(cb, pt);
    }
    int axis;
    size_t split;
    if (!find_best_split(p, n, cb, b, &axis, &split)) { make_leaf(); return idx; }
    std::sort(p, p + n, [axis](const Prim &x, const Prim &y) {
        if (x.c[axis] < y.c[axis]) return true;
        if (y.c[axis] < x.c[axis]) return false;
        return x.id < y.id;
    });
    build_recursive(p, split, nodes, order);
    uint32_t right = (uint32_t)nodes.size();
    build_recursive(p + split, n - split, nodes, order);
    orc_node nd{};
    for (int i = 0; i < 3; ++i) { nd.aabb_min[i] = b.mn[i]; nd.aabb_max[i] = b.mx[i]; }
    nd.right_or_offset = right;
    nd.prim_count = 0;
    nodes[idx] = nd;
    return idx;
}

int n_threads(int threads) {
#ifdef _OPENMP
    return threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

} // namespace

extern "C" {

uint32_t orc_pcg_hash(uint32_t v) { return pcg_hash(v); }

/* compute_camera, camera.rs:76-127 (glam Vec3 arithmetic; tan = sin / cos of
 * the shared elementary functions).  out: the 112-byte CameraUniform. */
void orc_compute_camera(uint32_t width, uint32_t height, const float look_from[3], const float look_at[3],
                        float vfov_deg, float aperture, float focus_dist, orc_camera *out) {
    const float aspect = (float)width / (float)height;
    const V3 vup = {0.0f, 1.0f, 0.0f};
    const float vfov_rad = vfov_deg * (PI_F / 180.0f);                      /* to_radians */
    const float hh = of_tan(vfov_rad * 0.5f);
    const float viewport_h = 2.0f * hh;
    const float viewport_w = aspect * viewport_h;
    const V3 from = ld3(look_from), at = ld3(look_at);
    const V3 w = normalize(from - at);                                       /* backward */
    const V3 c0 = cross(vup, w);
    const V3 vup_safe = dot(c0, c0) > 1e-10f ? vup : V3{0.0f, 0.0f, 1.0f};   /* gimbal-lock guard */
    const V3 u = normalize(cross(vup_safe, w));
    const V3 v = cross(w, u);
    const V3 horizontal = (focus_dist * viewport_w) * u;
    const V3 vertical = (focus_dist * viewport_h) * v;
    const V3 lower_left = ((from - 0.5f * horizontal) - 0.5f * vertical) - focus_dist * w;
    const float lens_radius = aperture * 0.5f;
    const V3 du = lens_radius * u, dv = lens_radius * v;
    std::memset(out, 0, sizeof(*out));
    auto put = [](float *dst, V3 x) { dst[0] = x.x; dst[1] = x.y; dst[2] = x.z; dst[3] = 0.0f; };
    put(out->origin, from);
    put(out->lower_left, lower_left);
    put(out->horizontal, horizontal);
    put(out->vertical, vertical);
    put(out->defocus_u, du);
    put(out->defocus_v, dv);
}

uint32_t orc_build_sphere_bvh(const orc_sphere *spheres, uint32_t n, orc_node *out_nodes,
                              orc_sphere *out_ordered, uint32_t *out_ids) {
    if (n == 0) return 0;                                                   /* bvh.rs:240-245 */
    std::vector<Prim> prims(n);
    for (uint32_t i = 0; i < n; ++i) {                                     /* bvh.rs:247-260, :133-143 */
        const float *c = spheres[i].center_r;
        float r = c[3];
        Prim &p = prims[i];
        for (int k = 0; k < 3; ++k) { p.b.mn[k] = c[k] - r; p.b.mx[k] = c[k] + r; }
        centroid(p.b, p.c);
        p.id = i;
    }
    std::vector<orc_node> nodes;
    nodes.reserve(2 * (size_t)n);
    std::vector<uint32_t> order;
    order.reserve(n);
    build_recursive(prims.data(), n, nodes, order);
    std::memcpy(out_nodes, nodes.data(), nodes.size() * sizeof(orc_node));
    for (uint32_t i = 0; i < n; ++i) {
        if (out_ordered) out_ordered[i] = spheres[order[i]];
        if (out_ids) out_ids[i] = order[i];
    }
    return (uint32_t)nodes.size();
}

uint32_t orc_build_mesh_bvh(const orc_vertex *verts, uint32_t nv, const orc_triangle *tris, uint32_t nt,
                            orc_node *out_nodes, orc_triangle *out_ordered, uint32_t *out_ids) {
    (void)nv;
    if (nt == 0) return 0;                                                  /* mesh.rs:83-89 */
    std::vector<Prim> prims(nt);
    for (uint32_t i = 0; i < nt; ++i) {                                    /* mesh.rs:99-111, :282-291 */
        Aabb b = aabb_empty();
        for (int k = 0; k < 3; ++k) {
            const float *q = verts[tris[i].v[k]].position;
            for (int a = 0; a < 3; ++a) { b.mn[a] = fminf(b.mn[a], q[a]); b.mx[a] = fmaxf(b.mx[a], q[a]); }
        }
        prims[i].b = padded(b);
        centroid(prims[i].b, prims[i].c);
        prims[i].id = i;
    }
    std::vector<orc_node> nodes;
    nodes.reserve(2 * (size_t)nt);
    std::vector<uint32_t> order;
    order.reserve(nt);
    build_recursive(prims.data(), nt, nodes, order);
    std::memcpy(out_nodes, nodes.data(), nodes.size() * sizeof(orc_node));
    for (uint32_t i = 0; i < nt; ++i) {
        if (out_ordered) out_ordered[i] = tris[order[i]];
        if (out_ids) out_ids[i] = order[i];
    }
    return (uint32_t)nodes.size();
}

void orc_trace(const orc_scene *sc, const orc_ray *rays, uint32_t n, orc_hit *hits, int mode,
               uint32_t *stats, int threads) {
#pragma omp parallel for schedule(dynamic, 256) num_threads(n_threads(threads))
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        Ray r{ld3(rays[i].org), ld3(rays[i].dir)};
        uint32_t nv = 0, pt = 0;
        Closest c = mode == 1 ? brute_hit(sc, r, rays[i].tmin, rays[i].tmax)
                              : world_hit(sc, r, rays[i].tmin, rays[i].tmax, &nv, &pt);
        hits[i].t = c.t;
        hits[i].prim = c.prim;
        hits[i].u = c.u;
        hits[i].v = c.v;
        if (stats) { stats[2 * i] = nv; stats[2 * i + 1] = pt; }
    }
}

void orc_render_ex(const orc_scene *sc, const orc_camera *cam, uint32_t w, uint32_t h, uint32_t x0, uint32_t y0,
                   uint32_t cw, uint32_t ch, uint32_t spp, uint32_t first_frame, uint32_t max_depth, uint32_t flags,
                   float *out_mean, double *out_sum, float *out_gbuf, int threads, uint64_t *out_stats) {
    int64_t npx = (int64_t)cw * ch;
    Lights lights;
    const Lights *lp = nullptr;
    if (flags & ORC_RENDER_NEE) {
        make_lights(sc, lights);
        lp = &lights;
    }
    uint64_t tot[3] = {0, 0, 0};
#pragma omp parallel num_threads(n_threads(threads))
    {
    uint64_t loc[3] = {0, 0, 0};
    uint64_t *st = out_stats ? loc : nullptr;
#pragma omp for schedule(dynamic, 16)
    for (int64_t i = 0; i < npx; ++i) {
        uint32_t x = x0 + (uint32_t)(i % cw), y = y0 + (uint32_t)(i / cw);
        float mean[3] = {0, 0, 0};
        if (out_mean) { mean[0] = out_mean[4 * i]; mean[1] = out_mean[4 * i + 1]; mean[2] = out_mean[4 * i + 2]; }
        double sum[3] = {0, 0, 0};
        float g[4] = {0, 0, 0, 0};
        for (uint32_t k = 0; k < spp; ++k) {
            uint32_t frame = first_frame + k;
            uint32_t rng = pcg_hash(pcg_hash(x + y * w) ^ (frame * 2654435761u));   /* :636-637 */
            Ray r = camera_ray(cam, x, y, w, h, rng);
            V3 s = path_color(sc, r, rng, max_depth, g, st, lp, nullptr);
            float wgt = 1.0f / (float)(std::min(frame, MAX_FRAME_COUNT) + 1u);      /* :657 */
            float omw = 1.0f - wgt;
            mean[0] = mean[0] * omw + s.x * wgt;                                     /* :659 mix */
            mean[1] = mean[1] * omw + s.y * wgt;
            mean[2] = mean[2] * omw + s.z * wgt;
            sum[0] += (double)s.x; sum[1] += (double)s.y; sum[2] += (double)s.z;
        }
        if (out_mean) {
            out_mean[4 * i] = mean[0]; out_mean[4 * i + 1] = mean[1]; out_mean[4 * i + 2] = mean[2];
            out_mean[4 * i + 3] = 1.0f;
        }
        if (out_sum) { out_sum[3 * i] += sum[0]; out_sum[3 * i + 1] += sum[1]; out_sum[3 * i + 2] += sum[2]; }
        if (out_gbuf) for (int c = 0; c < 4; ++c) out_gbuf[4 * i + c] = g[c];
    }
    if (out_stats) {
#pragma omp critical
        for (int k = 0; k < 3; ++k) tot[k] += loc[k];
    }
    }
    if (out_stats) for (int k = 0; k < 3; ++k) out_stats[k] = tot[k];
}

void orc_dump_rays(const orc_scene *sc, const orc_camera *cam, uint32_t w, uint32_t h, uint32_t x0, uint32_t y0,
                   uint32_t cw, uint32_t ch, uint32_t spp, uint32_t first_frame, uint32_t max_depth, uint32_t flags,
                   uint32_t bmax, orc_ray *out_rays, orc_hit *out_hits, int threads) {
    const int64_t npx = (int64_t)cw * ch;
    Lights lights;
    const Lights *lp = nullptr;
    if (flags & ORC_RENDER_NEE) {
        make_lights(sc, lights);
        lp = &lights;
    }
#pragma omp parallel for schedule(dynamic, 16) num_threads(n_threads(threads))
    for (int64_t i = 0; i < npx; ++i) {
        const uint32_t x = x0 + (uint32_t)(i % cw), y = y0 + (uint32_t)(i / cw);
        for (uint32_t k = 0; k < spp; ++k) {
            const size_t base = ((size_t)i * spp + k) * bmax;
            for (uint32_t b = 0; b < bmax; ++b) {                /* entries the path does not reach */
                out_rays[base + b] = orc_ray{{0, 0, 0}, 0.0f, {0, 0, 0}, -1.0f};
                out_hits[base + b] = orc_hit{-1.0f, ORC_HIT_MISS, 0.0f, 0.0f};
            }
            const uint32_t frame = first_frame + k;
            uint32_t rng = pcg_hash(pcg_hash(x + y * w) ^ (frame * 2654435761u));   /* :636-637 */
            Ray r = camera_ray(cam, x, y, w, h, rng);
            PathLog log{out_rays + base, out_hits + base, bmax};
            (void)path_color(sc, r, rng, max_depth, nullptr, nullptr, lp, nullptr, nullptr, &log);
        }
    }
}

void orc_render_cache_const(const orc_scene *sc, const orc_camera *cam, uint32_t w, uint32_t h, uint32_t spp,
                            uint32_t first_frame, uint32_t max_depth, uint32_t flags, uint32_t spp_pass,
                            uint32_t train_stride, uint32_t query_vertex, const float *c3, float *out_mean,
                            double *out_sum, int threads) {
    const int64_t npx = (int64_t)w * h;
    Lights lights;
    const Lights *lp = nullptr;
    if (flags & ORC_RENDER_NEE) {
        make_lights(sc, lights);
        lp = &lights;
    }
    const CacheStop stop{query_vertex, ld3(c3)};
#pragma omp parallel for schedule(dynamic, 16) num_threads(n_threads(threads))
    for (int64_t i = 0; i < npx; ++i) {
        uint32_t x = (uint32_t)(i % w), y = (uint32_t)(i / w);
        float mean[3] = {0, 0, 0};
        double sum[3] = {0, 0, 0};
        for (uint32_t k = 0; k < spp; ++k) {
            uint32_t frame = first_frame + k;
            uint32_t rng = pcg_hash(pcg_hash(x + y * w) ^ (frame * 2654435761u));
            Ray r = camera_ray(cam, x, y, w, h, rng);
            const uint32_t pass_start = k - k % spp_pass, planes = std::min(spp_pass, spp - pass_start);
            const uint64_t slot = (uint64_t)i * planes + (k - pass_start);
            const bool training = slot % train_stride == 0;
            V3 s = path_color(sc, r, rng, max_depth, nullptr, nullptr, lp, nullptr, training ? nullptr : &stop);
            float wgt = 1.0f / (float)(std::min(frame, MAX_FRAME_COUNT) + 1u);
            float omw = 1.0f - wgt;
            mean[0] = mean[0] * omw + s.x * wgt;
            mean[1] = mean[1] * omw + s.y * wgt;
            mean[2] = mean[2] * omw + s.z * wgt;
            sum[0] += (double)s.x; sum[1] += (double)s.y; sum[2] += (double)s.z;
        }
        if (out_mean) {
            out_mean[4 * i] = mean[0]; out_mean[4 * i + 1] = mean[1]; out_mean[4 * i + 2] = mean[2];
            out_mean[4 * i + 3] = 1.0f;
        }
        if (out_sum) { out_sum[3 * i] += sum[0]; out_sum[3 * i + 1] += sum[1]; out_sum[3 * i + 2] += sum[2]; }
    }
}

void orc_render_rect_stats(const orc_scene *sc, const orc_camera *cam, uint32_t w, uint32_t h,
                           uint32_t x0, uint32_t y0, uint32_t cw, uint32_t ch, uint32_t spp, uint32_t first_frame,
                           uint32_t max_depth, float *out_mean, double *out_sum, float *out_gbuf, int threads,
                           uint64_t *out_stats) {
    orc_render_ex(sc, cam, w, h, x0, y0, cw, ch, spp, first_frame, max_depth, 0u, out_mean, out_sum, out_gbuf,
                  threads, out_stats);
}

void orc_adjoint(const orc_scene *sc, const orc_camera *cam, uint32_t w, uint32_t h, uint32_t spp,
                 uint32_t first_frame, uint32_t max_depth, uint32_t flags, const float *d_image, double *grad,
                 double *out_sum, int threads) {
    Lights lights;
    const Lights *lp = nullptr;
    if (flags & ORC_RENDER_NEE) {
        make_lights(sc, lights);
        lp = &lights;
    }
    /* parameters of the material slots the scene references */
    uint32_t nmat = 0;
    for (uint32_t s = 0; s < sc->n_triangles; ++s)
        nmat = std::max(nmat, std::min(sc->triangles[s].mat_idx & 0x7fffffffu, MAX_MAT_IDX) + 1u);
    for (uint32_t s = 0; s < sc->n_spheres; ++s)
        nmat = std::max(nmat, std::min(sc->spheres[s].mat_and_pad[0], MAX_MAT_IDX) + 1u);
    const uint32_t np = 4 * nmat;
    std::vector<double> total(4 * 64, 0.0);
    const int64_t npx = (int64_t)w * h;
    const double inv_spp = 1.0 / (double)spp;
#pragma omp parallel num_threads(n_threads(threads))
    {
        Deriv D;
        D.np = np;
        D.dthr.assign(3 * (size_t)np, 0.0);
        D.dL.assign(3 * (size_t)np, 0.0);
        std::vector<double> loc(4 * 64, 0.0);
#pragma omp for schedule(dynamic, 16)
        for (int64_t i = 0; i < npx; ++i) {
            uint32_t x = (uint32_t)(i % w), y = (uint32_t)(i / w);
            const double dx = d_image[4 * i] * inv_spp, dy = d_image[4 * i + 1] * inv_spp,
                         dz = d_image[4 * i + 2] * inv_spp;
            double sum[3] = {0, 0, 0};
            for (uint32_t k = 0; k < spp; ++k) {
                uint32_t frame = first_frame + k;
                uint32_t rng = pcg_hash(pcg_hash(x + y * w) ^ (frame * 2654435761u));
                Ray r = camera_ray(cam, x, y, w, h, rng);
                V3 s = path_color(sc, r, rng, max_depth, nullptr, nullptr, lp, &D);
                sum[0] += (double)s.x; sum[1] += (double)s.y; sum[2] += (double)s.z;
                for (uint32_t p = 0; p < np; ++p)
                    loc[p] += (dx * D.dL[3 * p] + dy * D.dL[3 * p + 1]) + dz * D.dL[3 * p + 2];
            }
            if (out_sum) { out_sum[3 * i] += sum[0]; out_sum[3 * i + 1] += sum[1]; out_sum[3 * i + 2] += sum[2]; }
        }
#pragma omp critical
        for (uint32_t p = 0; p < np; ++p) total[p] += loc[p];
    }
    for (int p = 0; p < 4 * 64; ++p) grad[p] = total[p];
}

void orc_render_rect(const orc_scene *sc, const orc_camera *cam, uint32_t w, uint32_t h, uint32_t x0, uint32_t y0,
                     uint32_t cw, uint32_t ch, uint32_t spp, uint32_t first_frame, uint32_t max_depth,
                     float *out_mean, double *out_sum, float *out_gbuf, int threads) {
    orc_render_rect_stats(sc, cam, w, h, x0, y0, cw, ch, spp, first_frame, max_depth, out_mean, out_sum, out_gbuf,
                          threads, nullptr);
}

void orc_render(const orc_scene *sc, const orc_camera *cam, uint32_t w, uint32_t h, uint32_t spp,
                uint32_t first_frame, uint32_t max_depth, float *out_mean, double *out_sum, float *out_gbuf,
                int threads) {
    orc_render_rect(sc, cam, w, h, 0, 0, w, h, spp, first_frame, max_depth, out_mean, out_sum, out_gbuf, threads);
}

/* cs_denoise, denoise.wgsl:52-120 */
void orc_denoise(const float *accum, const float *gbuf, uint32_t w, uint32_t h, int radius, float sigma_s,
                 float sigma_d, float normal_pow, float *out) {
    orc_denoise_ex(accum, gbuf, w, h, radius, sigma_s, sigma_d, normal_pow, 0.0f, 0.0f, out);
}

/* cs_denoise with the two extension terms (0 = off): a colour term
 * exp(-|c_p - c_q|^2 / (2 sigma_color^2)) multiplied into the weight, and a
 * Gaussian normal term exp(-(1 - n_p.n_q)^2 / (2 sigma_normal^2)) in place of
 * max(0, n_p.n_q)^normal_pow. */
void orc_denoise_ex(const float *accum, const float *gbuf, uint32_t w, uint32_t h, int radius, float sigma_s,
                    float sigma_d, float normal_pow, float sigma_color, float sigma_normal, float *out) {
    const int W = (int)w, H = (int)h;
    float inv2ss = 1.0f / ((2.0f * sigma_s) * sigma_s);
    float inv2ds = 1.0f / ((2.0f * sigma_d) * sigma_d);
    const bool color_term = sigma_color > 0.0f;
    const float inv2cs = color_term ? 1.0f / ((2.0f * sigma_color) * sigma_color) : 0.0f;
    const bool gauss_normal = sigma_normal > 0.0f;
    const float inv2ns = gauss_normal ? 1.0f / ((2.0f * sigma_normal) * sigma_normal) : 0.0f;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const float *gp = gbuf + 4 * ((size_t)y * W + x);
            V3 np = ld3(gp);
            float dp = gp[3];
            bool on_sky = dp < 0.0f;
            V3 acc = {0, 0, 0};
            float wacc = 0.0f;
            for (int dy = -radius; dy <= radius; ++dy)
                for (int dx = -radius; dx <= radius; ++dx) {
                    int qx = std::min(std::max(x + dx, 0), W - 1);
                    int qy = std::min(std::max(y + dy, 0), H - 1);
                    const float *gq = gbuf + 4 * ((size_t)qy * W + qx);
                    V3 nq = ld3(gq);
                    float dq = gq[3];
                    bool q_sky = dq < 0.0f;
                    if (on_sky != q_sky) continue;
                    float dist_sq = (float)(dx * dx + dy * dy);
                    float ws = of_exp(-dist_sq * inv2ss);
                    float wn = 1.0f;
                    if (!on_sky) {
                        float nd = dot(np, nq);
                        if (gauss_normal) {
                            float e = 1.0f - nd;
                            wn = of_exp(-(e * e) * inv2ns);
                        } else {
                            wn = of_pow(fmaxf(0.0f, nd), normal_pow);
                        }
                    }
                    float rel = (dp - dq) / fmaxf(dp, 1e-4f);
                    float wd = on_sky ? 1.0f : of_exp(-(rel * rel) * inv2ds);
                    float wt = (ws * wn) * wd;
                    if (color_term) {
                        V3 dc = ld3(accum + 4 * ((size_t)qy * W + qx)) - ld3(accum + 4 * ((size_t)y * W + x));
                        wt = wt * of_exp(-dot(dc, dc) * inv2cs);
                    }
                    acc = acc + wt * ld3(accum + 4 * ((size_t)qy * W + qx));
                    wacc += wt;
                }
            V3 res = wacc > 0.0f ? acc / wacc : ld3(accum + 4 * ((size_t)y * W + x));
            float *o = out + 4 * ((size_t)y * W + x);
            o[0] = res.x; o[1] = res.y; o[2] = res.z; o[3] = 1.0f;
        }
}

/* headless.rs:93-98 and the non-finite sanitising at :350-368 */
void orc_tonemap_rgba8(const float *rgba, uint32_t n, uint8_t *out) {
    const float inv_gamma = 1.0f / 2.2f;
    for (uint32_t i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) {
            float v = rgba[4 * i + c];
            if (!std::isfinite(v)) v = 0.0f;
            v = fmaxf(v, 0.0f);
            float mapped = v / (v + 1.0f);
            float g = of_pow(mapped, inv_gamma);
            g = fminf(fmaxf(g, 0.0f), 1.0f);
            float q = g * 255.0f + 0.5f;
            out[4 * i + c] = (uint8_t)std::min(of_f2u_sat(q), 255u);
        }
        out[4 * i + 3] = 255;
    }
}

/* compare_images, regression.rs:120-181 (RGB only, f64) */
void orc_compare_images(const uint8_t *a, const uint8_t *b, uint32_t w, uint32_t h, double *out) {
    if (w == 0 || h == 0) { out[0] = 0.0; out[1] = INFINITY; out[2] = 0.0; return; }
    double sum = 0.0, mx = 0.0;
    for (size_t i = 0; i < (size_t)w * h; ++i)
        for (int c = 0; c < 3; ++c) {
            double va = a[4 * i + c] / 255.0, vb = b[4 * i + c] / 255.0;
            double d = std::fabs(va - vb);
            sum += d * d;
            if (d > mx) mx = d;
        }
    double mse = sum / ((double)w * (double)h * 3.0);
    out[0] = mse;
    out[1] = mse == 0.0 ? INFINITY : 10.0 * std::log10(1.0 / mse);
    out[2] = mx;
}

void orc_ggx_dg(double alpha, double mz, double cos_o, double cos_i, double *out) {
    ggx_dg_dalpha(alpha, mz, cos_o, cos_i, &out[0], &out[1]);
}

void orc_math_eval(int fn, const float *x, const float *y, float *out, uint32_t n) {
    for (uint32_t i = 0; i < n; ++i) {
        switch (fn) {
        case 0: out[i] = of_sin(x[i]); break;
        case 1: out[i] = of_cos(x[i]); break;
        case 2: out[i] = of_atan2(x[i], y[i]); break;
        case 3: out[i] = of_asin(x[i]); break;
        case 4: out[i] = of_exp(x[i]); break;
        case 5: out[i] = of_log(x[i]); break;
        case 6: out[i] = of_pow(x[i], y[i]); break;
        case 7: out[i] = of_tan(x[i]); break;
        default: out[i] = NAN;
        }
    }
}

} // extern "C"

extern "C" {
/* screenshot_to_u8 (gpu.rs:1904-1939): ACES filmic (Narkowicz 2016) then the
 * IEC 61966-2-1 transfer; Rust's f32::clamp lets NaN through. */
void orc_tonemap_aces_rgba8(const float *rgba, uint32_t n, uint8_t *out) {
    auto rclamp = [](float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); };
    for (uint32_t i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) {
            float x = rgba[4 * i + c];
            x = std::isnan(x) ? 0.0f : fmaxf(x, 0.0f);
            float a = rclamp((x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f), 0.0f, 1.0f);
            float s;
            if (a <= 0.0f) s = 0.0f;
            else if (a <= 0.0031308f) s = fminf(a * 12.92f, 1.0f);
            else if (a < 1.0f) s = rclamp(1.055f * of_pow(a, 1.0f / 2.4f) - 0.055f, 0.0f, 1.0f);
            else s = 1.0f;
            out[4 * i + c] = (uint8_t)std::min(of_f2u_sat(s * 255.0f + 0.5f), 255u);
        }
        out[4 * i + 3] = 255;
    }
}
}
