// render.cu — wavefront path tracer kernels: ray generation, closest-hit
// extension, shading (reference estimator or next-event estimation with MIS),
// shadow rays and per-pixel resolve; plus the closest-hit parity probe.
//
// One render pass traces `spp_pass` sample planes of the image at once (slot =
// pixel * spp_pass + plane: a pixel's samples sit in neighbouring lanes, so a
// warp's rays start together and stay close for the first bounces).  Each
// bounce is extend -> shade (-> shadow); shade
// appends surviving paths to the next ray queue with warp-aggregated atomics
// (one atomicAdd per warp), so later bounces run on compacted queues.  All
// per-path state is indexed by slot and every path owns its radiance, so the
// result is independent of queue order (deterministic, no float atomics).
#include "common.cuh"
#include "internal.h"
#include "traverse.cuh"

namespace mcrt {

namespace {

constexpr uint32_t kMatMetal = 1u, kMatDielectric = 2u, kMatEmissive = 3u, kMatGgx = 4u;

inline int grid_blocks_for(uint32_t n, int threads) { return (int)((n + threads - 1) / threads); }

// ------------------------------------------------------------------ sampling (path_trace.wgsl:210-227)
__device__ __forceinline__ f3 random_unit_sphere(uint32_t &rng) {
    float cos_phi = 1.0f - 2.0f * rand_f32(rng);
    float sin_phi = sqrtf(fmaxf(0.0f, 1.0f - cos_phi * cos_phi));
    float theta = kTau * rand_f32(rng);
    float s, c;
    dm_sincos(theta, &s, &c);
    return {sin_phi * c, sin_phi * s, cos_phi};
}
__device__ __forceinline__ f3 cosine_scatter(uint32_t &rng, f3 n) {
    f3 sc = n + random_unit_sphere(rng);
    if (dot(sc, sc) < 1e-6f) return n;
    return normalize(sc);
}

// sample_env_map, path_trace.wgsl:233-242
__device__ __forceinline__ f3 sample_env(const DeviceScene &S, f3 d) {
    if (S.env_w == 0 || S.env_h == 0) return {0.0f, 0.0f, 0.0f};
    float phi = dm_atan2(d.z, d.x);
    float theta = dm_asin(fminf(fmaxf(d.y, -1.0f), 1.0f));
    float u = phi / kTau + 0.5f;
    float v = 0.5f - theta / kPi;
    uint32_t ix = f2u_sat(u * (float)S.env_w) % S.env_w;
    uint32_t iy = f2u_sat(v * (float)S.env_h) % S.env_h;
    return xyz(__ldg(S.env + (size_t)iy * S.env_w + ix));
}

// path_trace.wgsl:485-500
__device__ __forceinline__ f3 reflect_vec(f3 v, f3 n) { return v - (2.0f * dot(v, n)) * n; }
__device__ __forceinline__ f3 refract_vec(f3 v, f3 n, float eta) {
    float cos_theta = fminf(dot(-v, n), 1.0f);
    f3 r_perp = eta * (v + cos_theta * n);
    f3 r_para = (-sqrtf(fmaxf(0.0f, 1.0f - dot(r_perp, r_perp)))) * n;
    return r_perp + r_para;
}
__device__ __forceinline__ float schlick(float cos_theta, float eta) {
    float r0 = (1.0f - eta) / (1.0f + eta);
    r0 = r0 * r0;
    return r0 + (1.0f - r0) * dm_pow(1.0f - cos_theta, 5.0f);
}

// cs_main ray generation, path_trace.wgsl:636-652
__device__ __forceinline__ void camera_ray(const mcrt_camera_uniform &cam, uint32_t x, uint32_t y, uint32_t w,
                                           uint32_t h, uint32_t &rng, f3 *o_out, f3 *d_out) {
    float u = ((float)x + rand_f32(rng)) / (float)w;
    float v = 1.0f - ((float)y + rand_f32(rng)) / (float)h;
    f3 focal = (ld3(cam.lower_left) + u * ld3(cam.horizontal)) + v * ld3(cam.vertical);
    float r = sqrtf(rand_f32(rng));
    float theta = kTau * rand_f32(rng);
    float s, c;
    dm_sincos(theta, &s, &c);
    float lx = r * c, ly = r * s;
    f3 lens = lx * ld3(cam.defocus_u) + ly * ld3(cam.defocus_v);
    f3 o = ld3(cam.origin) + lens;
    *o_out = o;
    *d_out = normalize(focal - o);
}

struct SurfaceHit { float t; f3 p; f3 n; bool front; uint32_t mat; };

__device__ __forceinline__ SurfaceHit surface(const DeviceScene &S, f3 o, f3 d, float4 h) {
    SurfaceHit s;
    s.t = h.x;
    s.p = o + h.x * d;                                          // path_trace.wgsl:283, :455
    uint32_t prim = __float_as_uint(h.y);
    if (prim & MCRT_HIT_SPHERE) {                               // :282-287
        uint32_t slot = __float_as_uint(h.z);
        float4 cr = __ldg(reinterpret_cast<const float4 *>(S.spheres + slot));
        f3 outn = (s.p - xyz(cr)) / cr.w;
        s.front = dot(d, outn) < 0.0f;
        s.n = s.front ? outn : -outn;
        s.mat = S.spheres[slot].mat_and_pad[0];
    } else {                                                    // :444-459
        f3 n = tri_shading_normal(S, prim, h.z, h.w);
        s.front = dot(d, n) < 0.0f;
        s.n = s.front ? n : -n;
        s.mat = tri_material_word(S, prim) & 0x7fffffffu;
    }
    return s;
}

// Texture coordinates of a hit, evaluated only for textured materials:
// triangles interpolate vertex uvs (path_trace.wgsl:459), spheres use the
// longitude/latitude mapping of the outward normal (:288-291).
__device__ __forceinline__ void hit_uv(const DeviceScene &S, f3 p, float4 h, float *u_out, float *v_out) {
    uint32_t prim = __float_as_uint(h.y);
    if (prim & MCRT_HIT_SPHERE) {
        float4 cr = __ldg(reinterpret_cast<const float4 *>(S.spheres + __float_as_uint(h.z)));
        f3 outn = (p - xyz(cr)) / cr.w;
        float phi = dm_atan2(outn.z, outn.x);
        float theta = dm_asin(fminf(fmaxf(outn.y, -1.0f), 1.0f));
        *u_out = phi / kTau + 0.5f;
        *v_out = 0.5f - theta / kPi;
        return;
    }
    mcrt_gpu_triangle tri = S.triangles[prim];
    const float *ua = S.vertices[tri.v[0]].uv, *ub = S.vertices[tri.v[1]].uv, *uc = S.vertices[tri.v[2]].uv;
    float u = h.z, v = h.w, w = 1.0f - u - v;
    *u_out = (w * ua[0] + u * ub[0]) + v * uc[0];
    *v_out = (w * ua[1] + u * ub[1]) + v * uc[1];
}

// textureSampleLevel with a linear, repeat sampler (headless.rs:184-191) on an
// RGBA8 sRGB array: texel centres at (i + 0.5) / N, channels decoded to linear
// before filtering, weights (1 - f, f) per axis.
__device__ __forceinline__ f3 sample_albedo(const DeviceScene &S, uint32_t layer, float u, float v) {
    const int N = (int)S.albedo_size;
    float x = u * (float)N - 0.5f, y = v * (float)N - 0.5f;
    if (!(fabsf(x) < 1e8f)) x = 0.0f;
    if (!(fabsf(y) < 1e8f)) y = 0.0f;
    float x0 = floorf(x), y0 = floorf(y);
    float fx = x - x0, fy = y - y0;
    int ix = (int)x0 % N, iy = (int)y0 % N;
    if (ix < 0) ix += N;
    if (iy < 0) iy += N;
    int ix1 = ix + 1 == N ? 0 : ix + 1, iy1 = iy + 1 == N ? 0 : iy + 1;
    const uchar4 *base = S.albedo + (size_t)layer * N * N;
    auto texel = [&](int tx, int ty) {
        uchar4 t = __ldg(base + (size_t)ty * N + tx);
        return mk3(__ldg(S.srgb_lut + t.x), __ldg(S.srgb_lut + t.y), __ldg(S.srgb_lut + t.z));
    };
    f3 t00 = texel(ix, iy), t10 = texel(ix1, iy), t01 = texel(ix, iy1), t11 = texel(ix1, iy1);
    float gx = 1.0f - fx, gy = 1.0f - fy;
    f3 top = gx * t00 + fx * t10;
    f3 bot = gx * t01 + fx * t11;
    return gy * top + fy * bot;
}

// material_albedo, path_trace.wgsl:506-515
__device__ __forceinline__ f3 material_albedo(const DeviceScene &S, const mcrt_gpu_material &m, f3 p, float4 h) {
    f3 albedo = ld3(m.albedo_fuzz);
    uint32_t layer = m.type_pad[1];
    if (layer == 0u || S.albedo_layers == 0u) return albedo;
    uint32_t safe = min(layer, S.albedo_layers - 1u);
    float u, v;
    hit_uv(S, p, h, &u, &v);
    return sample_albedo(S, safe, u, v) * albedo;
}

// GGX conductor (extension): Trowbridge-Reitz distribution, Smith
// height-correlated masking-shadowing, Schlick Fresnel with F0 = albedo;
// sampled by visible normals (Heitz 2018, "Sampling the GGX Distribution of
// Visible Normals", JCGT 7(4)).
__device__ __forceinline__ void onb(f3 n, f3 *t, f3 *b) {
    // Duff et al. 2017, "Building an Orthonormal Basis, Revisited"
    float sign = n.z >= 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float bb = n.x * n.y * a;
    *t = mk3(1.0f + sign * n.x * n.x * a, sign * bb, -sign * n.x);
    *b = mk3(bb, sign + n.y * n.y * a, -n.y);
}
__device__ __forceinline__ float ggx_lambda(float alpha, float cos_t) {
    float c2 = cos_t * cos_t;
    float t2 = fmaxf(0.0f, 1.0f - c2) / fmaxf(c2, 1e-12f);
    return 0.5f * (-1.0f + sqrtf(1.0f + alpha * alpha * t2));
}
__device__ __forceinline__ float ggx_d(float alpha, float cos_h) {
    float a2 = alpha * alpha;
    float c2 = cos_h * cos_h;
    float den = c2 * (a2 - 1.0f) + 1.0f;
    return a2 / (kPi * den * den);
}
// Sample wi for wo (both in the local frame, z = normal); returns the weight f*cos/pdf.
__device__ __forceinline__ bool ggx_sample(f3 wo, float alpha, f3 f0, float r1, float r2, f3 *wi_out, f3 *weight,
                                           float *pdf_out, float *mz_out = nullptr, float *fw_out = nullptr) {
    // stretch
    f3 vh = normalize(mk3(alpha * wo.x, alpha * wo.y, wo.z));
    float lensq = vh.x * vh.x + vh.y * vh.y;
    f3 t1 = lensq > 0.0f ? mk3(-vh.y, vh.x, 0.0f) / sqrtf(lensq) : mk3(1.0f, 0.0f, 0.0f);
    f3 t2 = cross(vh, t1);
    float r = sqrtf(r1);
    float phi = 2.0f * kPi * r2;
    float sp, cp;
    dm_sincos(phi, &sp, &cp);
    float p1 = r * cp;
    float p2 = r * sp;
    float s = 0.5f * (1.0f + vh.z);
    p2 = (1.0f - s) * sqrtf(fmaxf(0.0f, 1.0f - p1 * p1)) + s * p2;
    f3 nh = (p1 * t1 + p2 * t2) + sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2)) * vh;
    f3 m = normalize(mk3(alpha * nh.x, alpha * nh.y, fmaxf(1e-6f, nh.z)));
    float wo_m = dot(wo, m);
    f3 wi = (2.0f * wo_m) * m - wo;
    if (wi.z <= 0.0f) return false;
    float l_o = ggx_lambda(alpha, wo.z), l_i = ggx_lambda(alpha, wi.z);
    float g1 = 1.0f / (1.0f + l_o);
    float g2 = 1.0f / ((1.0f + l_o) + l_i);
    float fw = dm_pow(1.0f - fmaxf(0.0f, wo_m), 5.0f);
    f3 F = f0 + fw * (mk3(1.0f, 1.0f, 1.0f) - f0);
    *weight = (g2 / g1) * F;
    // pdf(wi) = D_v(m) / (4 wo.m) = G1(wo) max(0, wo.m) D(m) / (wo.z 4 wo.m)
    *pdf_out = g1 * ggx_d(alpha, m.z) / (4.0f * wo.z);
    *wi_out = wi;
    if (mz_out) *mz_out = m.z;
    if (fw_out) *fw_out = fw;
    return true;
}
__device__ __forceinline__ f3 ggx_eval(f3 wo, f3 wi, float alpha, f3 f0, float *pdf_out, float *mz_out = nullptr,
                                       float *fw_out = nullptr) {
    // returns f * cos(wi)
    *pdf_out = 0.0f;
    if (wo.z <= 0.0f || wi.z <= 0.0f) return mk3(0.0f, 0.0f, 0.0f);
    f3 m = normalize(wo + wi);
    float l_o = ggx_lambda(alpha, wo.z), l_i = ggx_lambda(alpha, wi.z);
    float g1 = 1.0f / (1.0f + l_o);
    float g2 = 1.0f / ((1.0f + l_o) + l_i);
    float D = ggx_d(alpha, m.z);
    float wo_m = dot(wo, m);
    float fw = dm_pow(1.0f - fmaxf(0.0f, wo_m), 5.0f);
    f3 F = f0 + fw * (mk3(1.0f, 1.0f, 1.0f) - f0);
    *pdf_out = g1 * D / (4.0f * wo.z);
    if (mz_out) *mz_out = m.z;
    if (fw_out) *fw_out = fw;
    return (D * g2 / (4.0f * wo.z)) * F;
}

// d log(D(m) G2(wo, wi)) / d alpha: the roughness derivative of log(f cos) of
// the GGX lobe (the Fresnel term does not depend on alpha).
//   d log D / d a  = 2/a - 4 a c^2 / (c^2 (a^2 - 1) + 1),   c = m.z
//   d log G2 / d a = -(dL(wo) + dL(wi)) / (1 + L(wo) + L(wi)),
//   dL/da = a t^2 / (2 sqrt(1 + a^2 t^2)),  t^2 = tan^2 of the direction.
__device__ __forceinline__ float ggx_dlog_dalpha(float alpha, float mz, float cos_o, float cos_i) {
    float c2 = mz * mz;
    float den = c2 * (alpha * alpha - 1.0f) + 1.0f;
    float dlog_d = 2.0f / alpha - 4.0f * alpha * c2 / den;
    auto lam = [&](float c, float *dl) {
        float cc = c * c;
        float t2 = fmaxf(0.0f, 1.0f - cc) / fmaxf(cc, 1e-12f);
        float sq = sqrtf(1.0f + alpha * alpha * t2);
        *dl = 0.5f * alpha * t2 / sq;
        return 0.5f * (sq - 1.0f);
    };
    float dlo, dli;
    float lo = lam(cos_o, &dlo), li = lam(cos_i, &dli);
    return dlog_d - (dlo + dli) / ((1.0f + lo) + li);
}

// Texture factor of a material at a hit (material_albedo = factor * albedo).
__device__ __forceinline__ f3 material_tex(const DeviceScene &S, const mcrt_gpu_material &m, f3 p, float4 h) {
    uint32_t layer = m.type_pad[1];
    if (layer == 0u || S.albedo_layers == 0u) return mk3(1.0f, 1.0f, 1.0f);
    float u, v;
    hit_uv(S, p, h, &u, &v);
    return sample_albedo(S, min(layer, S.albedo_layers - 1u), u, v);
}
__device__ __forceinline__ float safe_ratio(float a, float b) { return b != 0.0f ? a / b : 0.0f; }

// ------------------------------------------------------------------ light sampling (NEE)
// Lights are the emissive triangles (by original id) and emissive spheres (by
// ordered slot | MCRT_HIT_SPHERE).  A light is chosen with probability
// proportional to area * luminance(emission); the same weight function is
// evaluated when a BSDF-sampled ray hits an emitter, for the MIS weight.
__device__ __forceinline__ float luminance(f3 c) { return (0.2126f * c.x + 0.7152f * c.y) + 0.0722f * c.z; }

__device__ __forceinline__ f3 emission_of(const DeviceScene &S, uint32_t mat) {
    const mcrt_gpu_material &m = S.materials->materials[min(mat, kMaxMatIdx)];
    if (m.type_pad[0] != kMatEmissive) return mk3(0.0f, 0.0f, 0.0f);
    return m.ior_pad[0] * ld3(m.albedo_fuzz);
}

}  // namespace

__device__ float light_weight(const DeviceScene &S, uint32_t code) {
    if (code & MCRT_HIT_SPHERE) {
        uint32_t slot = code & ~MCRT_HIT_SPHERE;
        float r = S.spheres[slot].center_r[3];
        return ((4.0f * kPi) * (r * r)) * luminance(emission_of(S, S.spheres[slot].mat_and_pad[0]));
    }
    mcrt_gpu_triangle tri = S.triangles[code];
    f3 a = ld3(S.vertices[tri.v[0]].position), b = ld3(S.vertices[tri.v[1]].position),
       c = ld3(S.vertices[tri.v[2]].position);
    f3 ng = cross(b - a, c - a);
    return (0.5f * sqrtf(dot(ng, ng))) * luminance(emission_of(S, tri.mat_idx & 0x7fffffffu));
}

namespace {

__device__ __forceinline__ uint32_t pick_light(const DeviceScene &S, float u) {
    uint32_t lo = 0, hi = S.n_lights;               // largest k with cdf[k] <= u
    while (lo + 1 < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(S.light_cdf + mid) <= u) lo = mid; else hi = mid;
    }
    return lo;
}

struct LightSample { f3 dir; float dist; float pdf; f3 Le; uint32_t mat; bool ok; bool delta; };

// Probability of choosing among the area lights: with a directional light as
// well, each kind is chosen with probability 1/2.
__device__ __forceinline__ float area_light_selection(const DeviceScene &S) {
    return (S.has_sun && S.n_lights > 0) ? 0.5f : 1.0f;
}

// Uniform point on an emissive triangle, or a direction in the cone subtended by
// an emissive sphere.  pdf is per unit solid angle at x (including the choice of
// the light).  The directional light is a delta light: pdf is its selection
// probability, dist reaches past the scene, and no MIS applies.
__device__ __forceinline__ LightSample sample_light(const DeviceScene &S, f3 x, uint32_t &rng) {
    LightSample ls{};
    ls.ok = false;
    ls.delta = false;
    const float sel = area_light_selection(S);
    if (S.has_sun) {
        const bool sun = S.n_lights == 0 || rand_f32(rng) < 0.5f;
        if (sun) {
            ls.dir = xyz(S.sun_dir);
            ls.dist = kTMax;
            ls.pdf = sel;
            ls.Le = xyz(S.sun_E);
            ls.mat = 0xffu;
            ls.ok = true;
            ls.delta = true;
            return ls;
        }
    }
    uint32_t li = pick_light(S, rand_f32(rng));
    uint32_t code = __ldg(S.lights + li);
    float prob = sel * (light_weight(S, code) / S.light_total);
    float r1 = rand_f32(rng), r2 = rand_f32(rng);
    if (!(prob > 0.0f)) return ls;
    if (code & MCRT_HIT_SPHERE) {
        uint32_t slot = code & ~MCRT_HIT_SPHERE;
        float4 cr = __ldg(reinterpret_cast<const float4 *>(S.spheres + slot));
        f3 wc = xyz(cr) - x;
        float d2 = dot(wc, wc);
        float r2s = cr.w * cr.w;
        if (d2 <= r2s) return ls;
        float dc = sqrtf(d2);
        f3 w = wc / dc;
        float cosmax = sqrtf(fmaxf(0.0f, 1.0f - r2s / d2));
        if (!(cosmax < 1.0f)) return ls;
        float cos_t = (1.0f - r1) + r1 * cosmax;
        float sin_t = sqrtf(fmaxf(0.0f, 1.0f - cos_t * cos_t));
        float sp, cp;
        dm_sincos(kTau * r2, &sp, &cp);
        f3 t, b;
        onb(w, &t, &b);
        f3 dir = normalize(((sin_t * cp) * t + (sin_t * sp) * b) + cos_t * w);
        float proj = dot(wc, dir);
        float disc = r2s - (d2 - proj * proj);
        float dist = proj - sqrtf(fmaxf(0.0f, disc));
        ls.dir = dir;
        ls.dist = dist;
        ls.pdf = prob / (kTau * (1.0f - cosmax));
        ls.mat = min(S.spheres[slot].mat_and_pad[0], kMaxMatIdx);
        ls.Le = emission_of(S, S.spheres[slot].mat_and_pad[0]);
        ls.ok = dist > 0.0f;
        return ls;
    }
    mcrt_gpu_triangle tri = S.triangles[code];
    f3 a = ld3(S.vertices[tri.v[0]].position), bq = ld3(S.vertices[tri.v[1]].position),
       cq = ld3(S.vertices[tri.v[2]].position);
    float su = sqrtf(r1);
    float b0 = 1.0f - su, b1 = r2 * su, b2 = (1.0f - b0) - b1;
    f3 y = (b0 * a + b1 * bq) + b2 * cq;
    f3 ng = cross(bq - a, cq - a);
    float area2 = sqrtf(dot(ng, ng));
    if (!(area2 > 0.0f)) return ls;
    f3 wv = y - x;
    float dist2 = dot(wv, wv);
    float dist = sqrtf(dist2);
    if (!(dist > 0.0f)) return ls;
    f3 dir = wv / dist;
    float cos_l = fabsf(dot(ng, dir)) / area2;
    if (!(cos_l > 1e-7f)) return ls;
    if (tri.mat_idx & MCRT_BACKFACE_CULL_FLAG) {        // invisible from behind (path_trace.wgsl:452)
        f3 ns = tri_shading_normal(S, code, b1, b2);
        if (!(dot(dir, ns) < 0.0f)) return ls;
    }
    ls.dir = dir;
    ls.dist = dist;
    ls.pdf = prob * dist2 / (cos_l * (0.5f * area2));
    ls.mat = min(tri.mat_idx & 0x7fffffffu, kMaxMatIdx);
    ls.Le = emission_of(S, tri.mat_idx & 0x7fffffffu);
    ls.ok = true;
    return ls;
}

// Solid-angle pdf (at the ray origin o) with which NEE would have produced the
// emitter hit h along d.
__device__ __forceinline__ float light_pdf_of_hit(const DeviceScene &S, float4 h, f3 o, f3 d) {
    uint32_t prim = __float_as_uint(h.y);
    const float sel = area_light_selection(S);
    if (prim & MCRT_HIT_SPHERE) {
        uint32_t slot = __float_as_uint(h.z);
        float prob = sel * (light_weight(S, slot | MCRT_HIT_SPHERE) / S.light_total);
        float4 cr = __ldg(reinterpret_cast<const float4 *>(S.spheres + slot));
        f3 wc = xyz(cr) - o;
        float d2 = dot(wc, wc);
        float r2s = cr.w * cr.w;
        if (d2 <= r2s) return 0.0f;
        float cosmax = sqrtf(fmaxf(0.0f, 1.0f - r2s / d2));
        if (!(cosmax < 1.0f)) return 0.0f;
        return prob / (kTau * (1.0f - cosmax));
    }
    float prob = sel * (light_weight(S, prim) / S.light_total);
    mcrt_gpu_triangle tri = S.triangles[prim];
    f3 a = ld3(S.vertices[tri.v[0]].position), bq = ld3(S.vertices[tri.v[1]].position),
       cq = ld3(S.vertices[tri.v[2]].position);
    f3 ng = cross(bq - a, cq - a);
    float area2 = sqrtf(dot(ng, ng));
    if (!(area2 > 0.0f)) return 0.0f;
    float cos_l = fabsf(dot(ng, d)) / area2;
    if (!(cos_l > 1e-7f)) return 0.0f;
    float t = h.x;
    return prob * (t * t) / (cos_l * (0.5f * area2));
}

}  // namespace

// ------------------------------------------------------------------ kernels

__global__ void k_trace_closest(DeviceScene S, const mcrt_ray *rays, uint32_t n, mcrt_hit *hits, int ref_layout) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    mcrt_ray ry = rays[i];
    RayInv r = make_ray(mk3(ry.org[0], ry.org[1], ry.org[2]), mk3(ry.dir[0], ry.dir[1], ry.dir[2]));
    uint32_t nn = 0;
    Closest c = world_hit(S, r, ry.tmin, ry.tmax, ref_layout != 0, &nn);
    mcrt_hit h;
    h.t = c.t;
    h.prim = c.prim;
    h.u = c.u;
    h.v = c.v;
    hits[i] = h;
}

__global__ void k_raygen(DeviceScene S, RenderParams P, PathBuffers B, int keep_radiance) {
    uint32_t n = P.npix * P.spp_pass;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        B.counters[0] = n; B.counters[1] = 0; B.counters[2] = 0; B.counters[3] = 0; B.counters[4] = 0;
        B.counters[5] = 0; B.counters[6] = 0; B.counters[7] = 0;
    }
    if (i >= n) return;
    if (P.cache_query_vertex && i % P.train_stride == 0u) {        // training path: no vertex recorded yet
        float4 *rec = P.train_records + (size_t)(i / P.train_stride) * P.max_depth * kTrainRecordFloat4;
        for (uint32_t j = 0; j < P.max_depth; ++j) rec[(size_t)j * kTrainRecordFloat4].w = 0.0f;
    }
    uint32_t p = i / P.spp_pass;
    uint32_t k = i - p * P.spp_pass;
    uint32_t frame = (P.pass_state ? P.pass_state[0] : P.frame0) + k;
    uint32_t x, y, w, h;
    const mcrt_camera_uniform *cam = &P.cam;
    if (P.n_views) {                       // the view holding pixel p: largest v with view_px[v] <= p
        uint32_t lo = 0, hi = P.n_views;
        while (lo + 1 < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (__ldg(P.view_px + mid) <= p) lo = mid; else hi = mid;
        }
        const uint2 wh = __ldg(P.view_wh + lo);
        const uint32_t lp = p - __ldg(P.view_px + lo);
        w = wh.x; h = wh.y;
        x = lp % w; y = lp / w;
        cam = P.view_cam + lo;
    } else {
        w = P.w; h = P.h;
        x = p % w; y = p / w;
    }
    uint32_t rng = pcg_hash(pcg_hash(x + y * w) ^ (frame * 2654435761u));   // path_trace.wgsl:636-637
    f3 o, d;
    camera_ray(*cam, x, y, w, h, rng, &o, &d);
    B.thr[i] = make_float4(1.0f, 1.0f, 1.0f, -1.0f);
    if (!keep_radiance) B.L[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (keep_radiance) B.pend_mat[i] = 0u;
    // the path's random state travels with its ray (the direction's w)
    B.q_o[0][i] = make_float4(o.x, o.y, o.z, __uint_as_float(i));
    B.q_d[0][i] = make_float4(d.x, d.y, d.z, __uint_as_float(rng));
}

// Closest hit for the queued rays: persistent warps with dynamic ray refill and
// speculative while-while traversal of the compact BVH.
//  * A warp fetches rays for its idle lanes in batches (one atomicAdd on the
//    work counter counters[4] per batch) whenever at least kRefill lanes are
//    idle, so lanes do not sit out the longest ray of a fixed assignment.
//  * Traversal phase: a lane walks internal nodes; a leaf it reaches is
//    postponed and the lane keeps traversing until every active lane of the
//    warp holds a postponed leaf (warp vote); then the lanes test their leaves
//    together.  The vote only shapes scheduling: every order enters every box
//    that can hold a hit at or before the closest t (the cull's slack,
//    kCullSlack), so the hit is the reference order's.
// Sphere BVHs (the reference's binding 5) are traversed at ray fetch with the
// reference-order walk (spheres_hit); their count is small.

// Closest-hit kernel variants, chosen per scene by mcrt_autotune: BVH width
// (compact binary or quantised 4-wide), block size, minimum resident blocks per
// SM (the register budget ptxas must meet), traversal stack depth (entries of 8
// bytes in local memory; a ray that would overflow it leaves the kernel's queue
// for the overflow list, whose rays k_extend_retry traces without a stack, so
// a short stack costs time on a deep tree but never a wrong or missing hit)
// and the number of idle lanes at which a warp fetches new rays, and whether
// the block stages the top 7 levels of the compact tree in shared memory
// (top = kTopNodes records, 8 KB per block, loaded once per block; the nodes
// below are read through L1 as in the other variants).
struct ExtendVariant { int width, block, min_blocks, stack, refill, top; };
constexpr int kExtendVariants = 8;
constexpr ExtendVariant kVariantTable[kExtendVariants] = {
    {2, 128, 8, 64, 8, 0},  {2, 64, 20, 32, 8, 0},  {2, 64, 20, 32, 4, 0},   {2, 128, 10, 32, 8, (int)kTopNodes},
    {2, 64, 18, 32, 8, (int)kTopNodes}, {4, 128, 8, 64, 8, 0}, {2, 128, 10, 32, 8, 0}, {2, 64, 18, 32, 8, 0}};

// Visit an internal node of the compact binary layout: test both children,
// continue with the nearer hit child, push the farther one.  TOP: a code with
// kTopBit is an entry of the top tree staged in shared memory (s_top).
template <int STACK, int TOP>
__device__ __forceinline__ void visit_compact2(const DeviceScene &S, const float4 *s_top, const RayInv &r,
                                               float tmax, uint32_t *cur, float *cur_t, uint2 *stack, uint32_t *sp,
                                               bool *overflow) {
    float4 a, b, c;
    uint4 e;
    if (TOP > 0 && (*cur & kTopBit)) {
        const float4 *np = s_top + 4u * (*cur & ~kTopBit);
        a = np[0]; b = np[1]; c = np[2];
        e = *reinterpret_cast<const uint4 *>(np + 3);
    } else {
        const float4 *np = S.cnodes + 4ull * *cur;
        a = __ldg(np); b = __ldg(np + 1); c = __ldg(np + 2);
        e = __ldg(reinterpret_cast<const uint4 *>(np + 3));
    }
    float tl, tr;
    bool hl = e.x != kNoChild && slab(r, a.x, a.z, c.x, a.y, a.w, c.y, kTMin, tmax, &tl);
    bool hr = e.y != kNoChild && slab(r, b.x, b.z, c.z, b.y, b.w, c.w, kTMin, tmax, &tr);
    if (hl && hr) {
        uint32_t near = e.x, far = e.y;
        float tnear = tl, tfar = tr;
        if (tr < tl) { near = e.y; far = e.x; tnear = tr; tfar = tl; }
        if (*sp < (uint32_t)STACK) stack[(*sp)++] = make_uint2(far, __float_as_uint(tfar));
        else *overflow = true;
        *cur = near;
        *cur_t = tnear;
    } else if (hl) {
        *cur = e.x; *cur_t = tl;
    } else if (hr) {
        *cur = e.y; *cur_t = tr;
    } else {
        *cur = kNoChild;
    }
}

// Visit a quantised 4-wide node: slab-test each child box on the node's grid,
// order the hits by entry distance with a sorting network on (distance bits,
// child) keys, continue with the nearest and push the others farthest first.
// A plane origin + q * step (the builder guarantees that the exact real value
// lies outside the child box) is at distance q * a + b along the ray, with
// a = step * inv exact (step is a power of two) and b = (origin - o) * inv
// computed once per node and axis.  b carries two roundings, at most
// 2^-23 |b|; scaled by 1 -+ 2^-22 it becomes a bound from below for the plane
// that gives the entry on that axis and from above for the exit, so each
// child's fma(q, a, b) interval contains the exact one up to the fma's own
// relative rounding, which the cull's slack covers (as for slab()).
template <int STACK>
__device__ __forceinline__ void visit_wide4(const DeviceScene &S, const RayInv &r, float tmax, uint32_t *cur,
                                            float *cur_t, uint2 *stack, uint32_t *sp, bool *overflow) {
    const uint4 *np = S.wnodes + 4ull * *cur;
    const uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3);
    const float org[3] = {__uint_as_float(w0.x), __uint_as_float(w0.y), __uint_as_float(w0.z)};
    const float inv[3] = {r.inv.x, r.inv.y, r.inv.z}, o[3] = {r.o.x, r.o.y, r.o.z};
    float a[3], blo[3], bhi[3];                     // b bounds for the low and the high planes
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a[k] = __uint_as_float(((w0.w >> (8 * k)) & 0xffu) << 23) * inv[k];
        const float b = (org[k] - o[k]) * inv[k];
        const float p = b * 0.99999976158142089844f, q = b * 1.0000002384185791016f;   // b (1 -+ 2^-22)
        const float dn = fminf(p, q), up = fmaxf(p, q);
        blo[k] = inv[k] >= 0.0f ? dn : up;          // inv >= 0: the low plane is the entry
        bhi[k] = inv[k] >= 0.0f ? up : dn;
    }
    const uint32_t refs[4] = {w3.x, w3.y, w3.z, w3.w};
    // the byte j of a word as a float: 0x4B0000bb is 2^23 + byte, exactly
    auto qf = [](uint32_t w, uint32_t sel) { return __uint_as_float(__byte_perm(w, 0x4B000000u, sel)) - 8388608.0f; };
    const float reach = cull_t(tmax);
    // key = entry distance bits (non-negative floats order as integers) with the
    // child index in the two low bits: the distance loses at most 3 ulp
    // downward, which only makes the later cull (distance <= closest t) looser.
    uint32_t key[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        key[j] = 0xffffffffu;
        if (refs[j] == kNoChild) continue;
        const uint32_t sel = 0x7440u + (uint32_t)j;
        const float t0x = fmaf(qf(w1.x, sel), a[0], blo[0]), t1x = fmaf(qf(w1.w, sel), a[0], bhi[0]);
        const float t0y = fmaf(qf(w1.y, sel), a[1], blo[1]), t1y = fmaf(qf(w2.x, sel), a[1], bhi[1]);
        const float t0z = fmaf(qf(w1.z, sel), a[2], blo[2]), t1z = fmaf(qf(w2.y, sel), a[2], bhi[2]);
        const float te = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
        const float tx = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
        if (cull_t(tx) > fmaxf(te, kTMin) && te <= reach)
            key[j] = (__float_as_uint(fmaxf(te, 0.0f)) & ~3u) | (uint32_t)j;
    }
    auto cx = [](uint32_t &a, uint32_t &b) {
        uint32_t lo = min(a, b), hi = max(a, b);
        a = lo; b = hi;
    };
    cx(key[0], key[1]); cx(key[2], key[3]); cx(key[0], key[2]); cx(key[1], key[3]); cx(key[1], key[2]);
    auto ref_of = [&](uint32_t k) {
        uint32_t j = k & 3u;
        return j == 0 ? refs[0] : (j == 1 ? refs[1] : (j == 2 ? refs[2] : refs[3]));
    };
#pragma unroll
    for (int j = 3; j >= 1; --j) {
        if (key[j] == 0xffffffffu) continue;
        if (*sp < (uint32_t)STACK) stack[(*sp)++] = make_uint2(ref_of(key[j]), key[j] & ~3u);
        else *overflow = true;
    }
    if (key[0] == 0xffffffffu) {
        *cur = kNoChild;
    } else {
        *cur = ref_of(key[0]);
        *cur_t = __uint_as_float(key[0] & ~3u);
    }
}

// The end of a traced queue entry.  Closest hit: the hit record, in queue
// order.  Any hit (a shadow ray of path `slot`): an unoccluded ray adds its
// contribution to the path's radiance; ADJ: the adjoint replay's shadow ray,
// whose next-event term N leaves the radiance still ahead of its path
// (B.L -= N) and contributes delta * N * dlog(f)/d(params) to its vertex's
// material and delta * N / albedo to the emitter's radiance colour, collected
// in the block's shared gacc.
template <bool ANY, bool ADJ>
__device__ __forceinline__ void finish_ray(const DeviceScene &S, const PathBuffers &B, const AdjointParams &A,
                                           float *gacc, uint32_t ray, uint32_t slot, bool occl, Closest best) {
    if (ANY) {
        if (occl) return;
        const float4 c = B.sh_c[ray];              // one shadow ray per path and bounce: no race on L
        const float4 L = B.L[slot];
        if (!ADJ) {
            B.L[slot] = make_float4(L.x + c.x, L.y + c.y, L.z + c.z, 0.0f);
            return;
        }
        B.L[slot] = make_float4(L.x - c.x, L.y - c.y, L.z - c.z, 0.0f);
        auto gadd = [&](uint32_t k, float v) {
            if (v != 0.0f) atomicAdd(&gacc[k], v);
        };
        const uint32_t bits = __float_as_uint(c.w);
        const uint32_t mi = bits & 0xffu, lm = (bits >> 8) & 0xffu;
        const float4 di = A.dimg[slot / A.planes];
        const f3 dn = (A.inv_spp * xyz(di)) * xyz(c);
        const float4 g = B.sh_g[ray];
        gadd(4u * mi + 0, dn.x * g.x);
        gadd(4u * mi + 1, dn.y * g.y);
        gadd(4u * mi + 2, dn.z * g.z);
        gadd(4u * mi + 3, ((dn.x + dn.y) + dn.z) * g.w);
        if (lm <= kMaxMatIdx) {                    // not the directional light
            const float *la = S.materials->materials[lm].albedo_fuzz;
            gadd(4u * lm + 0, safe_ratio(dn.x, la[0]));
            gadd(4u * lm + 1, safe_ratio(dn.y, la[1]));
            gadd(4u * lm + 2, safe_ratio(dn.z, la[2]));
        }
    } else {
        if (best.prim == MCRT_HIT_MISS) best.t = -1.0f;
        float u = (best.prim != MCRT_HIT_MISS && (best.prim & MCRT_HIT_SPHERE)) ? __uint_as_float(best.slot) : best.u;
        __stcs(B.hits + ray, make_float4(best.t, __uint_as_float(best.prim), u, best.v));
    }
}

// Overflow lists of the closest-hit and the any-hit launches: counters[3] and
// counters[7] count the queue entries in B.ovf that k_extend_retry traces.
// The closest-hit list is cleared by the shading kernel, the any-hit list by
// the next closest-hit launch (neither runs while the list is in use).
constexpr uint32_t kOvfClosest = 3u, kOvfAny = 7u;

// ANY = true: the same persistent, refilled, speculative traversal for the
// shadow-ray queue of next-event estimation, as an any-hit test: the cull
// threshold stays the ray's t_max, so the set of boxes entered does not depend
// on the visit order, and any accepted triangle hit in it (leaf_any) proves
// the ray occluded, the answer of the closest-hit test; an unoccluded ray
// adds its contribution to its path's radiance.
// ADJ (with ANY): the adjoint replay's shadow rays (finish_ray), their
// gradients collected in shared memory per block and added once per block.
// A ray whose next push would overflow the stack stops here and joins the
// overflow list (finished by k_extend_retry).
// COUNT: the traversal's own record fetches, for the bytes-per-ray model of
// the kernel (outside timed runs): stats[3] += internal nodes visited (one
// 64-byte record each, those of the shared-memory top tree included),
// stats[4] += triangles tested (one 48-byte record each).
// TOP > 0 (binary layout): the block first copies the top tree (S.top, TOP
// records) into shared memory and starts every ray at its entry 0.
template <int WIDTH, int BLOCK, int MINB, int STACK, int REFILL, int TOP, bool ANY, bool ADJ, bool COUNT = false>
__global__ void __launch_bounds__(BLOCK, MINB) k_extend(DeviceScene S, PathBuffers B, int qi, AdjointParams A) {
    __shared__ float gacc[ADJ ? 256 : 1];
    __shared__ float4 s_top[TOP > 0 ? 4 * TOP : 1];
    if (ADJ) {
        for (uint32_t k = threadIdx.x; k < 256u; k += BLOCK) gacc[k] = 0.0f;
    }
    if constexpr (TOP > 0) {
        for (uint32_t k = threadIdx.x; k < 4u * TOP; k += BLOCK) s_top[k] = __ldg(S.top + k);
    }
    if (ADJ || TOP > 0) __syncthreads();
    const uint32_t n = ANY ? B.counters[2] : B.counters[qi];
    if (!ANY && blockIdx.x == 0 && threadIdx.x == 0) {
        B.counters[qi ^ 1] = 0; B.counters[2] = 0; B.counters[kOvfAny] = 0;
    }
    const float4 *qo = ANY ? B.sh_o : B.q_o[qi];
    const float4 *qd = ANY ? B.sh_d : B.q_d[qi];
    uint32_t *work = B.counters + (ANY ? 5 : 4);    // the queue's next unclaimed entry
    const uint32_t lane = threadIdx.x & 31u;
    const bool has_mesh = S.n_mesh_nodes > 0;
    uint32_t ray = 0xffffffffu;       // queue index of the lane's ray, or none
    bool exhausted = false;           // the queue has been handed out (warp-uniform)
    RayInv r;
    Closest best;
    uint2 stack[STACK];
    uint32_t sp = 0;
    uint32_t cur = kNoChild;          // next node code to visit
    float cur_t = 0.0f;               // its entry distance
    uint32_t leaf = kNoChild;         // postponed leaf code
    uint32_t traced = 0;
    uint32_t nn = 0;
    uint32_t ntri = 0;                // COUNT: triangles tested
    uint32_t slot = 0;                // ANY: the shadow ray's path
    bool occl = false;                // ANY: an accepted hit was found
    // a ray whose stack would overflow keeps its queue index with bit 31 set
    // (indices are below 2^31) until it joins the overflow list
    constexpr uint32_t kOvfBit = 0x80000000u;
    for (;;) {
        // ---- refill idle lanes
        const bool idle = ray == 0xffffffffu;
        const unsigned idle_mask = __ballot_sync(0xffffffffu, idle);
        if (!exhausted && (__popc(idle_mask) >= REFILL || idle_mask == 0xffffffffu)) {
            const int leader = __ffs(idle_mask) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(work, (uint32_t)__popc(idle_mask));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base + (uint32_t)__popc(idle_mask) >= n) exhausted = true;
            if (idle) {
                const uint32_t mine = base + __popc(idle_mask & ((1u << lane) - 1u));
                if (mine < n) {
                    ray = mine;
                    float4 o4 = __ldcs(qo + mine), d4 = __ldcs(qd + mine);   // streamed: evict first
                    r = make_ray(xyz(o4), xyz(d4));
                    const float tmax = ANY ? d4.w : kTMax;
                    best = Closest{tmax, MCRT_HIT_MISS, 0u, 0.0f, 0.0f};
                    spheres_hit(S, r, kTMin, tmax, best, &nn);       // path_trace.wgsl:472-474
                    sp = 0;
                    leaf = kNoChild;
                    cur = kNoChild;
                    if (ANY) {
                        slot = __float_as_uint(o4.w);
                        occl = best.prim != MCRT_HIT_MISS;
                        best.t = tmax;
                    }
                    if (has_mesh && !(ANY && occl)) {
                        const float4 *np = reinterpret_cast<const float4 *>(S.mesh_nodes);
                        float4 mn = __ldg(np), mx = __ldg(np + 1);
                        float te;
                        if (slab(r, mn.x, mn.y, mn.z, mx.x, mx.y, mx.z, kTMin, best.t, &te)) {
                            if (S.n_cnodes == 0) {
                                uint4 meta = __ldg(reinterpret_cast<const uint4 *>(np + 2));
                                cur = leaf_code(meta.x, meta.y);
                            } else {
                                cur = TOP > 0 ? kTopBit : 0u;
                            }
                            cur_t = te;
                        }
                    }
                }
            }
        }
        if (__ballot_sync(0xffffffffu, ray != 0xffffffffu) == 0) break;   // exhausted and all idle
        if (ray != 0xffffffffu) {
            // ---- traversal phase
            for (;;) {
                if (cur != kNoChild && cur_t > cull_t(best.t)) cur = kNoChild;   // culled since it was queued
                if (cur == kNoChild) {                                        // pop the next live entry
                    while (sp > 0) {
                        uint2 s = stack[--sp];
                        if (__uint_as_float(s.y) <= cull_t(best.t)) { cur = s.x; cur_t = __uint_as_float(s.y); break; }
                    }
                    if (cur == kNoChild) break;
                }
                if (cur & kLeafBit) {
                    if (leaf != kNoChild) break;                              // one leaf already waits
                    leaf = cur;
                    cur = kNoChild;
                    continue;
                }
                ++nn;
                bool full = false;
                if (WIDTH == 4) visit_wide4<STACK>(S, r, best.t, &cur, &cur_t, stack, &sp, &full);
                else visit_compact2<STACK, TOP>(S, s_top, r, best.t, &cur, &cur_t, stack, &sp, &full);
                if (full) {                                                   // to the overflow list
                    ray |= kOvfBit;
                    cur = kNoChild;
                    sp = 0;
                    leaf = kNoChild;
                    break;
                }
                if (__all_sync(__activemask(), leaf != kNoChild)) break;
            }
            // ---- leaf phase
            while (leaf != kNoChild) {
                if (ANY) {
                    if (leaf_any(S, r, (leaf & ~kLeafBit) >> 4, leaf_count(S, leaf), kTMin, best.t)) {
                        occl = true;                                          // done: drop what is left
                        cur = kNoChild;
                        sp = 0;
                    }
                } else {
                    const uint32_t cnt = leaf_count(S, leaf);
                    if (COUNT) ntri += cnt;
                    leaf_tris(S, r, (leaf & ~kLeafBit) >> 4, cnt, kTMin, best);
                }
                leaf = kNoChild;
                if (cur != kNoChild && (cur & kLeafBit) && cur_t <= cull_t(best.t)) {
                    leaf = cur;
                    cur = kNoChild;
                }
            }
            // ---- finished ray
            if (cur == kNoChild && sp == 0) {
                if (ray & kOvfBit) {
                    B.ovf[atomicAdd(B.counters + (ANY ? kOvfAny : kOvfClosest), 1u)] = ray & ~kOvfBit;
                } else {
                    finish_ray<ANY, ADJ>(S, B, A, gacc, ray, slot, occl, best);
                    ++traced;
                }
                ray = 0xffffffffu;
            }
        }
    }
    if (traced) atomicAdd(B.stats + (ANY ? 1 : 0), (unsigned long long)traced);
    if (COUNT) {
        atomicAdd(B.stats + 3, (unsigned long long)nn);
        atomicAdd(B.stats + 4, (unsigned long long)ntri);
    }
    if (ADJ) {
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < 256u; k += BLOCK) {
            const float v = gacc[k];
            if (v != 0.0f) atomicAdd(A.grad + k, (double)v);
        }
    }
}

// The overflow list of the preceding closest-hit (ANY = false) or any-hit
// launch: each ray traced again from the start, spheres first, with the
// stackless walk, and finished as k_extend would (finish_ray).  Launched
// after every extend launch; with an empty list its threads return at once.
// stats[2] counts the rays it traced.
constexpr int kRetryBlock = 128;
template <bool ANY, bool ADJ>
__global__ void __launch_bounds__(kRetryBlock) k_extend_retry(DeviceScene S, PathBuffers B, int qi, AdjointParams A) {
    __shared__ float gacc[ADJ ? 256 : 1];
    if (ADJ) {
        for (uint32_t k = threadIdx.x; k < 256u; k += kRetryBlock) gacc[k] = 0.0f;
        __syncthreads();
    }
    const uint32_t n = B.counters[ANY ? kOvfAny : kOvfClosest];
    const float4 *qo = ANY ? B.sh_o : B.q_o[qi];
    const float4 *qd = ANY ? B.sh_d : B.q_d[qi];
    uint32_t traced = 0, nn = 0;
    for (uint32_t i = blockIdx.x * kRetryBlock + threadIdx.x; i < n; i += gridDim.x * kRetryBlock) {
        const uint32_t ray = B.ovf[i];
        const float4 o4 = __ldcs(qo + ray), d4 = __ldcs(qd + ray);
        const RayInv r = make_ray(xyz(o4), xyz(d4));
        const float tmax = ANY ? d4.w : kTMax;
        Closest best{tmax, MCRT_HIT_MISS, 0u, 0.0f, 0.0f};
        spheres_hit(S, r, kTMin, tmax, best, &nn);
        bool occl = false;
        const uint32_t slot = __float_as_uint(o4.w);
        if (ANY) {
            occl = best.prim != MCRT_HIT_MISS;
            best.t = tmax;
            if (!occl) occl = mesh_walk_stackless<true>(S, r, kTMin, best, &nn);
        } else {
            mesh_walk_stackless<false>(S, r, kTMin, best, &nn);
        }
        finish_ray<ANY, ADJ>(S, B, A, gacc, ray, slot, occl, best);
        ++traced;
    }
    if (traced) {
        atomicAdd(B.stats + (ANY ? 1 : 0), (unsigned long long)traced);
        atomicAdd(B.stats + 2, (unsigned long long)traced);
    }
    if (ADJ) {
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < 256u; k += kRetryBlock) {
            const float v = gacc[k];
            if (v != 0.0f) atomicAdd(A.grad + k, (double)v);
        }
    }
}

// Closest hit for the primary rays (bounce 0), one warp per packet of 32
// consecutive queue entries.  Slots are pixel-major, so a packet holds a pixel's
// samples: nearly the same ray 32 times.  The warp walks one node stream: a
// child is entered when any lane's ray enters its box before that lane's
// closest t (each lane culls with its own), and every lane tests the same
// node and leaf records from one broadcast load, so a packet costs about one
// ray's traversal with all lanes busy.  The set of boxes a lane sees is a
// superset of its own traversal's and every triangle test is exact, so the
// closest hit under the tie rule is the per-ray kernel's.
//  * Near child: the one most lanes enter first.
//  * Stack: distributed over the lanes (entry k in lane k % 32, register
//    k / 32), each entry the child code and the smallest entry distance of the
//    lanes that entered it; popped entries no lane can still reach are dropped.
//    A packet whose stack would overflow joins the overflow list (its rays
//    are traced again by k_extend_retry).
//  * COUNT: the warp's record fetches (one per node or triangle for the whole
//    packet) into stats[3] / stats[4], as k_extend's COUNT.
constexpr int kPacketBlock = 128;
constexpr uint32_t kPacketStack = 64;
template <bool COUNT = false>
__global__ void __launch_bounds__(kPacketBlock) k_extend_packet(DeviceScene S, PathBuffers B, int qi) {
    const uint32_t n = B.counters[qi];
    if (blockIdx.x == 0 && threadIdx.x == 0) { B.counters[qi ^ 1] = 0; B.counters[2] = 0; B.counters[kOvfAny] = 0; }
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = (blockIdx.x * kPacketBlock + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * kPacketBlock) >> 5;
    const bool has_mesh = S.n_mesh_nodes > 0;
    uint32_t traced = 0, nn = 0, nodes = 0, ntri = 0;
    for (uint32_t base = warp * 32u; base < n; base += n_warps * 32u) {
        const uint32_t ray = base + lane;
        const bool active = ray < n;
        RayInv r;
        Closest best{kTMax, MCRT_HIT_MISS, 0u, 0.0f, 0.0f};
        bool want = false;
        if (active) {
            const float4 o4 = __ldcs(B.q_o[qi] + ray), d4 = __ldcs(B.q_d[qi] + ray);
            r = make_ray(xyz(o4), xyz(d4));
            spheres_hit(S, r, kTMin, kTMax, best, &nn);                   // path_trace.wgsl:472-474
            if (has_mesh) {
                const float4 *np = reinterpret_cast<const float4 *>(S.mesh_nodes);
                const float4 mn = __ldg(np), mx = __ldg(np + 1);
                float te;
                want = slab(r, mn.x, mn.y, mn.z, mx.x, mx.y, mx.z, kTMin, best.t, &te);
            }
        }
        uint32_t cur = kNoChild;
        if (__any_sync(0xffffffffu, want)) {
            if (S.n_cnodes == 0) {
                const uint4 meta = __ldg(reinterpret_cast<const uint4 *>(S.mesh_nodes) + 2);
                cur = leaf_code(meta.x, meta.y);
            } else {
                cur = 0;
            }
        }
        uint32_t sn0 = 0, sn1 = 0, st0 = 0, st1 = 0;   // this lane's stack entries k = lane, lane + 32
        uint32_t sp = 0;
        bool ovf = false;                               // warp-uniform
        while (cur != kNoChild) {
            if (cur & kLeafBit) {
                if (COUNT && lane == 0) ntri += leaf_count(S, cur);
                if (active) leaf_tris(S, r, (cur & ~kLeafBit) >> 4, leaf_count(S, cur), kTMin, best);
                cur = kNoChild;
            } else {
                if (COUNT && lane == 0) ++nodes;
                const float4 *np = S.cnodes + 4ull * cur;
                const float4 a = __ldg(np), b = __ldg(np + 1), c = __ldg(np + 2);
                const uint4 e = __ldg(reinterpret_cast<const uint4 *>(np + 3));
                float tl = 0.0f, tr = 0.0f;
                const bool hl = active && e.x != kNoChild && slab(r, a.x, a.z, c.x, a.y, a.w, c.y, kTMin, best.t, &tl);
                const bool hr = active && e.y != kNoChild && slab(r, b.x, b.z, c.z, b.y, b.w, c.w, kTMin, best.t, &tr);
                const uint32_t ml = __ballot_sync(0xffffffffu, hl), mr = __ballot_sync(0xffffffffu, hr);
                if (ml && mr) {
                    const uint32_t pref_r = __ballot_sync(0xffffffffu, hr && (!hl || tr < tl));
                    const bool right_first = 2u * __popc(pref_r) > (uint32_t)__popc(ml | mr);
                    const bool hit_far = right_first ? hl : hr;
                    const float t_far = right_first ? tl : tr;
                    // entry distances >= 0 order as their bits; no lane: +inf
                    const uint32_t key = hit_far ? __float_as_uint(fmaxf(t_far, 0.0f)) : 0x7f800000u;
                    const uint32_t far_t = __reduce_min_sync(0xffffffffu, key);
                    const uint32_t far = right_first ? e.x : e.y;
                    if (sp == kPacketStack) {
                        ovf = true;
                        break;
                    }
                    if (lane == (sp & 31u)) {
                        if (sp < 32u) { sn0 = far; st0 = far_t; } else { sn1 = far; st1 = far_t; }
                    }
                    ++sp;
                    cur = right_first ? e.y : e.x;
                } else if (ml) {
                    cur = e.x;
                } else if (mr) {
                    cur = e.y;
                } else {
                    cur = kNoChild;
                }
            }
            if (cur == kNoChild && sp > 0) {
                // pop the next entry some lane can still reach
                const float reach =
                    cull_t(__uint_as_float(__reduce_max_sync(0xffffffffu, active ? __float_as_uint(best.t) : 0u)));
                while (sp > 0) {
                    --sp;
                    const uint32_t node = __shfl_sync(0xffffffffu, sp < 32u ? sn0 : sn1, sp & 31u);
                    const uint32_t t = __shfl_sync(0xffffffffu, sp < 32u ? st0 : st1, sp & 31u);
                    if (__uint_as_float(t) <= reach) { cur = node; break; }
                }
            }
        }
        if (active) {
            if (ovf) {
                B.ovf[atomicAdd(B.counters + kOvfClosest, 1u)] = ray;
            } else {
                if (best.prim == MCRT_HIT_MISS) best.t = -1.0f;
                const float u = (best.prim != MCRT_HIT_MISS && (best.prim & MCRT_HIT_SPHERE))
                                    ? __uint_as_float(best.slot) : best.u;
                __stcs(B.hits + ray, make_float4(best.t, __uint_as_float(best.prim), u, best.v));
                ++traced;
            }
        }
    }
    if (traced) atomicAdd(B.stats, (unsigned long long)traced);
    if (COUNT && lane == 0) {
        atomicAdd(B.stats + 3, (unsigned long long)nodes);
        atomicAdd(B.stats + 4, (unsigned long long)ntri);
    }
}

// Shading of the queued hits.  ADJ = false: the forward estimator.  ADJ = true:
// the adjoint replay of the same paths (path-replay backpropagation, Vicini et
// al. 2021): the sampling is the forward code's, consuming the same random
// numbers, and B.L starts as each path's forward radiance and is reduced, vertex
// by vertex, to the radiance still ahead of the path (Lrem).  With the sampling
// held fixed (detached), a parameter pi of the vertex's material changes
//   an emitted term E               by  E * dlog(Le)/dpi,
//   a next-event term N             by  N * dlog(f)/dpi       (shadow rays),
//   every term after the BSDF sample by Lrem * dlog(f cos / pdf)/dpi,
// each weighted by delta = dLoss/dImage(pixel) / spp.  The last one needs Lrem
// after this vertex's next-event term, which the shadow rays subtract after this
// kernel: it is stored (B.pend, material in B.pend_mat bits 8..15) and applied at
// the path's next vertex.  Gradients collect in shared memory per block, then
// one double atomic per parameter and block.
// Four resident blocks per SM (a 64-register budget) for the forward kernel:
// it is bound by the latency of its scattered loads, and at the natural 88
// registers only two blocks fit.  The replay variant keeps its registers.
// Radiance-cache training path: the path ends at this bounce (a miss or an
// emitter); record the radiance gathered before this event (which includes the
// previous vertex's light sample) in place of a vertex.
__device__ __forceinline__ void record_end(const RenderParams &P, uint32_t slot, uint32_t bounce, float4 L) {
    float4 *rec = P.train_records + ((size_t)(slot / P.train_stride) * P.max_depth + bounce) * kTrainRecordFloat4;
    rec[0] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    rec[5] = make_float4(L.x, L.y, L.z, 0.0f);
}

template <bool ADJ>
__global__ void __launch_bounds__(256, ADJ ? 2 : 4) k_shade(DeviceScene S, RenderParams P, PathBuffers B, int qi,
                                                uint32_t bounce, float4 *gbuf, AdjointParams A) {
    __shared__ float gacc[ADJ ? 256 : 1];
    if (ADJ) {
        gacc[threadIdx.x] = 0.0f;
        __syncthreads();
    }
    auto gadd = [&](uint32_t k, float v) {
        if (ADJ && v != 0.0f) atomicAdd(&gacc[k], v);
    };
    const uint32_t n = B.counters[qi];
    const bool nee = (P.flags & MCRT_RENDER_NEE) != 0 && (S.n_lights > 0 || S.has_sun);
    const uint32_t lane = threadIdx.x & 31u;
    // work counters of the next extend and shadow launches, and the closest-hit
    // overflow list (traced by now); no kernel reads them while this one runs
    if (blockIdx.x == 0 && threadIdx.x == 0) { B.counters[4] = 0; B.counters[5] = 0; B.counters[kOvfClosest] = 0; }
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        bool cont = false, shadow = false, queried = false;
        f3 no = {0, 0, 0}, nd = {0, 0, 0}, so = {0, 0, 0}, sd = {0, 0, 0}, sc = {0, 0, 0};
        float4 cq0, cq1, cq2, cq3;             // radiance-cache query of this path
        float smax = 0.0f;
        uint32_t slot = 0;
        uint32_t rng_next = 0;                 // random state of the continuing ray
        uint32_t sh_bits = 0;                  // adjoint: material | light material << 8
        float4 sh_dlog = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (i < n) {
            // the queues and hits are streamed once per bounce (GBs per frame):
            // cache-streaming accesses keep them from evicting the BVH in L2
            float4 o4 = __ldcs(B.q_o[qi] + i), d4 = __ldcs(B.q_d[qi] + i);
            float4 h = __ldcs(B.hits + i);
            slot = __float_as_uint(o4.w);
            f3 o = xyz(o4), d = xyz(d4);
            float4 thr4 = B.thr[slot];
            const uint32_t pixel = slot / P.spp_pass;
            f3 thr = xyz(thr4);
            uint32_t rng = __float_as_uint(d4.w);
            f3 delta = {0.0f, 0.0f, 0.0f};
            if (ADJ) {
                float4 di = A.dimg[pixel];
                delta = A.inv_spp * xyz(di);
                const uint32_t pm = (B.pend_mat[slot] >> 8) & 0xffu;
                if (pm) {                                   // BSDF term of the previous vertex
                    float4 L = B.L[slot], pd = B.pend[slot];
                    const uint32_t k0 = 4u * (pm - 1u);
                    f3 dl = delta * xyz(L);
                    gadd(k0 + 0, dl.x * pd.x);
                    gadd(k0 + 1, dl.y * pd.y);
                    gadd(k0 + 2, dl.z * pd.z);
                    gadd(k0 + 3, ((dl.x + dl.y) + dl.z) * pd.w);
                }
            }
            const bool write_g = gbuf && bounce == 0 && (int)(slot % P.spp_pass) == P.gbuf_plane;
            if (h.x < 0.0f) {                                                   // miss, :592-597
                if (write_g) gbuf[pixel] = make_float4(0.0f, 0.0f, 0.0f, kTMax);
                if (!ADJ) {
                    f3 e = thr * sample_env(S, d);
                    if (P.cache_query_vertex && slot % P.train_stride == 0u)   // training path ends here
                        record_end(P, slot, bounce, B.L[slot]);
                    float4 L = B.L[slot];
                    if (nee) B.L[slot] = make_float4(L.x + e.x, L.y + e.y, L.z + e.z, 0.0f);
                    else B.L[slot] = make_float4(e.x, e.y, e.z, 0.0f);
                }
            } else {
                SurfaceHit sh = surface(S, o, d, h);
                if (write_g) gbuf[pixel] = make_float4(sh.n.x, sh.n.y, sh.n.z, sh.t);   // :599-602
                const uint32_t mi = min(sh.mat, kMaxMatIdx);
                const mcrt_gpu_material &m = S.materials->materials[mi];
                const uint32_t mtype = m.type_pad[0];
                f3 albedo = ld3(m.albedo_fuzz);
                if (mtype == kMatEmissive) {                                    // :608-610
                    f3 e = m.ior_pad[0] * (thr * albedo);
                    float wmis = 1.0f;
                    if (nee) {
                        if (thr4.w > 0.0f && S.n_lights > 0) {   // pdf <= 0: specular or camera
                            float pl = light_pdf_of_hit(S, h, o, d);
                            float pb = thr4.w;
                            wmis = (pb * pb) / (pb * pb + pl * pl);
                        }
                    }
                    if (ADJ) {                                                  // d E / d(radiance colour)
                        f3 g = (wmis * m.ior_pad[0]) * (delta * thr);
                        gadd(4u * mi + 0, g.x);
                        gadd(4u * mi + 1, g.y);
                        gadd(4u * mi + 2, g.z);
                    } else {
                        if (P.cache_query_vertex && slot % P.train_stride == 0u)   // training path ends here
                            record_end(P, slot, bounce, B.L[slot]);
                        if (nee) {
                            float4 L = B.L[slot];
                            B.L[slot] = make_float4(L.x + wmis * e.x, L.y + wmis * e.y, L.z + wmis * e.z, 0.0f);
                        } else {
                            B.L[slot] = make_float4(e.x, e.y, e.z, 0.0f);
                        }
                    }
                } else {
                    albedo = material_albedo(S, m, sh.p, h);                    // :506-515
                    const f3 tex = ADJ ? material_tex(S, m, sh.p, h) : mk3(1.0f, 1.0f, 1.0f);
                    f3 dir = {0, 0, 0}, atten = {0, 0, 0};
                    bool absorbed = false;
                    float pdf = -1.0f;
                    float4 dlw = make_float4(0.0f, 0.0f, 0.0f, 0.0f);   // adjoint: dlog(weight)/d(params)
                    bool has_params = false;
                    if (!ADJ && P.cache_query_vertex) {                         // radiance cache
                        if (slot % P.train_stride == 0u) {                      // training path: record the vertex
                            float4 *rec = P.train_records +
                                          ((size_t)(slot / P.train_stride) * P.max_depth + bounce) * kTrainRecordFloat4;
                            const float4 Lnow = B.L[slot];
                            rec[0] = make_float4(sh.p.x, sh.p.y, sh.p.z, 1.0f);
                            rec[1] = make_float4(-d.x, -d.y, -d.z, 0.0f);
                            rec[2] = make_float4(sh.n.x, sh.n.y, sh.n.z, 0.0f);
                            rec[3] = make_float4(albedo.x, albedo.y, albedo.z, 0.0f);
                            rec[4] = make_float4(thr.x, thr.y, thr.z, 0.0f);
                            rec[5] = make_float4(Lnow.x, Lnow.y, Lnow.z, 0.0f);
                        } else if (bounce + 1 == P.cache_query_vertex) {        // stop here: ask the cache
                            queried = true;
                            cq0 = make_float4(sh.p.x, sh.p.y, sh.p.z, __uint_as_float(slot));
                            cq1 = make_float4(-d.x, -d.y, -d.z, 0.0f);
                            cq2 = make_float4(sh.n.x, sh.n.y, sh.n.z, 0.0f);
                            cq3 = make_float4(albedo.x, albedo.y, albedo.z, 0.0f);
                        }
                    }
                    if (mtype == kMatMetal) {                                   // :530-541
                        float fuzz = m.albedo_fuzz[3];
                        f3 refl = reflect_vec(normalize(d), sh.n);
                        f3 pert = refl + fuzz * random_unit_sphere(rng);
                        dir = normalize(dot(pert, pert) >= 1e-6f ? pert : refl);
                        atten = albedo;
                        absorbed = dot(dir, sh.n) <= 0.0f;
                        if (ADJ) {
                            dlw = make_float4(safe_ratio(tex.x, albedo.x), safe_ratio(tex.y, albedo.y),
                                              safe_ratio(tex.z, albedo.z), 0.0f);
                            has_params = true;
                        }
                    } else if (mtype == kMatDielectric) {                       // :543-564
                        atten = mk3(1.0f, 1.0f, 1.0f);
                        float ior = m.ior_pad[0];
                        float eta = sh.front ? 1.0f / ior : ior;
                        float cos_t = fminf(dot(-d, sh.n), 1.0f);
                        float sin_t = sqrtf(fmaxf(0.0f, 1.0f - cos_t * cos_t));
                        bool cannot = eta * sin_t > 1.0f;
                        float scos = (!sh.front && !cannot)
                                         ? sqrtf(fmaxf(0.0f, 1.0f - (eta * eta) * (1.0f - cos_t * cos_t)))
                                         : cos_t;
                        float refl = schlick(scos, eta);
                        if (cannot || refl > rand_f32(rng)) dir = reflect_vec(d, sh.n);
                        else dir = normalize(refract_vec(d, sh.n, eta));
                    } else if (mtype == kMatGgx) {
                        f3 t, b;
                        onb(sh.n, &t, &b);
                        f3 wo = mk3(-dot(d, t), -dot(d, b), -dot(d, sh.n));
                        float rough = m.albedo_fuzz[3];
                        float alpha = fmaxf(rough * rough, 1e-4f);
                        const float dadr = rough * rough > 1e-4f ? 2.0f * rough : 0.0f;
                        float r1 = rand_f32(rng), r2 = rand_f32(rng);
                        f3 wi, wgt;
                        float gpdf, mz = 0.0f, fw = 0.0f;
                        if (wo.z > 0.0f && ggx_sample(wo, alpha, albedo, r1, r2, &wi, &wgt, &gpdf, &mz, &fw)) {
                            dir = normalize((wi.x * t + wi.y * b) + wi.z * sh.n);
                            atten = wgt;
                            pdf = gpdf;
                            if (ADJ) {
                                const f3 one = mk3(1.0f, 1.0f, 1.0f);
                                f3 F = albedo + fw * (one - albedo);
                                dlw = make_float4(safe_ratio((1.0f - fw) * tex.x, F.x),
                                                  safe_ratio((1.0f - fw) * tex.y, F.y),
                                                  safe_ratio((1.0f - fw) * tex.z, F.z),
                                                  ggx_dlog_dalpha(alpha, mz, wo.z, wi.z) * dadr);
                                has_params = true;
                            }
                            if (nee) {                                          // light sample at a GGX vertex
                                LightSample ls = sample_light(S, sh.p, rng);
                                if (ls.ok) {
                                    f3 wl = mk3(dot(ls.dir, t), dot(ls.dir, b), dot(ls.dir, sh.n));
                                    float bp, lmz = 0.0f, lfw = 0.0f;
                                    f3 fc = ggx_eval(wo, wl, alpha, albedo, &bp, &lmz, &lfw);
                                    if (wl.z > 0.0f && (fc.x > 0.0f || fc.y > 0.0f || fc.z > 0.0f)) {
                                        float wmis = ls.delta ? 1.0f : (ls.pdf * ls.pdf) / (ls.pdf * ls.pdf + bp * bp);
                                        sc = (wmis / ls.pdf) * (thr * (fc * ls.Le));
                                        so = sh.p; sd = ls.dir; smax = ls.dist * (1.0f - 1e-4f);
                                        shadow = true;
                                        if (ADJ) {
                                            const f3 one = mk3(1.0f, 1.0f, 1.0f);
                                            f3 F = albedo + lfw * (one - albedo);
                                            sh_dlog = make_float4(safe_ratio((1.0f - lfw) * tex.x, F.x),
                                                                  safe_ratio((1.0f - lfw) * tex.y, F.y),
                                                                  safe_ratio((1.0f - lfw) * tex.z, F.z),
                                                                  ggx_dlog_dalpha(alpha, lmz, wo.z, wl.z) * dadr);
                                            sh_bits = mi | (ls.mat << 8);
                                        }
                                    }
                                }
                            }
                        } else {
                            absorbed = true;
                        }
                    } else {                                                    // :521-528
                        if (nee) {
                            LightSample ls = sample_light(S, sh.p, rng);
                            float cs = dot(ls.dir, sh.n);
                            if (ls.ok && cs > 0.0f) {
                                float bp = cs / kPi;
                                float wmis = ls.delta ? 1.0f : (ls.pdf * ls.pdf) / (ls.pdf * ls.pdf + bp * bp);
                                sc = (wmis * bp / ls.pdf) * (thr * (albedo * ls.Le));
                                so = sh.p; sd = ls.dir; smax = ls.dist * (1.0f - 1e-4f);
                                shadow = true;
                                if (ADJ) {
                                    sh_dlog = make_float4(safe_ratio(tex.x, albedo.x), safe_ratio(tex.y, albedo.y),
                                                          safe_ratio(tex.z, albedo.z), 0.0f);
                                    sh_bits = mi | (ls.mat << 8);
                                }
                            }
                        }
                        dir = cosine_scatter(rng, sh.n);
                        atten = albedo;
                        pdf = fmaxf(dot(dir, sh.n), 0.0f) / kPi;
                        if (ADJ) {
                            dlw = make_float4(safe_ratio(tex.x, albedo.x), safe_ratio(tex.y, albedo.y),
                                              safe_ratio(tex.z, albedo.z), 0.0f);
                            has_params = true;
                        }
                    }
                    // a cache stop keeps this vertex's light sample (above) and ends
                    // the path: the cache stands for what BSDF sampling would gather
                    if (queried) absorbed = true;
                    uint32_t pend_bits = 0;
                    if (!absorbed) {
                        thr = thr * atten;
                        if (bounce + 1 < P.max_depth) {
                            cont = true;
                            no = sh.p;
                            nd = dir;
                            if (ADJ && has_params) {
                                B.pend[slot] = dlw;
                                pend_bits = (mi + 1u) << 8;
                            }
                        }
                        B.thr[slot] = make_float4(thr.x, thr.y, thr.z, pdf);
                    }
                    if (ADJ) B.pend_mat[slot] = pend_bits;
                    rng_next = rng;
                }
            }
        }
        // warp-aggregated append to the next ray queue
        unsigned mask = __ballot_sync(0xffffffffu, cont);
        if (mask) {
            int leader = __ffs(mask) - 1;
            uint32_t basepos = 0;
            if ((int)lane == leader) basepos = atomicAdd(B.counters + (qi ^ 1), (uint32_t)__popc(mask));
            basepos = __shfl_sync(0xffffffffu, basepos, leader);
            if (cont) {
                uint32_t pos = basepos + __popc(mask & ((1u << lane) - 1u));
                __stcs(B.q_o[qi ^ 1] + pos, make_float4(no.x, no.y, no.z, __uint_as_float(slot)));
                __stcs(B.q_d[qi ^ 1] + pos, make_float4(nd.x, nd.y, nd.z, __uint_as_float(rng_next)));
            }
        }
        unsigned smask = __ballot_sync(0xffffffffu, shadow);
        if (smask) {
            int leader = __ffs(smask) - 1;
            uint32_t basepos = 0;
            if ((int)lane == leader) basepos = atomicAdd(B.counters + 2, (uint32_t)__popc(smask));
            basepos = __shfl_sync(0xffffffffu, basepos, leader);
            if (shadow) {
                uint32_t pos = basepos + __popc(smask & ((1u << lane) - 1u));
                B.sh_o[pos] = make_float4(so.x, so.y, so.z, __uint_as_float(slot));
                B.sh_d[pos] = make_float4(sd.x, sd.y, sd.z, smax);
                B.sh_c[pos] = make_float4(sc.x, sc.y, sc.z, __uint_as_float(sh_bits));
                if (ADJ) B.sh_g[pos] = sh_dlog;
            }
        }
        if (!ADJ && P.cache_query_vertex) {
            unsigned qmask = __ballot_sync(0xffffffffu, queried);
            if (qmask) {
                int leader = __ffs(qmask) - 1;
                uint32_t basepos = 0;
                if ((int)lane == leader) basepos = atomicAdd(B.counters + 6, (uint32_t)__popc(qmask));
                basepos = __shfl_sync(0xffffffffu, basepos, leader);
                if (queried) {
                    uint32_t pos = basepos + __popc(qmask & ((1u << lane) - 1u));
                    float4 *q = P.cache_queries + 4 * (size_t)pos;
                    q[0] = cq0; q[1] = cq1; q[2] = cq2; q[3] = cq3;
                }
            }
        }
    }
    if (ADJ) {
        __syncthreads();
        const float v = gacc[threadIdx.x];
        if (v != 0.0f) atomicAdd(A.grad + threadIdx.x, (double)v);
    }
}

// Per pixel, in frame order: the reference's f32 running mean
// (path_trace.wgsl:656-661, mix = a*(1-t) + b*t) and the f64 sum.
__global__ void k_resolve(RenderParams P, PathBuffers B, float4 *mean, double *sum, int keep) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.npix) return;
    if (P.pass_state) keep = (int)P.pass_state[1];
    const uint32_t frame0 = P.pass_state ? P.pass_state[0] : P.frame0;
    float4 m = keep ? mean[p] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    double s0 = keep ? sum[3 * (size_t)p] : 0.0, s1 = keep ? sum[3 * (size_t)p + 1] : 0.0,
           s2 = keep ? sum[3 * (size_t)p + 2] : 0.0;
    for (uint32_t k = 0; k < P.spp_pass; ++k) {
        float4 s = B.L[(size_t)p * P.spp_pass + k];
        uint32_t frame = frame0 + k;
        float w = 1.0f / (float)(min(frame, kMaxFrameCount) + 1u);
        float omw = 1.0f - w;
        m.x = m.x * omw + s.x * w;
        m.y = m.y * omw + s.y * w;
        m.z = m.z * omw + s.z * w;
        s0 += (double)s.x; s1 += (double)s.y; s2 += (double)s.z;
    }
    m.w = 1.0f;
    mean[p] = m;
    sum[3 * (size_t)p] = s0; sum[3 * (size_t)p + 1] = s1; sum[3 * (size_t)p + 2] = s2;
}

// Tone map of the running mean into RGBA8 on the device: mode 0 is
// tonemap_to_u8 (headless.rs:93-98) after the non-finite sanitising
// (:356-358); mode 1 is screenshot_to_u8 (gpu.rs:1904-1939).
__device__ __forceinline__ float rclamp(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }

__global__ void k_tonemap(const float4 *mean, uint32_t npix, uint32_t mode, uchar4 *out) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float4 m = mean[p];
    float v[3] = {m.x, m.y, m.z};
    unsigned char q[3];
    for (int c = 0; c < 3; ++c) {
        float x = v[c], s;
        if (mode == MCRT_TONEMAP_ACES_SRGB) {
            x = isnan(x) ? 0.0f : fmaxf(x, 0.0f);
            float a = rclamp((x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f), 0.0f, 1.0f);
            if (a <= 0.0f) s = 0.0f;
            else if (a <= 0.0031308f) s = fminf(a * 12.92f, 1.0f);
            else if (a < 1.0f) s = rclamp(1.055f * dm_pow(a, 1.0f / 2.4f) - 0.055f, 0.0f, 1.0f);
            else s = 1.0f;
        } else {
            if (!isfinite(x)) x = 0.0f;
            x = fmaxf(x, 0.0f);
            float mapped = x / (x + 1.0f);
            s = fminf(fmaxf(dm_pow(mapped, 1.0f / 2.2f), 0.0f), 1.0f);
        }
        q[c] = (unsigned char)min(f2u_sat(s * 255.0f + 0.5f), 255u);
    }
    out[p] = make_uchar4(q[0], q[1], q[2], 255);
}

void launch_tonemap(const float4 *mean, uint32_t npix, uint32_t mode, uchar4 *out, cudaStream_t st) {
    k_tonemap<<<(npix + 255) / 256, 256, 0, st>>>(mean, npix, mode, out); ::mcrt::note_launch();
}

// Light-selection CDF: one block; each thread sums a contiguous chunk of light
// weights, a block scan gives chunk offsets, cdf[k] = prefix / total.
__global__ void __launch_bounds__(1024) k_light_cdf(DeviceScene S, float *cdf, float *total_out) {
    __shared__ float part[1024];
    const uint32_t n = S.n_lights;
    const uint32_t chunk = (n + 1023) / 1024;
    const uint32_t b = threadIdx.x * chunk, e = min(b + chunk, n);
    float local = 0.0f;
    for (uint32_t k = b; k < e; ++k) local += light_weight(S, __ldg(S.lights + k));
    part[threadIdx.x] = local;
    __syncthreads();
    if (threadIdx.x == 0) {            // sequential scan of 1024 partial sums: fixed order
        float run = 0.0f;
        for (int k = 0; k < 1024; ++k) { float v = part[k]; part[k] = run; run += v; }
        *total_out = run;
    }
    __syncthreads();
    const float total = *total_out;
    float run = part[threadIdx.x];
    for (uint32_t k = b; k < e; ++k) {
        cdf[k] = total > 0.0f ? run / total : 0.0f;
        run += light_weight(S, __ldg(S.lights + k));
    }
    if (threadIdx.x == 0) { cdf[0] = 0.0f; cdf[n] = 1.0f; }
}

void launch_light_cdf(const DeviceScene &S, float *d_cdf, float *d_total, cudaStream_t st) {
    k_light_cdf<<<1, 1024, 0, st>>>(S, d_cdf, d_total); ::mcrt::note_launch();
}

// ------------------------------------------------------------------ launchers

int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

void launch_trace_closest(const DeviceScene &S, const mcrt_ray *rays, uint32_t n, mcrt_hit *hits, bool ref_layout,
                          cudaStream_t st) {
    if (n == 0) return;
    k_trace_closest<<<(n + 127) / 128, 128, 0, st>>>(S, rays, n, hits, ref_layout ? 1 : 0); ::mcrt::note_launch();
}

void launch_raygen(const DeviceScene &S, const RenderParams &P, PathBuffers &B, cudaStream_t st, bool keep_radiance) {
    uint32_t n = P.npix * P.spp_pass;
    k_raygen<<<(n + 255) / 256, 256, 0, st>>>(S, P, B, keep_radiance ? 1 : 0); ::mcrt::note_launch();
}

int extend_variant_count() { return kExtendVariants; }

namespace {
using ExtendKernel = void (*)(DeviceScene, PathBuffers, int, AdjointParams);
#define MCRT_EXTEND_KERNEL(i, any, adj)                                                                  \
    k_extend<kVariantTable[i].width, kVariantTable[i].block, kVariantTable[i].min_blocks, kVariantTable[i].stack, \
             kVariantTable[i].refill, kVariantTable[i].top, any, adj>
#define MCRT_EXTEND_TABLE(any, adj)                                                                      \
    {MCRT_EXTEND_KERNEL(0, any, adj), MCRT_EXTEND_KERNEL(1, any, adj), MCRT_EXTEND_KERNEL(2, any, adj),    \
     MCRT_EXTEND_KERNEL(3, any, adj), MCRT_EXTEND_KERNEL(4, any, adj), MCRT_EXTEND_KERNEL(5, any, adj),    \
     MCRT_EXTEND_KERNEL(6, any, adj), MCRT_EXTEND_KERNEL(7, any, adj)}
const ExtendKernel kExtendKernels[kExtendVariants] = MCRT_EXTEND_TABLE(false, false);
// the any-hit instantiations, for the shadow rays of next-event estimation
const ExtendKernel kShadowKernels[kExtendVariants] = MCRT_EXTEND_TABLE(true, false);
// the same for the adjoint replay, which adds gradients per unoccluded shadow ray
const ExtendKernel kShadowAdjKernels[kExtendVariants] = MCRT_EXTEND_TABLE(true, true);
// the closest-hit instantiations that count their record fetches (MCRT_RENDER_COUNT)
#define MCRT_COUNT_KERNEL(i)                                                                            \
    k_extend<kVariantTable[i].width, kVariantTable[i].block, kVariantTable[i].min_blocks, kVariantTable[i].stack, \
             kVariantTable[i].refill, kVariantTable[i].top, false, false, true>
const ExtendKernel kCountKernels[kExtendVariants] = {
    MCRT_COUNT_KERNEL(0), MCRT_COUNT_KERNEL(1), MCRT_COUNT_KERNEL(2), MCRT_COUNT_KERNEL(3),
    MCRT_COUNT_KERNEL(4), MCRT_COUNT_KERNEL(5), MCRT_COUNT_KERNEL(6), MCRT_COUNT_KERNEL(7)};
#undef MCRT_COUNT_KERNEL
#undef MCRT_EXTEND_TABLE
#undef MCRT_EXTEND_KERNEL
int g_extend_per_sm[kExtendVariants] = {0, 0, 0, 0, 0, 0, 0, 0};
int g_shadow_per_sm[kExtendVariants] = {0, 0, 0, 0, 0, 0, 0, 0};
int g_shadow_adj_per_sm[kExtendVariants] = {0, 0, 0, 0, 0, 0, 0, 0};
int g_packet_per_sm = 0;
int g_count_per_sm[kExtendVariants] = {0, 0, 0, 0, 0, 0, 0, 0};
}  // namespace

void extend_variant_info(int v, int out[6]) {
    const ExtendVariant &e = kVariantTable[(v >= 0 && v < kExtendVariants) ? v : 0];
    out[0] = e.width; out[1] = e.block; out[2] = e.min_blocks; out[3] = e.stack; out[4] = e.refill; out[5] = e.top;
}

// Resident blocks per SM of every variant and of the packet kernel (occupancy
// queries, made before any stream capture of a render).
void prepare_extend_variants() {
    if (g_packet_per_sm == 0) {
        int n = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_extend_packet<false>, kPacketBlock, 0);
        g_packet_per_sm = n > 0 ? n : 1;
    }
    for (int v = 0; v < kExtendVariants; ++v) {
        if (g_extend_per_sm[v] == 0) {
            int n = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kExtendKernels[v], kVariantTable[v].block, 0);
            g_extend_per_sm[v] = n > 0 ? n : 1;
        }
        if (g_shadow_per_sm[v] == 0) {
            int n = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kShadowKernels[v], kVariantTable[v].block, 0);
            g_shadow_per_sm[v] = n > 0 ? n : 1;
        }
        if (g_shadow_adj_per_sm[v] == 0) {
            int n = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kShadowAdjKernels[v], kVariantTable[v].block, 0);
            g_shadow_adj_per_sm[v] = n > 0 ? n : 1;
        }
        if (g_count_per_sm[v] == 0) {
            int n = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kCountKernels[v], kVariantTable[v].block, 0);
            g_count_per_sm[v] = n > 0 ? n : 1;
        }
    }
}

// The rays of the overflow list (a stack too short for the tree), after each extend launch.
static void launch_retry(const DeviceScene &S, PathBuffers &B, int qi, bool any, const AdjointParams *adj,
                         cudaStream_t st) {
    const int blocks = sm_count();
    if (adj) k_extend_retry<true, true><<<blocks, kRetryBlock, 0, st>>>(S, B, qi, *adj);
    else if (any) k_extend_retry<true, false><<<blocks, kRetryBlock, 0, st>>>(S, B, qi, AdjointParams{});
    else k_extend_retry<false, false><<<blocks, kRetryBlock, 0, st>>>(S, B, qi, AdjointParams{});
    ::mcrt::note_launch();
}

void launch_extend(const DeviceScene &S, const RenderParams &P, PathBuffers &B, int qi, cudaStream_t st,
                   bool primary) {
    const int v = (P.extend_variant >= 0 && P.extend_variant < kExtendVariants) ? P.extend_variant : 0;
    prepare_extend_variants();
    const uint32_t nmax = P.npix * P.spp_pass;
    const bool count = (P.flags & MCRT_RENDER_COUNT) != 0;
    if (primary) {                    // the camera rays: warp packets, every warp resident at once
        const int blocks = min(grid_blocks_for(nmax, kPacketBlock), sm_count() * g_packet_per_sm);
        if (count) k_extend_packet<true><<<blocks, kPacketBlock, 0, st>>>(S, B, qi);
        else k_extend_packet<false><<<blocks, kPacketBlock, 0, st>>>(S, B, qi);
        ::mcrt::note_launch();
    } else {
        // persistent: as many resident blocks as fit, never more warps than rays
        const int block = kVariantTable[v].block;
        const int per_sm = count ? g_count_per_sm[v] : g_extend_per_sm[v];
        const int blocks = min(grid_blocks_for(nmax, block), sm_count() * per_sm);
        (count ? kCountKernels[v] : kExtendKernels[v])<<<blocks, block, 0, st>>>(S, B, qi, AdjointParams{});
        ::mcrt::note_launch();
    }
    launch_retry(S, B, qi, false, nullptr, st);
}

void launch_shade(const DeviceScene &S, const RenderParams &P, PathBuffers &B, int qi, uint32_t bounce,
                  float4 *gbuf, cudaStream_t st, const AdjointParams *adj) {
    uint32_t nmax = P.npix * P.spp_pass;
    int blocks = min(grid_blocks_for(nmax, 256), sm_count() * 8);
    if (adj) k_shade<true><<<blocks, 256, 0, st>>>(S, P, B, qi, bounce, gbuf, *adj);
    else k_shade<false><<<blocks, 256, 0, st>>>(S, P, B, qi, bounce, gbuf, AdjointParams{});
    ::mcrt::note_launch();
}

void launch_shadow(const DeviceScene &S, const RenderParams &P, PathBuffers &B, cudaStream_t st,
                   const AdjointParams *adj) {
    // persistent any-hit traversal with the render's variant; the adjoint
    // replay's instantiation also adds the gradients of unoccluded rays
    uint32_t nmax = P.npix * P.spp_pass;
    const int v = (P.extend_variant >= 0 && P.extend_variant < kExtendVariants) ? P.extend_variant : 0;
    prepare_extend_variants();
    const int block = kVariantTable[v].block;
    const int per_sm = adj ? g_shadow_adj_per_sm[v] : g_shadow_per_sm[v];
    int blocks = min(grid_blocks_for(nmax, block), sm_count() * per_sm);
    if (adj) kShadowAdjKernels[v]<<<blocks, block, 0, st>>>(S, B, 0, *adj);
    else kShadowKernels[v]<<<blocks, block, 0, st>>>(S, B, 0, AdjointParams{});
    ::mcrt::note_launch();
    launch_retry(S, B, 0, true, adj, st);
}

void launch_resolve(const RenderParams &P, const PathBuffers &B, float4 *mean, double *sum, bool keep,
                    cudaStream_t st) {
    k_resolve<<<(P.npix + 255) / 256, 256, 0, st>>>(P, B, mean, sum, keep ? 1 : 0); ::mcrt::note_launch();
}

}  // namespace mcrt
