// common.cuh — device-side types, RNG and float32 elementary functions shared by
// the path-tracing kernels.
//
// Every kernel translation unit is compiled with -fmad=false: the arithmetic is
// the IEEE-754 sequence written in the source (no contraction to fused
// multiply-add), so hit distances and per-sample radiance are reproducible and
// identical to a CPU evaluation of the same sequence.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "mcrt_cuda.h"
#include "fmath.h"

namespace mcrt {

// ---------------------------------------------------------------- constants
// path_trace.wgsl:36-66
constexpr float kTau = 6.283185307179586f;
constexpr float kPi = 3.141592653589793f;
constexpr uint32_t kMaxMatIdx = 63u;
constexpr uint32_t kStackSize = 64u;
constexpr float kTMin = 1e-4f;
constexpr float kTMax = 1e9f;
constexpr uint32_t kMaxFrameCount = 65535u;
constexpr uint32_t kDefaultBounces = 8u;
// Relative slack of every box test against the current closest t (entry) and
// of the box exit: a box is entered when texit * kCullSlack > max(tenter, tmin)
// and tenter <= t * kCullSlack.  A hit on a shared edge or vertex lies on the
// boundary of its triangle's box, and the Moller-Trumbore t can lie outside it
// by rounding (a few ulps, hundreds for a grazing ray); the exact test would
// make the closest hit depend on which triangle the visit order found first.
// With the slack (1 + 2^-12) every box that can hold a hit at or before t is
// entered, so every traversal order gives the tie rule's answer over all
// triangles the test accepts.
constexpr float kCullSlack = 1.000244140625f;
// Top levels of the compact BVH held in shared memory by the top-tree kernel
// variants: 7 levels, 127 records of 64 bytes (8 KB per block).
constexpr uint32_t kTopNodes = 127u;
constexpr uint32_t kTopBit = 0x40000000u;   // node code of a top-tree entry (bit 31 clear: internal)
__host__ __device__ __forceinline__ float cull_t(float t) { return t * kCullSlack; }

// ---------------------------------------------------------------- vectors
struct f3 { float x, y, z; };
__host__ __device__ __forceinline__ f3 mk3(float x, float y, float z) { return {x, y, z}; }
__host__ __device__ __forceinline__ f3 xyz(float4 a) { return {a.x, a.y, a.z}; }
__host__ __device__ __forceinline__ f3 ld3(const float *p) { return {p[0], p[1], p[2]}; }
__host__ __device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__host__ __device__ __forceinline__ f3 operator*(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
__host__ __device__ __forceinline__ f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__host__ __device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
// dot(a, b) = (ax*bx + ay*by) + az*bz
__host__ __device__ __forceinline__ float dot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__host__ __device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// normalize(v) = v * (1 / sqrt(dot(v, v)))
__host__ __device__ __forceinline__ f3 normalize(f3 a) {
    float inv = 1.0f / sqrtf(dot(a, a));
    return {a.x * inv, a.y * inv, a.z * inv};
}

// ---------------------------------------------------------------- RNG
// pcg_hash / rand_f32, path_trace.wgsl:64-66, :194-204
__host__ __device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
    uint32_t s = v * 747796405u + 2891336453u;
    uint32_t rot = s >> 28u;
    s = ((s >> (rot + 4u)) ^ s) * 277803737u;
    return (s >> 22u) ^ s;
}
__device__ __forceinline__ float rand_f32(uint32_t &rng) {
    rng = pcg_hash(rng);
    return __uint_as_float((rng >> 9u) | 0x3f800000u) - 1.0f;
}

// ---------------------------------------------------------------- elementary functions
// fmath.h (shared with the host code of the library).
__device__ __forceinline__ void dm_sincos(float x, float *s, float *c) { fm_sincos(x, s, c); }
__device__ __forceinline__ float dm_atan2(float y, float x) { return fm_atan2(y, x); }
__device__ __forceinline__ float dm_asin(float x) { return fm_asin(x); }
__device__ __forceinline__ float dm_exp(float x) { return fm_exp(x); }
__device__ __forceinline__ float dm_log(float x) { return fm_log(x); }
__device__ __forceinline__ float dm_pow(float x, float y) { return fm_pow(x, y); }
__device__ __forceinline__ uint32_t f2u_sat(float f) { return fm_f2u_sat(f); }

// ---------------------------------------------------------------- device scene
// Fast triangle record (leaf order): v0.xyz | orig id, e1.xyz | mat bits, e2.xyz | unused.
// e1 = v1 - v0 and e2 = v2 - v0 are the exact differences the reference forms in
// ray_triangle_uvt (path_trace.wgsl:302-303), so precomputing them changes no bit.
struct TriRec { float4 v0; float4 e1; float4 e2; };

struct DeviceScene {
    // spheres (ordered by the sphere BVH) and their original ids
    const mcrt_gpu_sphere *spheres; uint32_t n_spheres;
    const uint32_t *sphere_ids;
    const mcrt_gpu_bvh_node *sphere_nodes; uint32_t n_sphere_nodes;
    // triangles in original order (shading) and vertices
    const mcrt_gpu_vertex *vertices; uint32_t n_vertices;
    const mcrt_gpu_triangle *triangles; uint32_t n_triangles;
    // shading records, 3 float4 per triangle in original order: the three
    // vertex normals, the first with the triangle's material word in w (48 B:
    // two 32-byte sectors per record instead of one per vertex and triangle)
    const float4 *shade_recs;
    // reference-layout mesh BVH, ordered slots -> original ids, fast leaf-ordered records
    const mcrt_gpu_bvh_node *mesh_nodes; uint32_t n_mesh_nodes;
    const uint32_t *tri_ids;
    const TriRec *tris;
    // compact BVH2 (children boxes in the parent) for the fast traversal
    const float4 *cnodes; uint32_t n_cnodes;
    // the compact tree's top levels in heap order (kTopNodes records: entry j's
    // children at 2j+1, 2j+2), staged in shared memory by the top-tree variants;
    // internal children inside it are coded kTopBit | entry
    const float4 *top;
    // quantised 4-wide BVH collapsed from the same tree
    const uint4 *wnodes; uint32_t n_wnodes;
    const mcrt_gpu_material_data *materials;
    const float4 *env; uint32_t env_w, env_h;
    // light list for next-event estimation
    const uint32_t *lights; uint32_t n_lights;      // MCRT_HIT_SPHERE|sphere slot, or triangle id
    const float *light_cdf;                          // n_lights+1 entries, light_cdf[n] = 1
    float light_total;                               // sum of unnormalised weights
    // albedo texture array (RGBA8 sRGB), layers x size x size texels, and the
    // sRGB -> linear decode table of an 8-bit channel (IEC 61966-2-1, evaluated
    // on the host in double precision and rounded to float)
    const uchar4 *albedo; uint32_t albedo_layers, albedo_size;
    const float *srgb_lut;
    // directional light: unit direction towards it, irradiance at normal incidence
    int has_sun;
    float4 sun_dir, sun_E;
};

}  // namespace mcrt
