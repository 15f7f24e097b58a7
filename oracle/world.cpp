/* oracle/world.cpp — CPU restatement of the voxel-world generator and of the
 * reference's greedy chunk mesher.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the kernels in world.cu.
 *
 * Mesher: world/mesher.rs:97-366 (mesh_chunk, mesh_face_direction,
 * sample_neighbour, emit_quad) run chunk by chunk over a voxel grid, each chunk
 * with its in-grid neighbours (missing neighbours are air, mesher.rs:261-300),
 * and concatenated as merge_chunk_meshes (:377-400), chunks in (x outer, z
 * inner) order as visible_chunk_coords lists them (world/mod.rs:65-76).
 * Opacity: BLOCK_META (world/block.rs:53-125), ids 1..10 opaque.
 * Grid layout: (x * ny + y) * nz + z, the chunk's XZY-major order
 * (world/chunk.rs:26-31).
 *
 * Generator: the project's own terrain rule (lattice value noise fBm
 * heightmap, 3D fBm caves), restated here operation for operation. */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace {

inline uint32_t pcg(uint32_t v) {                  /* path_trace.wgsl:194-199 */
    uint32_t s = v * 747796405u + 2891336453u;
    uint32_t rot = s >> 28u;
    s = ((s >> (rot + 4u)) ^ s) * 277803737u;
    return (s >> 22u) ^ s;
}
inline uint32_t lhash(int32_t x, int32_t y, int32_t z, uint32_t seed) {
    uint32_t h = pcg((uint32_t)x * 0x8da6b343u ^ seed);
    h = pcg(h ^ ((uint32_t)y * 0xd8163841u));
    return pcg(h ^ ((uint32_t)z * 0xcb1ab31fu));
}
inline float lvalue(int32_t x, int32_t y, int32_t z, uint32_t seed) {
    return (float)(lhash(x, y, z, seed) >> 8) * (1.0f / 16777216.0f);
}
inline float fade(float t) { return t * t * (3.0f - 2.0f * t); }
inline float lerp(float a, float b, float t) { return a + (b - a) * t; }

float noise2(float x, float z, uint32_t seed) {
    float fx0 = std::floor(x), fz0 = std::floor(z);
    int32_t ix = (int32_t)fx0, iz = (int32_t)fz0;
    float tx = fade(x - fx0), tz = fade(z - fz0);
    float a = lerp(lvalue(ix, 0, iz, seed), lvalue(ix + 1, 0, iz, seed), tx);
    float b = lerp(lvalue(ix, 0, iz + 1, seed), lvalue(ix + 1, 0, iz + 1, seed), tx);
    return lerp(a, b, tz);
}
float noise3(float x, float y, float z, uint32_t seed) {
    float fx0 = std::floor(x), fy0 = std::floor(y), fz0 = std::floor(z);
    int32_t ix = (int32_t)fx0, iy = (int32_t)fy0, iz = (int32_t)fz0;
    float tx = fade(x - fx0), ty = fade(y - fy0), tz = fade(z - fz0);
    float c[2];
    for (int k = 0; k < 2; ++k) {
        float a = lerp(lvalue(ix, iy, iz + k, seed), lvalue(ix + 1, iy, iz + k, seed), tx);
        float b = lerp(lvalue(ix, iy + 1, iz + k, seed), lvalue(ix + 1, iy + 1, iz + k, seed), tx);
        c[k] = lerp(a, b, ty);
    }
    return lerp(c[0], c[1], tz);
}
float fbm2(float x, float z, uint32_t oct, float lac, float gain, uint32_t seed) {
    float sum = 0.0f, amp = 1.0f, norm = 0.0f, f = 1.0f;
    for (uint32_t o = 0; o < oct; ++o) {
        sum += amp * noise2(x * f, z * f, seed + o * 0x9e3779b9u);
        norm += amp;
        amp *= gain;
        f *= lac;
    }
    return sum / norm;
}
float fbm3(float x, float y, float z, uint32_t oct, float lac, float gain, uint32_t seed) {
    float sum = 0.0f, amp = 1.0f, norm = 0.0f, f = 1.0f;
    for (uint32_t o = 0; o < oct; ++o) {
        sum += amp * noise3(x * f, y * f, z * f, seed + o * 0x9e3779b9u);
        norm += amp;
        amp *= gain;
        f *= lac;
    }
    return sum / norm;
}

/* world/block.rs:14-24 */
constexpr uint8_t AIR = 0, LIMESTONE = 1, RED_SOIL = 2, GRASS = 3, SAND = 4, WATER = 5, SHRUB = 8, GRAVEL = 9,
                  CAVE_GLOW = 10;
inline bool opaque(uint8_t id) { return id >= 1 && id <= 10; }

constexpr uint32_t CHUNK_XZ = 16;                  /* world/chunk.rs:15 */

struct Mesh { std::vector<orc_vertex> v; std::vector<orc_triangle> t; };

/* emit_quad, mesher.rs:308-366 */
void emit_quad(float ox, float oz, int axis, int ua, int va, uint32_t layer, uint32_t u0, uint32_t v0, uint32_t h,
               uint32_t w, int sign, uint32_t mat, float voxel, Mesh &m) {
    const uint32_t face_offset = sign > 0 ? 1u : 0u;
    float normal[3] = {0.0f, 0.0f, 0.0f};
    normal[axis] = (float)sign;
    auto make_pos = [&](uint32_t u, uint32_t v, float out[3]) {
        float p[3] = {0.0f, 0.0f, 0.0f};
        p[axis] = (float)(layer + face_offset) * voxel;
        p[ua] = (float)u * voxel;
        p[va] = (float)v * voxel;
        out[0] = ox + p[0];
        out[1] = 0.0f + p[1];
        out[2] = oz + p[2];
    };
    float p[4][3];
    make_pos(u0, v0, p[0]);
    make_pos(u0 + h, v0, p[1]);
    make_pos(u0 + h, v0 + w, p[2]);
    make_pos(u0, v0 + w, p[3]);
    const float uv[4][2] = {{0.0f, 0.0f}, {1.0f, 0.0f}, {1.0f, 1.0f}, {0.0f, 1.0f}};
    const uint32_t base = (uint32_t)m.v.size();
    for (int k = 0; k < 4; ++k)
        m.v.push_back(orc_vertex{{p[k][0], p[k][1], p[k][2], 1.0f}, {normal[0], normal[1], normal[2], 0.0f},
                                 {uv[k][0], uv[k][1], 0.0f, 0.0f}});
    if (sign > 0) {
        m.t.push_back(orc_triangle{{base, base + 1, base + 2}, mat});
        m.t.push_back(orc_triangle{{base, base + 2, base + 3}, mat});
    } else {
        m.t.push_back(orc_triangle{{base, base + 2, base + 1}, mat});
        m.t.push_back(orc_triangle{{base, base + 3, base + 2}, mat});
    }
}

/* mesh_chunk + mesh_face_direction (mesher.rs:97-245) for chunk (i, k) of the grid */
void mesh_chunk(const uint8_t *vox, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t ci, uint32_t ck, int32_t cx0,
                int32_t cz0, bool greedy, const uint32_t *mat_of, float voxel, Mesh &m) {
    const uint32_t dim[3] = {CHUNK_XZ, ny, CHUNK_XZ};
    auto get = [&](int32_t gx, int32_t gy, int32_t gz) -> uint8_t {
        if (gx < 0 || gy < 0 || gz < 0 || gx >= (int32_t)nx || gy >= (int32_t)ny || gz >= (int32_t)nz) return AIR;
        return vox[((size_t)gx * ny + (size_t)gy) * nz + (size_t)gz];
    };
    const float ox = (float)(cx0 + (int32_t)ci) * (float)CHUNK_XZ * voxel;   /* chunk_world_origin, chunk.rs:131 */
    const float oz = (float)(cz0 + (int32_t)ck) * (float)CHUNK_XZ * voxel;
    const int dirs[6][2] = {{0, 1}, {0, -1}, {1, 1}, {1, -1}, {2, 1}, {2, -1}};
    for (const auto &fd : dirs) {
        const int axis = fd[0], sign = fd[1];
        const int ua = axis == 0 ? 1 : 0, va = axis == 2 ? 1 : 2;
        const uint32_t ud = dim[ua], vd = dim[va];
        std::vector<uint8_t> mask((size_t)ud * vd), visited((size_t)ud * vd);
        for (uint32_t layer = 0; layer < dim[axis]; ++layer) {
            std::fill(mask.begin(), mask.end(), 0);
            std::fill(visited.begin(), visited.end(), 0);
            for (uint32_t u = 0; u < ud; ++u)
                for (uint32_t v = 0; v < vd; ++v) {
                    int32_t pos[3];
                    pos[axis] = (int32_t)layer;
                    pos[ua] = (int32_t)u;
                    pos[va] = (int32_t)v;
                    const int32_t g[3] = {(int32_t)(ci * CHUNK_XZ) + pos[0], pos[1], (int32_t)(ck * CHUNK_XZ) + pos[2]};
                    const uint8_t id = get(g[0], g[1], g[2]);
                    if (id == AIR || !opaque(id)) continue;
                    int32_t q[3] = {g[0], g[1], g[2]};
                    q[axis] += sign;
                    if (!opaque(get(q[0], q[1], q[2]))) mask[(size_t)u * vd + v] = id;
                }
            for (uint32_t u0 = 0; u0 < ud; ++u0) {
                uint32_t v0 = 0;
                while (v0 < vd) {
                    const uint8_t id = mask[(size_t)u0 * vd + v0];
                    if (id == 0 || visited[(size_t)u0 * vd + v0]) { ++v0; continue; }
                    uint32_t w = 1, h = 1;
                    if (greedy) {
                        while (v0 + w < vd && mask[(size_t)u0 * vd + v0 + w] == id && !visited[(size_t)u0 * vd + v0 + w])
                            ++w;
                        for (bool grow = true; grow && u0 + h < ud;) {
                            for (uint32_t dv = 0; dv < w; ++dv)
                                if (mask[(size_t)(u0 + h) * vd + v0 + dv] != id ||
                                    visited[(size_t)(u0 + h) * vd + v0 + dv]) { grow = false; break; }
                            if (grow) ++h;
                        }
                    }
                    for (uint32_t du = 0; du < h; ++du)
                        for (uint32_t dv = 0; dv < w; ++dv) visited[(size_t)(u0 + du) * vd + v0 + dv] = 1;
                    emit_quad(ox, oz, axis, ua, va, layer, u0, v0, h, w, sign, mat_of[id], voxel, m);
                    v0 += w;
                }
            }
        }
    }
}

}  // namespace

extern "C" {

void orc_world_generate(const orc_world_params *P, uint8_t *vox) {
    const uint32_t ny = P->ny;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t t = 0; t < (int64_t)P->nx * P->nz; ++t) {
        const uint32_t x = (uint32_t)(t / P->nz), z = (uint32_t)(t % P->nz);
        const int32_t gx = P->chunk_x0 * 16 + (int32_t)x, gz = P->chunk_z0 * 16 + (int32_t)z;
        const float hn = fbm2((float)gx * P->height_freq, (float)gz * P->height_freq, P->height_octaves,
                              P->lacunarity, P->gain, P->seed);
        const float hf = P->height_base + P->height_amp * (2.0f * hn - 1.0f);
        int32_t surface = (int32_t)std::floor(hf);
        surface = std::max(1, std::min(surface, (int32_t)ny - 2));
        const bool beach = (float)surface <= P->sand_line;
        auto at = [&](uint32_t y) -> uint8_t & { return vox[((size_t)x * ny + y) * P->nz + z]; };
        for (uint32_t y = 0; y < ny; ++y) {
            const int32_t yi = (int32_t)y;
            uint8_t b = AIR;
            if (yi <= surface) {
                if (yi == surface) b = beach ? SAND : GRASS;
                else if (yi >= surface - 3) b = beach ? SAND : RED_SOIL;
                else {
                    b = LIMESTONE;
                    if (noise3((float)gx * 0.11f, (float)yi * 0.11f, (float)gz * 0.11f, P->seed ^ 0x5bd1e995u) > 0.72f)
                        b = GRAVEL;
                }
                if (y >= P->cave_min_y) {
                    const float c = fbm3((float)gx * P->cave_freq, (float)yi * P->cave_freq, (float)gz * P->cave_freq,
                                         P->cave_octaves, P->lacunarity, P->gain, P->seed ^ 0x6c62272eu);
                    if (0.5f + (c - 0.5f) * P->cave_contrast > P->cave_threshold) b = AIR;
                }
            } else if ((float)yi <= P->sea_level) {
                b = WATER;
            }
            at(y) = b;
        }
        for (uint32_t y = 1; y + 1 < ny && (int32_t)y < surface; ++y)
            if (at(y) != AIR && at(y + 1) == AIR && (lhash(gx, (int32_t)y, gz, P->seed ^ 0x27d4eb2fu) & 7u) == 0u)
                at(y) = CAVE_GLOW;
        if (at((uint32_t)surface) == GRASS && at((uint32_t)surface + 1) == AIR &&
            (lhash(gx, 0, gz, P->seed ^ 0x165667b1u) & 15u) == 0u)
            at((uint32_t)surface + 1) = SHRUB;
    }
}

uint64_t orc_world_mesh(const uint8_t *vox, uint32_t nx, uint32_t ny, uint32_t nz, int32_t chunk_x0, int32_t chunk_z0,
                        int greedy, const uint32_t *mat_of, float voxel, orc_vertex *out_v, orc_triangle *out_t,
                        uint64_t cap_quads) {
    const uint32_t ncx = nx / CHUNK_XZ, ncz = nz / CHUNK_XZ;
    std::vector<Mesh> meshes((size_t)ncx * ncz);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t c = 0; c < (int64_t)ncx * ncz; ++c)
        mesh_chunk(vox, nx, ny, nz, (uint32_t)(c / ncz), (uint32_t)(c % ncz), chunk_x0, chunk_z0, greedy != 0,
                   mat_of, voxel, meshes[(size_t)c]);
    /* merge_chunk_meshes: concatenate, offsetting vertex indices */
    uint64_t quads = 0;
    for (const Mesh &m : meshes) quads += m.v.size() / 4;
    if (!out_v || !out_t || quads > cap_quads) return quads;
    uint64_t vbase = 0, tbase = 0;
    for (const Mesh &m : meshes) {
        for (size_t i = 0; i < m.v.size(); ++i) out_v[vbase + i] = m.v[i];
        for (size_t i = 0; i < m.t.size(); ++i) {
            orc_triangle t = m.t[i];
            for (int k = 0; k < 3; ++k) t.v[k] += (uint32_t)vbase;
            out_t[tbase + i] = t;
        }
        vbase += m.v.size();
        tbase += m.t.size();
    }
    return quads;
}

}  // extern "C"
