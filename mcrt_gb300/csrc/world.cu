// world.cu — the procedural voxel world on the GPU: a seeded terrain generator
// and the chunked face mesher that turns the voxel grid into the triangle mesh
// the tracer renders.
//
// Voxel grid: one byte per voxel (block id), index (x * ny + y) * nz + z — the
// XZY-major order of the reference's chunks (world/chunk.rs:26-31) extended to
// the whole grid.  Chunks are 16 x ny x 16 columns; chunk (i, k) of the grid has
// chunk coordinates (chunk_x0 + i, chunk_z0 + k) and world origin
// chunk_world_origin (world/chunk.rs:131-137).
//
// Mesher: world/mesher.rs:97-366.  Every (chunk, face direction, layer) slice
// is one thread: it rebuilds the slice's visibility mask on the fly from the
// grid (a face is visible when its block is opaque and the neighbour along the
// normal is not; outside the grid counts as air, as the reference's missing
// neighbour chunks do) and runs the reference's greedy rectangle growth with a
// visited bitset in shared memory.  A count pass, an exclusive scan and an emit
// pass place every quad where the reference's sequential loop would: chunks in
// (x outer, z inner) order, then +X, -X, +Y, -Y, +Z, -Z, layers, then the greedy
// order within the slice.  MCRT_MESH_FACES emits one quad per visible face in
// the same order (the exposed-face mesh).
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace mcrt {

namespace {

// ------------------------------------------------------------------ noise
// Lattice value noise: a PCG hash of the integer lattice point and the seed
// gives a value in [0, 1); values are blended with the smoothstep fade
// t^2 (3 - 2t).  fBm sums octaves with frequency * lacunarity and
// amplitude * gain per octave, normalised by the amplitude sum.
__device__ __forceinline__ uint32_t lattice_hash(int32_t x, int32_t y, int32_t z, uint32_t seed) {
    uint32_t h = pcg_hash((uint32_t)x * 0x8da6b343u ^ seed);
    h = pcg_hash(h ^ ((uint32_t)y * 0xd8163841u));
    return pcg_hash(h ^ ((uint32_t)z * 0xcb1ab31fu));
}
__device__ __forceinline__ float lattice_value(int32_t x, int32_t y, int32_t z, uint32_t seed) {
    return (float)(lattice_hash(x, y, z, seed) >> 8) * (1.0f / 16777216.0f);
}
__device__ __forceinline__ float fade(float t) { return t * t * (3.0f - 2.0f * t); }
__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + (b - a) * t; }

__device__ float value_noise2(float x, float z, uint32_t seed) {
    float fx0 = floorf(x), fz0 = floorf(z);
    int32_t ix = (int32_t)fx0, iz = (int32_t)fz0;
    float tx = fade(x - fx0), tz = fade(z - fz0);
    float a = lerpf(lattice_value(ix, 0, iz, seed), lattice_value(ix + 1, 0, iz, seed), tx);
    float b = lerpf(lattice_value(ix, 0, iz + 1, seed), lattice_value(ix + 1, 0, iz + 1, seed), tx);
    return lerpf(a, b, tz);
}
__device__ float value_noise3(float x, float y, float z, uint32_t seed) {
    float fx0 = floorf(x), fy0 = floorf(y), fz0 = floorf(z);
    int32_t ix = (int32_t)fx0, iy = (int32_t)fy0, iz = (int32_t)fz0;
    float tx = fade(x - fx0), ty = fade(y - fy0), tz = fade(z - fz0);
    float c[2];
    for (int k = 0; k < 2; ++k) {
        float a = lerpf(lattice_value(ix, iy, iz + k, seed), lattice_value(ix + 1, iy, iz + k, seed), tx);
        float b = lerpf(lattice_value(ix, iy + 1, iz + k, seed), lattice_value(ix + 1, iy + 1, iz + k, seed), tx);
        c[k] = lerpf(a, b, ty);
    }
    return lerpf(c[0], c[1], tz);
}
__device__ float fbm2(float x, float z, uint32_t octaves, float lac, float gain, uint32_t seed) {
    float sum = 0.0f, amp = 1.0f, norm = 0.0f, f = 1.0f;
    for (uint32_t o = 0; o < octaves; ++o) {
        sum += amp * value_noise2(x * f, z * f, seed + o * 0x9e3779b9u);
        norm += amp;
        amp *= gain;
        f *= lac;
    }
    return sum / norm;
}
__device__ float fbm3(float x, float y, float z, uint32_t octaves, float lac, float gain, uint32_t seed) {
    float sum = 0.0f, amp = 1.0f, norm = 0.0f, f = 1.0f;
    for (uint32_t o = 0; o < octaves; ++o) {
        sum += amp * value_noise3(x * f, y * f, z * f, seed + o * 0x9e3779b9u);
        norm += amp;
        amp *= gain;
        f *= lac;
    }
    return sum / norm;
}

// ------------------------------------------------------------------ generator
// Block ids of the reference's registry (world/block.rs:14-24).
constexpr uint8_t kAir = 0, kLimestone = 1, kRedSoil = 2, kGrass = 3, kSand = 4, kWater = 5, kShrub = 8,
                  kGravel = 9, kCaveGlow = 10;

// One thread per (x, z) column, z fastest so that a warp's writes of one y are
// contiguous.  Column: limestone (gravel patches) below, 3 blocks of red soil
// (sand near the sea), a grass (sand) top, caves carved by 3D fBm above
// cave_min_y, glowing flora on some cave floors, water up to the sea level,
// shrubs on some grass tops.
__global__ void k_world_generate(mcrt_world_params P, uint8_t *vox) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.nx * P.nz) return;
    const uint32_t x = t / P.nz, z = t - x * P.nz;
    const uint32_t ny = P.ny;
    const int32_t gx = P.chunk_x0 * 16 + (int32_t)x, gz = P.chunk_z0 * 16 + (int32_t)z;
    const float hn = fbm2((float)gx * P.height_freq, (float)gz * P.height_freq, P.height_octaves, P.lacunarity,
                          P.gain, P.seed);
    const float hf = P.height_base + P.height_amp * (2.0f * hn - 1.0f);
    int32_t surface = (int32_t)floorf(hf);
    surface = max(1, min(surface, (int32_t)ny - 2));
    const bool beach = (float)surface <= P.sand_line;
    uint8_t *col = vox + (size_t)x * ny * P.nz + z;
    auto at = [&](uint32_t y) -> uint8_t & { return col[(size_t)y * P.nz]; };
    for (uint32_t y = 0; y < ny; ++y) {
        const int32_t yi = (int32_t)y;
        uint8_t b = kAir;
        if (yi <= surface) {
            if (yi == surface) b = beach ? kSand : kGrass;
            else if (yi >= surface - 3) b = beach ? kSand : kRedSoil;
            else {
                b = kLimestone;
                if (value_noise3((float)gx * 0.11f, (float)yi * 0.11f, (float)gz * 0.11f, P.seed ^ 0x5bd1e995u) > 0.72f)
                    b = kGravel;
            }
            if (y >= P.cave_min_y) {
                const float c = fbm3((float)gx * P.cave_freq, (float)yi * P.cave_freq, (float)gz * P.cave_freq,
                                     P.cave_octaves, P.lacunarity, P.gain, P.seed ^ 0x6c62272eu);
                if (0.5f + (c - 0.5f) * P.cave_contrast > P.cave_threshold) b = kAir;
            }
        } else if ((float)yi <= P.sea_level) {
            b = kWater;
        }
        at(y) = b;
    }
    // cave floors: a solid block under a carved voxel below the surface
    for (uint32_t y = 1; y + 1 < ny && (int32_t)y < surface; ++y)
        if (at(y) != kAir && at(y + 1) == kAir && (lattice_hash(gx, (int32_t)y, gz, P.seed ^ 0x27d4eb2fu) & 7u) == 0u)
            at(y) = kCaveGlow;
    // shrubs on some grass tops
    if (at((uint32_t)surface) == kGrass && at((uint32_t)surface + 1) == kAir &&
        (lattice_hash(gx, 0, gz, P.seed ^ 0x165667b1u) & 15u) == 0u)
        at((uint32_t)surface + 1) = kShrub;
}

// ------------------------------------------------------------------ mesher
// BLOCK_META[id].opaque (world/block.rs:53-125): ids 1..10 occlude, air and
// unassigned ids do not.
__device__ __forceinline__ bool opaque(uint8_t id) { return id >= 1 && id <= 10; }

struct MeshGrid {
    const uint8_t *vox;
    uint32_t nx, ny, nz, ncz;
    int32_t chunk_x0, chunk_z0;
    uint32_t per_chunk;     // slices per chunk: 16 + 16 + ny + ny + 16 + 16
};

struct Slice {
    uint32_t cx, cz;        // chunk index in the grid
    int axis, sign, ua, va;
    uint32_t layer, udim, vdim;
};

__device__ __forceinline__ Slice slice_of(const MeshGrid &G, uint32_t s) {
    Slice sl;
    const uint32_t c = s / G.per_chunk;
    uint32_t r = s - c * G.per_chunk;
    sl.cx = c / G.ncz;
    sl.cz = c - sl.cx * G.ncz;
    const uint32_t dims[3] = {16u, G.ny, 16u};
    int dir = 0;
    for (; dir < 6; ++dir) {                       // +X, -X, +Y, -Y, +Z, -Z (mesher.rs:77-84)
        uint32_t n = dims[dir >> 1];
        if (r < n) break;
        r -= n;
    }
    sl.axis = dir >> 1;
    sl.sign = (dir & 1) ? -1 : 1;
    sl.layer = r;
    sl.ua = sl.axis == 0 ? 1 : 0;                  // mesher.rs:137-141
    sl.va = sl.axis == 2 ? 1 : 2;
    sl.udim = dims[sl.ua];
    sl.vdim = dims[sl.va];
    return sl;
}

// Block id of the visible face at (u, v) of the slice, 0 when hidden.
__device__ __forceinline__ uint8_t face_at(const MeshGrid &G, const Slice &sl, uint32_t u, uint32_t v) {
    uint32_t p[3];
    p[sl.axis] = sl.layer;
    p[sl.ua] = u;
    p[sl.va] = v;
    const int32_t gx = (int32_t)(sl.cx * 16 + p[0]), gy = (int32_t)p[1], gz = (int32_t)(sl.cz * 16 + p[2]);
    const uint8_t id = G.vox[((size_t)gx * G.ny + gy) * G.nz + gz];
    if (!opaque(id)) return 0;
    int32_t q[3] = {gx, gy, gz};
    q[sl.axis] += sl.sign;
    if (q[0] < 0 || q[1] < 0 || q[2] < 0 || q[0] >= (int32_t)G.nx || q[1] >= (int32_t)G.ny || q[2] >= (int32_t)G.nz)
        return id;                                 // beyond the grid: air (mesher.rs:261-300)
    const uint8_t nb = G.vox[((size_t)q[0] * G.ny + q[1]) * G.nz + q[2]];
    return opaque(nb) ? 0 : id;
}

struct MeshOut {
    mcrt_gpu_vertex *v;
    mcrt_gpu_triangle *t;
    const uint32_t *quad_base;   // per slice
    const uint32_t *mat_of;      // 256 block -> material slot
    float voxel;
};

// emit_quad, mesher.rs:308-366
__device__ void emit_quad(const MeshGrid &G, const Slice &sl, const MeshOut &O, uint32_t q, uint32_t u0, uint32_t v0,
                          uint32_t h, uint32_t w, uint8_t id) {
    const float s = O.voxel;
    const float ox = (float)(G.chunk_x0 + (int32_t)sl.cx) * 16.0f * s;
    const float oz = (float)(G.chunk_z0 + (int32_t)sl.cz) * 16.0f * s;
    const uint32_t face = sl.sign > 0 ? 1u : 0u;
    auto corner = [&](uint32_t uu, uint32_t vv, float tu, float tv, mcrt_gpu_vertex *out) {
        float p[3];
        p[sl.axis] = (float)(sl.layer + face) * s;
        p[sl.ua] = (float)uu * s;
        p[sl.va] = (float)vv * s;
        float n[3] = {0.0f, 0.0f, 0.0f};
        n[sl.axis] = (float)sl.sign;
        *out = mcrt_gpu_vertex{{ox + p[0], 0.0f + p[1], oz + p[2], 1.0f}, {n[0], n[1], n[2], 0.0f},
                               {tu, tv, 0.0f, 0.0f}};
    };
    const uint32_t b = 4 * q;
    corner(u0, v0, 0.0f, 0.0f, O.v + b);
    corner(u0 + h, v0, 1.0f, 0.0f, O.v + b + 1);
    corner(u0 + h, v0 + w, 1.0f, 1.0f, O.v + b + 2);
    corner(u0, v0 + w, 0.0f, 1.0f, O.v + b + 3);
    const uint32_t mat = O.mat_of[id];
    if (sl.sign > 0) {
        O.t[2 * q] = mcrt_gpu_triangle{{b, b + 1, b + 2}, mat};
        O.t[2 * q + 1] = mcrt_gpu_triangle{{b, b + 2, b + 3}, mat};
    } else {
        O.t[2 * q] = mcrt_gpu_triangle{{b, b + 2, b + 1}, mat};
        O.t[2 * q + 1] = mcrt_gpu_triangle{{b, b + 3, b + 2}, mat};
    }
}

// Greedy expansion of one slice (mesher.rs:185-243); EMIT = false counts quads.
template <bool EMIT>
__global__ void k_world_mesh(MeshGrid G, uint32_t n_slices, int greedy, uint32_t words_per_thread, uint32_t *counts,
                             MeshOut O) {
    extern __shared__ uint32_t visited_all[];
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_slices) return;
    uint32_t *visited = visited_all + (size_t)threadIdx.x * words_per_thread;
    const Slice sl = slice_of(G, s);
    const uint32_t cells = sl.udim * sl.vdim;
    auto vis = [&](uint32_t u, uint32_t v) {
        uint32_t k = u * sl.vdim + v;
        return (visited[k >> 5] >> (k & 31u)) & 1u;
    };
    auto mark = [&](uint32_t u, uint32_t v) {
        uint32_t k = u * sl.vdim + v;
        visited[k >> 5] |= 1u << (k & 31u);
    };
    uint32_t q = 0;
    uint32_t qbase = EMIT ? O.quad_base[s] : 0u;
    if (!greedy) {
        for (uint32_t u = 0; u < sl.udim; ++u)
            for (uint32_t v = 0; v < sl.vdim; ++v) {
                uint8_t id = face_at(G, sl, u, v);
                if (!id) continue;
                if (EMIT) emit_quad(G, sl, O, qbase + q, u, v, 1, 1, id);
                ++q;
            }
    } else {
        for (uint32_t k = 0; k < (cells + 31) / 32; ++k) visited[k] = 0u;
        for (uint32_t u0 = 0; u0 < sl.udim; ++u0) {
            uint32_t v0 = 0;
            while (v0 < sl.vdim) {
                const uint8_t id = face_at(G, sl, u0, v0);
                if (id == 0 || vis(u0, v0)) { ++v0; continue; }
                uint32_t w = 1;
                while (v0 + w < sl.vdim && face_at(G, sl, u0, v0 + w) == id && !vis(u0, v0 + w)) ++w;
                uint32_t h = 1;
                while (u0 + h < sl.udim) {
                    bool row = true;
                    for (uint32_t dv = 0; dv < w; ++dv)
                        if (face_at(G, sl, u0 + h, v0 + dv) != id || vis(u0 + h, v0 + dv)) { row = false; break; }
                    if (!row) break;
                    ++h;
                }
                for (uint32_t du = 0; du < h; ++du)
                    for (uint32_t dv = 0; dv < w; ++dv) mark(u0 + du, v0 + dv);
                if (EMIT) emit_quad(G, sl, O, qbase + q, u0, v0, h, w, id);
                ++q;
                v0 += w;
            }
        }
    }
    if (!EMIT) counts[s] = q;
}

}  // namespace

void launch_world_generate(const mcrt_world_params &P, uint8_t *vox, cudaStream_t st) {
    const uint32_t n = P.nx * P.nz;
    k_world_generate<<<(n + 127) / 128, 128, 0, st>>>(P, vox);
    ::mcrt::note_launch();
}

cudaError_t world_mesh(const uint8_t *d_vox, uint32_t nx, uint32_t ny, uint32_t nz, int32_t chunk_x0, int32_t chunk_z0,
                       bool greedy, const uint32_t *d_mat_of, float voxel, WorldMeshBuffers &M, cudaStream_t st) {
    MeshGrid G;
    G.vox = d_vox;
    G.nx = nx; G.ny = ny; G.nz = nz;
    G.ncz = nz / 16;
    G.chunk_x0 = chunk_x0;
    G.chunk_z0 = chunk_z0;
    G.per_chunk = 64 + 2 * ny;
    const uint32_t n_slices = (nx / 16) * (nz / 16) * G.per_chunk;
    // visited bits of the largest slice: 16 x ny cells (X and Z faces) or 16 x 16 (Y faces)
    const uint32_t words = (std::max(16u * ny, 256u) + 31) / 32;
    int threads = 128;
    while (threads > 16 && (size_t)threads * words * 4 > 48 * 1024) threads >>= 1;
    const size_t smem = (size_t)threads * words * 4;
    if (smem > 48 * 1024) return cudaErrorInvalidValue;
    const size_t scan_words = scan_tmp_words(n_slices + 1);
    cudaError_t e;
    if ((e = M.counts.ensure((size_t)(n_slices + 1) * 4 * 2 + scan_words * 4)) != cudaSuccess) return e;
    uint32_t *counts = M.counts.as<uint32_t>();
    uint32_t *base = counts + n_slices + 1;
    uint32_t *tmp = base + n_slices + 1;
    if ((e = cudaMemsetAsync(counts + n_slices, 0, 4, st)) != cudaSuccess) return e;
    const int blocks = (int)((n_slices + threads - 1) / threads);
    MeshOut O{};
    k_world_mesh<false><<<blocks, threads, smem, st>>>(G, n_slices, greedy ? 1 : 0, words, counts, O);
    ::mcrt::note_launch();
    exclusive_scan_u32(counts, base, n_slices + 1, tmp, st);
    uint32_t total = 0;
    if ((e = cudaMemcpyAsync(&total, base + n_slices, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    if ((uint64_t)total * 2 >= (1ull << 27) - 1) return cudaErrorInvalidValue;   // triangle-id bound of the tracer
    if ((e = M.vertices.ensure((size_t)std::max(total, 1u) * 4 * sizeof(mcrt_gpu_vertex))) != cudaSuccess) return e;
    if ((e = M.triangles.ensure((size_t)std::max(total, 1u) * 2 * sizeof(mcrt_gpu_triangle))) != cudaSuccess) return e;
    O.v = M.vertices.as<mcrt_gpu_vertex>();
    O.t = M.triangles.as<mcrt_gpu_triangle>();
    O.quad_base = base;
    O.mat_of = d_mat_of;
    O.voxel = voxel;
    k_world_mesh<true><<<blocks, threads, smem, st>>>(G, n_slices, greedy ? 1 : 0, words, counts, O);
    ::mcrt::note_launch();
    M.n_quads = total;
    return cudaGetLastError();
}

}  // namespace mcrt
