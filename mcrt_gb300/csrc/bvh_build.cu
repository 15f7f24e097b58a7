// bvh_build.cu — GPU binned SAH BVH builder, compact-layout conversion, scan.
//
// The builder is a level-synchronous parallel restatement of the reference's
// recursive CPU builder (src/mesh.rs:82-291 with src/bvh.rs:87-463):
//   * primitive bounds: the triangle AABB padded by 1e-4 on degenerate axes
//     (mesh.rs:282-291, bvh.rs:194-207), centroid = (min+max)*0.5;
//   * a node with <= 4 primitives is a leaf (bvh.rs:32, :302);
//   * otherwise 8 bins per axis over the node's centroid bounds (axes with
//     extent < 1e-8 skipped), left-prefix / right-suffix sweep, half-area SAH
//     cost (Ct = 0, Ci = 1) against a parent area clamped to 1e-8, a split is
//     taken only when strictly cheaper than the leaf (bvh.rs:388-463);
//   * the split sends the primitives of bins 0..s left.  Binning is monotone in
//     the centroid, so this is exactly the set of the l smallest centroids the
//     reference takes after sorting (bvh.rs:303-306);
//   * pre-order layout, left child = i+1, right = right_or_offset, leaves
//     reference consecutive ranges of the ordered triangle list.
// All arithmetic is the same IEEE sequence (compiled with -fmad=false), so the
// output nodes equal the reference builder's bit for bit; only the order of the
// primitives inside a leaf may differ (the partition here is stable, starting
// from the Morton order of the centroids; the reference uses an unstable sort).
#include <algorithm>
#include <utility>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "traverse.cuh"

namespace mcrt {

// ------------------------------------------------------------------ scan
namespace {
constexpr uint32_t kScanBlock = 1024;   // elements per block (256 threads x 4)

__global__ void k_scan_block(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *block_sums) {
    __shared__ uint32_t sh[256];
    uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * 4;
    uint32_t v[4];
    uint32_t local = 0;
    for (int k = 0; k < 4; ++k) {
        uint32_t idx = base + k;
        v[k] = idx < n ? in[idx] : 0u;
        local += v[k];
    }
    sh[threadIdx.x] = local;
    __syncthreads();
    for (uint32_t off = 1; off < 256; off <<= 1) {
        uint32_t t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0u;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    uint32_t run = sh[threadIdx.x] - local;   // exclusive prefix of this thread
    for (int k = 0; k < 4; ++k) {
        uint32_t idx = base + k;
        if (idx < n) out[idx] = run;
        run += v[k];
    }
    if (threadIdx.x == 255 && block_sums) block_sums[blockIdx.x] = sh[255];
}

__global__ void k_scan_add(uint32_t *out, uint32_t n, const uint32_t *block_offsets) {
    uint32_t idx = blockIdx.x * kScanBlock + threadIdx.x;
    uint32_t add = block_offsets[blockIdx.x];
    for (int k = 0; k < 4; ++k, idx += 256)
        if (idx < n) out[idx] += add;
}
}  // namespace

size_t scan_tmp_words(uint32_t n) {
    size_t words = 0;
    while (n > kScanBlock) {
        n = (n + kScanBlock - 1) / kScanBlock;
        words += 2 * (size_t)n;
    }
    return words + 2;
}

void exclusive_scan_u32(const uint32_t *d_in, uint32_t *d_out, uint32_t n, uint32_t *d_tmp, cudaStream_t st) {
    if (n == 0) return;
    uint32_t nb = (n + kScanBlock - 1) / kScanBlock;
    if (nb == 1) {
        k_scan_block<<<1, 256, 0, st>>>(d_in, d_out, n, nullptr); ::mcrt::note_launch();
        return;
    }
    uint32_t *sums = d_tmp;
    uint32_t *offs = d_tmp + nb;
    k_scan_block<<<nb, 256, 0, st>>>(d_in, d_out, n, sums); ::mcrt::note_launch();
    exclusive_scan_u32(sums, offs, nb, d_tmp + 2 * (size_t)nb, st);
    k_scan_add<<<nb, 256, 0, st>>>(d_out, n, offs); ::mcrt::note_launch();
}

// ------------------------------------------------------------------ float atomics
namespace {
__device__ __forceinline__ void atomic_min_f(float *a, float v) {
    if (v >= 0.0f) atomicMin(reinterpret_cast<int *>(a), __float_as_int(v));
    else atomicMax(reinterpret_cast<unsigned *>(a), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float *a, float v) {
    if (v >= 0.0f) atomicMax(reinterpret_cast<int *>(a), __float_as_int(v));
    else atomicMin(reinterpret_cast<unsigned *>(a), __float_as_uint(v));
}

// Order-preserving map of floats onto unsigned integers (the order the float
// atomics above use: -0 below +0), so min / max reduce as integers (redux.sync).
__device__ __forceinline__ unsigned f2ord(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}
constexpr unsigned kOrdPosInf = 0xff800000u;     // f2ord(+inf): empty minimum
constexpr unsigned kOrdNegInf = 0x007fffffu;     // f2ord(-inf): empty maximum
constexpr unsigned kFull = 0xffffffffu;

// Positions per block of the whole-array passes (4 per thread).
constexpr uint32_t kPosPerBlock = 1024;

constexpr int kBins = 8;
constexpr uint32_t kLeafMax = 4;
constexpr int kBinStride = 7;                    // count, min xyz, max xyz
constexpr int kTaskBinWords = 3 * kBins * kBinStride;

struct Aabb { float mn[3], mx[3]; };
__device__ __forceinline__ Aabb aabb_empty() {
    Aabb a;
    for (int i = 0; i < 3; ++i) { a.mn[i] = __int_as_float(0x7f800000); a.mx[i] = __int_as_float(0xff800000); }
    return a;
}
__device__ __forceinline__ Aabb aabb_union(const Aabb &a, const Aabb &b) {
    Aabb r;
    for (int i = 0; i < 3; ++i) { r.mn[i] = fminf(a.mn[i], b.mn[i]); r.mx[i] = fmaxf(a.mx[i], b.mx[i]); }
    return r;
}
__device__ __forceinline__ float half_area(const Aabb &a) {          // bvh.rs:168-175
    float d0 = a.mx[0] - a.mn[0], d1 = a.mx[1] - a.mn[1], d2 = a.mx[2] - a.mn[2];
    return d0 * d1 + d1 * d2 + d0 * d2;
}

// Build state (device pointers), sized for nt primitives.
struct BuildState {
    uint32_t nt;
    float4 *pmin, *pmax, *pcen;       // per original primitive
    uint32_t *perm[2];                // position -> original id
    int32_t *ptask[2];                // position -> task (-1: in a finished leaf)
    uint32_t *flags, *scan;           // partition flags and their exclusive scan
    // tasks (per level, double-buffered)
    uint32_t *t_start[2], *t_count[2], *t_node[2];
    float *t_bounds[2];               // 6 per task
    float *t_cb;                      // centroid bounds, 6 per task (current level)
    float *t_bins;                    // kTaskBinWords per task (current level)
    int32_t *t_split;                 // per task: axis*16 + bin, or -1 (leaf)
    uint32_t *t_lcount;
    // BFS nodes
    float4 *n_min, *n_max;            // bounds
    uint32_t *n_a, *n_b;              // internal: left bfs, right bfs; leaf: start, count
    uint32_t *n_leaf;                 // 1 = leaf
    uint32_t *n_size, *n_pre;         // subtree size, pre-order index
    // Tasks of a level: large ones (above kSmallTask primitives) at indices
    // 0, 1, ... of a task buffer, built by the whole-array passes; small ones
    // at tcap - 1, tcap - 2, ... of the same buffer, one warp each; tiny ones
    // (at most kTinyTask) in their own buffers, one thread each.
    uint32_t tcap;                    // task buffer capacity (a level has at most nt / 5 tasks)
    uint32_t *y_start[2], *y_count[2], *y_node[2];
    float *y_bounds[2];               // tiny tasks (double-buffered), 6 bounds each
    uint32_t *counters;               // [0] large tasks of the next level, [1] bfs node count,
                                      // [4] small tasks of the next level, [5] of the current level,
                                      // [6] tiny tasks of the next level, [7] of the current level
    uint32_t *level_end;              // bfs node count at the start of each level
    // spatial order: primitives are built in the order of their centroids'
    // Morton codes (radix-sorted), so a warp's positions are neighbours
    uint32_t *rkey[2], *rval[2];      // sort keys / primitive ids (ping-pong)
    uint32_t *rhist, *roffs;          // digit counts per tile and their exclusive scan
    float4 *qmin, *qmax, *qcen;       // second set of primitive bounds: the reordering target
    // single-pass partition scan of a level (k_flag_scan): [0] tile ticket,
    // [1] error word (a look-back wait gave up), [2 + t] status of tile t:
    // flag << 32 | value (flag 1: the tile's own sum, 2: inclusive prefix)
    unsigned long long *part;
};
constexpr uint32_t kFlagThreads = 256, kFlagItems = 8;   // k_flag_scan: positions per thread, per block
constexpr uint32_t kFlagTile = kFlagThreads * kFlagItems;
constexpr uint32_t kLookbackPolls = 1u << 20;              // polls of one predecessor before giving up
constexpr uint32_t kSmallTask = 256;       // tasks up to this size are built by one warp each
constexpr uint32_t kTinyTask = 8;          // and up to this size by one thread each
constexpr uint32_t kMaxLevels = 4096;
}  // namespace

struct BvhScratch {
    uint32_t cap = 0;
    void *mem = nullptr;
    BuildState s{};
    uint32_t *scan_tmp = nullptr;
};

void free_bvh_scratch(BvhScratch *s) {
    if (!s) return;
    if (s->mem) cudaFree(s->mem);
    delete s;
}

namespace {

__global__ void k_prim_bounds(const mcrt_gpu_vertex *verts, const mcrt_gpu_triangle *tris, BuildState S) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.nt) return;
    mcrt_gpu_triangle t = tris[i];
    Aabb b = aabb_empty();
    for (int k = 0; k < 3; ++k) {                                   // from_points_3, bvh.rs:113-126
        const float *p = verts[t.v[k]].position;
        for (int a = 0; a < 3; ++a) { b.mn[a] = fminf(b.mn[a], p[a]); b.mx[a] = fmaxf(b.mx[a], p[a]); }
    }
    const float EPS = 1e-4f;                                        // padded, bvh.rs:194-207
    Aabb pb;
    for (int a = 0; a < 3; ++a) { pb.mn[a] = fminf(b.mn[a], b.mx[a] - EPS); pb.mx[a] = fmaxf(b.mx[a], b.mn[a] + EPS); }
    float c[3];
    for (int a = 0; a < 3; ++a) c[a] = (pb.mn[a] + pb.mx[a]) * 0.5f;   // centroid, bvh.rs:179-185
    S.pmin[i] = make_float4(pb.mn[0], pb.mn[1], pb.mn[2], 0.0f);
    S.pmax[i] = make_float4(pb.mx[0], pb.mx[1], pb.mx[2], 0.0f);
    S.pcen[i] = make_float4(c[0], c[1], c[2], 0.0f);
    S.perm[0][i] = i;
    S.ptask[0][i] = 0;
}

// Sphere primitive bounds: Aabb::from_sphere (bvh.rs:133-143), not padded.
__global__ void k_sphere_bounds(const mcrt_gpu_sphere *sph, BuildState S) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.nt) return;
    float4 cr = *reinterpret_cast<const float4 *>(sph + i);
    float mn[3] = {cr.x - cr.w, cr.y - cr.w, cr.z - cr.w};
    float mx[3] = {cr.x + cr.w, cr.y + cr.w, cr.z + cr.w};
    float c[3];
    for (int a = 0; a < 3; ++a) c[a] = (mn[a] + mx[a]) * 0.5f;
    S.pmin[i] = make_float4(mn[0], mn[1], mn[2], 0.0f);
    S.pmax[i] = make_float4(mx[0], mx[1], mx[2], 0.0f);
    S.pcen[i] = make_float4(c[0], c[1], c[2], 0.0f);
    S.perm[0][i] = i;
    S.ptask[0][i] = 0;
}

// root bounds: one task covering everything
__global__ void k_root_init(BuildState S) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        S.t_start[0][0] = 0;
        S.t_count[0][0] = S.nt;
        S.t_node[0][0] = 0;
        for (int a = 0; a < 3; ++a) {
            S.t_bounds[0][a] = __int_as_float(0x7f800000);
            S.t_bounds[0][3 + a] = __int_as_float(0xff800000);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < 16) S.counters[threadIdx.x] = threadIdx.x == 1 ? 1u : 0u;
}

// Root bounds: per-thread min / max over 4 primitives, warp and block
// reductions on the ordered integers, six global atomics per block.
__global__ void __launch_bounds__(256) k_root_bounds(BuildState S) {
    __shared__ unsigned sh[6];
    if (threadIdx.x < 6) sh[threadIdx.x] = threadIdx.x < 3 ? kOrdPosInf : kOrdNegInf;
    __syncthreads();
    const uint32_t first = blockIdx.x * kPosPerBlock, end = min(first + kPosPerBlock, S.nt);
    unsigned o[6] = {kFull, kFull, kFull, 0u, 0u, 0u};
    for (uint32_t i = first + threadIdx.x; i < end; i += 256) {
        const float4 a = S.pmin[i], b = S.pmax[i];
        o[0] = min(o[0], f2ord(a.x)); o[1] = min(o[1], f2ord(a.y)); o[2] = min(o[2], f2ord(a.z));
        o[3] = max(o[3], f2ord(b.x)); o[4] = max(o[4], f2ord(b.y)); o[5] = max(o[5], f2ord(b.z));
    }
    for (int a = 0; a < 3; ++a) {
        o[a] = __reduce_min_sync(kFull, o[a]);
        o[3 + a] = __reduce_max_sync(kFull, o[3 + a]);
    }
    if ((threadIdx.x & 31u) == 0)
        for (int a = 0; a < 3; ++a) { atomicMin(&sh[a], o[a]); atomicMax(&sh[3 + a], o[3 + a]); }
    __syncthreads();
    if (threadIdx.x < 3) atomic_min_f(&S.t_bounds[0][threadIdx.x], ord2f(sh[threadIdx.x]));
    else if (threadIdx.x < 6) atomic_max_f(&S.t_bounds[0][threadIdx.x], ord2f(sh[threadIdx.x]));
}

// ---- spatial order of the primitives
// The tree does not depend on the order the primitives start in (binning and
// the stable partition are decided by centroids alone); only the order inside
// a leaf does.  Starting from Morton order keeps the 32 positions of a warp
// neighbours in space at every level, so their bins mostly agree and the
// warp reductions above take one pass.

__device__ __forceinline__ uint32_t morton_expand10(uint32_t v) {
    v &= 1023u;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// 30-bit Morton code of each centroid on a 1024^3 grid over the root bounds.
__global__ void k_morton(BuildState S) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.nt) return;
    const float4 c = S.pcen[i];
    const float cc[3] = {c.x, c.y, c.z};
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
        const float lo = S.t_bounds[0][a], ext = S.t_bounds[0][3 + a] - lo;
        const float f = ext > 0.0f ? (cc[a] - lo) / ext * 1024.0f : 0.0f;
        q[a] = min(f2u_sat(f), 1023u);
    }
    S.rkey[0][i] = (morton_expand10(q[0]) << 2) | (morton_expand10(q[1]) << 1) | morton_expand10(q[2]);
    S.rval[0][i] = i;
}

constexpr uint32_t kRadixTile = 2048;      // keys per block of a radix pass (256 threads x 8 rounds)

// Digit counts of one tile, stored digit-major (digit * tiles + tile) so that
// their exclusive scan is each tile's output offset per digit.
__global__ void __launch_bounds__(256) k_radix_hist(const uint32_t *keys, uint32_t n, int shift, uint32_t tiles,
                                                    uint32_t *hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kRadixTile;
    for (uint32_t k = threadIdx.x; k < kRadixTile; k += 256) {
        const uint32_t i = base + k;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile by its digit: rounds of 256 keys in tile order;
// within a round, a key's rank = the tile's running offset of its digit + the
// counts of earlier warps + the lanes before it with the same digit.
__global__ void __launch_bounds__(256) k_radix_scatter(const uint32_t *kin, const uint32_t *vin, uint32_t n, int shift,
                                                       uint32_t tiles, const uint32_t *offs, uint32_t *kout,
                                                       uint32_t *vout) {
    __shared__ uint32_t wcnt[8][256];
    __shared__ uint32_t wpre[8][256];
    __shared__ uint32_t run[256];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    for (int k = 0; k < 8; ++k) wcnt[k][threadIdx.x] = 0;
    run[threadIdx.x] = offs[threadIdx.x * tiles + blockIdx.x];
    __syncthreads();
    const uint32_t base = blockIdx.x * kRadixTile;
    const unsigned lanes_below = (1u << lane) - 1u;
    for (uint32_t r = 0; r < kRadixTile / 256; ++r) {
        const uint32_t i = base + r * 256 + threadIdx.x;
        const bool valid = i < n;
        uint32_t key = 0, val = 0, d = 256;             // 256: no key (its own group)
        if (valid) { key = kin[i]; val = vin[i]; d = (key >> shift) & 255u; }
        const unsigned peers = __match_any_sync(kFull, d);
        const uint32_t prank = __popc(peers & lanes_below);
        if (valid && prank == 0) wcnt[w][d] = __popc(peers);
        __syncthreads();
        {
            const uint32_t dd = threadIdx.x;             // one digit per thread: prefix over the warps
            uint32_t acc = run[dd];
            for (int k = 0; k < 8; ++k) {
                const uint32_t c = wcnt[k][dd];
                wpre[k][dd] = acc;
                acc += c;
                wcnt[k][dd] = 0;
            }
            run[dd] = acc;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = wpre[w][d] + prank;
            kout[pos] = key;
            vout[pos] = val;
        }
    }
}

// Primitive bounds into Morton order; positions start as the identity of that order.
__global__ void k_reorder(BuildState S) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= S.nt) return;
    const uint32_t id = S.rval[0][j];
    S.qmin[j] = S.pmin[id];
    S.qmax[j] = S.pmax[id];
    S.qcen[j] = S.pcen[id];
    S.perm[0][j] = j;
    S.ptask[0][j] = 0;
}

// Output order: the primitive ids of the final positions (Morton index -> id).
__global__ void k_final_order(const uint32_t *perm, const uint32_t *sorted_ids, uint32_t n, uint32_t *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = sorted_ids[perm[i]];
}

// The start of a level: the current level's small and tiny task counts (those
// of the level before), the node count at its start, and fresh child-task
// counters.  One thread.
__device__ __forceinline__ void level_advance(BuildState &S, uint32_t level) {
    S.counters[0] = 0;
    S.counters[5] = S.counters[4];
    S.counters[4] = 0;
    S.counters[7] = S.counters[6];
    S.counters[6] = 0;
    S.level_end[level] = S.counters[1];
}

// The start of a level with large tasks, in one launch: level_advance, the
// status words of the level's partition scan zeroed (n_part), and the large
// tasks' centroid bounds and bins set to empty.
__global__ void k_task_reset(BuildState S, uint32_t level, uint32_t ntasks, uint32_t n_part) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) level_advance(S, level);
    if (i < n_part) S.part[i] = 0ull;
    if (i >= ntasks * (6 + kTaskBinWords)) return;
    uint32_t t = i / (6 + kTaskBinWords), k = i % (6 + kTaskBinWords);
    if (k < 6) {
        S.t_cb[6 * t + k] = __int_as_float(k < 3 ? 0x7f800000 : 0xff800000);
    } else {
        uint32_t w = k - 6;
        uint32_t f = w % kBinStride;
        float v = f == 0 ? 0.0f : __int_as_float(f < 4 ? 0x7f800000 : 0xff800000);
        S.t_bins[(size_t)t * kTaskBinWords + w] = v;
    }
}

// First and last position of a block; the block's task if every position in
// between belongs to it (tasks are contiguous ranges, so the ends decide), else -1.
__device__ __forceinline__ int block_single_task(const BuildState &S, int cur, uint32_t first, uint32_t end) {
    const int t0 = S.ptask[cur][first], t1 = S.ptask[cur][end - 1];
    return (t0 == t1 && t0 >= 0) ? t0 : -1;
}

// Centroid bounds per task.  Lanes reduce first (one pass per distinct task in
// the warp, redux.sync on the ordered integers); a block inside one task
// combines its warps in shared memory and issues six global atomics.
__global__ void __launch_bounds__(256) k_centroid_bounds(BuildState S, int cur) {
    __shared__ unsigned sh[6];
    __shared__ int block_task;
    const uint32_t first = blockIdx.x * kPosPerBlock;
    const uint32_t end = min(first + kPosPerBlock, S.nt);
    const uint32_t lane = threadIdx.x & 31u;
    if (threadIdx.x == 0) block_task = block_single_task(S, cur, first, end);
    if (threadIdx.x < 6) sh[threadIdx.x] = threadIdx.x < 3 ? kOrdPosInf : kOrdNegInf;
    __syncthreads();
    const int bt = block_task;
    if (bt >= 0) {
        unsigned o[6] = {kFull, kFull, kFull, 0u, 0u, 0u};
        for (uint32_t i = first + threadIdx.x; i < end; i += 256) {
            const float4 c = S.pcen[S.perm[cur][i]];
            const unsigned q[3] = {f2ord(c.x), f2ord(c.y), f2ord(c.z)};
            for (int a = 0; a < 3; ++a) { o[a] = min(o[a], q[a]); o[3 + a] = max(o[3 + a], q[a]); }
        }
        for (int a = 0; a < 3; ++a) {
            o[a] = __reduce_min_sync(kFull, o[a]);
            o[3 + a] = __reduce_max_sync(kFull, o[3 + a]);
        }
        if (lane == 0)
            for (int a = 0; a < 3; ++a) { atomicMin(&sh[a], o[a]); atomicMax(&sh[3 + a], o[3 + a]); }
        __syncthreads();
        if (threadIdx.x < 3) atomic_min_f(&S.t_cb[6 * bt + threadIdx.x], ord2f(sh[threadIdx.x]));
        else if (threadIdx.x < 6) atomic_max_f(&S.t_cb[6 * bt + threadIdx.x], ord2f(sh[threadIdx.x]));
        return;
    }
    for (uint32_t base = first + (threadIdx.x & ~31u); base < end; base += 256) {   // warp-uniform
        const uint32_t i = base + lane;
        const int task = i < end ? S.ptask[cur][i] : -1;
        float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (task >= 0) c = S.pcen[S.perm[cur][i]];
        const unsigned q[3] = {f2ord(c.x), f2ord(c.y), f2ord(c.z)};
        unsigned pending = __ballot_sync(kFull, task >= 0);
        while (pending) {
            const int leader = __ffs(pending) - 1;
            const int lt = __shfl_sync(kFull, task, leader);
            const bool mine = task == lt;
            pending &= ~__ballot_sync(kFull, mine);
            unsigned r[6];
            for (int a = 0; a < 3; ++a) {
                r[a] = __reduce_min_sync(kFull, mine ? q[a] : kFull);
                r[3 + a] = __reduce_max_sync(kFull, mine ? q[a] : 0u);
            }
            if ((int)lane == leader)
                for (int a = 0; a < 3; ++a) {
                    atomic_min_f(&S.t_cb[6 * lt + a], ord2f(r[a]));
                    atomic_max_f(&S.t_cb[6 * lt + 3 + a], ord2f(r[3 + a]));
                }
        }
    }
}

__device__ __forceinline__ uint32_t bin_of(float c, float cmin, float len) {
    float t = (c - cmin) / len;                                     // bvh.rs:412-415
    uint32_t b = f2u_sat(t * (float)kBins);
    return b > (uint32_t)(kBins - 1) ? (uint32_t)(kBins - 1) : b;
}

// One warp's contribution to the bins of one axis: lanes with the same
// (task, bin) key form a group (match.any) and reduce within it (redux.sync
// on the group's mask, the ordered integers); the group's first lane adds the
// result — into the shared bins `sh` (ordered-integer form) when given, else
// into the task's global bins.
__device__ __forceinline__ void bin_axis_warp(BuildState &S, unsigned *sh, int axis, bool valid, int task,
                                              uint32_t b, const unsigned mn[3], const unsigned mx[3],
                                              uint32_t lane) {
    const unsigned key = valid ? ((unsigned)task << 3) | b : kFull;
    const unsigned peers = __match_any_sync(kFull, key);
    if (!valid) return;
    unsigned r[6];
    for (int a = 0; a < 3; ++a) {
        r[a] = __reduce_min_sync(peers, mn[a]);
        r[3 + a] = __reduce_max_sync(peers, mx[a]);
    }
    if ((int)lane != __ffs(peers) - 1) return;
    const int o = (axis * kBins + (int)b) * kBinStride;
    if (sh) {
        atomicAdd(sh + o, (unsigned)__popc(peers));
        for (int a = 0; a < 3; ++a) { atomicMin(sh + o + 1 + a, r[a]); atomicMax(sh + o + 4 + a, r[3 + a]); }
    } else {
        float *g = S.t_bins + (size_t)task * kTaskBinWords + o;
        atomicAdd(reinterpret_cast<unsigned *>(g), (unsigned)__popc(peers));
        for (int a = 0; a < 3; ++a) {
            atomic_min_f(g + 1 + a, ord2f(r[a]));
            atomic_max_f(g + 4 + a, ord2f(r[3 + a]));
        }
    }
}

// One warp's contribution to the bins of all three axes (task < 0: lane
// without a primitive).  An axis on which every lane has the same (task, bin)
// adds the warp's union of primitive bounds, reduced once for all such axes;
// the other axes reduce by groups (bin_axis_warp).  b[axis] = the lane's bin
// on each axis with an extent (0 otherwise).
__device__ __forceinline__ void bins_warp(BuildState &S, unsigned *sh, int task, float4 c, const float cb[6],
                                          const unsigned mn[3], const unsigned mx[3], uint32_t lane,
                                          uint32_t b[3]) {
    const float cc[3] = {c.x, c.y, c.z};
    bool valid[3];
    bool uni[3];
    for (int axis = 0; axis < 3; ++axis) {
        const float len = cb[3 + axis] - cb[axis];
        valid[axis] = task >= 0 && !(len < 1e-8f);
        b[axis] = valid[axis] ? bin_of(cc[axis], cb[axis], len) : 0u;
        const unsigned key = valid[axis] ? ((unsigned)task << 3) | b[axis] : kFull;
        const unsigned k0 = __shfl_sync(kFull, key, 0);
        uni[axis] = __all_sync(kFull, key == k0) && k0 != kFull;
    }
    if (uni[0] || uni[1] || uni[2]) {                 // warp-uniform; every lane holds a primitive
        unsigned r[6];
        for (int a = 0; a < 3; ++a) {
            r[a] = __reduce_min_sync(kFull, mn[a]);
            r[3 + a] = __reduce_max_sync(kFull, mx[a]);
        }
        if (lane == 0)
            for (int axis = 0; axis < 3; ++axis) {
                if (!uni[axis]) continue;
                const int o = (axis * kBins + (int)b[axis]) * kBinStride;
                if (sh) {
                    atomicAdd(sh + o, 32u);
                    for (int a = 0; a < 3; ++a) { atomicMin(sh + o + 1 + a, r[a]); atomicMax(sh + o + 4 + a, r[3 + a]); }
                } else {
                    float *g = S.t_bins + (size_t)task * kTaskBinWords + o;
                    atomicAdd(reinterpret_cast<unsigned *>(g), 32u);
                    for (int a = 0; a < 3; ++a) {
                        atomic_min_f(g + 1 + a, ord2f(r[a]));
                        atomic_max_f(g + 4 + a, ord2f(r[3 + a]));
                    }
                }
            }
    }
    for (int axis = 0; axis < 3; ++axis)
        if (!uni[axis]) bin_axis_warp(S, sh, axis, valid[axis], task, b[axis], mn, mx, lane);
}

// Bin accumulation (count and primitive-bounds union per bin and axis).  Warps
// reduce lanes of equal (task, bin) first; a block inside one task collects
// its warps in shared memory and adds the block's bins to the global ones.
__global__ void __launch_bounds__(256) k_bins(BuildState S, int cur) {
    __shared__ unsigned sh[kTaskBinWords];
    __shared__ int block_task;
    const uint32_t first = blockIdx.x * kPosPerBlock;
    const uint32_t end = min(first + kPosPerBlock, S.nt);
    const uint32_t lane = threadIdx.x & 31u;
    if (threadIdx.x == 0) block_task = block_single_task(S, cur, first, end);
    for (int k = threadIdx.x; k < kTaskBinWords; k += blockDim.x) {
        const uint32_t f = k % kBinStride;
        sh[k] = f == 0 ? 0u : (f < 4 ? kOrdPosInf : kOrdNegInf);
    }
    __syncthreads();
    const int bt = block_task;
    unsigned *dst = bt >= 0 ? sh : nullptr;
    for (uint32_t base = first + (threadIdx.x & ~31u); base < end; base += 256) {   // warp-uniform
        const uint32_t i = base + lane;
        const int task = i < end ? S.ptask[cur][i] : -1;
        if (__all_sync(kFull, task < 0)) continue;              // leaves and small tasks only
        float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f), bmn = c, bmx = c;
        float cb[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        if (task >= 0) {
            const uint32_t id = S.perm[cur][i];
            c = S.pcen[id]; bmn = S.pmin[id]; bmx = S.pmax[id];
            for (int k = 0; k < 6; ++k) cb[k] = S.t_cb[6 * task + k];
        }
        const unsigned mn[3] = {f2ord(bmn.x), f2ord(bmn.y), f2ord(bmn.z)};
        const unsigned mx[3] = {f2ord(bmx.x), f2ord(bmx.y), f2ord(bmx.z)};
        uint32_t b[3];
        bins_warp(S, dst, task, c, cb, mn, mx, lane, b);
    }
    if (bt < 0) return;
    __syncthreads();
    float *g = S.t_bins + (size_t)bt * kTaskBinWords;
    for (int k = threadIdx.x; k < kTaskBinWords; k += blockDim.x) {
        const uint32_t f = k % kBinStride;
        if (f == 0) {
            if (sh[k]) atomicAdd(reinterpret_cast<unsigned *>(g + k), sh[k]);
        } else if (f < 4) {
            if (sh[k] != kOrdPosInf) atomic_min_f(g + k, ord2f(sh[k]));
        } else {
            if (sh[k] != kOrdNegInf) atomic_max_f(g + k, ord2f(sh[k]));
        }
    }
}

// SAH split choice of one task (bvh.rs:388-463) from its node bounds tb,
// centroid bounds cb and bins.  Returns the split (axis * 16 + bin), or -1 when
// the task stays a leaf; *lcount = primitives going left, *bl / *br = the
// children's bounds.
// Best split so far of the serial SAH sweep.
struct SplitBest {
    float cost;                    // starts at the leaf cost n
    int axis = 0, bin = 0;
    uint32_t l = 0;
    bool found = false;
    Aabb lb, rb;
};
__device__ __forceinline__ SplitBest split_best_init(uint32_t n) {
    SplitBest b;
    b.cost = (float)n;
    b.lb = aabb_empty();
    b.rb = aabb_empty();
    return b;
}

// One axis of the SAH sweep (bvh.rs:388-463): prefix unions of bins 0..s,
// suffix unions of bins 7..s+1, cost (A_l * n_l + A_r * n_r) / A_parent,
// replaced only on a strictly smaller cost.  get(k, f) = field f of bin k
// (0: count as bits, 1-3: min, 4-6: max).
template <class Get>
__device__ __forceinline__ void split_axis(int axis, float parent, Get get, SplitBest &best) {
    Aabb bb[kBins];
    uint32_t bc[kBins];
    for (int k = 0; k < kBins; ++k) {
        bc[k] = __float_as_uint(get(k, 0));
        for (int a = 0; a < 3; ++a) { bb[k].mn[a] = get(k, 1 + a); bb[k].mx[a] = get(k, 4 + a); }
    }
    Aabb lb[kBins];
    uint32_t lc[kBins];
    lb[0] = bb[0]; lc[0] = bc[0];
    for (int k = 1; k < kBins; ++k) { lb[k] = aabb_union(lb[k - 1], bb[k]); lc[k] = lc[k - 1] + bc[k]; }
    Aabb rb = aabb_empty();
    uint32_t rc = 0;
    for (int s = kBins - 2; s >= 0; --s) {
        rb = aabb_union(rb, bb[s + 1]);
        rc += bc[s + 1];
        const uint32_t l = lc[s];
        if (l == 0 || rc == 0) continue;
        const float cost = (half_area(lb[s]) * (float)l + half_area(rb) * (float)rc) / parent;
        if (cost < best.cost) {
            best.cost = cost; best.axis = axis; best.bin = s; best.l = l; best.found = true;
            best.lb = lb[s]; best.rb = rb;
        }
    }
}

// The split of a finished sweep: axis * 16 + bin, or -1 for a leaf.
__device__ __forceinline__ int split_result(const SplitBest &best, uint32_t n, uint32_t *lcount, Aabb *bl, Aabb *br) {
    if (!(best.found && best.l > 0 && best.l < n)) return -1;
    *lcount = best.l;
    *bl = best.lb;
    *br = best.rb;
    return best.axis * 16 + best.bin;
}

__device__ __forceinline__ float node_half_area(const float *tb) {
    Aabb nb;
    for (int a = 0; a < 3; ++a) { nb.mn[a] = tb[a]; nb.mx[a] = tb[3 + a]; }
    return fmaxf(half_area(nb), 1e-8f);
}

__device__ int choose_split(uint32_t n, const float *tb, const float *cb, const float *bins, uint32_t *lcount,
                            Aabb *bl, Aabb *br) {
    const float parent = node_half_area(tb);
    SplitBest best = split_best_init(n);
    for (int axis = 0; axis < 3; ++axis) {
        const float len = cb[3 + axis] - cb[axis];
        if (len < 1e-8f) continue;
        const float *q = bins + axis * kBins * kBinStride;
        split_axis(axis, parent, [&](int k, int f) { return q[k * kBinStride + f]; }, best);
    }
    return split_result(best, n, lcount, bl, br);
}

// choose_split evaluated by a warp.  Lane j < 21 takes the serial loop's j-th
// candidate (axis j / 7, split 6 - j % 7) and forms its left union over bins
// 0..s ascending and its right union over bins 7..s+1 descending — the serial
// loop's operation order, so every cost has the same bits — and the cheapest
// candidate below the leaf cost wins, ties to the earliest (the serial loop
// replaces only on a strictly smaller cost).  Every lane gets the result.
__device__ int choose_split_warp(uint32_t n, const float *tb, const float *cb, const float *bins, uint32_t lane,
                                 uint32_t *lcount, Aabb *bl, Aabb *br) {
    Aabb nb;
    for (int a = 0; a < 3; ++a) { nb.mn[a] = tb[a]; nb.mx[a] = tb[3 + a]; }
    const float parent = fmaxf(half_area(nb), 1e-8f);
    const int axis = (int)lane / 7, s = 6 - (int)lane % 7;
    bool ok = lane < 21u;
    float cost = 0.0f;
    uint32_t l = 0, rc = 0;
    Aabb lb = aabb_empty(), rb = aabb_empty();
    if (ok) {
        const float len = cb[3 + axis] - cb[axis];
        if (len < 1e-8f) {
            ok = false;
        } else {
            const float *q = bins + axis * kBins * kBinStride;
            auto box = [&](int k) {
                Aabb b;
                for (int a = 0; a < 3; ++a) { b.mn[a] = q[k * kBinStride + 1 + a]; b.mx[a] = q[k * kBinStride + 4 + a]; }
                return b;
            };
            lb = box(0);
            l = __float_as_uint(q[0]);
            for (int k = 1; k <= s; ++k) { lb = aabb_union(lb, box(k)); l += __float_as_uint(q[k * kBinStride]); }
            for (int k = kBins - 1; k > s; --k) { rb = aabb_union(rb, box(k)); rc += __float_as_uint(q[k * kBinStride]); }
            if (l == 0 || rc == 0) ok = false;
            else cost = (half_area(lb) * (float)l + half_area(rb) * (float)rc) / parent;
            ok = ok && cost < (float)n;
        }
    }
    const unsigned oc = ok ? f2ord(cost) : kFull;
    const unsigned best = __reduce_min_sync(kFull, oc);
    if (best == kFull) return -1;
    const int win = (int)__reduce_min_sync(kFull, (ok && oc == best) ? lane : kFull);
    *lcount = __shfl_sync(kFull, l, win);
    for (int a = 0; a < 3; ++a) {
        bl->mn[a] = __shfl_sync(kFull, lb.mn[a], win); bl->mx[a] = __shfl_sync(kFull, lb.mx[a], win);
        br->mn[a] = __shfl_sync(kFull, rb.mn[a], win); br->mx[a] = __shfl_sync(kFull, rb.mx[a], win);
    }
    return (win / 7) * 16 + (6 - win % 7);
}

// Child tasks a split creates, by class: large (above kSmallTask primitives),
// small (above kTinyTask) and tiny (above the leaf size).
__device__ __forceinline__ uint32_t child_large(uint32_t n, uint32_t lcount) {
    return (lcount > kSmallTask ? 1u : 0u) + (n - lcount > kSmallTask ? 1u : 0u);
}
__device__ __forceinline__ uint32_t child_small(uint32_t n, uint32_t lcount) {
    auto small = [](uint32_t c) { return c > kTinyTask && c <= kSmallTask; };
    return (small(lcount) ? 1u : 0u) + (small(n - lcount) ? 1u : 0u);
}
__device__ __forceinline__ uint32_t child_tiny(uint32_t n, uint32_t lcount) {
    auto tiny = [](uint32_t c) { return c > kLeafMax && c <= kTinyTask; };
    return (tiny(lcount) ? 1u : 0u) + (tiny(n - lcount) ? 1u : 0u);
}
constexpr uint32_t kSmallFlag = 0x80000000u;     // task map: the child is a small or tiny task

// Node records of a task.  A leaf (sp < 0) keeps its range.  A split gets the
// BFS ids child0, child0 + 1 for its children; its large children get the task
// ids large0, large0 + 1, its small children small0, small0 + 1 (a small task
// k is stored at index tcap - 1 - k) and its tiny children tiny0, tiny0 + 1
// (in child order) in buffer nxt.  child_task[c] = -1 for a leaf child.  Ids
// come from the caller, which reserves them for a whole warp with one atomic
// each (same-address atomics per task serialise at the L2).
__device__ void record_task(BuildState &S, int nxt, uint32_t start, uint32_t n, uint32_t node, int sp,
                            uint32_t lcount, const Aabb &bl, const Aabb &br, uint32_t child0, uint32_t large0,
                            uint32_t small0, uint32_t tiny0, int child_task[2]) {
    child_task[0] = child_task[1] = -1;
    if (sp < 0) {
        S.n_leaf[node] = 1; S.n_a[node] = start; S.n_b[node] = n;
        return;
    }
    S.n_leaf[node] = 0;
    const uint32_t counts[2] = {lcount, n - lcount};
    const uint32_t starts[2] = {start, start + lcount};
    const Aabb *cbx[2] = {&bl, &br};
    for (int c = 0; c < 2; ++c) {
        const uint32_t id = child0 + (uint32_t)c;
        S.n_min[id] = make_float4(cbx[c]->mn[0], cbx[c]->mn[1], cbx[c]->mn[2], 0.0f);
        S.n_max[id] = make_float4(cbx[c]->mx[0], cbx[c]->mx[1], cbx[c]->mx[2], 0.0f);
        if (counts[c] <= kLeafMax) {
            S.n_leaf[id] = 1; S.n_a[id] = starts[c]; S.n_b[id] = counts[c];
            continue;
        }
        S.n_leaf[id] = 0;
        if (counts[c] <= kTinyTask) {
            const uint32_t task = tiny0++;
            S.y_start[nxt][task] = starts[c];
            S.y_count[nxt][task] = counts[c];
            S.y_node[nxt][task] = id;
            for (int a = 0; a < 3; ++a) {
                S.y_bounds[nxt][6 * task + a] = cbx[c]->mn[a];
                S.y_bounds[nxt][6 * task + 3 + a] = cbx[c]->mx[a];
            }
            S.n_size[id] = kSmallFlag;
            child_task[c] = (int)task;
            continue;
        }
        const bool small = counts[c] <= kSmallTask;
        const uint32_t task = small ? S.tcap - 1u - small0++ : large0++;
        S.t_start[nxt][task] = starts[c];
        S.t_count[nxt][task] = counts[c];
        S.t_node[nxt][task] = id;
        for (int a = 0; a < 3; ++a) {
            S.t_bounds[nxt][6 * task + a] = cbx[c]->mn[a];
            S.t_bounds[nxt][6 * task + 3 + a] = cbx[c]->mx[a];
        }
        // the child's positions learn their new task id in k_scatter through this map
        S.n_size[id] = small ? kSmallFlag : task;      // temporary: child node -> task id
        child_task[c] = (int)task;
    }
    S.n_a[node] = child0;
    S.n_b[node] = child0 + 1;
}

// One thread per task: split choice, then ids for the children reserved per
// warp (prefix sums by shuffles, one atomic per counter).
__global__ void k_split(BuildState S, int cur, uint32_t ntasks) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u;
    if ((t & ~31u) >= ntasks) return;                     // whole warps
    const bool active = t < ntasks;
    uint32_t start = 0, n = 0, node = 0, lcount = 0;
    int sp = -1;
    Aabb bl = aabb_empty(), br = aabb_empty();
    if (active) {
        start = S.t_start[cur][t]; n = S.t_count[cur][t]; node = S.t_node[cur][t];
        sp = choose_split(n, S.t_bounds[cur] + 6 * t, S.t_cb + 6 * t, S.t_bins + (size_t)t * kTaskBinWords, &lcount,
                          &bl, &br);
    }
    const uint32_t my_nodes = sp >= 0 ? 2u : 0u;
    const uint32_t my_large = sp >= 0 ? child_large(n, lcount) : 0u;
    const uint32_t my_small = sp >= 0 ? child_small(n, lcount) : 0u;
    const uint32_t my_tiny = sp >= 0 ? child_tiny(n, lcount) : 0u;
    uint32_t pn = my_nodes, pl = my_large, ps = my_small, py = my_tiny;   // inclusive prefix sums over the warp
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t a = __shfl_up_sync(kFull, pn, off), b = __shfl_up_sync(kFull, pl, off);
        const uint32_t c = __shfl_up_sync(kFull, ps, off), d = __shfl_up_sync(kFull, py, off);
        if ((int)lane >= off) { pn += a; pl += b; ps += c; py += d; }
    }
    const uint32_t tn = __shfl_sync(kFull, pn, 31), tl = __shfl_sync(kFull, pl, 31);
    const uint32_t ts = __shfl_sync(kFull, ps, 31), ty = __shfl_sync(kFull, py, 31);
    uint32_t bn = 0, bl0 = 0, bs = 0, by = 0;
    if (lane == 0) {
        if (tn) bn = atomicAdd(S.counters + 1, tn);
        if (tl) bl0 = atomicAdd(S.counters, tl);
        if (ts) bs = atomicAdd(S.counters + 4, ts);
        if (ty) by = atomicAdd(S.counters + 6, ty);
    }
    bn = __shfl_sync(kFull, bn, 0);
    bl0 = __shfl_sync(kFull, bl0, 0);
    bs = __shfl_sync(kFull, bs, 0);
    by = __shfl_sync(kFull, by, 0);
    if (!active) return;
    int ct[2];
    record_task(S, cur ^ 1, start, n, node, sp, lcount, bl, br, bn + pn - my_nodes, bl0 + pl - my_large,
                bs + ps - my_small, by + py - my_tiny, ct);
    S.t_split[t] = sp;
    if (sp >= 0) S.t_lcount[t] = lcount;
}

// Levels whose tasks are all small: one warp per task does what the per-level
// kernels above do for the whole array — centroid bounds (warp reduction),
// bins (shared-memory atomics private to the warp), the split of lane 0, and a
// stable partition by ballot — so a level is one launch.  Positions that land
// in a leaf are written to both permutation buffers (they never move again).
__global__ void __launch_bounds__(256) k_small_level(BuildState S, int cur) {
    __shared__ float wbins[8][kTaskBinWords];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (k >= S.counters[5]) return;                            // whole warps leave together
    const uint32_t t = S.tcap - 1u - k;                        // small tasks from the top of the buffer
    const uint32_t start = S.t_start[cur][t], n = S.t_count[cur][t], node = S.t_node[cur][t];
    const uint32_t *perm_in = S.perm[cur];
    // A task of at most 32 primitives keeps one per lane in registers for all
    // passes (one load each); a larger one streams chunks of 32 per pass.
    const bool one = n <= 32u;                                 // warp-uniform
    const bool in0 = one && lane < n;
    uint32_t id0 = 0;
    float4 c0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), mn0 = c0, mx0 = c0;
    if (in0) {
        id0 = perm_in[start + lane];
        c0 = S.pcen[id0]; mn0 = S.pmin[id0]; mx0 = S.pmax[id0];
    }
    // centroid bounds
    unsigned co[6] = {kFull, kFull, kFull, 0u, 0u, 0u};
    auto add_centroid = [&](float4 c) {
        const unsigned q[3] = {f2ord(c.x), f2ord(c.y), f2ord(c.z)};
        for (int a = 0; a < 3; ++a) { co[a] = min(co[a], q[a]); co[3 + a] = max(co[3 + a], q[a]); }
    };
    if (one) {
        if (in0) add_centroid(c0);
    } else {
        for (uint32_t i = start + lane; i < start + n; i += 32) add_centroid(S.pcen[perm_in[i]]);
    }
    float cb[6];
    for (int a = 0; a < 3; ++a) {
        cb[a] = ord2f(__reduce_min_sync(kFull, co[a]));
        cb[3 + a] = ord2f(__reduce_max_sync(kFull, co[3 + a]));
    }
    // bins (ordered-integer form while accumulating, then floats for the split);
    // lane j < 24 initialises and converts bin j
    unsigned *ubins = reinterpret_cast<unsigned *>(wbins[w]);
    if (lane < 3u * kBins) {
        unsigned *q = ubins + lane * kBinStride;
        q[0] = 0u;
        for (int a = 0; a < 3; ++a) { q[1 + a] = kOrdPosInf; q[4 + a] = kOrdNegInf; }
    }
    __syncwarp();
    uint32_t b0[3] = {0u, 0u, 0u};                             // one: the lane's bins
    if (one) {
        const unsigned mn[3] = {f2ord(mn0.x), f2ord(mn0.y), f2ord(mn0.z)};
        const unsigned mx[3] = {f2ord(mx0.x), f2ord(mx0.y), f2ord(mx0.z)};
        bins_warp(S, ubins, in0 ? 0 : -1, c0, cb, mn, mx, lane, b0);
    } else {
        for (uint32_t base = start; base < start + n; base += 32) {     // warp-uniform
            const uint32_t i = base + lane;
            const bool in = i < start + n;
            float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f), bmn = c, bmx = c;
            if (in) {
                const uint32_t id = perm_in[i];
                c = S.pcen[id]; bmn = S.pmin[id]; bmx = S.pmax[id];
            }
            const unsigned mn[3] = {f2ord(bmn.x), f2ord(bmn.y), f2ord(bmn.z)};
            const unsigned mx[3] = {f2ord(bmx.x), f2ord(bmx.y), f2ord(bmx.z)};
            uint32_t b[3];
            bins_warp(S, ubins, in ? 0 : -1, c, cb, mn, mx, lane, b);
        }
    }
    __syncwarp();
    if (lane < 3u * kBins) {
        unsigned *q = ubins + lane * kBinStride;
        for (int j = 1; j < kBinStride; ++j) q[j] = __float_as_uint(ord2f(q[j]));
    }
    __syncwarp();
    const float *bins = wbins[w];
    // split (the whole warp), child ids (lane 0)
    int ct0 = -1, ct1 = -1;
    uint32_t lcount = 0;
    Aabb bl = aabb_empty(), br = aabb_empty();
    const int sp = choose_split_warp(n, S.t_bounds[cur] + 6 * t, cb, bins, lane, &lcount, &bl, &br);
    if (lane == 0) {
        uint32_t c0 = 0, s0 = 0, y0 = 0;
        if (sp >= 0) {
            c0 = atomicAdd(S.counters + 1, 2u);
            const uint32_t m = child_small(n, lcount);           // a small task has no large child
            if (m) s0 = atomicAdd(S.counters + 4, m);
            const uint32_t q = child_tiny(n, lcount);
            if (q) y0 = atomicAdd(S.counters + 6, q);
        }
        int ct[2];
        record_task(S, cur ^ 1, start, n, node, sp, lcount, bl, br, c0, 0u, s0, y0, ct);
        ct0 = ct[0];
        ct1 = ct[1];
    }
    ct0 = __shfl_sync(0xffffffffu, ct0, 0);
    ct1 = __shfl_sync(0xffffffffu, ct1, 0);
    uint32_t *out0 = S.perm[cur ^ 1], *out1 = S.perm[cur];
    const unsigned below = (1u << lane) - 1u;
    const int axis = sp >> 4, bin = sp & 15;
    if (one) {
        if (sp < 0) {                                          // a leaf: positions stay
            if (in0) out0[start + lane] = id0;
            return;
        }
        // the split axis has an extent, so b0[axis] is the lane's bin on it
        const uint32_t my_bin = axis == 0 ? b0[0] : (axis == 1 ? b0[1] : b0[2]);
        const bool left = in0 && my_bin <= (uint32_t)bin;
        const unsigned lm = __ballot_sync(kFull, left);
        const unsigned rm = __ballot_sync(kFull, in0 && !left);
        if (in0) {
            const uint32_t pos = left ? start + __popc(lm & below) : start + lcount + __popc(rm & below);
            out0[pos] = id0;
            if ((left ? ct0 : ct1) < 0) out1[pos] = id0;       // in a leaf: final in both buffers
        }
        return;
    }
    if (sp < 0) {                                              // a leaf: positions stay
        for (uint32_t i = start + lane; i < start + n; i += 32) out0[i] = perm_in[i];
        return;
    }
    // stable partition by ballot, in position order
    const float len = cb[3 + axis] - cb[axis];
    uint32_t lbase = start, rbase = start + lcount;
    for (uint32_t base = start; base < start + n; base += 32) {
        const uint32_t i = base + lane;
        const bool valid = i < start + n;
        uint32_t id = 0;
        bool left = false;
        if (valid) {
            id = perm_in[i];
            const float4 c = S.pcen[id];
            const float cc = axis == 0 ? c.x : (axis == 1 ? c.y : c.z);
            left = bin_of(cc, cb[axis], len) <= (uint32_t)bin;
        }
        const unsigned lm = __ballot_sync(0xffffffffu, valid && left);
        const unsigned rm = __ballot_sync(0xffffffffu, valid && !left);
        if (valid) out0[left ? lbase + __popc(lm & below) : rbase + __popc(rm & below)] = id;
        lbase += __popc(lm);
        rbase += __popc(rm);
    }
    // a child that is a leaf: its positions are final, copy them into the input
    // buffer too (after every read of that buffer above)
    __syncwarp();
    if (ct0 < 0)
        for (uint32_t i = start + lane; i < start + lcount; i += 32) out1[i] = out0[i];
    if (ct1 < 0)
        for (uint32_t i = start + lcount + lane; i < start + n; i += 32) out1[i] = out0[i];
}

constexpr int kTinyThreads = 128;

// Tiny tasks (at most kTinyTask primitives): one thread each runs the serial
// algorithm — centroid bounds, the 8 bins of one axis at a time in its own
// column of shared memory (a column per thread, so lanes never share a bank),
// the sweep of split_axis, and the stable partition.  Child ids are reserved
// per warp; every child of a tiny task is a leaf or tiny.
__global__ void __launch_bounds__(kTinyThreads) k_tiny_level(BuildState S, int cur) {
    __shared__ unsigned sb[kBins * kBinStride][kTinyThreads];
    const uint32_t tid = threadIdx.x, lane = tid & 31u;
    const uint32_t k = blockIdx.x * kTinyThreads + tid;
    const uint32_t ntiny = S.counters[7];
    if ((k & ~31u) >= ntiny) return;                           // whole warps
    const bool active = k < ntiny;
    uint32_t start = 0, n = 0, node = 0;
    if (active) { start = S.y_start[cur][k]; n = S.y_count[cur][k]; node = S.y_node[cur][k]; }
    const uint32_t *perm_in = S.perm[cur];
    unsigned co[6] = {kFull, kFull, kFull, 0u, 0u, 0u};
    for (uint32_t j = 0; j < n; ++j) {
        const float4 c = S.pcen[perm_in[start + j]];
        const unsigned q[3] = {f2ord(c.x), f2ord(c.y), f2ord(c.z)};
        for (int a = 0; a < 3; ++a) { co[a] = min(co[a], q[a]); co[3 + a] = max(co[3 + a], q[a]); }
    }
    float cb[6], tb[6];
    for (int a = 0; a < 6; ++a) {
        cb[a] = ord2f(co[a]);
        tb[a] = active ? S.y_bounds[cur][6 * k + a] : 0.0f;
    }
    const float parent = node_half_area(tb);
    SplitBest best = split_best_init(n);
    for (int axis = 0; axis < 3; ++axis) {
        const float len = cb[3 + axis] - cb[axis];
        if (!active || len < 1e-8f) continue;
        for (int b = 0; b < kBins; ++b) {
            sb[b * kBinStride][tid] = 0u;
            for (int a = 0; a < 3; ++a) {
                sb[b * kBinStride + 1 + a][tid] = kOrdPosInf;
                sb[b * kBinStride + 4 + a][tid] = kOrdNegInf;
            }
        }
        for (uint32_t j = 0; j < n; ++j) {
            const uint32_t id = perm_in[start + j];
            const float4 c = S.pcen[id], bmn = S.pmin[id], bmx = S.pmax[id];
            const float cc = axis == 0 ? c.x : (axis == 1 ? c.y : c.z);
            const uint32_t o = bin_of(cc, cb[axis], len) * kBinStride;
            const unsigned mn[3] = {f2ord(bmn.x), f2ord(bmn.y), f2ord(bmn.z)};
            const unsigned mx[3] = {f2ord(bmx.x), f2ord(bmx.y), f2ord(bmx.z)};
            sb[o][tid] += 1u;
            for (int a = 0; a < 3; ++a) {
                sb[o + 1 + a][tid] = min(sb[o + 1 + a][tid], mn[a]);
                sb[o + 4 + a][tid] = max(sb[o + 4 + a][tid], mx[a]);
            }
        }
        split_axis(axis, parent, [&](int b, int f) {
            const unsigned v = sb[b * kBinStride + f][tid];
            return f == 0 ? __uint_as_float(v) : ord2f(v);
        }, best);
    }
    uint32_t lcount = 0;
    Aabb bl = aabb_empty(), br = aabb_empty();
    const int sp = active ? split_result(best, n, &lcount, &bl, &br) : -1;
    // child ids for the warp: prefix sums by shuffles, one atomic per counter
    const uint32_t my_nodes = sp >= 0 ? 2u : 0u;
    const uint32_t my_tiny = sp >= 0 ? child_tiny(n, lcount) : 0u;
    uint32_t pn = my_nodes, py = my_tiny;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t a = __shfl_up_sync(kFull, pn, off), b = __shfl_up_sync(kFull, py, off);
        if ((int)lane >= off) { pn += a; py += b; }
    }
    const uint32_t tn = __shfl_sync(kFull, pn, 31), ty = __shfl_sync(kFull, py, 31);
    uint32_t bn = 0, by = 0;
    if (lane == 0) {
        if (tn) bn = atomicAdd(S.counters + 1, tn);
        if (ty) by = atomicAdd(S.counters + 6, ty);
    }
    bn = __shfl_sync(kFull, bn, 0);
    by = __shfl_sync(kFull, by, 0);
    if (!active) return;
    int ct[2];
    record_task(S, cur ^ 1, start, n, node, sp, lcount, bl, br, bn + pn - my_nodes, 0u, 0u, by + py - my_tiny, ct);
    uint32_t *out0 = S.perm[cur ^ 1], *out1 = S.perm[cur];
    if (sp < 0) {                                              // a leaf: positions stay
        for (uint32_t j = 0; j < n; ++j) out0[start + j] = perm_in[start + j];
        return;
    }
    // stable partition, then the positions of leaf children into the input
    // buffer too (after every read of it)
    const int axis = sp >> 4, bin = sp & 15;
    const float len = cb[3 + axis] - cb[axis];
    uint32_t lp = start, rp = start + lcount;
    for (uint32_t j = 0; j < n; ++j) {
        const uint32_t id = perm_in[start + j];
        const float4 c = S.pcen[id];
        const float cc = axis == 0 ? c.x : (axis == 1 ? c.y : c.z);
        const bool left = bin_of(cc, cb[axis], len) <= (uint32_t)bin;
        out0[left ? lp++ : rp++] = id;
    }
    if (ct[0] < 0)
        for (uint32_t p = start; p < start + lcount; ++p) out1[p] = out0[p];
    if (ct[1] < 0)
        for (uint32_t p = start + lcount; p < start + n; ++p) out1[p] = out0[p];
}

// The start of a level without large tasks (level_advance alone).
__global__ void k_level_advance(BuildState S, uint32_t level) {
    if (threadIdx.x == 0 && blockIdx.x == 0) level_advance(S, level);
}

// Partition flag of position i: 1 when its primitive goes to the left child of
// its large task's split, else 0.
__device__ __forceinline__ uint32_t partition_flag(const BuildState &S, int cur, uint32_t i) {
    const int task = S.ptask[cur][i];
    if (task < 0) return 0u;
    const int sp = S.t_split[task];
    if (sp < 0) return 0u;
    const int axis = sp >> 4, bin = sp & 15;
    const float *cb = S.t_cb + 6 * task;
    const float4 c = S.pcen[S.perm[cur][i]];
    const float cc = axis == 0 ? c.x : (axis == 1 ? c.y : c.z);
    const float len = cb[3 + axis] - cb[axis];
    return bin_of(cc, cb[axis], len) <= (uint32_t)bin ? 1u : 0u;
}

// The partition flags of every position and their exclusive scan in one pass
// (decoupled look-back, Merrill and Garland 2016): a block takes the next tile
// from a ticket (tiles start in order, so every predecessor of a tile is
// running or done), scans its kFlagTile flags, publishes its sum, adds its
// predecessors' published sums walking back to the first inclusive prefix,
// and publishes its own.  The walk reads 32 predecessors per step, one per lane
// of the first warp: the nearest inclusive prefix among them (ballot) ends it,
// else their sums are added and the window moves back.  Every wait is bounded:
// after kLookbackPolls polls of a predecessor the tile records the error word
// and goes on (the host fails the build).
__global__ void __launch_bounds__(kFlagThreads) k_flag_scan(BuildState S, int cur) {
    __shared__ uint32_t s_tile, s_excl, s_warp[kFlagThreads / 32];
    const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
    unsigned long long *status = S.part + 2;
    if (t == 0) s_tile = atomicAdd(reinterpret_cast<unsigned int *>(S.part), 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t i0 = tile * kFlagTile + t * kFlagItems;
    uint32_t f[kFlagItems], sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < kFlagItems; ++k) {
        f[k] = i0 + k < S.nt ? partition_flag(S, cur, i0 + k) : 0u;
        sum += f[k];
    }
    uint32_t x = sum;                                          // inclusive scan over the warp
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    if (w == 0) {                                              // inclusive scan of the warp totals
        uint32_t v = lane < kFlagThreads / 32 ? s_warp[lane] : 0u;
#pragma unroll
        for (uint32_t d = 1; d < kFlagThreads / 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, v, d);
            if (lane >= d) v += y;
        }
        if (lane < kFlagThreads / 32) s_warp[lane] = v;
    }
    __syncthreads();
    const uint32_t block_total = s_warp[kFlagThreads / 32 - 1];
    const uint32_t thread_excl = (w ? s_warp[w - 1] : 0u) + x - sum;
    if (w == 0) {
        uint32_t excl = 0;
        if (tile == 0) {
            if (lane == 0) {
                __threadfence();
                atomicExch(status, (2ull << 32) | block_total);
            }
        } else {
            if (lane == 0) atomicExch(status + tile, (1ull << 32) | block_total);
            bool gave_up = false;
            for (int j = (int)tile - 1; !gave_up;) {            // window: predecessors j, j - 1, ..., j - 31
                const int idx = j - (int)lane;
                unsigned long long v = 2ull << 32;              // before tile 0: an inclusive prefix of 0
                if (idx >= 0) {
                    uint32_t polls = 0;
                    for (;;) {
                        v = *reinterpret_cast<volatile unsigned long long *>(status + idx);
                        if ((uint32_t)(v >> 32) != 0u) break;
                        if (++polls > kLookbackPolls) { v = 2ull << 32; gave_up = true; break; }
                    }
                }
                gave_up = __any_sync(kFull, gave_up);
                const unsigned incl = __ballot_sync(kFull, (uint32_t)(v >> 32) == 2u);
                const uint32_t last = incl ? (uint32_t)__ffs(incl) - 1u : 31u;   // nearest inclusive lane
                excl += __reduce_add_sync(kFull, lane <= last ? (uint32_t)v : 0u);
                if (incl) break;
                j -= 32;
            }
            if (lane == 0) {
                if (gave_up) atomicExch(reinterpret_cast<unsigned int *>(S.part + 1), 1u);
                __threadfence();
                atomicExch(status + tile, (2ull << 32) | (excl + block_total));
            }
        }
        if (lane == 0) s_excl = excl;
    }
    __syncthreads();
    uint32_t run = s_excl + thread_excl;
#pragma unroll
    for (uint32_t k = 0; k < kFlagItems; ++k) {
        if (i0 + k < S.nt) {
            S.flags[i0 + k] = f[k];
            S.scan[i0 + k] = run;
        }
        run += f[k];
    }
}

__global__ void k_scatter(BuildState S, int cur) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.nt) return;
    int task = S.ptask[cur][i];
    if (task == -2) { S.ptask[cur ^ 1][i] = -2; return; }     // a small task's position: k_small_level moves it
    uint32_t id = S.perm[cur][i];
    if (task < 0) { S.perm[cur ^ 1][i] = id; S.ptask[cur ^ 1][i] = -1; return; }
    int sp = S.t_split[task];
    uint32_t start = S.t_start[cur][task], node = S.t_node[cur][task];
    if (sp < 0) { S.perm[cur ^ 1][i] = id; S.ptask[cur ^ 1][i] = -1; return; }
    uint32_t lcount = S.t_lcount[task];
    uint32_t left_rank = S.scan[i] - S.scan[start];
    uint32_t pos;
    uint32_t child;
    if (S.flags[i]) { pos = start + left_rank; child = S.n_a[node]; }
    else { pos = start + lcount + ((i - start) - left_rank); child = S.n_b[node]; }
    S.perm[cur ^ 1][pos] = id;
    const uint32_t map = S.n_size[child];
    S.ptask[cur ^ 1][pos] = S.n_leaf[child] ? -1 : (map == kSmallFlag ? -2 : (int)map);
}

// subtree sizes, bottom-up over a BFS id range
__global__ void k_sizes(BuildState S, uint32_t begin, uint32_t end) {
    uint32_t i = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    S.n_size[i] = S.n_leaf[i] ? 1u : 1u + S.n_size[S.n_a[i]] + S.n_size[S.n_b[i]];
}
// pre-order indices, top-down
__global__ void k_preorder(BuildState S, uint32_t begin, uint32_t end) {
    uint32_t i = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    if (S.n_leaf[i]) return;
    uint32_t p = S.n_pre[i];
    uint32_t l = S.n_a[i], r = S.n_b[i];
    S.n_pre[l] = p + 1;
    S.n_pre[r] = p + 1 + S.n_size[l];
}
__global__ void k_emit(BuildState S, uint32_t n_bfs, mcrt_gpu_bvh_node *out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_bfs) return;
    mcrt_gpu_bvh_node nd;
    float4 mn = S.n_min[i], mx = S.n_max[i];
    nd.aabb_min[0] = mn.x; nd.aabb_min[1] = mn.y; nd.aabb_min[2] = mn.z; nd.aabb_min[3] = 0.0f;
    nd.aabb_max[0] = mx.x; nd.aabb_max[1] = mx.y; nd.aabb_max[2] = mx.z; nd.aabb_max[3] = 0.0f;
    if (S.n_leaf[i]) { nd.right_or_offset = S.n_a[i]; nd.prim_count = S.n_b[i]; }
    else { nd.right_or_offset = S.n_pre[S.n_b[i]]; nd.prim_count = 0; }
    nd._pad[0] = 0; nd._pad[1] = 0;
    out[S.n_pre[i]] = nd;
}

template <typename T> T *carve(char *&p, size_t count) {
    T *r = reinterpret_cast<T *>(p);
    size_t bytes = (count * sizeof(T) + 255) & ~(size_t)255;
    p += bytes;
    return r;
}

}  // namespace

static cudaError_t gpu_build(const mcrt_gpu_vertex *d_verts, const mcrt_gpu_triangle *d_tris,
                             const mcrt_gpu_sphere *d_sph, uint32_t nt, mcrt_gpu_bvh_node *d_nodes,
                             uint32_t *d_order, uint32_t *n_nodes_out, BvhScratch **scratch_io, cudaStream_t st,
                             std::string *err) {
    *n_nodes_out = 0;
    if (nt == 0) return cudaSuccess;
    BvhScratch *sc = *scratch_io;
    if (!sc || sc->cap < nt) {
        free_bvh_scratch(sc);
        sc = new BvhScratch();
        *scratch_io = sc;
        size_t n = nt, nn = 2 * (size_t)nt, tc = (size_t)nt / 4 + 1;   // tasks hold > 4 primitives
        size_t bytes = 0;
        auto acc = [&](size_t b) { bytes += (b + 255) & ~(size_t)255; };
        acc(n * 16); acc(n * 16); acc(n * 16);               // pmin, pmax, pcen
        acc(n * 4); acc(n * 4); acc(n * 4); acc(n * 4);      // perm x2, ptask x2
        acc(n * 4); acc(n * 4);                              // flags, scan
        for (int k = 0; k < 2; ++k) { acc(tc * 4); acc(tc * 4); acc(tc * 4); acc(tc * 24); }
        acc(tc * 24); acc(tc * 4 * kTaskBinWords); acc(tc * 4); acc(tc * 4);
        acc(nn * 16); acc(nn * 16); acc(nn * 4); acc(nn * 4); acc(nn * 4); acc(nn * 4); acc(nn * 4);
        acc(64);
        acc(kMaxLevels * 4);
        const size_t tiles = (n + kRadixTile - 1) / kRadixTile;
        const size_t scan_words = std::max(scan_tmp_words(nt), scan_tmp_words((uint32_t)(256 * tiles)));
        acc(scan_words * 4);
        acc(n * 4); acc(n * 4); acc(n * 4); acc(n * 4);      // sort keys, ids (ping-pong)
        acc(256 * tiles * 4); acc(256 * tiles * 4);          // digit counts, offsets
        acc(n * 16); acc(n * 16); acc(n * 16);               // reordered bounds
        for (int k = 0; k < 2; ++k) { acc(tc * 4); acc(tc * 4); acc(tc * 4); acc(tc * 24); }   // tiny tasks
        acc((2 + (n + kFlagTile - 1) / kFlagTile) * 8);     // partition scan state
        cudaError_t e = cudaMalloc(&sc->mem, bytes);
        if (e != cudaSuccess) { if (err) *err = "BVH scratch allocation failed"; return e; }
        sc->cap = nt;
        char *p = static_cast<char *>(sc->mem);
        BuildState &S = sc->s;
        S.pmin = carve<float4>(p, n); S.pmax = carve<float4>(p, n); S.pcen = carve<float4>(p, n);
        S.perm[0] = carve<uint32_t>(p, n); S.perm[1] = carve<uint32_t>(p, n);
        S.ptask[0] = carve<int32_t>(p, n); S.ptask[1] = carve<int32_t>(p, n);
        S.flags = carve<uint32_t>(p, n); S.scan = carve<uint32_t>(p, n);
        for (int k = 0; k < 2; ++k) {
            S.t_start[k] = carve<uint32_t>(p, tc); S.t_count[k] = carve<uint32_t>(p, tc);
            S.t_node[k] = carve<uint32_t>(p, tc); S.t_bounds[k] = carve<float>(p, 6 * tc);
        }
        S.t_cb = carve<float>(p, 6 * tc); S.t_bins = carve<float>(p, tc * kTaskBinWords);
        S.t_split = carve<int32_t>(p, tc); S.t_lcount = carve<uint32_t>(p, tc);
        S.n_min = carve<float4>(p, nn); S.n_max = carve<float4>(p, nn);
        S.n_a = carve<uint32_t>(p, nn); S.n_b = carve<uint32_t>(p, nn); S.n_leaf = carve<uint32_t>(p, nn);
        S.n_size = carve<uint32_t>(p, nn); S.n_pre = carve<uint32_t>(p, nn);
        S.counters = carve<uint32_t>(p, 16);
        S.level_end = carve<uint32_t>(p, kMaxLevels);
        sc->scan_tmp = carve<uint32_t>(p, scan_words);
        S.rkey[0] = carve<uint32_t>(p, n); S.rkey[1] = carve<uint32_t>(p, n);
        S.rval[0] = carve<uint32_t>(p, n); S.rval[1] = carve<uint32_t>(p, n);
        S.rhist = carve<uint32_t>(p, 256 * tiles); S.roffs = carve<uint32_t>(p, 256 * tiles);
        S.qmin = carve<float4>(p, n); S.qmax = carve<float4>(p, n); S.qcen = carve<float4>(p, n);
        for (int k = 0; k < 2; ++k) {
            S.y_start[k] = carve<uint32_t>(p, tc); S.y_count[k] = carve<uint32_t>(p, tc);
            S.y_node[k] = carve<uint32_t>(p, tc); S.y_bounds[k] = carve<float>(p, 6 * tc);
        }
        S.part = carve<unsigned long long>(p, 2 + (n + kFlagTile - 1) / kFlagTile);
    }
    BuildState S = sc->s;
    S.nt = nt;
    S.tcap = nt / 4 + 1;                                 // tasks hold > 4 primitives
    const uint32_t TB = 256;
    const uint32_t nb = (nt + TB - 1) / TB;
    if (d_sph) k_sphere_bounds<<<nb, TB, 0, st>>>(d_sph, S);
    else k_prim_bounds<<<nb, TB, 0, st>>>(d_verts, d_tris, S);
    ::mcrt::note_launch();
    k_root_init<<<1, 32, 0, st>>>(S); ::mcrt::note_launch();
    k_root_bounds<<<(nt + kPosPerBlock - 1) / kPosPerBlock, 256, 0, st>>>(S); ::mcrt::note_launch();
    if (nt <= kLeafMax) {
        // the root is a single leaf (bvh.rs:301-304)
        std::vector<float> tb(6);
        cudaMemcpyAsync(tb.data(), S.t_bounds[0], 24, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        mcrt_gpu_bvh_node nd{};
        for (int a = 0; a < 3; ++a) { nd.aabb_min[a] = tb[a]; nd.aabb_max[a] = tb[3 + a]; }
        nd.right_or_offset = 0;
        nd.prim_count = nt;
        cudaMemcpyAsync(d_nodes, &nd, sizeof(nd), cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(d_order, S.perm[0], 4 * (size_t)nt, cudaMemcpyDeviceToDevice, st);
        cudaError_t e = cudaStreamSynchronize(st);
        *n_nodes_out = 1;
        return e;
    }
    // Morton order: 4 stable radix passes of 8 bits over the 30-bit codes
    // (ends in buffer 0), then the bounds are gathered into that order and the
    // build runs on Morton indices; the output order maps them back to ids.
    {
        const uint32_t tiles = (nt + kRadixTile - 1) / kRadixTile;
        k_morton<<<nb, TB, 0, st>>>(S); ::mcrt::note_launch();
        for (int pass = 0; pass < 4; ++pass) {
            const int in = pass & 1;
            k_radix_hist<<<tiles, 256, 0, st>>>(S.rkey[in], nt, 8 * pass, tiles, S.rhist); ::mcrt::note_launch();
            exclusive_scan_u32(S.rhist, S.roffs, 256 * tiles, sc->scan_tmp, st);
            k_radix_scatter<<<tiles, 256, 0, st>>>(S.rkey[in], S.rval[in], nt, 8 * pass, tiles, S.roffs,
                                                  S.rkey[in ^ 1], S.rval[in ^ 1]);
            ::mcrt::note_launch();
        }
        k_reorder<<<nb, TB, 0, st>>>(S); ::mcrt::note_launch();
        std::swap(S.pmin, S.qmin);
        std::swap(S.pmax, S.qmax);
        std::swap(S.pcen, S.qcen);
    }
    // BFS node 0 = root
    cudaMemcpyAsync(S.n_min, S.t_bounds[0], 12, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(S.n_max, S.t_bounds[0] + 3, 12, cudaMemcpyDeviceToDevice, st);
    // Levels.  Round r builds the tasks of level r: the large ones by the
    // whole-array passes (while any exist; the host reads their count after
    // each round), the small ones by k_small_level in the same round.  Once no
    // large task is left, rounds run in batches of 8 with one host round trip
    // per batch.  level_end[r] = the BFS node count when round r starts, so
    // round r creates the nodes [level_end[r], level_end[r + 1]).
    const uint32_t tcap = S.tcap;
    const uint32_t nbp = (nt + kPosPerBlock - 1) / kPosPerBlock;
    uint32_t n_large = 1, n_small = 0, n_tiny = 0;       // tasks of the current level
    uint32_t level = 0;
    int cur = 0;
    uint32_t host_counters[8] = {};
    uint32_t scan_error = 0;
    const uint32_t n_flag_tiles = (nt + kFlagTile - 1) / kFlagTile;
    auto level_ok = [&]() -> bool {
        if (level + 1 >= kMaxLevels) {
            if (err) *err = "BVH build exceeded 4096 levels";
            return false;
        }
        return true;
    };
    auto advance = [&]() -> bool {
        if (!level_ok()) return false;
        k_level_advance<<<1, 1, 0, st>>>(S, level++); ::mcrt::note_launch();
        return true;
    };
    // small and tiny tasks of the current level (bounds: at least their counts)
    auto small_round = [&](uint64_t small_bound, uint64_t tiny_bound) {
        const uint32_t warps = (uint32_t)std::min<uint64_t>(small_bound, tcap);
        if (warps) { k_small_level<<<(warps + 7) / 8, 256, 0, st>>>(S, cur); ::mcrt::note_launch(); }
        const uint32_t threads = (uint32_t)std::min<uint64_t>(tiny_bound, tcap);
        if (threads) {
            k_tiny_level<<<(threads + kTinyThreads - 1) / kTinyThreads, kTinyThreads, 0, st>>>(S, cur);
            ::mcrt::note_launch();
        }
    };
    const uint32_t n_part = 2 + n_flag_tiles;
    while (n_large > 0) {
        if (!level_ok()) return cudaErrorUnknown;
        const uint32_t nw = std::max(n_large * (6 + kTaskBinWords), n_part);
        k_task_reset<<<(nw + TB - 1) / TB, TB, 0, st>>>(S, level++, n_large, n_part); ::mcrt::note_launch();
        k_centroid_bounds<<<nbp, 256, 0, st>>>(S, cur); ::mcrt::note_launch();
        k_bins<<<nbp, 256, 0, st>>>(S, cur); ::mcrt::note_launch();
        k_split<<<(n_large + 127) / 128, 128, 0, st>>>(S, cur, n_large); ::mcrt::note_launch();
        k_flag_scan<<<n_flag_tiles, kFlagThreads, 0, st>>>(S, cur); ::mcrt::note_launch();
        k_scatter<<<nb, TB, 0, st>>>(S, cur); ::mcrt::note_launch();
        small_round(n_small, n_tiny);
        cur ^= 1;
        cudaMemcpyAsync(host_counters, S.counters, sizeof(host_counters), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&scan_error, S.part + 1, 4, cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { if (err) *err = "BVH build level failed"; return e; }
        if (scan_error) { if (err) *err = "BVH build: partition scan look-back gave up"; return cudaErrorUnknown; }
        n_large = host_counters[0];
        n_small = host_counters[4];
        n_tiny = host_counters[6];
    }
    // positions the whole-array passes finished (leaves) are in perm[cur] only
    cudaMemcpyAsync(S.perm[cur ^ 1], S.perm[cur], 4 * (size_t)nt, cudaMemcpyDeviceToDevice, st);
    // upper bounds of a level's small and tiny tasks: a small task has at most
    // two small or tiny children, a tiny one at most two tiny children
    uint64_t small_bound = n_small, tiny_bound = n_tiny;
    while (n_small > 0 || n_tiny > 0) {
        for (int k = 0; k < 8; ++k) {
            if (!advance()) return cudaErrorUnknown;
            small_round(small_bound, tiny_bound);
            cur ^= 1;
            tiny_bound = std::min<uint64_t>(2 * (small_bound + tiny_bound), tcap);
            small_bound = std::min<uint64_t>(2 * small_bound, tcap);
        }
        cudaMemcpyAsync(host_counters, S.counters, sizeof(host_counters), cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { if (err) *err = "BVH build level failed"; return e; }
        n_small = host_counters[4];
        n_tiny = host_counters[6];
        small_bound = n_small;
        tiny_bound = n_tiny;
    }
    if (!advance()) return cudaErrorUnknown;             // the node count after the last level
    std::vector<uint32_t> level_begin(level + 1);
    level_begin[0] = 0;                                  // level 0 is the root alone: [0, 1)
    cudaMemcpyAsync(level_begin.data() + 1, S.level_end, 4 * (size_t)level, cudaMemcpyDeviceToHost, st);
    {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { if (err) *err = "BVH build level failed"; return e; }
    }
    const uint32_t n_bfs = level_begin[level];
    // BFS ids are allocated level by level: the children of the nodes created by
    // one level are all created by the next, so subtree sizes are exact when the
    // levels are swept bottom-up and pre-order indices when swept top-down.
    {
        const size_t nl = level_begin.size() - 1;
        for (size_t k = nl; k-- > 0;) {
            const uint32_t b = level_begin[k], e = level_begin[k + 1];
            if (e > b) { k_sizes<<<(e - b + TB - 1) / TB, TB, 0, st>>>(S, b, e); ::mcrt::note_launch(); }
        }
        cudaMemsetAsync(S.n_pre, 0, 4, st);
        for (size_t k = 0; k < nl; ++k) {
            const uint32_t b = level_begin[k], e = level_begin[k + 1];
            if (e > b) { k_preorder<<<(e - b + TB - 1) / TB, TB, 0, st>>>(S, b, e); ::mcrt::note_launch(); }
        }
    }
    k_emit<<<(n_bfs + TB - 1) / TB, TB, 0, st>>>(S, n_bfs, d_nodes); ::mcrt::note_launch();
    k_final_order<<<nb, TB, 0, st>>>(S.perm[cur], S.rval[0], nt, d_order); ::mcrt::note_launch();
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { if (err) *err = "BVH emit failed"; return e; }
    *n_nodes_out = n_bfs;
    return cudaSuccess;
}

cudaError_t gpu_build_mesh_bvh(const mcrt_gpu_vertex *d_verts, const mcrt_gpu_triangle *d_tris, uint32_t nt,
                               mcrt_gpu_bvh_node *d_nodes, uint32_t *d_order, uint32_t *n_nodes_out,
                               BvhScratch **scratch, cudaStream_t st, std::string *err) {
    return gpu_build(d_verts, d_tris, nullptr, nt, d_nodes, d_order, n_nodes_out, scratch, st, err);
}

cudaError_t gpu_build_sphere_bvh(const mcrt_gpu_sphere *d_spheres, uint32_t n, mcrt_gpu_bvh_node *d_nodes,
                                 uint32_t *d_order, uint32_t *n_nodes_out, BvhScratch **scratch, cudaStream_t st,
                                 std::string *err) {
    return gpu_build(nullptr, nullptr, d_spheres, n, d_nodes, d_order, n_nodes_out, scratch, st, err);
}

// ------------------------------------------------------------------ compact layout
namespace {
__global__ void k_internal_flags(const mcrt_gpu_bvh_node *nodes, uint32_t n, uint32_t *flags) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = nodes[i].prim_count == 0 ? 1u : 0u;
}
__device__ __forceinline__ uint32_t child_code(const mcrt_gpu_bvh_node *nodes, const uint32_t *rank, uint32_t c) {
    const mcrt_gpu_bvh_node &nd = nodes[c];
    return nd.prim_count == 0 ? rank[c] : leaf_code(nd.right_or_offset, nd.prim_count);
}
__global__ void k_compact(const mcrt_gpu_bvh_node *nodes, uint32_t n, const uint32_t *rank, float4 *out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || nodes[i].prim_count != 0) return;
    uint32_t l = i + 1, r = nodes[i].right_or_offset;
    const mcrt_gpu_bvh_node &L = nodes[l], &R = nodes[r];
    float4 *o = out + 4ull * rank[i];
    o[0] = make_float4(L.aabb_min[0], L.aabb_max[0], L.aabb_min[1], L.aabb_max[1]);
    o[1] = make_float4(R.aabb_min[0], R.aabb_max[0], R.aabb_min[1], R.aabb_max[1]);
    o[2] = make_float4(L.aabb_min[2], L.aabb_max[2], R.aabb_min[2], R.aabb_max[2]);
    o[3] = make_float4(__uint_as_float(child_code(nodes, rank, l)), __uint_as_float(child_code(nodes, rank, r)),
                       __uint_as_float(kNoChild), 0.0f);
}
// Word 3.z of each compact record: its parent's index (the root keeps
// kNoChild), the up-link of the stackless walk.  Runs after k_compact.
__global__ void k_compact_parents(const mcrt_gpu_bvh_node *nodes, uint32_t n, const uint32_t *rank, float4 *out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || nodes[i].prim_count != 0) return;
    const uint32_t kids[2] = {i + 1, nodes[i].right_or_offset};
    for (int k = 0; k < 2; ++k)
        if (nodes[kids[k]].prim_count == 0)
            reinterpret_cast<uint32_t *>(out + 4ull * rank[kids[k]] + 3)[2] = rank[i];
}
// Shading records in original triangle order: the three vertex normals, the
// first carrying the material word.
__global__ void k_shade_recs(const mcrt_gpu_vertex *verts, const mcrt_gpu_triangle *tris, uint32_t nt, float4 *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt) return;
    const mcrt_gpu_triangle t = tris[i];
    float4 *r = out + 3ull * i;
    for (int k = 0; k < 3; ++k) {
        const float *n = verts[t.v[k]].normal;
        r[k] = make_float4(n[0], n[1], n[2], k == 0 ? __uint_as_float(t.mat_idx) : 0.0f);
    }
}

__global__ void k_trirecs(const uint32_t *order, const mcrt_gpu_vertex *verts, const mcrt_gpu_triangle *tris,
                          uint32_t nt, TriRec *out) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nt) return;
    uint32_t id = order[s];
    mcrt_gpu_triangle t = tris[id];
    f3 v0 = ld3(verts[t.v[0]].position), v1 = ld3(verts[t.v[1]].position), v2 = ld3(verts[t.v[2]].position);
    f3 e1 = v1 - v0, e2 = v2 - v0;                                 // path_trace.wgsl:302-303
    TriRec r;
    r.v0 = make_float4(v0.x, v0.y, v0.z, __uint_as_float(id));
    r.e1 = make_float4(e1.x, e1.y, e1.z, __uint_as_float(t.mat_idx));
    r.e2 = make_float4(e2.x, e2.y, e2.z, 0.0f);
    out[s] = r;
}
__global__ void k_leaf_counts(const mcrt_gpu_bvh_node *nodes, uint32_t n, TriRec *recs) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || nodes[i].prim_count == 0) return;
    recs[nodes[i].right_or_offset].e2.w = __uint_as_float(nodes[i].prim_count);
}
}  // namespace

void launch_shade_recs(const mcrt_gpu_vertex *d_verts, const mcrt_gpu_triangle *d_tris, uint32_t nt, float4 *out,
                       cudaStream_t st) {
    if (nt == 0) return;
    k_shade_recs<<<(nt + 255) / 256, 256, 0, st>>>(d_verts, d_tris, nt, out); ::mcrt::note_launch();
}

cudaError_t gpu_make_compact(const mcrt_gpu_bvh_node *d_nodes, uint32_t n_nodes, const uint32_t *d_order,
                             const mcrt_gpu_vertex *d_verts, const mcrt_gpu_triangle *d_tris, uint32_t nt,
                             float4 **d_cnodes, uint32_t *n_cnodes, void *d_trirecs, uint32_t *d_tmp,
                             size_t tmp_words, cudaStream_t st) {
    // d_tmp: 2*n_nodes + scan_tmp_words(n_nodes) words
    (void)tmp_words;
    const uint32_t TB = 256;
    TriRec *recs = static_cast<TriRec *>(d_trirecs);
    if (nt) k_trirecs<<<(nt + TB - 1) / TB, TB, 0, st>>>(d_order, d_verts, d_tris, nt, recs); ::mcrt::note_launch();
    *n_cnodes = 0;
    if (n_nodes == 0) return cudaGetLastError();
    k_leaf_counts<<<(n_nodes + TB - 1) / TB, TB, 0, st>>>(d_nodes, n_nodes, recs); ::mcrt::note_launch();
    if (n_nodes == 1) return cudaGetLastError();
    uint32_t *flags = d_tmp, *rank = d_tmp + n_nodes, *stmp = d_tmp + 2 * (size_t)n_nodes;
    k_internal_flags<<<(n_nodes + TB - 1) / TB, TB, 0, st>>>(d_nodes, n_nodes, flags); ::mcrt::note_launch();
    exclusive_scan_u32(flags, rank, n_nodes, stmp, st);
    uint32_t last_rank = 0, last_flag = 0;
    cudaMemcpyAsync(&last_rank, rank + n_nodes - 1, 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&last_flag, flags + n_nodes - 1, 4, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    uint32_t n_int = last_rank + last_flag;
    if (*d_cnodes == nullptr) return cudaErrorInvalidValue;
    k_compact<<<(n_nodes + TB - 1) / TB, TB, 0, st>>>(d_nodes, n_nodes, rank, *d_cnodes); ::mcrt::note_launch();
    k_compact_parents<<<(n_nodes + TB - 1) / TB, TB, 0, st>>>(d_nodes, n_nodes, rank, *d_cnodes);
    ::mcrt::note_launch();
    *n_cnodes = n_int;
    return cudaGetLastError();
}

// The top levels of the compact tree in heap order, for the shared-memory
// top-tree traversal: entry 0 is the root, entry j's children go to 2j+1 and
// 2j+2 while those fit (kTopNodes entries, 7 levels); an internal child that
// gets an entry is recoded kTopBit | entry, every other child keeps its code
// (a deeper internal node's compact index, a leaf, or none).  One block, one
// thread per entry, a level per step.
__global__ void k_top_tree(const float4 *cnodes, uint32_t n_cnodes, float4 *top) {
    __shared__ uint32_t src[kTopNodes];            // compact index held by an entry, or kNoChild
    const uint32_t j = threadIdx.x;
    if (j < kTopNodes) src[j] = (j == 0 && n_cnodes > 0) ? 0u : kNoChild;
    __syncthreads();
    for (uint32_t first = 0, width = 1; first < kTopNodes; first += width, width *= 2) {
        if (j >= first && j < first + width && j < kTopNodes) {
            float4 r[4] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f),
                           make_float4(0.f, 0.f, 0.f, 0.f),
                           make_float4(__uint_as_float(kNoChild), __uint_as_float(kNoChild), 0.f, 0.f)};
            if (src[j] != kNoChild) {
                const float4 *np = cnodes + 4ull * src[j];
                for (int k = 0; k < 4; ++k) r[k] = np[k];
                uint32_t code[2] = {__float_as_uint(r[3].x), __float_as_uint(r[3].y)};
                for (int side = 0; side < 2; ++side) {
                    const uint32_t slot = 2 * j + 1 + side;
                    if (code[side] != kNoChild && !(code[side] & kLeafBit) && slot < kTopNodes) {
                        src[slot] = code[side];
                        code[side] = kTopBit | slot;
                    }
                }
                r[3].x = __uint_as_float(code[0]);
                r[3].y = __uint_as_float(code[1]);
            }
            for (int k = 0; k < 4; ++k) top[4ull * j + k] = r[k];
        }
        __syncthreads();
    }
}

cudaError_t gpu_make_top(const float4 *d_cnodes, uint32_t n_cnodes, float4 *d_top, cudaStream_t st) {
    k_top_tree<<<1, 128, 0, st>>>(d_cnodes, n_cnodes, d_top); ::mcrt::note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ quantised 4-wide layout
// Collapse of the reference-layout binary BVH into 4-wide nodes (64 bytes):
//   w0: origin.xyz (float, the node box minimum) | exponent bytes ex, ey, ez
//       (grid step 2^(e-127) per axis) and the child count
//   w1: qlo.x[4] | qlo.y[4] | qlo.z[4] | qhi.x[4]   (8-bit grid coordinates)
//   w2: qhi.y[4] | qhi.z[4] | 0 | 0
//   w3: child codes (internal 4-wide node index, leaf code, or kNoChild)
// A node takes the two children of a binary node and repeatedly replaces the
// internal child of largest surface area by its two children until it has
// four.  Leaves are the reference's leaves.  Child boxes are rounded outward:
// the builder checks that every grid plane origin + q * step, as an exact real
// number, lies outside the exact child box (the traversal bounds its plane
// distances from that exact value), so a ray that reaches a leaf of the
// reference tree also reaches it here.
namespace {

__device__ __forceinline__ float step_of(uint32_t e) { return __uint_as_float(e << 23); }

// Smallest exponent byte e with extent / 2^(e-127) <= 250 (a normal power of two).
__device__ __forceinline__ uint32_t grid_exponent(float extent) {
    if (!(extent > 0.0f)) return 1u;
    float s = extent / 250.0f;
    uint32_t e = (__float_as_uint(s) >> 23) & 0xffu;     // 2^(e-127) <= s < 2^(e-126)
    if (e == 0u) e = 1u;
    while (e < 254u && step_of(e) * 250.0f < extent) ++e;
    while (e > 1u && step_of(e - 1u) * 250.0f >= extent) --e;
    return e;
}

// Sign of the exact real origin + qs - v (qs = q * step, exact: step is a
// power of two).  The rounded sum s lies within half an ulp of the exact one,
// so s != v decides; at s == v the error-free residual of the sum (Knuth's
// TwoSum: s + err is exactly origin + qs) does.
__device__ __forceinline__ int grid_plane_vs(float origin, float qs, float v) {
    const float s = origin + qs;
    if (s != v) return s < v ? -1 : 1;
    const float bb = s - origin;
    const float err = (origin - (s - bb)) + (qs - bb);
    return err < 0.0f ? -1 : (err > 0.0f ? 1 : 0);
}
__device__ __forceinline__ uint32_t quant_lo(float origin, float step, float v) {
    float q = floorf((v - origin) / step);
    int qi = q < 0.0f ? 0 : (q > 255.0f ? 255 : (int)q);
    while (qi > 0 && grid_plane_vs(origin, (float)qi * step, v) > 0) --qi;
    return (uint32_t)qi;
}
__device__ __forceinline__ uint32_t quant_hi(float origin, float step, float v, bool *ok) {
    float q = ceilf((v - origin) / step);
    int qi = q < 0.0f ? 0 : (q > 255.0f ? 255 : (int)q);
    while (qi < 255 && grid_plane_vs(origin, (float)qi * step, v) < 0) ++qi;
    if (grid_plane_vs(origin, (float)qi * step, v) < 0) *ok = false;
    return (uint32_t)qi;
}

__global__ void k_widen(const mcrt_gpu_bvh_node *nodes, const uint32_t *front, uint32_t n_front, uint32_t level_base,
                        uint32_t next_base, uint32_t *next_front, uint32_t *counter, uint4 *out, uint32_t *bad) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_front) return;
    const uint32_t i = front[k];
    uint32_t set[4] = {i + 1, nodes[i].right_or_offset, kNoChild, kNoChild};
    uint32_t cnt = 2;
    auto area = [&](uint32_t c) {
        const mcrt_gpu_bvh_node &nd = nodes[c];
        float d0 = nd.aabb_max[0] - nd.aabb_min[0], d1 = nd.aabb_max[1] - nd.aabb_min[1],
              d2 = nd.aabb_max[2] - nd.aabb_min[2];
        return d0 * d1 + d1 * d2 + d0 * d2;
    };
    while (cnt < 4) {
        int pick = -1;
        float best = -1.0f;
        for (uint32_t j = 0; j < cnt; ++j) {
            if (nodes[set[j]].prim_count != 0) continue;
            float a = area(set[j]);
            if (a > best) { best = a; pick = (int)j; }
        }
        if (pick < 0) break;
        uint32_t c = set[pick];
        set[pick] = c + 1;
        set[cnt++] = nodes[c].right_or_offset;
    }
    uint32_t n_int = 0;
    for (uint32_t j = 0; j < cnt; ++j) n_int += nodes[set[j]].prim_count == 0 ? 1u : 0u;
    uint32_t base = n_int ? atomicAdd(counter, n_int) : 0u;
    const mcrt_gpu_bvh_node &nd = nodes[i];
    float org[3], stp[3];
    uint32_t ex[3];
    for (int a = 0; a < 3; ++a) {
        org[a] = nd.aabb_min[a];
        ex[a] = grid_exponent(nd.aabb_max[a] - nd.aabb_min[a]);
        stp[a] = step_of(ex[a]);
    }
    uint32_t qlo[3] = {0, 0, 0}, qhi[3] = {0, 0, 0}, refs[4];
    bool ok = true;
    uint32_t r = 0;
    for (uint32_t j = 0; j < 4; ++j) {
        if (j >= cnt) { refs[j] = kNoChild; continue; }
        const mcrt_gpu_bvh_node &c = nodes[set[j]];
        for (int a = 0; a < 3; ++a) {
            qlo[a] |= quant_lo(org[a], stp[a], c.aabb_min[a]) << (8 * j);
            qhi[a] |= quant_hi(org[a], stp[a], c.aabb_max[a], &ok) << (8 * j);
        }
        if (c.prim_count == 0) {
            refs[j] = next_base + base + r;
            next_front[base + r] = set[j];
            ++r;
        } else {
            refs[j] = leaf_code(c.right_or_offset, c.prim_count);
        }
    }
    if (!ok) atomicOr(bad, 1u);
    uint4 *o = out + 4ull * (level_base + k);
    o[0] = make_uint4(__float_as_uint(org[0]), __float_as_uint(org[1]), __float_as_uint(org[2]),
                      ex[0] | (ex[1] << 8) | (ex[2] << 16) | (cnt << 24));
    o[1] = make_uint4(qlo[0], qlo[1], qlo[2], qhi[0]);
    o[2] = make_uint4(qhi[1], qhi[2], 0u, 0u);
    o[3] = make_uint4(refs[0], refs[1], refs[2], refs[3]);
}

}  // namespace

// d_tmp: 2 * n_nodes + 4 words.  d_wide: capacity (n_nodes / 2 + 1) nodes of 64 bytes.
cudaError_t gpu_make_wide4(const mcrt_gpu_bvh_node *d_nodes, uint32_t n_nodes, uint4 *d_wide, uint32_t *n_wide,
                           uint32_t *d_tmp, cudaStream_t st) {
    *n_wide = 0;
    if (n_nodes <= 1) return cudaSuccess;           // a single leaf: traversed without wide nodes
    uint32_t *front[2] = {d_tmp, d_tmp + n_nodes};
    uint32_t *counter = d_tmp + 2 * (size_t)n_nodes;
    uint32_t *bad = counter + 1;
    uint32_t zero = 0;
    cudaMemcpyAsync(front[0], &zero, 4, cudaMemcpyHostToDevice, st);   // root
    cudaMemsetAsync(bad, 0, 4, st);
    uint32_t n_front = 1, level_base = 0;
    int cur = 0;
    for (int guard = 0; n_front > 0; ++guard) {
        if (guard > 4096) return cudaErrorUnknown;
        cudaMemsetAsync(counter, 0, 4, st);
        const uint32_t next_base = level_base + n_front;
        k_widen<<<(n_front + 127) / 128, 128, 0, st>>>(d_nodes, front[cur], n_front, level_base, next_base,
                                                      front[cur ^ 1], counter, d_wide, bad); ::mcrt::note_launch();
        uint32_t n_next = 0;
        cudaMemcpyAsync(&n_next, counter, 4, cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        level_base = next_base;
        n_front = n_next;
        cur ^= 1;
    }
    uint32_t b = 0;
    cudaMemcpyAsync(&b, bad, 4, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    if (b) return cudaErrorInvalidValue;            // a child box could not be enclosed on the grid
    *n_wide = level_base;
    return cudaSuccess;
}

}  // namespace mcrt
