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
// primitives inside a leaf may differ (the partition here is stable by the
// previous order, the reference uses an unstable sort).
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
    uint32_t *counters;               // [0] next task count, [1] bfs node count, [2] tasks of the
                                      // current level (small-task levels), [3] largest new task
    uint32_t *level_end;              // small-task levels: bfs node count after each level
};
constexpr uint32_t kSmallTask = 256;       // tasks up to this size are built by one warp each
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
        S.counters[1] = 1;
    }
}

__global__ void k_root_bounds(BuildState S) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float mn[3], mx[3];
    bool valid = i < S.nt;
    if (valid) {
        float4 a = S.pmin[i], b = S.pmax[i];
        mn[0] = a.x; mn[1] = a.y; mn[2] = a.z; mx[0] = b.x; mx[1] = b.y; mx[2] = b.z;
    } else {
        for (int k = 0; k < 3; ++k) { mn[k] = __int_as_float(0x7f800000); mx[k] = __int_as_float(0xff800000); }
    }
    for (int off = 16; off > 0; off >>= 1)
        for (int k = 0; k < 3; ++k) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], off));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], off));
        }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; ++k) { atomic_min_f(&S.t_bounds[0][k], mn[k]); atomic_max_f(&S.t_bounds[0][3 + k], mx[k]); }
}

__global__ void k_task_reset(BuildState S, uint32_t ntasks) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
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

// Warp-level segmented reduction helper: lanes with the same task combine first.
__global__ void k_centroid_bounds(BuildState S, int cur) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    int task = i < S.nt ? S.ptask[cur][i] : -1;
    float c[3] = {0, 0, 0};
    if (task >= 0) {
        float4 cc = S.pcen[S.perm[cur][i]];
        c[0] = cc.x; c[1] = cc.y; c[2] = cc.z;
    }
    unsigned same = __match_any_sync(0xffffffffu, task);
    int leader = __ffs(same) - 1;
    float mn[3] = {c[0], c[1], c[2]}, mx[3] = {c[0], c[1], c[2]};
    if (same == 0xffffffffu) {
        for (int off = 16; off > 0; off >>= 1)
            for (int k = 0; k < 3; ++k) {
                mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], off));
                mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], off));
            }
        if ((threadIdx.x & 31) != 0 || task < 0) return;
    } else if (task < 0) {
        return;
    }
    (void)leader;
    for (int k = 0; k < 3; ++k) {
        atomic_min_f(&S.t_cb[6 * task + k], mn[k]);
        atomic_max_f(&S.t_cb[6 * task + 3 + k], mx[k]);
    }
}

__device__ __forceinline__ uint32_t bin_of(float c, float cmin, float len) {
    float t = (c - cmin) / len;                                     // bvh.rs:412-415
    uint32_t b = f2u_sat(t * (float)kBins);
    return b > (uint32_t)(kBins - 1) ? (uint32_t)(kBins - 1) : b;
}

// Bin accumulation.  A block whose positions all belong to one task reduces in
// shared memory first; otherwise each primitive adds to global bins.
__global__ void __launch_bounds__(256) k_bins(BuildState S, int cur) {
    __shared__ float sh[kTaskBinWords];
    __shared__ int block_task;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    int task = i < S.nt ? S.ptask[cur][i] : -1;
    uint32_t last = min((uint32_t)(blockIdx.x + 1) * blockDim.x, S.nt) - 1;
    if (threadIdx.x == 0) {
        int t0 = S.ptask[cur][blockIdx.x * blockDim.x];
        int t1 = S.ptask[cur][last];
        block_task = (t0 == t1 && t0 >= 0) ? t0 : -1;
    }
    for (int k = threadIdx.x; k < kTaskBinWords; k += blockDim.x) {
        uint32_t f = k % kBinStride;
        sh[k] = f == 0 ? 0.0f : __int_as_float(f < 4 ? 0x7f800000 : 0xff800000);
    }
    __syncthreads();
    // a block is single-task only if every position agrees (tasks are contiguous, so ends suffice)
    const bool shared_mode = block_task >= 0;
    if (task >= 0) {
        uint32_t id = S.perm[cur][i];
        float4 c = S.pcen[id], bmn = S.pmin[id], bmx = S.pmax[id];
        const float *cb = S.t_cb + 6 * task;
        float cc[3] = {c.x, c.y, c.z};
        for (int axis = 0; axis < 3; ++axis) {
            float len = cb[3 + axis] - cb[axis];
            if (len < 1e-8f) continue;
            uint32_t b = bin_of(cc[axis], cb[axis], len);
            int o = (axis * kBins + (int)b) * kBinStride;
            float *dst = shared_mode ? sh : S.t_bins + (size_t)task * kTaskBinWords;
            atomicAdd(reinterpret_cast<unsigned *>(dst + o), 1u);
            atomic_min_f(dst + o + 1, bmn.x); atomic_min_f(dst + o + 2, bmn.y); atomic_min_f(dst + o + 3, bmn.z);
            atomic_max_f(dst + o + 4, bmx.x); atomic_max_f(dst + o + 5, bmx.y); atomic_max_f(dst + o + 6, bmx.z);
        }
    }
    if (!shared_mode) return;
    __syncthreads();
    float *g = S.t_bins + (size_t)block_task * kTaskBinWords;
    for (int k = threadIdx.x; k < kTaskBinWords; k += blockDim.x) {
        uint32_t f = k % kBinStride;
        if (f == 0) {
            uint32_t cnt = __float_as_uint(sh[k]);
            if (cnt) atomicAdd(reinterpret_cast<unsigned *>(g + k), cnt);
        } else if (f < 4) {
            if (sh[k] != __int_as_float(0x7f800000)) atomic_min_f(g + k, sh[k]);
        } else {
            if (sh[k] != __int_as_float(0xff800000)) atomic_max_f(g + k, sh[k]);
        }
    }
}

__device__ __forceinline__ uint32_t new_bfs_node(BuildState &S, const Aabb &b) {
    uint32_t id = atomicAdd(S.counters + 1, 1u);
    S.n_min[id] = make_float4(b.mn[0], b.mn[1], b.mn[2], 0.0f);
    S.n_max[id] = make_float4(b.mx[0], b.mx[1], b.mx[2], 0.0f);
    return id;
}

// SAH split selection of one task (bvh.rs:388-463) from its node bounds tb,
// centroid bounds cb and bins, and child creation: child nodes, and child
// tasks (buffer cur ^ 1) for children above the leaf size.  Returns the split
// (axis * 16 + bin) or -1 when the task becomes a leaf; *lcount = primitives
// going left; child_task[c] = the child's task id or -1 (leaf).
__device__ int split_task(BuildState &S, int cur, uint32_t start, uint32_t n, uint32_t node, const float *tb,
                          const float *cb, const float *bins, uint32_t *lcount, int child_task[2]) {
    child_task[0] = child_task[1] = -1;
    Aabb nb;
    for (int a = 0; a < 3; ++a) { nb.mn[a] = tb[a]; nb.mx[a] = tb[3 + a]; }
    float parent = fmaxf(half_area(nb), 1e-8f);
    float best_cost = (float)n;
    int best_axis = 0, best_bin = 0;
    uint32_t best_split = 0;
    bool found = false;
    Aabb best_l = aabb_empty(), best_r = aabb_empty();
    for (int axis = 0; axis < 3; ++axis) {
        float len = cb[3 + axis] - cb[axis];
        if (len < 1e-8f) continue;
        Aabb bb[kBins];
        uint32_t bc[kBins];
        for (int k = 0; k < kBins; ++k) {
            const float *q = bins + (axis * kBins + k) * kBinStride;
            bc[k] = __float_as_uint(q[0]);
            for (int a = 0; a < 3; ++a) { bb[k].mn[a] = q[1 + a]; bb[k].mx[a] = q[4 + a]; }
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
            uint32_t l = lc[s];
            if (l == 0 || rc == 0) continue;
            float cost = (half_area(lb[s]) * (float)l + half_area(rb) * (float)rc) / parent;
            if (cost < best_cost) {
                best_cost = cost; best_axis = axis; best_bin = s; best_split = l; found = true;
                best_l = lb[s]; best_r = rb;
            }
        }
    }
    if (!(found && best_split > 0 && best_split < n)) {
        S.n_leaf[node] = 1; S.n_a[node] = start; S.n_b[node] = n;
        return -1;
    }
    *lcount = best_split;
    S.n_leaf[node] = 0;
    uint32_t counts[2] = {best_split, n - best_split};
    uint32_t starts[2] = {start, start + best_split};
    const Aabb *cbx[2] = {&best_l, &best_r};
    uint32_t child[2];
    for (int c = 0; c < 2; ++c) {
        child[c] = new_bfs_node(S, *cbx[c]);
        if (counts[c] <= kLeafMax) {
            S.n_leaf[child[c]] = 1; S.n_a[child[c]] = starts[c]; S.n_b[child[c]] = counts[c];
        } else {
            S.n_leaf[child[c]] = 0;
            atomicMax(S.counters + 3, counts[c]);
            uint32_t nt2 = atomicAdd(S.counters, 1u);
            S.t_start[cur ^ 1][nt2] = starts[c];
            S.t_count[cur ^ 1][nt2] = counts[c];
            S.t_node[cur ^ 1][nt2] = child[c];
            for (int a = 0; a < 3; ++a) {
                S.t_bounds[cur ^ 1][6 * nt2 + a] = cbx[c]->mn[a];
                S.t_bounds[cur ^ 1][6 * nt2 + 3 + a] = cbx[c]->mx[a];
            }
            // the child's positions learn their new task id in k_scatter through this map
            S.n_size[child[c]] = nt2;      // temporary: child node -> task id
            child_task[c] = (int)nt2;
        }
    }
    S.n_a[node] = child[0];
    S.n_b[node] = child[1];
    return best_axis * 16 + best_bin;
}

// One thread per task: split selection and child creation.
__global__ void k_split(BuildState S, int cur, uint32_t ntasks) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    uint32_t lcount = 0;
    int child_task[2];
    const int sp = split_task(S, cur, S.t_start[cur][t], S.t_count[cur][t], S.t_node[cur][t], S.t_bounds[cur] + 6 * t,
                              S.t_cb + 6 * t, S.t_bins + (size_t)t * kTaskBinWords, &lcount, child_task);
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
    const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t ntasks = S.counters[2];
    if (t >= ntasks) return;                                   // whole warps leave together
    const uint32_t start = S.t_start[cur][t], n = S.t_count[cur][t], node = S.t_node[cur][t];
    const uint32_t *perm_in = S.perm[cur];
    // centroid bounds
    float cmn[3], cmx[3];
    for (int k = 0; k < 3; ++k) { cmn[k] = __int_as_float(0x7f800000); cmx[k] = __int_as_float(0xff800000); }
    for (uint32_t i = start + lane; i < start + n; i += 32) {
        const float4 c = S.pcen[perm_in[i]];
        cmn[0] = fminf(cmn[0], c.x); cmn[1] = fminf(cmn[1], c.y); cmn[2] = fminf(cmn[2], c.z);
        cmx[0] = fmaxf(cmx[0], c.x); cmx[1] = fmaxf(cmx[1], c.y); cmx[2] = fmaxf(cmx[2], c.z);
    }
    for (int off = 16; off > 0; off >>= 1)
        for (int k = 0; k < 3; ++k) {
            cmn[k] = fminf(cmn[k], __shfl_xor_sync(0xffffffffu, cmn[k], off));
            cmx[k] = fmaxf(cmx[k], __shfl_xor_sync(0xffffffffu, cmx[k], off));
        }
    const float cb[6] = {cmn[0], cmn[1], cmn[2], cmx[0], cmx[1], cmx[2]};
    // bins
    float *bins = wbins[w];
    for (int k = lane; k < kTaskBinWords; k += 32) {
        const uint32_t f = k % kBinStride;
        bins[k] = f == 0 ? 0.0f : __int_as_float(f < 4 ? 0x7f800000 : 0xff800000);
    }
    __syncwarp();
    for (uint32_t i = start + lane; i < start + n; i += 32) {
        const uint32_t id = perm_in[i];
        const float4 c = S.pcen[id], bmn = S.pmin[id], bmx = S.pmax[id];
        const float cc[3] = {c.x, c.y, c.z};
        for (int axis = 0; axis < 3; ++axis) {
            const float len = cb[3 + axis] - cb[axis];
            if (len < 1e-8f) continue;
            const uint32_t b = bin_of(cc[axis], cb[axis], len);
            float *dst = bins + (axis * kBins + (int)b) * kBinStride;
            atomicAdd(reinterpret_cast<unsigned *>(dst), 1u);
            atomic_min_f(dst + 1, bmn.x); atomic_min_f(dst + 2, bmn.y); atomic_min_f(dst + 3, bmn.z);
            atomic_max_f(dst + 4, bmx.x); atomic_max_f(dst + 5, bmx.y); atomic_max_f(dst + 6, bmx.z);
        }
    }
    __syncwarp();
    // split (lane 0), broadcast
    int sp = -1, ct0 = -1, ct1 = -1;
    uint32_t lcount = 0;
    if (lane == 0) {
        int child_task[2];
        sp = split_task(S, cur, start, n, node, S.t_bounds[cur] + 6 * t, cb, bins, &lcount, child_task);
        ct0 = child_task[0];
        ct1 = child_task[1];
    }
    sp = __shfl_sync(0xffffffffu, sp, 0);
    lcount = __shfl_sync(0xffffffffu, lcount, 0);
    ct0 = __shfl_sync(0xffffffffu, ct0, 0);
    ct1 = __shfl_sync(0xffffffffu, ct1, 0);
    uint32_t *out0 = S.perm[cur ^ 1], *out1 = S.perm[cur];
    if (sp < 0) {                                              // a leaf: positions stay
        for (uint32_t i = start + lane; i < start + n; i += 32) out0[i] = perm_in[i];
        return;
    }
    // stable partition by ballot, in position order
    const int axis = sp >> 4, bin = sp & 15;
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
        const unsigned below = (1u << lane) - 1u;
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

// Between small-task levels: the next level's task count, the node count of
// the level just built, and a fresh child-task counter.
__global__ void k_level_advance(BuildState S, uint32_t level) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        S.counters[2] = S.counters[0];
        S.counters[0] = 0;
        S.level_end[level] = S.counters[1];
    }
}

__global__ void k_flags(BuildState S, int cur) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.nt) return;
    int task = S.ptask[cur][i];
    uint32_t f = 0;
    if (task >= 0) {
        int sp = S.t_split[task];
        if (sp >= 0) {
            int axis = sp >> 4, bin = sp & 15;
            const float *cb = S.t_cb + 6 * task;
            float4 c = S.pcen[S.perm[cur][i]];
            float cc = axis == 0 ? c.x : (axis == 1 ? c.y : c.z);
            float len = cb[3 + axis] - cb[axis];
            f = bin_of(cc, cb[axis], len) <= (uint32_t)bin ? 1u : 0u;
        }
    }
    S.flags[i] = f;
}

__global__ void k_scatter(BuildState S, int cur) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.nt) return;
    int task = S.ptask[cur][i];
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
    S.ptask[cur ^ 1][pos] = S.n_leaf[child] ? -1 : (int)S.n_size[child];
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
        acc(scan_tmp_words(nt) * 4);
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
        sc->scan_tmp = carve<uint32_t>(p, scan_tmp_words(nt));
    }
    BuildState S = sc->s;
    S.nt = nt;
    const uint32_t TB = 256;
    const uint32_t nb = (nt + TB - 1) / TB;
    if (d_sph) k_sphere_bounds<<<nb, TB, 0, st>>>(d_sph, S);
    else k_prim_bounds<<<nb, TB, 0, st>>>(d_verts, d_tris, S);
    ::mcrt::note_launch();
    k_root_init<<<1, 32, 0, st>>>(S); ::mcrt::note_launch();
    k_root_bounds<<<nb, TB, 0, st>>>(S); ::mcrt::note_launch();
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
    // BFS node 0 = root
    cudaMemcpyAsync(S.n_min, S.t_bounds[0], 12, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(S.n_max, S.t_bounds[0] + 3, 12, cudaMemcpyDeviceToDevice, st);
    std::vector<uint32_t> level_begin;
    level_begin.push_back(0);
    uint32_t ntasks = 1;
    int cur = 0;
    uint32_t host_counters[4] = {0, 1, 0, 0};
    uint32_t max_task = nt;
    int guard = 0;
    // levels with a large task: per-level kernels over the whole array
    while (ntasks > 0 && max_task > kSmallTask) {
        if (++guard > (int)kMaxLevels) { if (err) *err = "BVH build exceeded 4096 levels"; return cudaErrorUnknown; }
        cudaMemsetAsync(S.counters, 0, 4, st);
        cudaMemsetAsync(S.counters + 3, 0, 4, st);
        uint32_t nw = ntasks * (6 + kTaskBinWords);
        k_task_reset<<<(nw + TB - 1) / TB, TB, 0, st>>>(S, ntasks); ::mcrt::note_launch();
        k_centroid_bounds<<<nb, TB, 0, st>>>(S, cur); ::mcrt::note_launch();
        k_bins<<<nb, TB, 0, st>>>(S, cur); ::mcrt::note_launch();
        k_split<<<(ntasks + 127) / 128, 128, 0, st>>>(S, cur, ntasks); ::mcrt::note_launch();
        k_flags<<<nb, TB, 0, st>>>(S, cur); ::mcrt::note_launch();
        exclusive_scan_u32(S.flags, S.scan, nt, sc->scan_tmp, st);
        k_scatter<<<nb, TB, 0, st>>>(S, cur); ::mcrt::note_launch();
        cudaMemcpyAsync(host_counters, S.counters, 16, cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { if (err) *err = "BVH build level failed"; return e; }
        level_begin.push_back(host_counters[1]);      // the nodes this level created: [previous, this)
        ntasks = host_counters[0];
        max_task = host_counters[3];
        cur ^= 1;
    }
    // the remaining levels: every task small, one warp per task, launched in
    // batches with one host round trip per batch
    if (ntasks > 0) {
        const uint32_t tcap = nt / 4 + 1;                // tasks hold > 4 primitives
        // finished positions so far live in perm[cur]; give the other buffer them too
        cudaMemcpyAsync(S.perm[cur ^ 1], S.perm[cur], 4 * (size_t)nt, cudaMemcpyDeviceToDevice, st);
        host_counters[0] = ntasks;                        // the tasks of buffer cur
        cudaMemcpyAsync(S.counters, host_counters, 4, cudaMemcpyHostToDevice, st);
        uint32_t level = 0;
        uint64_t bound = ntasks;                          // upper bound of the next level's tasks
        while (ntasks > 0) {
            for (int k = 0; k < 8; ++k) {
                if (level + 1 >= kMaxLevels) { if (err) *err = "BVH build exceeded 4096 levels"; return cudaErrorUnknown; }
                k_level_advance<<<1, 1, 0, st>>>(S, level++); ::mcrt::note_launch();
                const uint32_t warps = (uint32_t)std::min<uint64_t>(bound, tcap);
                k_small_level<<<(warps + 7) / 8, 256, 0, st>>>(S, cur); ::mcrt::note_launch();
                cur ^= 1;
                bound = std::min<uint64_t>(2 * bound, tcap);
            }
            cudaMemcpyAsync(host_counters, S.counters, 16, cudaMemcpyDeviceToHost, st);
            cudaError_t e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) { if (err) *err = "BVH build level failed"; return e; }
            ntasks = host_counters[0];
            bound = ntasks;
        }
        k_level_advance<<<1, 1, 0, st>>>(S, level++); ::mcrt::note_launch();
        std::vector<uint32_t> ends(level);
        cudaMemcpyAsync(ends.data(), S.level_end, 4 * (size_t)level, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(host_counters, S.counters, 16, cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { if (err) *err = "BVH build level failed"; return e; }
        for (uint32_t k = 1; k < level; ++k) level_begin.push_back(ends[k]);   // ends[0]: the last level above
    }
    const uint32_t n_bfs = host_counters[1];
    // BFS ids are allocated level by level: the children of the nodes created by
    // one level are all created by the next, so subtree sizes are exact when the
    // levels are swept bottom-up and pre-order indices when swept top-down.
    {
        level_begin[0] = 0;
        level_begin.insert(level_begin.begin() + 1, 1u);   // level 0 is the root alone
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
    cudaMemcpyAsync(d_order, S.perm[cur], 4 * (size_t)nt, cudaMemcpyDeviceToDevice, st);
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
                       0.0f, 0.0f);
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
    *n_cnodes = n_int;
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
// the builder checks, in the float arithmetic the traversal uses
// (origin + q * step), that every dequantised plane lies outside the exact
// child box, so a ray that reaches a leaf of the reference tree also reaches it
// here.
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

__device__ __forceinline__ uint32_t quant_lo(float origin, float step, float v) {
    float q = floorf((v - origin) / step);
    int qi = q < 0.0f ? 0 : (q > 255.0f ? 255 : (int)q);
    while (qi > 0 && origin + (float)qi * step > v) --qi;
    return (uint32_t)qi;
}
__device__ __forceinline__ uint32_t quant_hi(float origin, float step, float v, bool *ok) {
    float q = ceilf((v - origin) / step);
    int qi = q < 0.0f ? 0 : (q > 255.0f ? 255 : (int)q);
    while (qi < 255 && origin + (float)qi * step < v) ++qi;
    if (origin + (float)qi * step < v) *ok = false;
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
