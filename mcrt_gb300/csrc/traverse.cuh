// traverse.cuh — closest-hit and any-hit traversal (device functions).
//
// Two node layouts:
//  * the reference's 48-byte pre-order GpuBvhNode (bvh.rs:56-68), traversed in
//    the reference's visit order (path_trace.wgsl:343-465) — the parity probe;
//  * the compact layout: one 64-byte record per internal node holding both
//    children's boxes (the same float boxes as the reference nodes), children
//    visited nearest-first with a short stack of (child code, entry distance).
// Both use the same slab arithmetic and the same triangle/sphere tests, so the
// closest hit under the tie rule (smallest t, then smallest original id;
// spheres win over triangles at equal t) does not depend on the layout.
#pragma once

#include "common.cuh"

namespace mcrt {

struct Closest {
    float t;
    uint32_t prim;   // MCRT_HIT_MISS, MCRT_HIT_SPHERE | sphere id, or triangle id
    uint32_t slot;   // ordered slot (sphere) or original id (triangle)
    float u, v;
};

// Leaf code in the compact layout: bit 31 set, first slot << 4, count (15 = read e2.w).
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kNoChild = 0xffffffffu;
__host__ __device__ __forceinline__ uint32_t leaf_code(uint32_t first, uint32_t count) {
    return kLeafBit | (first << 4) | (count < 15u ? count : 15u);
}

// 1/d with the clamp of the reference's traversal test (bvh.rs:808-812,
// mesh.rs:950-954): |d| < 1e-7 -> +-1e30, so a ray lying in a slab plane counts
// as inside the slab instead of producing 0 * inf = NaN.
__device__ __forceinline__ float inv_dir(float d) {
    return fabsf(d) < 1e-7f ? (d >= 0.0f ? 1e30f : -1e30f) : 1.0f / d;
}
struct RayInv { f3 o, d, inv; };
__device__ __forceinline__ RayInv make_ray(f3 o, f3 d) {
    return {o, d, mk3(inv_dir(d.x), inv_dir(d.y), inv_dir(d.z))};
}

// ray_aabb_hit, path_trace.wgsl:248-256, with the slack kCullSlack on the
// entry cull and the exit, so that the closest hit does not depend on the
// visit order.  Each plane distance (plane - o) * inv carries relative errors
// only (the difference, the product and 1/d rounded once each), a few ulps,
// inside the slack, so a box is still entered whenever the exact interval
// reaches the closest hit, and the hit found is the same (the box test only
// decides which boxes are visited).  The fused form fma(plane, inv, -o * inv)
// is not used: rounding o * inv adds an ABSOLUTE error of up to |o * inv|
// 2^-24, beyond any relative slack for a ray that barely moves along an axis
// and starts near a box plane of that axis far from the world origin.
__device__ __forceinline__ bool slab(const RayInv &r, float lx, float ly, float lz, float hx, float hy, float hz,
                                     float tmin, float tmax, float *tenter_out) {
    float t0x = (lx - r.o.x) * r.inv.x, t1x = (hx - r.o.x) * r.inv.x;
    float t0y = (ly - r.o.y) * r.inv.y, t1y = (hy - r.o.y) * r.inv.y;
    float t0z = (lz - r.o.z) * r.inv.z, t1z = (hz - r.o.z) * r.inv.z;
    float tenter = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
    float texit = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    *tenter_out = tenter;
    return cull_t(texit) > fmaxf(tenter, tmin) && tenter <= cull_t(tmax);
}

// ray_sphere_hit root selection, path_trace.wgsl:262-281 (t_max applied by the caller).
__device__ __forceinline__ bool sphere_t(const RayInv &r, float4 cr, float tmin, float *t_out) {
    f3 oc = r.o - mk3(cr.x, cr.y, cr.z);
    float a = dot(r.d, r.d);
    float h = dot(oc, r.d);
    float c = dot(oc, oc) - cr.w * cr.w;
    float disc = h * h - a * c;
    if (disc < 0.0f) return false;
    float sq = sqrtf(disc);
    float t = (-h - sq) / a;
    if (t <= tmin) {
        t = (-h + sq) / a;
        if (t <= tmin) return false;
    }
    *t_out = t;
    return true;
}

// ray_triangle_uvt, path_trace.wgsl:300-317 on precomputed e1/e2 (t_max applied by the caller).
__device__ __forceinline__ bool tri_test(const RayInv &r, f3 v0, f3 e1, f3 e2, float tmin, float *t, float *uu,
                                         float *vv) {
    f3 h = cross(r.d, e2);
    float a = dot(e1, h);
    if (fabsf(a) < 1e-8f) return false;
    float f = 1.0f / a;
    f3 s = r.o - v0;
    float u = f * dot(s, h);
    if (u < 0.0f || u > 1.0f) return false;
    f3 q = cross(s, e1);
    float v = f * dot(r.d, q);
    if (v < 0.0f || u + v > 1.0f) return false;
    float tt = f * dot(e2, q);
    if (tt < tmin) return false;
    *t = tt; *uu = u; *vv = v;
    return true;
}

__device__ __forceinline__ bool tie_better_tri(float t, uint32_t id, const Closest &b) {
    if (t < b.t) return true;
    return t == b.t && b.prim != MCRT_HIT_MISS && !(b.prim & MCRT_HIT_SPHERE) && id < b.prim;
}

// Interpolated shading normal (path_trace.wgsl:448-450), from the triangle's
// shading record (the vertex normals, copied bit for bit).
__device__ __forceinline__ f3 tri_shading_normal(const DeviceScene &S, uint32_t tri_id, float u, float v) {
    const float4 *r = S.shade_recs + 3ull * tri_id;
    f3 na = xyz(__ldg(r)), nb = xyz(__ldg(r + 1)), nc = xyz(__ldg(r + 2));
    float w = 1.0f - u - v;
    return normalize((w * na + u * nb) + v * nc);
}

// The triangle's material word (bit 31: backface flag), from its shading record.
__device__ __forceinline__ uint32_t tri_material_word(const DeviceScene &S, uint32_t tri_id) {
    return __float_as_uint(__ldg(S.shade_recs + 3ull * tri_id).w);
}

// Test the triangles of one leaf (fast records) and update best.
__device__ __forceinline__ void leaf_tris(const DeviceScene &S, const RayInv &r, uint32_t first, uint32_t count,
                                          float tmin, Closest &best) {
    for (uint32_t j = 0; j < count; ++j) {
        const TriRec *tr = S.tris + first + j;
        float4 a = __ldg(&tr->v0), b = __ldg(&tr->e1), c = __ldg(&tr->e2);
        float t, u, v;
        if (!tri_test(r, xyz(a), xyz(b), xyz(c), tmin, &t, &u, &v)) continue;
        uint32_t id = __float_as_uint(a.w);
        if (!tie_better_tri(t, id, best)) continue;
        if (__float_as_uint(b.w) & MCRT_BACKFACE_CULL_FLAG) {       // path_trace.wgsl:438-452
            f3 n = tri_shading_normal(S, id, u, v);
            if (!(dot(r.d, n) < 0.0f)) continue;
        }
        best.t = t; best.prim = id; best.slot = id; best.u = u; best.v = v;
    }
}

__device__ __forceinline__ uint32_t leaf_count(const DeviceScene &S, uint32_t code) {
    uint32_t c = code & 15u;
    if (c == 15u) c = __float_as_uint(__ldg(&S.tris[(code & ~kLeafBit) >> 4].e2.w));
    return c;
}

// sphere_bvh_hit, path_trace.wgsl:343-364, :393-413.
__device__ __forceinline__ void spheres_hit(const DeviceScene &S, const RayInv &r, float tmin, float tmax,
                                            Closest &best, uint32_t *n_nodes) {
    if (S.n_sphere_nodes == 0) return;
    uint32_t stack[kStackSize];
    uint32_t top = 0;
    stack[top++] = 0;
    while (top > 0) {
        uint32_t ni = stack[--top];
        const float4 *np = reinterpret_cast<const float4 *>(S.sphere_nodes + ni);
        float4 mn = __ldg(np), mx = __ldg(np + 1);
        uint4 meta = __ldg(reinterpret_cast<const uint4 *>(np + 2));
        ++*n_nodes;
        float te;
        if (!slab(r, mn.x, mn.y, mn.z, mx.x, mx.y, mx.z, tmin, best.t, &te)) continue;
        if (meta.y > 0) {
            for (uint32_t j = 0; j < meta.y; ++j) {
                uint32_t slot = meta.x + j;
                float4 cr = __ldg(reinterpret_cast<const float4 *>(S.spheres + slot));
                float t;
                if (!sphere_t(r, cr, tmin, &t) || !(t < tmax)) continue;
                uint32_t id = S.sphere_ids[slot] | MCRT_HIT_SPHERE;
                if (t < best.t || (t == best.t && best.prim != MCRT_HIT_MISS && id < best.prim)) {
                    best.t = t; best.prim = id; best.slot = slot; best.u = 0.0f; best.v = 0.0f;
                }
            }
            continue;
        }
        if (top + 2u <= kStackSize) {
            stack[top++] = meta.x;
            stack[top++] = ni + 1u;
        }
    }
}

// mesh_bvh_hit over the reference layout, path_trace.wgsl:368-387, :419-465.
__device__ __forceinline__ void mesh_hit_ref(const DeviceScene &S, const RayInv &r, float tmin, Closest &best,
                                             uint32_t *n_nodes) {
    if (S.n_mesh_nodes == 0) return;
    uint32_t stack[kStackSize];
    uint32_t top = 0;
    stack[top++] = 0;
    while (top > 0) {
        uint32_t ni = stack[--top];
        const float4 *np = reinterpret_cast<const float4 *>(S.mesh_nodes + ni);
        float4 mn = __ldg(np), mx = __ldg(np + 1);
        uint4 meta = __ldg(reinterpret_cast<const uint4 *>(np + 2));
        ++*n_nodes;
        float te;
        if (!slab(r, mn.x, mn.y, mn.z, mx.x, mx.y, mx.z, tmin, best.t, &te)) continue;
        if (meta.y > 0) { leaf_tris(S, r, meta.x, meta.y, tmin, best); continue; }
        if (top + 2u <= kStackSize) {
            stack[top++] = meta.x;
            stack[top++] = ni + 1u;
        }
    }
}

// Any hit in (tmin, tmax) with the same visibility rules (backface-culled
// triangles are invisible from behind); used by shadow rays.
// Any triangle of a leaf that mesh_hit_fast would accept as a hit before its
// first one: tri_test passes, t < tmax, not culled by the backface flag.
__device__ __forceinline__ bool leaf_any(const DeviceScene &S, const RayInv &r, uint32_t first, uint32_t count,
                                         float tmin, float tmax) {
    for (uint32_t j = 0; j < count; ++j) {
        const TriRec *tr = S.tris + first + j;
        float4 a = __ldg(&tr->v0), b = __ldg(&tr->e1), c = __ldg(&tr->e2);
        float t, u, v;
        if (!tri_test(r, xyz(a), xyz(b), xyz(c), tmin, &t, &u, &v)) continue;
        if (!(t < tmax)) continue;
        if (__float_as_uint(b.w) & MCRT_BACKFACE_CULL_FLAG) {       // path_trace.wgsl:438-452
            f3 n = tri_shading_normal(S, __float_as_uint(a.w), u, v);
            if (!(dot(r.d, n) < 0.0f)) continue;
        }
        return true;
    }
    return false;
}

// ---------------------------------------------------------------- stackless walk
// Closest hit and any hit over the compact layout without a stack, for rays
// whose short stack overflowed (trees deeper than the stack: a degenerate
// mesh can make the binned SAH tree as deep as it has triangles).  Each
// compact record keeps its parent's index in word 3.z (kNoChild at the root),
// so the walk goes down and back up (Hapala et al. 2011, "Efficient
// stack-less BVH traversal for ray tracing"): a node's children are ordered
// by entry distance with no far cull (ties: left first), so the order seen
// on the way down is the order seen on the way back; the near child is
// entered when its entry distance is <= the current closest t, the far one
// when the walk comes back from the near one and the same test passes, and
// after the far one the walk returns to the parent.  A child is skipped only
// when its box starts beyond the current closest t, as in the stacked walk,
// so every triangle that can be the closest hit is tested and the tie rule
// gives the same answer.
__device__ __forceinline__ uint32_t cnode_parent(const DeviceScene &S, uint32_t node) {
    return __ldg(reinterpret_cast<const uint32_t *>(S.cnodes + 4ull * node + 3) + 2);
}

// Children of compact node `node` in visit order: c[0] nearer, c[1] farther
// (kNoChild where a box is missed even with no far bound), entry distances t[].
__device__ __forceinline__ void cnode_order(const DeviceScene &S, const RayInv &r, uint32_t node, float tmin,
                                            uint32_t c[2], float t[2]) {
    const float4 *np = S.cnodes + 4ull * node;
    float4 a = __ldg(np), b = __ldg(np + 1), cc = __ldg(np + 2);
    uint4 e = __ldg(reinterpret_cast<const uint4 *>(np + 3));
    const float inf = __uint_as_float(0x7f800000u);
    float tl = 0.0f, tr = 0.0f;
    bool hl = e.x != kNoChild && slab(r, a.x, a.z, cc.x, a.y, a.w, cc.y, tmin, inf, &tl);
    bool hr = e.y != kNoChild && slab(r, b.x, b.z, cc.z, b.y, b.w, cc.w, tmin, inf, &tr);
    if (hl && hr && tr < tl) {
        c[0] = e.y; t[0] = tr; c[1] = e.x; t[1] = tl;
    } else {
        c[0] = hl ? e.x : (hr ? e.y : kNoChild);
        t[0] = hl ? tl : tr;
        c[1] = (hl && hr) ? e.y : kNoChild;
        t[1] = tr;
    }
}

// ANY = false: closest hit into best; ANY = true: returns whether some
// triangle is accepted before tmax (best.t must be tmax), stopping there.
template <bool ANY>
__device__ __noinline__ bool mesh_walk_stackless(const DeviceScene &S, const RayInv &r, float tmin, Closest &best,
                                                 uint32_t *n_nodes) {
    if (S.n_mesh_nodes == 0) return false;
    {
        const float4 *np = reinterpret_cast<const float4 *>(S.mesh_nodes);
        float4 mn = __ldg(np), mx = __ldg(np + 1);
        float te;
        if (!slab(r, mn.x, mn.y, mn.z, mx.x, mx.y, mx.z, tmin, best.t, &te)) return false;
        if (S.n_cnodes == 0) {                     // the whole tree is one leaf
            uint4 meta = __ldg(reinterpret_cast<const uint4 *>(np + 2));
            if (ANY) return leaf_any(S, r, meta.x, meta.y, tmin, best.t);
            leaf_tris(S, r, meta.x, meta.y, tmin, best);
            return false;
        }
    }
    uint32_t node = 0, from = kNoChild;            // from: the child the walk returns from
    for (;;) {
        uint32_t c[2];
        float t[2];
        cnode_order(S, r, node, tmin, c, t);
        if (from == kNoChild) ++*n_nodes;
        uint32_t k = from == kNoChild ? 0u : (from == c[0] ? 1u : 2u);
        uint32_t down = kNoChild;
        for (; k < 2u; ++k) {
            if (c[k] == kNoChild || !(t[k] <= cull_t(best.t))) continue;
            if (c[k] & kLeafBit) {
                const uint32_t first = (c[k] & ~kLeafBit) >> 4, cnt = leaf_count(S, c[k]);
                if (ANY) {
                    if (leaf_any(S, r, first, cnt, tmin, best.t)) return true;
                } else {
                    leaf_tris(S, r, first, cnt, tmin, best);
                }
                continue;
            }
            down = c[k];
            break;
        }
        if (down != kNoChild) {
            node = down;
            from = kNoChild;
            continue;
        }
        const uint32_t up = cnode_parent(S, node);
        if (up == kNoChild) return false;
        from = node;
        node = up;
    }
}

// Compact layout: node k = {Lx, Ly | Rx, Ry | Lz, Rz | codeL, codeR, parent, 0}.
// A ray that would overflow the stack is finished by the stackless walk from
// its current closest hit (which only tightens the cull).
__device__ __forceinline__ void mesh_hit_fast(const DeviceScene &S, const RayInv &r, float tmin, Closest &best,
                                              uint32_t *n_nodes) {
    if (S.n_mesh_nodes == 0) return;
    if (S.n_cnodes == 0) {                       // the whole tree is one leaf
        const float4 *np = reinterpret_cast<const float4 *>(S.mesh_nodes);
        float4 mn = __ldg(np), mx = __ldg(np + 1);
        uint4 meta = __ldg(reinterpret_cast<const uint4 *>(np + 2));
        float te;
        if (slab(r, mn.x, mn.y, mn.z, mx.x, mx.y, mx.z, tmin, best.t, &te)) leaf_tris(S, r, meta.x, meta.y, tmin, best);
        return;
    }
    // the root box itself (reference node 0) is tested first, as the reference does
    {
        const float4 *np = reinterpret_cast<const float4 *>(S.mesh_nodes);
        float4 mn = __ldg(np), mx = __ldg(np + 1);
        float te;
        if (!slab(r, mn.x, mn.y, mn.z, mx.x, mx.y, mx.z, tmin, best.t, &te)) return;
    }
    uint2 stack[kStackSize];
    uint32_t sp = 0;
    uint32_t node = 0;
    for (;;) {
        const float4 *np = S.cnodes + 4ull * node;
        float4 a = __ldg(np), b = __ldg(np + 1), c = __ldg(np + 2);
        uint4 e = __ldg(reinterpret_cast<const uint4 *>(np + 3));
        ++*n_nodes;
        float tl, tr;
        bool hl = e.x != kNoChild && slab(r, a.x, a.z, c.x, a.y, a.w, c.y, tmin, best.t, &tl);
        bool hr = e.y != kNoChild && slab(r, b.x, b.z, c.z, b.y, b.w, c.w, tmin, best.t, &tr);
        uint32_t next = kNoChild;
        if (hl && hr) {
            uint32_t near = e.x, far = e.y;
            float tfar = tr;
            if (tr < tl) { near = e.y; far = e.x; tfar = tl; }
            if (sp == kStackSize) {
                mesh_walk_stackless<false>(S, r, tmin, best, n_nodes);
                return;
            }
            stack[sp++] = make_uint2(far, __float_as_uint(tfar));
            next = near;
        } else if (hl) {
            next = e.x;
        } else if (hr) {
            next = e.y;
        }
        // descend through leaves and popped entries until an internal node is found
        for (;;) {
            if (next == kNoChild) {
                // pop, skipping entries that start beyond the current closest hit
                next = kNoChild;
                while (sp > 0) {
                    uint2 s = stack[--sp];
                    if (__uint_as_float(s.y) <= cull_t(best.t)) { next = s.x; break; }
                }
                if (next == kNoChild) return;
            }
            if (next & kLeafBit) {
                uint32_t first = (next & ~kLeafBit) >> 4;
                leaf_tris(S, r, first, leaf_count(S, next), tmin, best);
                next = kNoChild;
                continue;
            }
            break;
        }
        node = next;
    }
}

// world_hit, path_trace.wgsl:471-479: spheres first, then the mesh with t_max =
// the sphere distance; the mesh wins only when strictly closer.
__device__ __forceinline__ Closest world_hit(const DeviceScene &S, const RayInv &r, float tmin, float tmax,
                                             bool ref_layout, uint32_t *n_nodes) {
    Closest best{tmax, MCRT_HIT_MISS, 0u, 0.0f, 0.0f};
    spheres_hit(S, r, tmin, tmax, best, n_nodes);
    if (ref_layout) mesh_hit_ref(S, r, tmin, best, n_nodes);
    else mesh_hit_fast(S, r, tmin, best, n_nodes);
    if (best.prim == MCRT_HIT_MISS) best.t = -1.0f;
    return best;
}

// Is there a mesh hit in [tmin, tmax)?  mesh_hit_fast's traversal (same
// order, same cull against tmax) up to its first accepted hit, which alone
// decides whether it finds one, so the answer is the same; it stops there.
__device__ __forceinline__ bool mesh_any_hit(const DeviceScene &S, const RayInv &r, float tmin, float tmax) {
    if (S.n_mesh_nodes == 0) return false;
    const float4 *root = reinterpret_cast<const float4 *>(S.mesh_nodes);
    {
        float4 mn = __ldg(root), mx = __ldg(root + 1);
        float te;
        if (!slab(r, mn.x, mn.y, mn.z, mx.x, mx.y, mx.z, tmin, tmax, &te)) return false;
    }
    if (S.n_cnodes == 0) {                       // the whole tree is one leaf
        uint4 meta = __ldg(reinterpret_cast<const uint4 *>(root + 2));
        return leaf_any(S, r, meta.x, meta.y, tmin, tmax);
    }
    uint2 stack[kStackSize];
    uint32_t sp = 0;
    uint32_t node = 0;
    for (;;) {
        const float4 *np = S.cnodes + 4ull * node;
        float4 a = __ldg(np), b = __ldg(np + 1), c = __ldg(np + 2);
        uint4 e = __ldg(reinterpret_cast<const uint4 *>(np + 3));
        float tl, tr;
        bool hl = e.x != kNoChild && slab(r, a.x, a.z, c.x, a.y, a.w, c.y, tmin, tmax, &tl);
        bool hr = e.y != kNoChild && slab(r, b.x, b.z, c.z, b.y, b.w, c.w, tmin, tmax, &tr);
        uint32_t next = kNoChild;
        if (hl && hr) {
            uint32_t near = e.x, far = e.y;
            float tfar = tr;
            if (tr < tl) { near = e.y; far = e.x; tfar = tl; }
            if (sp == kStackSize) {                // too deep for the stack: walk without one
                uint32_t nn = 0;
                Closest b{tmax, MCRT_HIT_MISS, 0u, 0.0f, 0.0f};
                return mesh_walk_stackless<true>(S, r, tmin, b, &nn);
            }
            stack[sp++] = make_uint2(far, __float_as_uint(tfar));
            next = near;
        } else if (hl) {
            next = e.x;
        } else if (hr) {
            next = e.y;
        }
        for (;;) {
            if (next == kNoChild) {
                while (sp > 0) {
                    uint2 s = stack[--sp];
                    if (__uint_as_float(s.y) <= cull_t(tmax)) { next = s.x; break; }
                }
                if (next == kNoChild) return false;
            }
            if (next & kLeafBit) {
                if (leaf_any(S, r, (next & ~kLeafBit) >> 4, leaf_count(S, next), tmin, tmax)) return true;
                next = kNoChild;
                continue;
            }
            break;
        }
        node = next;
    }
}

__device__ __forceinline__ bool occluded(const DeviceScene &S, const RayInv &r, float tmin, float tmax) {
    uint32_t nn = 0;
    Closest best{tmax, MCRT_HIT_MISS, 0u, 0.0f, 0.0f};
    spheres_hit(S, r, tmin, tmax, best, &nn);
    if (best.prim != MCRT_HIT_MISS) return true;
    return mesh_any_hit(S, r, tmin, tmax);
}

}  // namespace mcrt
