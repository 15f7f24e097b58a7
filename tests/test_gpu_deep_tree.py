"""Trees deeper than the traversal stacks.

The reference's traversal keeps a 64-entry stack and drops children past it
(path_trace.wgsl:358), so a ray through a deeper tree can miss its hit.  The
closest-hit kernels here keep 32- or 64-entry stacks; a ray whose next push
would overflow is handed to the stackless walk (parent links in the compact
nodes), so every variant returns the exact closest hit on any tree.

The scene is the seeded Cornell box plus 150 thin layers across the view,
uploaded with a hand-made caterpillar BVH (each internal node: one leaf of one
triangle and an internal node holding the rest; 185 levels), the far layers
near the root, so a camera ray pushes one leaf per level.  The oracle traces
the same triangles through its own reference-algorithm BVH (a shallow tree, so
its 64-entry stack never drops), and every image must equal it bit for bit.
"""
import numpy as np
import pytest

import mcrt_gb300 as M
from mcrt_gb300 import scenes
from mcrt_gb300._native import NODE, TRIANGLE, VERTEX

pytestmark = pytest.mark.gpu

N_LAYERS = 150


def _layered_scene(seed=1234):
    sc = scenes.cornell_box(seed)
    verts = list(sc["vertices"])
    tris = [((int(t["v"][0]), int(t["v"][1]), int(t["v"][2])), int(t["mat_idx"])) for t in sc["triangles"]]
    lo, hi = 0.05, 0.95
    for i in range(N_LAYERS):                      # far (small z) to near
        z = 0.1 + 0.8 * i / (N_LAYERS - 1)
        corners = [(lo, lo), (hi, lo), (lo, hi)] if i % 2 == 0 else [(hi, hi), (lo, hi), (hi, lo)]
        base = len(verts)
        for k, (x, y) in enumerate(corners):
            v = np.zeros((), VERTEX)
            v["position"] = (x, y, z, 1.0)
            v["normal"] = (0.0, 0.0, 1.0, 0.0)
            v["uv"][:2] = [(0, 0), (1, 0), (0, 1)][k]
            verts.append(v)
        tris.append(((base, base + 1, base + 2), i % 3))
    V = np.array(verts, VERTEX)
    T = np.zeros(len(tris), TRIANGLE)
    T["v"] = [t[0] for t in tris]
    T["mat_idx"] = [t[1] for t in tris]
    return sc, V, T


def _padded_box(V, tri):
    p = V["position"][tri["v"]][:, :3]
    mn, mx = p.min(axis=0), p.max(axis=0)
    eps = np.float32(1e-4)
    return np.minimum(mn, mx - eps), np.maximum(mx, mn + eps)


def caterpillar_bvh(V, T):
    """Pre-order reference-layout nodes: node 2k (internal) has leaf 2k+1
    (triangle k) on the left and node 2k+2 on the right; the last internal node
    holds the last two triangles as leaves.  Depth len(T) - 1."""
    n = len(T)
    boxes = [_padded_box(V, T[i]) for i in range(n)]
    nodes = np.zeros(2 * n - 1, NODE)
    suffix_mn, suffix_mx = boxes[-1][0].copy(), boxes[-1][1].copy()
    sub = [None] * n                                 # box of triangles i .. n-1
    for i in range(n - 1, -1, -1):
        suffix_mn = np.minimum(suffix_mn, boxes[i][0])
        suffix_mx = np.maximum(suffix_mx, boxes[i][1])
        sub[i] = (suffix_mn.copy(), suffix_mx.copy())

    def put(idx, box, right_or_offset, count):
        nodes[idx]["aabb_min"][:3] = box[0]
        nodes[idx]["aabb_max"][:3] = box[1]
        nodes[idx]["right_or_offset"] = right_or_offset
        nodes[idx]["prim_count"] = count

    for k in range(n - 1):
        put(2 * k, sub[k], 2 * k + 2, 0)
        put(2 * k + 1, boxes[k], k, 1)
    put(2 * n - 2, boxes[n - 1], n - 1, 1)
    return nodes


def _tree_depth(nodes):
    depth, stack = 0, [(0, 0)]
    while stack:
        i, d = stack.pop()
        depth = max(depth, d)
        if nodes[i]["prim_count"] == 0:
            stack.append((i + 1, d + 1))
            stack.append((int(nodes[i]["right_or_offset"]), d + 1))
    return depth


@pytest.fixture(scope="module")
def deep():
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle"))
    import pyoracle as O
    sc, V, T = _layered_scene()
    nodes = caterpillar_bvh(V, T)
    env = M.gradient_env_map()
    osc = O.OracleScene(materials=sc["materials"], vertices=V, triangles=T, env=env)
    assert _tree_depth(nodes) == len(T) - 1 > 64
    assert _tree_depth(osc.mesh_nodes) < 32         # the oracle's own tree: no dropped children
    ctx = M.Context(0)
    ctx.upload_scene(vertices=V, triangles=T, materials=sc["materials"], env=env, mesh_bvh=nodes,
                     triangle_order=np.arange(len(T), dtype=np.uint32))
    c = sc["camera"]
    yield dict(ctx=ctx, osc=osc, V=V, T=T, sc=sc, env=env, cam=lambda w, h: M.compute_camera(
        w, h, c["look_from"], c["look_at"], c["vfov"], 0.0))
    ctx.close()


def test_deep_tree_closest_hits_equal_brute_force(deep):
    ctx, osc = deep["ctx"], deep["osc"]
    rng = np.random.default_rng(5)
    org = np.column_stack([rng.uniform(0.1, 0.9, 4096), rng.uniform(0.1, 0.9, 4096), np.full(4096, 2.0)])
    d = np.column_stack([rng.normal(0, 0.15, 4096), rng.normal(0, 0.15, 4096), -np.ones(4096)])
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = M.make_rays(org, d)
    got, want = ctx.trace_closest(rays), osc.trace(rays, brute_force=True)
    assert np.array_equal(got["prim"], want["prim"])
    assert np.array_equal(got["t"].view(np.uint32), want["t"].view(np.uint32))


@pytest.mark.parametrize("nee", [False, True])
def test_deep_tree_every_variant_renders_the_oracle_image(deep, nee):
    ctx, osc = deep["ctx"], deep["osc"]
    w, h, spp = 48, 40, 3
    cam = deep["cam"](w, h)
    want = osc.render(cam, w, h, spp, max_depth=8, nee=nee)["rgba"]
    for v in range(8):
        got = ctx.render(cam, w, h, spp, max_depth=8, nee=nee, variant=v)["rgba"]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"variant {v}"
        assert ctx.timings()["stackless_rays"] > 0


def test_deep_tree_autotuned_render(deep):
    ctx, osc = deep["ctx"], deep["osc"]
    w, h, spp = 48, 40, 2
    cam = deep["cam"](w, h)
    variant, ms = ctx.autotune(cam, w, h, spp, max_depth=8)
    assert all(t > 0 for t in ms)
    got = ctx.render(cam, w, h, spp, first_frame=7, max_depth=8, nee=True)["rgba"]
    want = osc.render(cam, w, h, spp, first_frame=7, max_depth=8, nee=True)["rgba"]
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_deep_tree_adjoint_equals_the_shallow_tree(deep):
    """The adjoint replay's shadow rays overflow too: gradients on the deep tree
    equal those of the same scene on the GPU-built tree (up to the order of the
    per-block float sums)."""
    ctx = deep["ctx"]
    w, h, spp = 32, 32, 2
    cam = deep["cam"](w, h)
    d_img = np.random.default_rng(1).standard_normal((h, w, 4)).astype(np.float32)
    g_deep = ctx.adjoint(cam, w, h, spp, d_img, max_depth=6, nee=True)
    with M.Context(0) as c2:
        c2.upload_scene(vertices=deep["V"], triangles=deep["T"], materials=deep["sc"]["materials"], env=deep["env"])
        g_flat = c2.adjoint(cam, w, h, spp, d_img, max_depth=6, nee=True)
    scale = float(np.abs(g_flat).max())
    assert scale > 0
    assert float(np.abs(g_deep - g_flat).max()) <= 2e-4 * scale
