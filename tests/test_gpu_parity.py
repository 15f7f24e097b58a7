"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Bit-exact for closest hits (primitive id and t bits), the GPU-built BVH, the
reference-estimator radiance (running mean, f64 sums, G-buffer) and the
denoiser; next-event estimation against the reference estimator by relMSE.
"""
import os

import numpy as np
import pytest

import mcrt_gb300 as M
from conftest import golden, load_fixture_scene

pytestmark = pytest.mark.gpu

SCENES = ["diffuse_sphere", "mirror_sphere", "glass_sphere", "emissive_box", "cornell_box_mini", "skymap_sphere"]


def env_for(name):
    z = np.load(golden(f"scene_{name}.npz"))
    return M.load_env_map(golden("test_sky_128x64.hdr")) if bool(z["uses_sky"][0]) else M.gradient_env_map()


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def upload_reference(ctx, osc):
    ctx.upload_scene(**osc.reference_buffers())


def oracle_scene(oracle, s, env):
    return oracle.OracleScene(materials=s["materials"], spheres=s["spheres"], vertices=s["vertices"],
                              triangles=s["triangles"], env=env)


def rel_mse(x, r):
    return float(np.mean((x - r) ** 2 / (r * r + 1e-2)))


# ---------------------------------------------------------------- closest hit
@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("ref_layout", [True, False])
def test_closest_hit_bit_exact_against_golden(ctx, oracle, name, ref_layout):
    s = load_fixture_scene(name)
    g = np.load(golden(f"oracle_{name}.npz"))
    rays = g["rays"].view(M.RAY).reshape(-1)
    want = g["hits"].view(M.HIT).reshape(-1)
    osc = oracle_scene(oracle, s, env_for(name))
    upload_reference(ctx, osc)
    got = ctx.trace_closest(rays, reference_layout=ref_layout)
    assert np.array_equal(got["prim"], want["prim"])
    assert np.array_equal(bits(got["t"]), bits(want["t"]))
    tri = (want["prim"] != M._native.HIT_MISS) & (want["prim"] < M._native.HIT_SPHERE)
    assert np.array_equal(bits(got["u"][tri]), bits(want["u"][tri]))
    assert np.array_equal(bits(got["v"][tri]), bits(want["v"][tri]))


def random_scene_rays(rng, n, lo=-3, hi=3):
    org = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    # a few exactly axis-parallel rays through vertices and planes
    d[:64] = 0
    d[np.arange(64), np.arange(64) % 3] = np.where(np.arange(64) % 2, 1.0, -1.0)
    return M.make_rays(org, d)


def test_closest_hit_large_mesh_gpu_built_bvh(ctx, oracle):
    from mcrt_gb300 import scenes
    sc = scenes.displaced_icosphere(seed=5, level=5, width=64, height=64)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"], env=sc["env"])
    osc = oracle.OracleScene(materials=sc["materials"], vertices=sc["vertices"], triangles=sc["triangles"])
    rng = np.random.default_rng(3)
    rays = random_scene_rays(rng, 200000, -2.5, 2.5)
    rays["org"][:, 1] += 1.2
    want = osc.trace(rays)
    got = ctx.trace_closest(rays)
    assert (want["prim"] != 0xFFFFFFFF).sum() > 50000
    assert np.array_equal(got["prim"], want["prim"])
    assert np.array_equal(bits(got["t"]), bits(want["t"]))


# ---------------------------------------------------------------- GPU BVH builder
def leaf_sets(nodes, order):
    out = []
    for nd in nodes:
        if nd["prim_count"] > 0:
            o, c = int(nd["right_or_offset"]), int(nd["prim_count"])
            out.append(tuple(sorted(order[o:o + c].tolist())))
        else:
            out.append(None)
    return out


@pytest.mark.parametrize("which", ["cornell", "ico4", "ico6", "torus", "degenerate"])
def test_gpu_bvh_equals_reference_builder(ctx, oracle, which):
    from mcrt_gb300 import scenes
    if which == "cornell":
        sc = scenes.cornell_box(1234)
        V, T = sc["vertices"], sc["triangles"]
    elif which.startswith("ico"):
        sc = scenes.displaced_icosphere(seed=9, level=int(which[3:]), width=8, height=8)
        V, T = sc["vertices"], sc["triangles"]
    elif which == "torus":
        from test_oracle_kats import torus
        V, T = torus(2.0, 0.5, 48, 24)
    else:   # many coincident and coplanar triangles
        V = np.zeros(3 * 300, M.VERTEX)
        rng = np.random.default_rng(1)
        base = rng.integers(0, 5, (300, 1)).astype(np.float32)
        V["position"][:, 0] = np.repeat(base[:, 0], 3) + np.tile([0, 1, 0], 300)
        V["position"][:, 1] = np.tile([0, 0, 1], 300)
        T = np.zeros(300, M.TRIANGLE)
        T["v"] = np.arange(900).reshape(300, 3)
    md = M.materials([(0, (0.5, 0.5, 0.5), 0, 1)])
    ctx.upload_scene(vertices=V, triangles=T, materials=md)
    g_nodes, g_order = ctx.mesh_bvh()
    o_nodes, _, o_ids = oracle.build_mesh_bvh(V, T)
    assert len(g_nodes) == len(o_nodes)
    for f in ("aabb_min", "aabb_max"):
        assert np.array_equal(bits(g_nodes[f]), bits(o_nodes[f]))
    assert np.array_equal(g_nodes["right_or_offset"], o_nodes["right_or_offset"])
    assert np.array_equal(g_nodes["prim_count"], o_nodes["prim_count"])
    assert leaf_sets(g_nodes, g_order) == leaf_sets(o_nodes, o_ids)


def test_gpu_sphere_bvh_and_update_vertices(ctx, oracle):
    rng = np.random.default_rng(4)
    S = np.zeros(300, M.SPHERE)
    S["center_r"][:, :3] = rng.uniform(-5, 5, (300, 3))
    S["center_r"][:, 3] = rng.uniform(0.05, 0.4, 300)
    from test_oracle_kats import torus
    V, T = torus(2.0, 0.5, 32, 16)
    md = M.materials([(0, (0.5, 0.5, 0.5), 0, 1)])
    ctx.upload_scene(spheres=S, vertices=V, triangles=T, materials=md)
    rays = random_scene_rays(rng, 50000, -5, 5)
    osc = oracle.OracleScene(materials=md, spheres=S, vertices=V, triangles=T)
    want, got = osc.trace(rays), ctx.trace_closest(rays)
    assert np.array_equal(got["prim"], want["prim"]) and np.array_equal(bits(got["t"]), bits(want["t"]))
    # move the mesh: the BVH is rebuilt on the GPU
    V2 = V.copy()
    V2["position"][:, 1] += 0.7
    ctx.update_vertices(V2)
    osc2 = oracle.OracleScene(materials=md, spheres=S, vertices=V2, triangles=T)
    want, got = osc2.trace(rays), ctx.trace_closest(rays)
    assert np.array_equal(got["prim"], want["prim"]) and np.array_equal(bits(got["t"]), bits(want["t"]))


# ---------------------------------------------------------------- radiance
@pytest.mark.parametrize("name", SCENES)
def test_render_reference_estimator_bit_exact_against_golden(ctx, oracle, name):
    s = load_fixture_scene(name)
    g = np.load(golden(f"oracle_{name}.npz"))
    cam = g["camera32"].view(M.CAMERA).reshape(())
    ctx.upload_scene(spheres=s["spheres"], vertices=s["vertices"], triangles=s["triangles"], materials=s["materials"],
                     env=env_for(name))
    r = ctx.render(cam, 32, 32, 4, max_depth=8)
    assert np.array_equal(bits(r["rgba"]), bits(g["rgba"]))
    assert np.array_equal(r["sum"].view(np.uint64), g["sum"].view(np.uint64))
    assert np.array_equal(bits(r["gbuf"]), bits(g["gbuf"]))


@pytest.mark.parametrize("spp_per_pass", [1, 3, 0])
def test_render_cornell_config0_bit_exact(ctx, oracle, spp_per_pass):
    from mcrt_gb300 import scenes
    sc = scenes.cornell_box(1234)
    c = sc["camera"]
    cam = M.compute_camera(96, 80, c["look_from"], c["look_at"], c["vfov"], 0.0)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"],
                     env=M.gradient_env_map())
    r = ctx.render(cam, 96, 80, 8, first_frame=5, max_depth=8, spp_per_pass=spp_per_pass)
    osc = oracle.OracleScene(materials=sc["materials"], vertices=sc["vertices"], triangles=sc["triangles"],
                             env=M.gradient_env_map())
    o = osc.render(cam, 96, 80, 8, first_frame=5, max_depth=8)
    assert np.array_equal(bits(r["rgba"]), bits(o["rgba"]))
    assert np.array_equal(r["sum"].view(np.uint64), o["sum"].view(np.uint64))
    # continuing the accumulation equals one longer run
    r2 = ctx.render(cam, 96, 80, 4, first_frame=13, max_depth=8, keep=True)
    o2 = osc.render(cam, 96, 80, 12, first_frame=5, max_depth=8)
    assert np.array_equal(bits(r2["rgba"]), bits(o2["rgba"]))


def test_nee_converges_to_reference_estimator(ctx):
    s = load_fixture_scene("cornell_box_mini")
    c = s["camera"]
    ctx.upload_scene(spheres=s["spheres"], vertices=s["vertices"], triangles=s["triangles"], materials=s["materials"],
                     env=M.gradient_env_map())
    w = h = 24
    cam = M.compute_camera(w, h, [0.0, 4.75, 8.0], [0.0, 4.0, 0.0], 60.0, 0.0)
    ref = ctx.render(cam, w, h, 131072, max_depth=8, outputs=("sum",))["sum"] / 131072
    nee = ctx.render(cam, w, h, 16384, max_depth=8, nee=True, outputs=("sum",))["sum"] / 16384
    e = rel_mse(nee, ref)
    assert e < 1e-3, e


# ---------------------------------------------------------------- denoiser
@pytest.mark.parametrize("radius", [3, 2, 11])
def test_denoise_bit_exact(ctx, oracle, radius):
    s = load_fixture_scene("cornell_box_mini")
    c = s["camera"]
    cam = M.compute_camera(77, 53, [0.0, 4.75, 8.0], [0.0, 4.0, 0.0], 60.0, 0.0)
    ctx.upload_scene(spheres=s["spheres"], vertices=s["vertices"], triangles=s["triangles"], materials=s["materials"],
                     env=M.gradient_env_map())
    r = ctx.render(cam, 77, 53, 4)
    gb = r["gbuf"].copy()
    gb[:5, :7, 3] = -1.0                      # a patch of sky pixels (depth < 0, denoise.wgsl:62)
    got = ctx.denoise(r["rgba"], gb, radius=radius, sigma_s=2.0, sigma_d=0.5, normal_pow=8.0)
    want = oracle.denoise(r["rgba"], gb, radius=radius, sigma_s=2.0, sigma_d=0.5, normal_pow=8.0)
    assert np.array_equal(bits(got), bits(want))


# ---------------------------------------------------------------- errors
def test_invalid_inputs_are_rejected(mcrt):
    with M.Context(0) as c:
        with pytest.raises(M.MCRTError) as e:
            c.render(M.compute_camera(4, 4, (0, 0, 1), (0, 0, 0)), 4, 4, 1)
        assert e.value.status == -6
        V = np.zeros(3, M.VERTEX)
        T = np.zeros(1, M.TRIANGLE)
        T["v"] = (0, 1, 3)
        md = M.materials([(0, (0.5, 0.5, 0.5), 0, 1)])
        with pytest.raises(M.MCRTError) as e:
            c.upload_scene(vertices=V, triangles=T, materials=md)
        assert e.value.status == -1
        T["v"] = (0, 1, 2)
        bad = np.zeros(3, M.NODE)
        bad[0]["right_or_offset"] = 0      # a child before its parent
        with pytest.raises(M.MCRTError) as e:
            c.upload_scene(vertices=V, triangles=T, materials=md, mesh_bvh=bad)
        assert e.value.status == -1
        c.upload_scene(vertices=V, triangles=T, materials=md)
        r = M.make_rays([(0, 0, 1)], [(0, 0, -1)], tmin=0.0)
        with pytest.raises(M.MCRTError) as e:
            c.trace_closest(r)
        assert e.value.status == -1
        with pytest.raises(M.MCRTError):
            c.update_vertices(np.zeros(4, M.VERTEX))
