"""GPU edge cases against the oracle, bit for bit: a scene with no geometry,
ragged image sizes with sample counts that do not divide into their passes, a
one-pixel image, single-bounce paths, an empty ray batch, a zero-area
triangle (the reference's Moller-Trumbore test rejects it by its determinant,
path_trace.wgsl:300-317), and rays that graze box planes far from the world
origin (traced, and rendered by every closest-hit variant)."""
import os
import sys

import numpy as np
import pytest

import mcrt_gb300 as M
from mcrt_gb300 import scenes

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import grazing_cases as G  # noqa: E402

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_scene_without_geometry_renders_the_environment(ctx, oracle):
    md = M.materials([(0, (0.5, 0.5, 0.5), 0, 1)])
    env = M.gradient_env_map()
    cam = M.compute_camera(7, 5, (0, 0, 1), (0, 0, 0), 40.0, 0.0)
    ctx.upload_scene(materials=md, env=env)
    osc = oracle.OracleScene(materials=md, env=env)
    want = osc.render(cam, 7, 5, 3, first_frame=2, max_depth=8)
    for nee in (False, True):                          # no lights: NEE changes nothing
        got = ctx.render(cam, 7, 5, 3, first_frame=2, max_depth=8, nee=nee)
        assert np.array_equal(bits(got["rgba"]), bits(want["rgba"]))
        assert np.array_equal(got["sum"].view(np.uint64), want["sum"].view(np.uint64))


@pytest.mark.parametrize("w,h,spp,per_pass,depth", [(37, 23, 5, 2, 8), (1, 1, 3, 0, 8), (16, 12, 2, 0, 1)])
def test_ragged_sizes_passes_and_depths(ctx, oracle, w, h, spp, per_pass, depth):
    sc = scenes.cornell_box(1234)
    c = sc["camera"]
    env = M.gradient_env_map()
    cam = M.compute_camera(w, h, c["look_from"], c["look_at"], c["vfov"], 0.0)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"], env=env)
    got = ctx.render(cam, w, h, spp, first_frame=3, max_depth=depth, spp_per_pass=per_pass)
    osc = oracle.OracleScene(materials=sc["materials"], vertices=sc["vertices"], triangles=sc["triangles"], env=env)
    want = osc.render(cam, w, h, spp, first_frame=3, max_depth=depth)
    assert np.array_equal(bits(got["rgba"]), bits(want["rgba"]))
    assert np.array_equal(got["sum"].view(np.uint64), want["sum"].view(np.uint64))


def test_empty_ray_batch_and_zero_area_triangle(ctx, oracle):
    sc = scenes.cornell_box(1234)
    n = len(sc["vertices"])
    V = np.concatenate([sc["vertices"], sc["vertices"][:3]])
    V["position"][n + 2] = 0.5 * V["position"][n] + 0.5 * V["position"][n + 1]     # collinear corners
    T = np.concatenate([sc["triangles"], sc["triangles"][:1]])
    T["v"][-1] = (n, n + 1, n + 2)
    ctx.upload_scene(vertices=V, triangles=T, materials=sc["materials"])
    assert len(ctx.trace_closest(M.make_rays(np.zeros((0, 3)), np.zeros((0, 3))))) == 0
    rng = np.random.default_rng(4)
    d = rng.normal(size=(4096, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = M.make_rays(np.tile(np.float32([0.5, 0.4, 0.5]), (4096, 1)), d)
    got = ctx.trace_closest(rays)
    want = oracle.OracleScene(materials=sc["materials"], vertices=V, triangles=T).trace(rays)
    assert np.array_equal(got["prim"], want["prim"])
    assert np.array_equal(bits(got["t"]), bits(want["t"]))
    assert not np.any(got["prim"] == len(T) - 1)       # the zero-area triangle is never hit


def test_grazing_rays_far_from_the_origin_find_their_hits(ctx, oracle):
    """Rays that graze box planes far from the world origin (grazing_cases):
    every ray still enters its triangle's box and returns the oracle's
    brute-force hit, through both node layouts."""
    V, T, rays = G.grazing_walls()
    md = M.materials([(0, (0.5, 0.5, 0.5), 0, 1)])
    ctx.upload_scene(vertices=V, triangles=T, materials=md)
    want = oracle.OracleScene(materials=md, vertices=V, triangles=T).trace(rays, brute_force=True)
    assert np.array_equal(want["prim"], np.arange(len(T), dtype=np.uint32))
    for ref_layout in (False, True):
        got = ctx.trace_closest(rays, reference_layout=ref_layout)
        assert np.array_equal(got["prim"], want["prim"])
        assert np.array_equal(bits(got["t"]), bits(want["t"]))


def test_grazing_camera_every_variant_renders_the_oracle_image(ctx, oracle):
    """Camera rays from x = 1234.5677 with direction x components of 1..21
    ulps of that origin per 100 units, onto a wall 2 ulps away in x that ends
    at z = 30: the wall's far edge is where the rounding of o / d decides the
    box test.  Every closest-hit variant renders the oracle's image."""
    X = np.float32(1234.5677)
    u = np.spacing(X)
    xw = np.float32(X + 2 * u)
    V = np.zeros(4, M._native.VERTEX)
    V["position"] = [[xw, -60, 0, 1], [xw, 60, 0, 1], [xw, 60, 30, 1], [xw, -60, 30, 1]]
    T = np.zeros(2, M._native.TRIANGLE)
    T["v"] = [(0, 1, 2), (0, 2, 3)]
    md = M.materials([(0, (0.7, 0.6, 0.5), 0, 1)])
    env = M.gradient_env_map()
    cam = np.zeros((), M._native.CAMERA)
    cam["origin"] = [X, 0, 0, 0]
    cam["lower_left"] = [np.float32(X + u), -50, 100, 0]
    cam["horizontal"] = [20 * u, 0, 0, 0]
    cam["vertical"] = [0, 100, 0, 0]
    w, h, spp = 48, 32, 2
    ctx.upload_scene(vertices=V, triangles=T, materials=md, env=env)
    want = oracle.OracleScene(materials=md, vertices=V, triangles=T, env=env).render(cam, w, h, spp, max_depth=3)
    for v in range(8):
        got = ctx.render(cam, w, h, spp, max_depth=3, variant=v)
        assert np.array_equal(bits(got["rgba"]), bits(want["rgba"])), f"variant {v}"
