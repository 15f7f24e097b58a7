"""Parity at the benchmark workloads' own sizes.

* Displaced icosphere (1,310,722 triangles, 1920 x 1080, 16 spp, depth 12),
  BVH built on the GPU: the closest-hit queries of 245,760 camera paths (8
  strips of 16 rows, one sample per pixel) at bounces 0-3, dumped by the oracle
  from its reference traversal of the reference-algorithm BVH
  (path_trace.wgsl:343-479), traced through mcrt_trace_closest: primitive ids
  and the bits of t, u and v equal; and 128 rows of the full frame rendered on
  the GPU equal the oracle's rows bit for bit (they include a shared-edge tie
  that the exact box test had resolved differently in the two visit orders).
* Voxel world (256 x 128 x 256, 4,943,232 exposed-face triangles, 1280 x 720,
  8 spp, depth 6, sun + sky, next-event estimation): the GPU mesh equals the
  oracle's mesher byte for byte, then the same two checks on 245,760 paths
  (8 strips of 24 rows) and 128 rows of the frame.
* Rays aimed at the vertices and edges of a displaced icosphere (ties between
  triangles meeting there): both GPU layouts equal the oracle's brute force.
"""
import os
import sys

import numpy as np
import pytest

import mcrt_gb300 as M
from mcrt_gb300 import scenes

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))


def _strips(h, n, rows):
    return [int((k + 0.5) * h / n) - rows // 2 for k in range(n)]


def _check_hits(ctx, osc, cam, w, h, strip_rows, nee, max_depth):
    rays, hits, bounce = [], [], []
    for y0 in _strips(h, 8, strip_rows):
        r, hh, b = osc.dump_rays(cam, w, h, 1, rect=(0, y0, w, strip_rows), max_depth=min(max_depth, 4), nee=nee,
                                 bounces=4)
        rays.append(r)
        hits.append(hh)
        bounce.append(b)
    rays, want, bounce = np.concatenate(rays), np.concatenate(hits), np.concatenate(bounce)
    assert int((bounce == 0).sum()) == 8 * strip_rows * w >= 200_000
    assert int((bounce > 0).sum()) > 20_000
    for ref_layout in (False, True):
        got = ctx.trace_closest(rays, reference_layout=ref_layout)
        assert np.array_equal(got["prim"], want["prim"])
        for f in ("t", "u", "v"):
            assert np.array_equal(got[f].view(np.uint32), want[f].view(np.uint32)), f
    return np.bincount(bounce)


def _check_rows(ctx, osc, cam, w, h, spp, depth, nee, rows=16):
    """8 strips of `rows` rows (the benchmark's oracle sample)."""
    got = ctx.render(cam, w, h, spp, max_depth=depth, nee=nee, outputs=("rgba",))["rgba"]
    for y0 in _strips(h, 8, rows):
        want = osc.render(cam, w, h, spp, rect=(0, y0, w, rows), max_depth=depth, nee=nee)["rgba"]
        assert np.array_equal(got[y0:y0 + rows].view(np.uint32), want.view(np.uint32)), f"rows {y0}..{y0 + rows - 1}"


@pytest.fixture(scope="module")
def icosphere_c1():
    import pyoracle as O
    sc = scenes.displaced_icosphere(seed=1234, level=8, width=1920, height=1080)
    osc = O.OracleScene(materials=sc["materials"], vertices=sc["vertices"], triangles=sc["triangles"], env=sc["env"])
    c = sc["camera"]
    cam = M.compute_camera(1920, 1080, c["look_from"], c["look_at"], c["vfov"], c["aperture"])
    with M.Context(0) as ctx:
        ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"], env=sc["env"])
        ctx.rebuild_bvh()                         # the benchmark's per-frame rebuild
        yield ctx, osc, cam


def test_displaced_icosphere_hits_bit_exact(icosphere_c1):
    ctx, osc, cam = icosphere_c1
    counts = _check_hits(ctx, osc, cam, 1920, 1080, 16, nee=False, max_depth=12)
    assert len(counts) == 4 and counts[3] > 0


def test_displaced_icosphere_frame_rows_bit_exact(icosphere_c1):
    ctx, osc, cam = icosphere_c1
    _check_rows(ctx, osc, cam, 1920, 1080, 16, 12, nee=False)


@pytest.fixture(scope="module")
def voxel_world_c2():
    import pyoracle as O
    w = scenes.voxel_world(1234)
    p = w["params"]
    env = M.gradient_env_map()
    c = w["camera"]
    cam = M.compute_camera(w["width"], w["height"], c["look_from"], c["look_at"], c["vfov"], 0.0)
    with M.Context(0) as ctx:
        ctx.world_generate(p)
        nv, nt = ctx.world_mesh(w["block_material"], greedy=False)
        v, t = ctx.world_read_mesh()
        ov, ot = O.world_mesh(O.world_generate(p), w["block_material"], greedy=False, chunk_x0=p["chunk_x0"],
                              chunk_z0=p["chunk_z0"])
        assert nt == len(ot) > 4_000_000
        assert np.array_equal(v.view(np.uint8), ov.view(np.uint8))
        assert np.array_equal(t.view(np.uint8), ot.view(np.uint8))
        ctx.upload_scene(materials=w["materials"], env=env, sun_dir=w["sun_dir"], sun_irradiance=w["sun_irradiance"],
                         world_mesh=True)
        osc = O.OracleScene(materials=w["materials"], vertices=v, triangles=t, env=env, sun_dir=w["sun_dir"],
                            sun_irradiance=w["sun_irradiance"])
        yield ctx, osc, cam, w


def test_voxel_world_hits_bit_exact(voxel_world_c2):
    ctx, osc, cam, w = voxel_world_c2
    counts = _check_hits(ctx, osc, cam, w["width"], w["height"], 24, nee=True, max_depth=w["max_depth"])
    assert len(counts) == 4


def test_voxel_world_frame_rows_bit_exact(voxel_world_c2):
    ctx, osc, cam, w = voxel_world_c2
    _check_rows(ctx, osc, cam, w["width"], w["height"], w["spp"], w["max_depth"], nee=True)


def test_shared_edge_rays_equal_brute_force():
    import pyoracle as O
    import test_oracle_kats as K
    sc = scenes.displaced_icosphere(seed=7, level=5, width=64, height=64)
    osc = O.OracleScene(materials=sc["materials"], vertices=sc["vertices"], triangles=sc["triangles"], env=sc["env"])
    rays = K.edge_aimed_rays(sc["vertices"], sc["triangles"], 100_000, seed=2)
    want = osc.trace(rays, brute_force=True)
    with M.Context(0) as ctx:
        ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"], env=sc["env"])
        for ref_layout in (False, True):
            assert ctx.trace_closest(rays, reference_layout=ref_layout).tobytes() == want.tobytes()
