"""GPU: batched multi-view rendering (every view equals its own single render,
bit for bit, and the oracle's render) and CUDA-graph replay of the passes (same
results as direct launches, re-captured when the configuration changes)."""
import numpy as np
import pytest

import mcrt_gb300 as M
from mcrt_gb300 import scenes

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def ico(ctx):
    sc = scenes.displaced_icosphere(seed=21, level=5, width=64, height=48)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"], env=sc["env"])
    return sc


def _views(sc, sizes):
    c = sc["camera"]
    out = []
    for k, (w, h) in enumerate(sizes):
        lf = np.asarray(c["look_from"], np.float32) + np.float32(0.3 * k)
        out.append((M.compute_camera(w, h, lf.tolist(), c["look_at"], c["vfov"] + 5 * k, 0.0), w, h))
    return out


@pytest.mark.parametrize("graph", [False, True])
def test_views_equal_single_renders(ctx, ico, graph):
    views = _views(ico, [(64, 48), (32, 32), (80, 20), (17, 13), (5, 7)])
    got = ctx.render_views(views, 6, first_frame=2, max_depth=12, spp_per_pass=2, graph=graph)
    for (cam, w, h), img in zip(views, got):
        want = ctx.render(cam, w, h, 6, first_frame=2, max_depth=12, outputs=("rgba",))["rgba"]
        assert np.array_equal(bits(img), bits(want))


def test_view_matches_oracle(ctx, oracle, ico):
    views = _views(ico, [(24, 16), (16, 20)])
    got = ctx.render_views(views, 3, max_depth=12, nee=True)
    osc = oracle.OracleScene(materials=ico["materials"], vertices=ico["vertices"], triangles=ico["triangles"],
                             env=ico["env"])
    for (cam, w, h), img in zip(views, got):
        want = osc.render(cam, w, h, 3, max_depth=12, nee=True)["rgba"]
        assert np.array_equal(bits(img), bits(want))


def test_graph_equals_direct_launches(ctx, ico):
    c = ico["camera"]
    cam = M.compute_camera(40, 30, c["look_from"], c["look_at"], c["vfov"], 0.0)
    for spp, per_pass in ((8, 2), (7, 3), (5, 5)):          # full passes, a remainder pass, one pass
        a = ctx.render(cam, 40, 30, spp, first_frame=9, max_depth=12, spp_per_pass=per_pass)
        b = ctx.render(cam, 40, 30, spp, first_frame=9, max_depth=12, spp_per_pass=per_pass, graph=True)
        assert np.array_equal(bits(a["rgba"]), bits(b["rgba"]))
        assert np.array_equal(a["sum"].view(np.uint64), b["sum"].view(np.uint64))
        assert np.array_equal(bits(a["gbuf"]), bits(b["gbuf"]))
    # continuing an accumulation, and a new camera (a new capture) with NEE
    ctx.render(cam, 40, 30, 4, max_depth=12, spp_per_pass=2)
    a = ctx.render(cam, 40, 30, 4, first_frame=4, max_depth=12, spp_per_pass=2, keep=True)
    ctx.render(cam, 40, 30, 4, max_depth=12, spp_per_pass=2, graph=True)
    b = ctx.render(cam, 40, 30, 4, first_frame=4, max_depth=12, spp_per_pass=2, keep=True, graph=True)
    assert np.array_equal(bits(a["rgba"]), bits(b["rgba"]))
    cam2 = M.compute_camera(40, 30, [0.0, 0.5, 3.0], c["look_at"], 50.0, 0.0)
    a = ctx.render(cam2, 40, 30, 4, max_depth=12, spp_per_pass=2, nee=True)
    b = ctx.render(cam2, 40, 30, 4, max_depth=12, spp_per_pass=2, nee=True, graph=True)
    assert np.array_equal(bits(a["rgba"]), bits(b["rgba"]))


def test_world_views_workload(ctx):
    """The batched workload's views over the voxel world: 16 seeded poses of
    uneven sizes between 256 x 256 and 1920 x 1080."""
    w = scenes.voxel_world()
    views = scenes.world_views(w, seed=1234)
    assert len(views) == 16
    sizes = [(v["width"], v["height"]) for v in views]
    assert all(256 <= a <= 1920 and 256 <= b <= 1080 for a, b in sizes)
    assert len(set(sizes)) == 16


@pytest.mark.parametrize("graph", [False, True])
def test_views_keep_accum_and_read_accum(ctx, ico, graph):
    """render_views in two calls with keep equals one call with all the samples
    (f64 sums from read_accum, running mean from the read-back), and each view's
    slice of the sums equals its own single render's sums."""
    views = _views(ico, [(40, 30), (23, 17), (9, 31)])
    whole = ctx.render_views(views, 8, first_frame=0, max_depth=8, nee=True, graph=graph)
    _, sum_whole = ctx.read_accum()
    ctx.render_views(views, 3, first_frame=0, max_depth=8, nee=True, graph=graph, read_back=False)
    split = ctx.render_views(views, 5, first_frame=3, max_depth=8, nee=True, graph=graph, keep=True)
    _, sum_split = ctx.read_accum()
    assert np.array_equal(sum_whole.view(np.uint64), sum_split.view(np.uint64))
    for a, b in zip(whole, split):
        assert np.array_equal(bits(a), bits(b))
    off = 0
    for cam, w, h in views:
        want = ctx.render(cam, w, h, 8, max_depth=8, nee=True, outputs=("sum",))["sum"].reshape(-1, 3)
        assert np.array_equal(sum_whole[0, off:off + w * h].view(np.uint64), want.view(np.uint64))
        off += w * h


def test_render_into_caller_buffer(ctx, ico):
    """render(out_rgba=...) fills a caller-owned (here pinned) array with the
    same image as the returned one; a wrong shape or dtype is refused."""
    torch = pytest.importorskip("torch")
    c = ico["camera"]
    cam = M.compute_camera(40, 24, c["look_from"], c["look_at"], c["vfov"], 0.0)
    want = ctx.render(cam, 40, 24, 4, max_depth=8, outputs=("rgba",))["rgba"]
    buf = torch.empty(24 * 40 * 4, dtype=torch.float32, pin_memory=True).numpy().reshape(24, 40, 4)
    ctx.render(cam, 40, 24, 4, max_depth=8, outputs=(), out_rgba=buf)
    assert np.array_equal(bits(buf), bits(want))
    with pytest.raises(TypeError):
        ctx.render(cam, 40, 24, 4, max_depth=8, outputs=(), out_rgba=np.zeros((24, 40, 3), np.float32))
