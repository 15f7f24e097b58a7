"""mcrt_render_noalloc — the render entry point for hosts that may not allocate
GPU memory while rendering (an engine or viewer with a fixed, pre-reserved
memory budget, where a mid-frame cudaMalloc would stall the device or fail).

Called through the C ABI with a caller-owned device output buffer, its image
must equal mcrt_render's bit for bit (the tolerance of the other render tests),
on two calls in a row: the second call reuses the same static scratch array and
must not see the first call's state.  This file is collected last so that a run
stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import mcrt_gb300 as M
from mcrt_gb300 import _native as N
from mcrt_gb300 import scenes

pytestmark = pytest.mark.gpu


def _noalloc(ctx, cam, w, h, spp, first, nee, out_ptr, spp_per_pass=0, flags=0):
    o = N.RenderOpts(max_depth=8, flags=(N.RENDER_NEE if nee else 0) | flags, spp_per_pass=spp_per_pass)
    return M.lib().mcrt_render_noalloc(ctx._h, N.ptr(cam), w, h, spp, first, ctypes.byref(o), ctypes.c_void_p(out_ptr))


def test_noalloc_render_matches_render_on_two_calls():
    torch = pytest.importorskip("torch")
    sc = scenes.cornell_box(1234)
    c = sc["camera"]
    w, h = 128, 96
    cam = M.compute_camera(w, h, c["look_from"], c["look_at"], c["vfov"], 0.0)
    with M.Context(0) as ctx:
        ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"],
                         env=M.gradient_env_map())
        out = torch.full((h * w * 4,), float("nan"), dtype=torch.float32, device="cuda")   # caller-owned output
        torch.cuda.synchronize()
        for first, spp, nee in [(0, 6, False), (6, 3, True)]:
            want = ctx.render(cam, w, h, spp, first_frame=first, max_depth=8, nee=nee, outputs=("rgba",))["rgba"]
            st = _noalloc(ctx, cam, w, h, spp, first, nee, out.data_ptr())
            M.check(st, ctx._h)
            got = out.cpu().numpy().reshape(h, w, 4)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_noalloc_rejects_images_beyond_the_static_limit():
    torch = pytest.importorskip("torch")
    sc = scenes.cornell_box(1234)
    c = sc["camera"]
    with M.Context(0) as ctx:
        ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"])
        out = torch.zeros(4, dtype=torch.float32, device="cuda")
        cam = M.compute_camera(600, 600, c["look_from"], c["look_at"], c["vfov"], 0.0)
        st = _noalloc(ctx, cam, 600, 600, 1, 0, False, out.data_ptr())
        assert st == -1
        assert b"262144" in M.lib().mcrt_last_error(ctx._h)


def test_noalloc_render_in_several_passes_at_the_pixel_limit():
    """512 x 512 (the pixel limit): the static scratch holds one sample per
    pixel at a time, so 3 samples take three passes, the later ones adding into
    the f64 sums the array keeps between passes."""
    torch = pytest.importorskip("torch")
    sc = scenes.cornell_box(1234)
    c = sc["camera"]
    w = h = 512
    cam = M.compute_camera(w, h, c["look_from"], c["look_at"], c["vfov"], 0.0)
    with M.Context(0) as ctx:
        ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"],
                         env=M.gradient_env_map())
        out = torch.full((h * w * 4,), float("nan"), dtype=torch.float32, device="cuda")
        for first, spp, nee in [(0, 3, True), (3, 2, False)]:
            want = ctx.render(cam, w, h, spp, first_frame=first, max_depth=8, nee=nee, spp_per_pass=1,
                              outputs=("rgba",))["rgba"]
            M.check(_noalloc(ctx, cam, w, h, spp, first, nee, out.data_ptr(), spp_per_pass=1), ctx._h)
            got = out.cpu().numpy().reshape(h, w, 4)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_noalloc_rejects_cache_and_gbuffer():
    torch = pytest.importorskip("torch")
    sc = scenes.cornell_box(1234)
    c = sc["camera"]
    with M.Context(0) as ctx:
        ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"])
        out = torch.zeros(16 * 16 * 4, dtype=torch.float32, device="cuda")
        cam = M.compute_camera(16, 16, c["look_from"], c["look_at"], c["vfov"], 0.0)
        for flag in (N.RENDER_CACHE, N.RENDER_GBUFFER):
            assert _noalloc(ctx, cam, 16, 16, 1, 0, False, out.data_ptr(), flags=flag) == -1
