"""GPU: the voxel-world generator and the chunk mesher bit-exact against the
oracle (including the reference mesher's own test cases), the world mesh
rendered with the directional light bit-exact, and the denoiser's extension
terms bit-exact."""
import numpy as np
import pytest

import mcrt_gb300 as M
from mcrt_gb300 import scenes

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_world_generate_bit_exact(ctx, oracle):
    for p in (scenes.world_params(seed=5, nx=32, ny=64, nz=48), scenes.world_params()):
        got = ctx.world_generate(p, read_back=True)
        assert np.array_equal(got, oracle.world_generate(p))


@pytest.mark.parametrize("greedy", [True, False])
def test_world_mesh_bit_exact(ctx, oracle, greedy):
    w = scenes.voxel_world(seed=9, nx=128, ny=96, nz=96)
    p = w["params"]
    ctx.world_generate(p)
    nv, nt = ctx.world_mesh(w["block_material"], greedy=greedy)
    v, t = ctx.world_read_mesh()
    ov, ot = oracle.world_mesh(oracle.world_generate(p), w["block_material"], greedy=greedy,
                               chunk_x0=p["chunk_x0"], chunk_z0=p["chunk_z0"])
    assert (nv, nt) == (len(ov), len(ot)) and nt > 0
    assert np.array_equal(v.view(np.uint8), ov.view(np.uint8))
    assert np.array_equal(t.view(np.uint8), ot.view(np.uint8))


def test_reference_mesher_cases(ctx, oracle):
    """The voxel sets of the reference's mesher tests (world/mesher.rs:430-491) and
    a random chunk pair, uploaded as grids and meshed on the GPU."""
    rng = np.random.default_rng(4)
    cases = []
    c = np.zeros((16, 256, 16), np.uint8)
    cases.append(c.copy())
    c[8, 8, 8] = 1
    cases.append(c.copy())
    c = np.zeros((16, 256, 16), np.uint8)
    c[0:2, 0, 0:2] = 1
    cases.append(c)
    c = np.zeros((16, 256, 16), np.uint8)
    c[0, 0, 0] = c[1, 0, 0] = 1
    cases.append(c)
    cases.append(rng.choice(np.array([0, 0, 1, 2, 9, 11], np.uint8), size=(32, 40, 16)))
    mm = np.arange(256, dtype=np.uint32) % 7
    for vox in cases:
        for greedy in (True, False):
            ctx.world_upload(vox, chunk_x0=-1, chunk_z0=2)
            ctx.world_mesh(mm, greedy=greedy)
            v, t = ctx.world_read_mesh()
            ov, ot = oracle.world_mesh(vox, mm, greedy=greedy, chunk_x0=-1, chunk_z0=2)
            assert np.array_equal(v.view(np.uint8), ov.view(np.uint8))
            assert np.array_equal(t.view(np.uint8), ot.view(np.uint8))
    ctx.world_upload(cases[1])
    assert ctx.world_mesh(mm, greedy=True) == (24, 12)


def _world_scene(ctx, seed=3, n=48):
    w = scenes.voxel_world(seed=seed, nx=n, ny=n, nz=n)
    ctx.world_generate(w["params"])
    ctx.world_mesh(w["block_material"], greedy=True)
    return w


def test_world_render_with_sun_bit_exact(ctx, oracle):
    w = _world_scene(ctx)
    env = M.gradient_env_map()
    ctx.upload_scene(materials=w["materials"], env=env, sun_dir=w["sun_dir"], sun_irradiance=w["sun_irradiance"],
                     world_mesh=True)
    c = w["camera"]
    cam = M.compute_camera(64, 40, c["look_from"], c["look_at"], c["vfov"], 0.0)
    r = ctx.render(cam, 64, 40, 3, max_depth=6, nee=True)
    v, t = ctx.world_read_mesh()
    o = oracle.OracleScene(materials=w["materials"], vertices=v, triangles=t, env=env, sun_dir=w["sun_dir"],
                           sun_irradiance=w["sun_irradiance"]).render(cam, 64, 40, 3, max_depth=6, nee=True)
    assert np.array_equal(bits(r["rgba"]), bits(o["rgba"]))
    assert np.array_equal(r["sum"].view(np.uint64), o["sum"].view(np.uint64))
    assert np.array_equal(bits(r["gbuf"]), bits(o["gbuf"]))
    # the sun contributes: the same render without it is darker
    ctx.upload_scene(materials=w["materials"], env=env, world_mesh=True)
    dark = ctx.render(cam, 64, 40, 3, max_depth=6, nee=True)["sum"].sum()
    assert dark < r["sum"].sum()


def test_sun_and_area_lights_bit_exact(ctx, oracle):
    """With both kinds of light, next-event estimation picks each with probability 1/2."""
    from test_gpu_regression import SCENE_YAML
    s = M.load_scene_yaml_str(SCENE_YAML.format(), "<textured>")
    c = s.camera
    cam = M.compute_camera(48, 32, c["look_from"], c["look_at"], c["vfov"], c["aperture"], c["focus_dist"])
    env = M.gradient_env_map()
    sun = dict(sun_dir=[-0.3, 1.0, 0.5], sun_irradiance=[2.0, 1.8, 1.5])
    ctx.upload_scene(spheres=s.spheres, vertices=s.vertices, triangles=s.triangles, materials=s.materials, env=env,
                     **sun)
    r = ctx.render(cam, 48, 32, 4, max_depth=8, nee=True)
    o = oracle.OracleScene(materials=s.materials, spheres=s.spheres, vertices=s.vertices, triangles=s.triangles,
                           env=env, **sun).render(cam, 48, 32, 4, max_depth=8, nee=True)
    assert np.array_equal(bits(r["rgba"]), bits(o["rgba"]))


def test_denoise_extension_terms_bit_exact(ctx, oracle):
    """The workload's 5 x 5 filter with sigma_color 0.1 and sigma_normal 0.2, on
    the device accumulation and on host images, against the oracle."""
    w = _world_scene(ctx, seed=11)
    ctx.upload_scene(materials=w["materials"], env=M.gradient_env_map(), sun_dir=w["sun_dir"],
                     sun_irradiance=w["sun_irradiance"], world_mesh=True)
    c = w["camera"]
    cam = M.compute_camera(96, 64, c["look_from"], c["look_at"], c["vfov"], 0.0)
    r = ctx.render(cam, 96, 64, 2, max_depth=6, nee=True)
    d = w["denoise"]
    got = ctx.denoise_accum(**d)
    want = oracle.denoise(r["rgba"], r["gbuf"], **d)
    assert np.array_equal(bits(got), bits(want))
    for radius, sc, sn in ((2, 0.1, 0.2), (7, 0.05, 0.0), (11, 0.0, 0.3)):
        got = ctx.denoise(r["rgba"], r["gbuf"], radius=radius, sigma_color=sc, sigma_normal=sn)
        want = oracle.denoise(r["rgba"], r["gbuf"], radius=radius, sigma_color=sc, sigma_normal=sn)
        assert np.array_equal(bits(got), bits(want))


def test_world_invalid_inputs(ctx):
    with pytest.raises(M.MCRTError):
        ctx.world_generate(dict(scenes.world_params(), nx=20))
    with pytest.raises(M.MCRTError):
        ctx.world_upload(np.zeros((16, 1, 16), np.uint8))
    ctx.world_upload(np.zeros((16, 8, 16), np.uint8))
    with pytest.raises(M.MCRTError):
        ctx.upload_scene(materials=scenes.voxel_world()["materials"], world_mesh=True)   # not meshed yet
