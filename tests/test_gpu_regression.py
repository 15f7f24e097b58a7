"""The reference's image-regression harness (tests/regression_tests.rs,
src/regression.rs) run against the CPU oracle, the headless command line, and
parity of the extensions the harness scenes do not reach (textures, GGX,
dielectric meshes under an HDR environment)."""
import os
import struct
import subprocess
import zlib

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


def read_png(path):
    data = open(path, "rb").read()
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    assert (raw[:, 0] == 0).all()
    return raw[:, 1:].reshape(h, w, 4)


@pytest.mark.parametrize("name", SCENES)
def test_regression_harness_against_oracle(ctx, oracle, name):
    """regression_suite (regression_tests.rs:211-428): render each scene at its
    sidecar [render] size and spp, tone-map, compare_images with the sidecar
    [regression] thresholds (fail when mse > threshold_mse or psnr < threshold_psnr)."""
    s = load_fixture_scene(name)
    w, h, spp = s["width"], s["height"], s["spp"]
    env = env_for(name)
    ctx.upload_scene(spheres=s["spheres"], vertices=s["vertices"], triangles=s["triangles"], materials=s["materials"],
                     env=env)
    got = M.tonemap_rgba8(ctx.render(s["camera"], w, h, spp, outputs=("rgba",))["rgba"])
    osc = oracle.OracleScene(materials=s["materials"], spheres=s["spheres"], vertices=s["vertices"],
                             triangles=s["triangles"], env=env)
    base = oracle.tonemap_rgba8(osc.render(s["camera"], w, h, spp)["rgba"])
    mse, psnr, mx = oracle.compare_images(got, base)
    assert mse <= s["threshold_mse"] and (psnr == float("inf") or psnr >= s["threshold_psnr"])
    assert mse == 0.0                                  # and in fact byte-identical


SCENE_YAML = """
camera:
  look_from: [0.0, 2.0, 6.0]
  look_at:   [0.0, 0.8, 0.0]
  vfov:      45.0
materials:
  floor:  {{ type: lambertian, albedo: [0.9, 0.9, 0.9], texture_layer: 1 }}
  ball:   {{ type: lambertian, albedo: [1.0, 1.0, 1.0], texture_layer: 2 }}
  chrome: {{ type: metal, albedo: [0.9, 0.9, 0.9], fuzz: 0.2, texture_layer: 3 }}
  gold:   {{ type: ggx, albedo: [1.0, 0.78, 0.34], roughness: 0.3 }}
  glass:  {{ type: dielectric, ior: 1.5 }}
  lamp:   {{ type: emissive, albedo: [1.0, 0.9, 0.8], emission_strength: 20.0 }}
objects:
  - type: plane
    normal: [0.0, 1.0, 0.0]
    half_extents: [4, 4]
    material: floor
    backface_culling: true
  - {{ type: sphere, center: [-1.2, 0.7, 0.0], radius: 0.7, material: ball }}
  - {{ type: sphere, center: [1.2, 0.7, 0.0], radius: 0.7, material: chrome }}
  - {{ type: sphere, center: [0.0, 0.5, 1.2], radius: 0.5, material: glass }}
  - type: box
    half_extents: [0.4, 0.4, 0.4]
    material: gold
    transform:
      translate: [0.0, 0.4, -1.2]
      rotate: [0.0, 30.0, 0.0]
  - {{ type: sphere, center: [0.0, 4.0, 0.0], radius: 0.5, material: lamp }}
"""


def test_textures_and_ggx_bit_exact(ctx, oracle):
    s = M.load_scene_yaml_str(SCENE_YAML.format(), "<textured>")
    c = s.camera
    cam = M.compute_camera(96, 64, c["look_from"], c["look_at"], c["vfov"], c["aperture"], c["focus_dist"])
    env = M.gradient_env_map()
    ctx.upload_scene(spheres=s.spheres, vertices=s.vertices, triangles=s.triangles, materials=s.materials, env=env)
    r = ctx.render(cam, 96, 64, 6, max_depth=8)
    osc = oracle.OracleScene(materials=s.materials, spheres=s.spheres, vertices=s.vertices, triangles=s.triangles,
                             env=env)
    o = osc.render(cam, 96, 64, 6, max_depth=8)
    assert np.array_equal(bits(r["rgba"]), bits(o["rgba"]))
    assert np.array_equal(r["sum"].view(np.uint64), o["sum"].view(np.uint64))


def test_displaced_icosphere_bit_exact(ctx, oracle):
    from mcrt_gb300 import scenes
    sc = scenes.displaced_icosphere(seed=1234, level=6, width=80, height=48)
    c = sc["camera"]
    cam = M.compute_camera(80, 48, c["look_from"], c["look_at"], c["vfov"], 0.0)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"], env=sc["env"])
    r = ctx.render(cam, 80, 48, 4, max_depth=12)
    osc = oracle.OracleScene(materials=sc["materials"], vertices=sc["vertices"], triangles=sc["triangles"],
                             env=sc["env"])
    o = osc.render(cam, 80, 48, 4, max_depth=12)
    assert np.array_equal(bits(r["rgba"]), bits(o["rgba"]))


def test_headless_cli_matches_oracle(tmp_path, oracle):
    """mcrt_headless --headless scene --output png (main.rs:62-80) with a sidecar
    [render] table (headless.rs:46-77): the PNG equals the oracle's tone-mapped image."""
    scene = tmp_path / "cli_scene.yaml"
    scene.write_text(SCENE_YAML.format())
    (tmp_path / "cli_scene.test.toml").write_text("[render]\nwidth = 40\nheight = 30\nspp = 3\n")
    out = tmp_path / "out" / "img.png"
    cli = os.path.join(os.path.dirname(M.__file__), "mcrt_headless")
    p = subprocess.run([cli, "--headless", str(scene), "--output", str(out)], capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 0, p.stderr
    img = read_png(str(out))
    assert img.shape == (30, 40, 4)
    s = M.load_scene_yaml(str(scene))
    c = s.camera
    cam = M.compute_camera(40, 30, c["look_from"], c["look_at"], c["vfov"], c["aperture"], c["focus_dist"])
    osc = oracle.OracleScene(materials=s.materials, spheres=s.spheres, vertices=s.vertices, triangles=s.triangles,
                             env=M.gradient_env_map())
    want = oracle.tonemap_rgba8(osc.render(cam, 40, 30, 3)["rgba"])
    assert np.array_equal(img, want)
    # failure path: exit code 1 and a message (main.rs:75-78)
    p = subprocess.run([cli, "--headless", str(tmp_path / "missing.yaml"), "--output", str(out)],
                       capture_output=True, text=True, timeout=60)
    assert p.returncode == 1 and "headless render failed" in p.stderr


@pytest.mark.parametrize("variant", [1, 6])   # compact binary BVH, quantised 4-wide BVH (kernel variants 0, 5)
def test_bvh_layouts_bit_exact_against_oracle(ctx, oracle, variant):
    import ctypes
    from mcrt_gb300 import scenes
    sc = scenes.displaced_icosphere(seed=77, level=7, width=96, height=64)
    c = sc["camera"]
    cam = M.compute_camera(96, 64, c["look_from"], c["look_at"], c["vfov"], 0.0)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"], env=sc["env"])
    o = M._native.RenderOpts(max_depth=12, variant=variant)
    rgba = np.zeros((64, 96, 4), np.float32)
    M.check(M.lib().mcrt_render(ctx._h, M._native.ptr(cam), 96, 64, 4, 0, ctypes.byref(o), M._native.ptr(rgba),
                                None, None), ctx._h)
    osc = oracle.OracleScene(materials=sc["materials"], vertices=sc["vertices"], triangles=sc["triangles"],
                             env=sc["env"])
    want = osc.render(cam, 96, 64, 4, max_depth=12)["rgba"]
    assert np.array_equal(bits(rgba), bits(want))


def test_autotuned_variants_are_bit_identical(ctx):
    from mcrt_gb300 import scenes
    sc = scenes.displaced_icosphere(seed=3, level=5, width=64, height=48)
    c = sc["camera"]
    cam = M.compute_camera(64, 48, c["look_from"], c["look_at"], c["vfov"], 0.0)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"], env=sc["env"])
    v, ms = ctx.autotune(cam, 64, 48, 2, max_depth=12)
    assert 0 <= v < len(ms) and len(ms) == 8 and ms[v] > 0
    assert {M.variant_info(k)["width"] for k in range(8)} == {2, 4}
    imgs = []
    for k in [k for k in range(len(ms)) if ms[k] > 0]:
        o = M._native.RenderOpts(max_depth=12, variant=k + 1)
        rgba = np.zeros((48, 64, 4), np.float32)
        import ctypes
        M.check(M.lib().mcrt_render(ctx._h, M._native.ptr(cam), 64, 48, 3, 0, ctypes.byref(o), M._native.ptr(rgba),
                                    None, None), ctx._h)
        imgs.append(rgba)
    for im in imgs[1:]:
        assert np.array_equal(bits(im), bits(imgs[0]))


def test_device_tonemaps_match_host(ctx, oracle):
    """mcrt_read_image_rgba8: Reinhard + gamma 2.2 and ACES + sRGB on the GPU equal
    the host restatements applied to the read-back running mean."""
    s = load_fixture_scene("cornell_box_mini")
    ctx.upload_scene(spheres=s["spheres"], vertices=s["vertices"], triangles=s["triangles"], materials=s["materials"],
                     env=M.gradient_env_map())
    cam = M.compute_camera(64, 48, [0.0, 4.75, 8.0], [0.0, 4.0, 0.0], 60.0, 0.0)
    rgba = ctx.render(cam, 64, 48, 4, outputs=("rgba",))["rgba"]
    assert np.array_equal(ctx.image_rgba8(aces=False), oracle.tonemap_rgba8(rgba))
    assert np.array_equal(ctx.image_rgba8(aces=True), oracle.tonemap_aces_rgba8(rgba))
