"""Host side of libmcrt_cuda.so (no GPU needed): exported symbols, every
entry point's refusal of NULL arguments, the scene YAML API against the
reference's scene/camera/texture unit-test known answers, tone mapping and the
PNG writer."""
import ctypes
import math
import os
import re
import struct
import zlib

import numpy as np
import pytest

import mcrt_gb300 as M
from mcrt_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "mcrt_cuda.h")).read()
    names = set(re.findall(r"^(?:const\s+)?\w+\s*\*?\s*(mcrt_[a-z0-9_]+)\s*\(", hdr, re.MULTILINE))
    assert len(names) >= 20
    L = M.lib()
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    assert {n for n, _, _ in N.SIGNATURES} == names
    assert b"sm_103a" in L.mcrt_version()


_NULL_CALLS = r"""
import ctypes, sys
sys.path.insert(0, sys.argv[1])
from mcrt_gb300 import _native as N
L = N.lib()
for name, res, args in N.SIGNATURES:
    vals = []
    for t in args:
        if t in (ctypes.c_float, ctypes.c_double):
            vals.append(0.0)
        elif t in (ctypes.c_int, ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_size_t, ctypes.c_uint8):
            vals.append(0)
        else:
            vals.append(None)
    r = getattr(L, name)(*vals)
    print(name, r, flush=True)
"""


def test_every_entry_point_returns_a_status_on_null_arguments():
    """Every declared function called with NULL for each pointer (the context
    included) and 0 for each number, in one child process: each returns (a
    status, or nothing for the void ones) and none crashes.  Every status
    function refuses the call, except the tone maps of zero pixels."""
    import subprocess
    import sys
    r = subprocess.run([sys.executable, "-c", _NULL_CALLS, ROOT], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    got = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())
    assert set(got) == {n for n, _, _ in N.SIGNATURES}
    ok_with_nothing = {"mcrt_tonemap_rgba8", "mcrt_tonemap_aces_rgba8"}
    for name, res, _ in N.SIGNATURES:
        if res is ctypes.c_int and name not in ok_with_nothing:
            assert int(got[name]) < 0, (name, got[name])


def test_record_sizes_match_reference_layouts():                    # bvh.rs:649, mesh.rs:683-690, scene.rs:1194
    assert (M.SPHERE.itemsize, M.NODE.itemsize, M.VERTEX.itemsize, M.TRIANGLE.itemsize) == (32, 48, 48, 16)
    assert (M.MATERIAL.itemsize, M.MATERIAL_DATA.itemsize, M.CAMERA.itemsize) == (48, 3088, 112)


FIXTURE = """
camera:
  look_from: [4.0, 3.0, 8.0]
  look_at:   [0.0, 0.5, 0.0]
  vfov:      40.0
  aperture:  0.1

materials:
  ground: { type: lambertian, albedo: [0.5, 0.5, 0.5] }
  glass:  { type: dielectric, ior: 1.5 }
  metal:  { type: metal,      albedo: [0.8, 0.6, 0.2], fuzz: 0.1 }
  red:    { type: lambertian, albedo: [0.7, 0.1, 0.1] }
  blue:   { type: lambertian, albedo: [0.1, 0.1, 0.65] }
  light:  { type: emissive,   albedo: [1.0, 0.85, 0.7], emission_strength: 8.0 }

objects:
  - { type: sphere, center: [0.0, -100.0, 0.0], radius: 100.0, material: ground }
  - { type: sphere, center: [0.0,   2.5,  0.0], radius: 1.0,   material: glass  }
  - { type: sphere, center: [-4.0,  1.0,  0.0], radius: 1.0,   material: metal  }
  - { type: sphere, center: [4.0,   1.0,  0.0], radius: 1.0,   material: red    }
  - { type: sphere, center: [-2.0,  4.0,  0.0], radius: 0.5,   material: light  }
  - type: mesh
    path: {obj}
    material: blue
    transform:
      scale: 8.0
      translate: [0.5, -0.264, 0.0]
"""

OBJ = "\n".join(["# small closed mesh: an octahedron with normals on half the faces"] +
                [f"v {x} {y} {z}" for x, y, z in [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]] +
                ["vn 0 1 0", "vt 0.5 0.5",
                 "f 1//1 3//1 5//1", "f 3 2 5", "f 2/1 4/1 5/1", "f 4 1 5", "f 3 1 6", "f 2 3 6", "f 4 2 6 ",
                 "f 1 4 6"]) + "\n"


@pytest.fixture()
def fixture_scene(tmp_path):
    p = tmp_path / "octa.obj"
    p.write_text(OBJ)
    return M.load_scene_yaml_str(FIXTURE.replace("{obj}", str(p)), "<fixture>")


def test_yaml_scene_counts_centers_materials(fixture_scene):        # scene.rs:1227-1270
    s = fixture_scene
    assert len(s.spheres) == 5
    assert s.spheres["center_r"][0].tolist() == [0.0, -100.0, 0.0, 100.0]
    assert s.spheres["center_r"][1].tolist() == [0.0, 2.5, 0.0, 1.0]
    assert s.spheres["center_r"][2].tolist() == [-4.0, 1.0, 0.0, 1.0]
    assert s.spheres["center_r"][3].tolist() == [4.0, 1.0, 0.0, 1.0]
    assert int(s.materials["mat_count"]) == 6
    assert (s.spheres["mat_and_pad"][:, 0] < 6).all()
    assert (s.triangles["mat_idx"] & 0x7FFFFFFF < 6).all()           # scene.rs:1739-1758
    assert len(s.emissive_spheres) == 1 and int(s.materials["n_emissive"]) == 1
    assert s.material_names == ["ground", "glass", "metal", "red", "blue", "light"]


def test_yaml_scene_camera_is_loaded(fixture_scene):                # scene.rs:1373-1385
    c = fixture_scene.camera
    assert c["look_from"] == [4.0, 3.0, 8.0] and c["look_at"] == [0.0, 0.5, 0.0]
    assert abs(c["vfov"] - 40.0) < 1e-4 and abs(c["aperture"] - 0.1) < 1e-5


def test_obj_loader_and_transform(fixture_scene):                   # mesh.rs:474-642, scene.rs:829-879
    s = fixture_scene
    assert len(s.triangles) == 8
    # 3 faces with normals share vertices through the (pos, uv, normal) cache: f 1//1 3//1 5//1 and
    # f 2/1 4/1 5/1 make 6 distinct keys; the other 6 faces make 3 fresh vertices each
    assert len(s.vertices) == 6 + 6 * 3
    p = s.vertices["position"][:, :3]
    assert np.allclose(np.abs(p - [0.5, -0.264, 0.0]).max(axis=0), 8.0, atol=1e-5)
    n = s.vertices["normal"][:, :3]
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-5)


def test_emissive_tracking_and_gpu_type():                          # scene.rs:1273-1342
    s = M.load_scene_yaml_str("""
materials:
  wall:  { type: lambertian, albedo: [0.8, 0.8, 0.8] }
  light: { type: emissive,   albedo: [1.0, 0.85, 0.7], emission_strength: 8.0 }
objects:
  - { type: sphere, center: [0.0, -100.0, 0.0], radius: 100.0, material: wall  }
  - { type: sphere, center: [-2.0,   4.0,  0.0], radius: 0.5,   material: light }
""")
    assert len(s.emissive_spheres) == 1 and s.emissive_spheres["center_r"][0].tolist() == [-2.0, 4.0, 0.0, 0.5]
    s = M.load_scene_yaml_str("materials:\n  wall: { type: lambertian, albedo: [0.8, 0.8, 0.8] }\n"
                              "objects:\n  - { type: sphere, center: [0, 0, 0], radius: 1, material: wall }\n")
    assert len(s.emissive_spheres) == 0 and int(s.materials["n_emissive"]) == 0
    s = M.load_scene_yaml_str("materials:\n  sun: { type: emissive, albedo: [1.0, 0.9, 0.7], emission_strength: 10.0 }\n"
                              "objects:\n  - { type: sphere, center: [0, 5, 0], radius: 1.0, material: sun }\n")
    m = s.materials["materials"][0]
    assert int(s.materials["mat_count"]) == 1 and m["type_pad"][0] == N.MAT_EMISSIVE
    assert abs(m["albedo_fuzz"][0] - 1.0) < 1e-5 and abs(m["ior_pad"][0] - 10.0) < 1e-5


def test_inline_material_is_appended():                             # scene.rs:1344-1361
    s = M.load_scene_yaml_str("""
materials:
  base: { type: lambertian, albedo: [0.5, 0.5, 0.5] }
objects:
  - type: sphere
    center: [0, 0, 0]
    radius: 1
    material: { type: metal, albedo: [0.8, 0.6, 0.2], fuzz: 0.1 }
""")
    assert int(s.materials["mat_count"]) == 2 and s.material_names == ["base", "inline-1"]


def test_plane_tessellation():                                      # scene.rs:1387-1440
    s = M.load_scene_yaml_str("""
materials:
  floor: { type: lambertian, albedo: [0.5, 0.5, 0.5] }
objects:
  - type: plane
    normal: [0.0, 1.0, 0.0]
    half_extents: [1.0, 1.0]
    material: floor
    transform:
      translate: [0.0, 0.0, 0.0]
""")
    assert len(s.vertices) == 4 and len(s.triangles) == 2
    p = s.vertices["position"][:, :3]
    t = s.triangles["v"][0]
    gn = np.cross(p[t[1]] - p[t[0]], p[t[2]] - p[t[0]])
    gn /= np.linalg.norm(gn)
    assert abs(gn[1] - 1.0) < 1e-5
    assert np.allclose(s.vertices["normal"][:, 1], 1.0, atol=1e-5)


def test_plane_backface_flag():                                     # scene.rs:1463-1502
    s = M.load_scene_yaml_str("""
materials:
  wall: { type: lambertian, albedo: [0.7, 0.7, 0.7] }
objects:
  - type: plane
    normal: [0.0, 1.0, 0.0]
    half_extents: [1.0, 1.0]
    material: wall
    backface_culling: true
    transform:
      translate: [0.0, 0.0, 0.0]
  - type: plane
    normal: [0.0, -1.0, 0.0]
    half_extents: [1.0, 1.0]
    material: wall
    transform:
      translate: [0.0, 5.0, 0.0]
""")
    assert ((s.triangles["mat_idx"][:2] & 0x80000000) != 0).all()
    assert ((s.triangles["mat_idx"][2:] & 0x80000000) == 0).all()
    assert ((s.triangles["mat_idx"] & 0x7FFFFFFF) < int(s.materials["mat_count"])).all()


BOX = """
materials:
  m: {{ type: lambertian, albedo: [1.0, 1.0, 1.0] }}
objects:
  - type: box
    half_extents: [{hx}, {hy}, {hz}]
    material: m
{extra}
"""


def test_box_faces_normals_and_spans():                             # scene.rs:1504-1641
    s = M.load_scene_yaml_str(BOX.format(hx=0.5, hy=0.5, hz=0.5, extra="    transform:\n      translate: [0.0, 0.5, 0.0]"))
    assert len(s.vertices) == 24 and len(s.triangles) == 12
    s = M.load_scene_yaml_str(BOX.format(hx=1.0, hy=2.0, hz=3.0, extra=""))
    axes = np.array([(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)], np.float32)
    n = s.vertices["normal"][:, :3]
    assert all(np.min(np.abs(axes - v).max(axis=1)) < 1e-5 for v in n)
    p = s.vertices["position"][:, :3]
    expect = {(1, 0, 0): (0, 4, 6), (-1, 0, 0): (0, 4, 6), (0, 1, 0): (2, 0, 6), (0, -1, 0): (2, 0, 6),
              (0, 0, 1): (2, 4, 0), (0, 0, -1): (2, 4, 0)}
    for ax, span in expect.items():
        sel = np.abs(n - ax).max(axis=1) < 1e-5
        assert sel.sum() == 4
        got = p[sel].max(axis=0) - p[sel].min(axis=0)
        assert np.allclose(got, span, atol=1e-4)


def test_box_rotate_y_90():                                         # scene.rs:1643-1714
    s = M.load_scene_yaml_str(BOX.format(hx=1.0, hy=1.0, hz=1.0, extra="    transform:\n      rotate: [0, 90, 0]"))
    n = s.vertices["normal"][:, :3]
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-5)
    sel = np.abs(n[:, 2] + 1.0) < 1e-5
    assert sel.sum() == 4
    assert np.allclose(s.vertices["position"][sel, 2], -1.0, atol=1e-5)


def test_camera_focus_dist_defaults_to_eye_distance():              # scene.rs:1716-1737
    s = M.load_scene_yaml_str("""
camera:
  look_from: [0.0, 0.0, 5.0]
  look_at:   [0.0, 0.0, 0.0]
objects:
  - { type: sphere, center: [0, 0, 0], radius: 1, material: { type: lambertian } }
""")
    assert abs(s.camera["focus_dist"] - 5.0) < 1e-4 and s.camera["vfov"] == 60.0


def test_stub_geometry_and_errors(tmp_path):                        # scene.rs:598-609, :887-907
    s = M.load_scene_yaml_str("materials:\n  a: { type: lambertian }\nobjects:\n"
                              "  - { type: sphere, center: [0, 0, 0], radius: 1, material: a }\n")
    assert len(s.vertices) == 1 and s.vertices["position"][0, 0] == 1e9 and s.triangles["v"][0].tolist() == [0, 0, 0]
    with pytest.raises(M.MCRTError) as e:
        M.load_scene_yaml_str("objects:\n  - { type: sphere, center: [0, 0, 0], radius: 1, material: nope }\n")
    assert e.value.status == -9 and "nope" in str(e.value)
    with pytest.raises(M.MCRTError) as e:
        M.load_scene_yaml_str("objects: [ {type: sphere, center: [0, 0, 0] }")
    assert e.value.status == -7
    with pytest.raises(M.MCRTError) as e:
        M.load_scene_yaml_str("objects:\n  - { type: torus, material: { type: lambertian } }\n")
    assert e.value.status == -7
    many = "objects:\n" + "".join(f"  - {{ type: sphere, center: [{i}, 0, 0], radius: 1, material: {{ type: lambertian }} }}\n"
                                  for i in range(65))
    with pytest.raises(M.MCRTError) as e:
        M.load_scene_yaml_str(many)
    assert e.value.status == -11
    with pytest.raises(M.MCRTError) as e:
        M.load_scene_yaml(str(tmp_path / "missing.yaml"))
    assert e.value.status == -8
    with pytest.raises(M.MCRTError) as e:
        M.load_scene_yaml_str("objects:\n  - type: mesh\n    path: /nonexistent.obj\n    material: { type: lambertian }\n")
    assert e.value.status == -10
    with pytest.raises(M.MCRTError) as e:
        M.load_scene_yaml_str("materials:\n  a: { type: lambertian }\n  a: { type: metal }\n")
    assert e.value.status == -7


# ---------------------------------------------------------------- camera.rs
def test_camera_kats():                                             # camera.rs:137-221
    c = M.compute_camera(800, 600, (0, 0, 3), (0, 0, 0), 60.0, 0.0, 3.0)
    assert c["defocus_u"].tolist() == [0, 0, 0, 0] and c["defocus_v"].tolist() == [0, 0, 0, 0]
    assert int(c["frame_count"]) == 0
    c = M.compute_camera(800, 600, (1, 2, 3), (0, 0, 0), 60.0, 0.0, 3.0)
    assert np.allclose(c["origin"][:3], [1, 2, 3], atol=1e-5)
    c = M.compute_camera(800, 600, (0, 5, 0), (0, 0, 0), 60.0, 0.0, 5.0)   # gimbal lock
    assert not np.isnan(np.frombuffer(c.tobytes()[:96], np.float32)).any()
    c = M.compute_camera(800, 600, (0, 0, 3), (0, 0, 0), 60.0, 0.5, 3.0)
    assert np.linalg.norm(c["defocus_u"][:3]) > 1e-5 and np.linalg.norm(c["defocus_v"][:3]) > 1e-5


def test_camera_basis_geometry():
    c = M.compute_camera(400, 200, (0, 0, 4), (0, 0, 0), 90.0, 0.0, 4.0)
    # focal plane through the look-at point: centre of the screen = look_at
    centre = c["lower_left"][:3] + 0.5 * c["horizontal"][:3] + 0.5 * c["vertical"][:3]
    assert np.allclose(centre, [0, 0, 0], atol=1e-5)
    assert np.allclose(c["vertical"][:3], [0, 8.0, 0], atol=1e-4)          # 2 * tan(45) * 4
    assert np.allclose(c["horizontal"][:3], [16.0, 0, 0], atol=1e-4)


# ---------------------------------------------------------------- texture.rs
def test_gradient_env_map_kats():                                   # texture.rs:316-351
    e = M.gradient_env_map()
    assert e.shape == (512, 1024, 4) and np.isfinite(e).all() and (e >= 0).all()
    lum = lambda p: 0.2126 * p[0] + 0.7152 * p[1] + 0.0722 * p[2]
    assert lum(e[0, 0]) > lum(e[-1, 0])
    assert np.array_equal(M.load_env_map(None), e)          # fallback chain ends at the gradient


# ---------------------------------------------------------------- tone map + PNG
def test_tonemap_kats_and_oracle_agreement(oracle):
    x = np.zeros((1, 6, 4), np.float32)
    x[0, :, 0] = [0.0, 1.0, -1.0, np.inf, np.nan, 1e30]
    t = M.tonemap_rgba8(x)
    assert t[0, :, 0].tolist()[:3] == [0, 186, 0]            # 0.5 ** (1/2.2) * 255 + 0.5 = 186.6
    assert t[0, 3, 0] == 0 and t[0, 4, 0] == 0 and t[0, 5, 0] == 255 and (t[..., 3] == 255).all()
    r = np.random.default_rng(1).exponential(1.0, (64, 64, 4)).astype(np.float32)
    assert np.array_equal(M.tonemap_rgba8(r), oracle.tonemap_rgba8(r))


def test_png_writer_roundtrip(tmp_path):
    img = (np.random.default_rng(2).integers(0, 256, (37, 53, 4))).astype(np.uint8)
    p = str(tmp_path / "out.png")
    M.write_png(p, img)
    data = open(p, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        assert zlib.crc32(typ + body) == struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if typ == b"IHDR":
            assert struct.unpack(">II", body[:8]) == (53, 37)
        if typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(37, 1 + 53 * 4)
    assert (raw[:, 0] == 0).all() and np.array_equal(raw[:, 1:].reshape(37, 53, 4), img)


def test_aces_tonemap_matches_oracle(oracle):                       # gpu.rs:1904-1939
    r = np.random.default_rng(5).exponential(2.0, (40, 30, 4)).astype(np.float32)
    r[0, 0, :3] = [np.nan, np.inf, -1.0]
    assert np.array_equal(M.tonemap_aces_rgba8(r), oracle.tonemap_aces_rgba8(r))
    z = np.zeros((1, 1, 4), np.float32)
    assert M.tonemap_aces_rgba8(z)[0, 0].tolist() == [0, 0, 0, 255]


def test_hdr_writer_roundtrip_and_sky_fixture(tmp_path):
    """The RGBE writer encodes as the reference's sky generator; the reader decodes
    the generator's own file (tests/golden/test_sky_128x64.hdr) to within RGBE
    precision of the float image it was made from."""
    img = np.random.default_rng(6).exponential(3.0, (512, 1024, 4)).astype(np.float32)
    p = str(tmp_path / "x.hdr")
    M.write_hdr(p, img)
    back = M.load_env_map(p)                                  # 1024x512: no resize
    rel = np.abs(back[..., :3] - img[..., :3]) / img[..., :3].max(axis=-1, keepdims=True)
    assert rel.max() < 1.0 / 128 and (back[..., 3] == 1.0).all()
    here = os.path.dirname(os.path.abspath(__file__))
    sky = np.load(os.path.join(here, "golden", "test_sky_128x64.npy"))
    env = M.load_env_map(os.path.join(here, "golden", "test_sky_128x64.hdr"))
    src = env[::8, ::8, :3]                                    # nearest 8x upsample of 128x64
    ref = sky.astype(np.float64)
    tol = ref.max(axis=-1, keepdims=True) / 128 + 1e-30
    assert (np.abs(src - ref) <= tol).all()
