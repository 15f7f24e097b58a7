"""Scene ingestion on the device: OBJ text parsed by the CUDA kernels
(mcrt_mesh_append_obj) against the oracle's load_obj (mesh.rs:474-642), bit
for bit, on the edge-case corpus, seeded irregular files, hard decimals, the
error cases, transforms and whole YAML scenes (scene.rs:687-899), and at the
benchmark sizes: the displaced icosphere (1.31 M triangles) against the
oracle, the voxel world's face mesh against the device mesher's own records."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import obj_cases as C  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["direct", "copy"], autouse=True)
def text_path(request, monkeypatch):
    """Every test twice: the parser's first pass reading the host text in place
    (where the device reaches pageable memory) and a copy of it first."""
    if request.param == "copy":
        monkeypatch.setenv("MCRT_OBJ_COPY_TEXT", "1")
    else:
        monkeypatch.delenv("MCRT_OBJ_COPY_TEXT", raising=False)
    return request.param


def dev_load(ctx, text, mat=0, **xf):
    ctx.mesh_reset()
    nv, nt = ctx.mesh_append_obj(text, mat, **xf)
    v, t = ctx.mesh_read()
    assert (len(v), len(t)) == (nv, nt)
    return v, t


def same(a_v, a_t, b_v, b_t):
    return np.array_equal(C.canon(a_v), C.canon(b_v)) and np.array_equal(a_t.view(np.uint32), b_t.view(np.uint32))


@pytest.mark.parametrize("name", sorted(C.EDGE_CASES))
def test_edge_cases_match_oracle(ctx, oracle, name):
    text = C.EDGE_CASES[name]
    v_o, t_o = oracle.obj_load(text, 3)
    v_d, t_d = dev_load(ctx, text, 3)
    assert same(v_d, t_d, v_o, t_o)


@pytest.mark.parametrize("seed", range(48))
def test_random_files_match_oracle(ctx, oracle, mcrt, seed):
    text = C.random_obj(seed, n_lines=int(200 + 40 * seed))
    try:
        v_o, t_o = oracle.obj_load(text, 1)
    except oracle.ObjError as e:
        with pytest.raises(mcrt.MCRTError) as ed:
            dev_load(ctx, text, 1)
        assert str(ed.value).endswith(str(e))
        return
    v_d, t_d = dev_load(ctx, text, 1)
    assert same(v_d, t_d, v_o, t_o)


@pytest.mark.parametrize("chunk", range(4))
def test_mutated_files_match_oracle(ctx, oracle, mcrt, chunk):
    """Seeded near-valid files (obj_cases.mutated_obj, 50 per chunk): the
    device parse gives the oracle's records, or fails with its message."""
    for seed in range(50 * chunk, 50 * chunk + 50):
        text = C.mutated_obj(seed)
        try:
            v_o, t_o = oracle.obj_load(text, 2)
        except oracle.ObjError as e:
            with pytest.raises(mcrt.MCRTError) as ed:
                dev_load(ctx, text, 2)
            assert str(ed.value).endswith(str(e)), seed
            continue
        v_d, t_d = dev_load(ctx, text, 2)
        assert same(v_d, t_d, v_o, t_o), seed


@pytest.mark.parametrize("case", C.ERROR_CASES, ids=[c[0] for c in C.ERROR_CASES])
def test_errors_leave_the_mesh_unchanged(ctx, mcrt, case):
    name, text, msg = case
    ctx.mesh_reset()
    ctx.mesh_append_obj(C.EDGE_CASES["shared_normals"])
    before = ctx.mesh_read()
    with pytest.raises(mcrt.MCRTError) as e:
        ctx.mesh_append_obj(text, source="m.obj")
    sep = " " if msg.startswith("is not") else ": "
    assert str(e.value) == f"MESH_LOAD: mesh load error: failed to load mesh 'm.obj': 'm.obj'{sep}{msg}"
    after = ctx.mesh_read()
    assert same(*after, *before)


def test_decimals_are_correctly_rounded(ctx, oracle):
    """v lines of hard and random decimals, each referenced by a face (vertices
    exist only through faces); positions against exact rational rounding."""
    rng = np.random.default_rng(11)
    decs = list(C.HARD_DECIMALS)
    for _ in range(6000):
        nd = int(rng.integers(1, 45))
        digits = "".join(str(d) for d in rng.integers(0, 10, nd))
        point = int(rng.integers(0, nd + 1))
        s = ("-" if rng.random() < 0.3 else "") + digits[:point] + "." + digits[point:]
        if rng.random() < 0.7:
            s += f"e{int(rng.integers(-70, 45))}"
        decs.append(s)
    for k in range(200):                     # exact float32 midpoints and their neighbours
        b = int(rng.integers(1, 0x7F7FFFFF))
        lo = float(np.array(b, np.uint32).view(np.float32))
        hi = float(np.array(b + 1, np.uint32).view(np.float32))
        from fractions import Fraction
        mid = (Fraction(lo) + Fraction(hi)) / 2
        num, den = mid.numerator, mid.denominator
        if den == 1:
            decs.append(str(num))
        else:
            k2 = den.bit_length() - 1             # den = 2^k2: mid = num * 5^k2 / 10^k2
            s = str(num * 5 ** k2)
            decs.append(f"{s}e-{k2}")
    lines = [f"v {d} {d} {d}" for d in decs]
    lines += [f"f {i + 1} {i + 1} {i + 1}" for i in range(len(decs))]
    v, t = dev_load(ctx, "\n".join(lines).encode())
    got = v["position"][:, :3].view(np.uint32)
    for i, d in enumerate(decs):
        want = C.exact_f32_bits(d)
        for k in range(3):
            g = int(got[3 * i + k, 0])
            if want in (0x7FC00000, 0xFFC00000):
                assert (g & 0x7F800000) == 0x7F800000 and (g & 0x7FFFFF), d
            else:
                assert g == want, (d, hex(g), hex(want))


@pytest.mark.parametrize("xf", [dict(scale=2.5), dict(translate=[0.5, -0.25, 3.0]), dict(rotate=[30, -45, 90]),
                                dict(scale=0.125, rotate=[0, 0, 0], translate=[0, 0, 0]),
                                dict(scale=3.0, rotate=[12.5, 200, -33], translate=[-1, 2, 0.75])])
def test_transform_matches_host_loader(ctx, mcrt, tmp_path, xf):
    text = C.EDGE_CASES["mixed_has_norm_fan"] + b"v -0.0 -0 1\nf -1 1 2\n"
    p = tmp_path / "m.obj"
    p.write_bytes(text)
    parts = []
    if "translate" in xf:
        parts.append(f"translate: {list(xf['translate'])}")
    if "rotate" in xf:
        parts.append(f"rotate: {list(xf['rotate'])}")
    if "scale" in xf:
        parts.append(f"scale: {xf['scale']}")
    yaml = (f"objects:\n  - type: mesh\n    path: {p}\n    material: {{ type: lambertian }}\n"
            "    transform: { " + ", ".join(parts) + " }\n")
    host = mcrt.load_scene_yaml_str(yaml)
    v_d, t_d = dev_load(ctx, text, 0, **xf)
    assert np.array_equal(C.canon(v_d), C.canon(host.vertices))
    assert np.array_equal(t_d["v"], host.triangles["v"])


def test_non_positive_scale_is_rejected_after_parsing(ctx, mcrt):
    ctx.mesh_reset()
    with pytest.raises(mcrt.MCRTError) as e:
        ctx.mesh_append_obj(C.EDGE_CASES["shared_normals"], scale=0.0, source="m.obj")
    assert "transform.scale must be positive" in str(e.value)
    assert ctx.mesh_counts() == (0, 0)
    with pytest.raises(mcrt.MCRTError) as e:          # a load error is reported first, as the reference does
        ctx.mesh_append_obj(b"v 0 0 0\n", scale=-1.0, source="m.obj")
    assert "no geometry" in str(e.value)


SCENE = """
camera:
  look_from: [0.0, 1.5, 4.0]
  look_at: [0.0, 0.5, 0.0]
  vfov: 45.0
objects:
  - type: plane
    normal: [0.0, 1.0, 0.0]
    half_extents: [4.0, 4.0]
    material: {{ type: lambertian, albedo: [0.7, 0.7, 0.7] }}
  - type: mesh
    path: {a}
    material: {{ type: metal, albedo: [0.9, 0.8, 0.6], fuzz: 0.1 }}
    transform: {{ scale: 0.6, rotate: [0.0, 30.0, 0.0], translate: [-0.8, 0.6, 0.0] }}
  - type: box
    half_extents: [0.3, 0.3, 0.3]
    transform: {{ translate: [0.9, 0.3, 0.2], rotate: [0.0, 20.0, 0.0] }}
    material: {{ type: lambertian, albedo: [0.2, 0.4, 0.8] }}
  - type: mesh
    path: {b}
    material: {{ type: lambertian, albedo: [0.8, 0.3, 0.2] }}
    transform: {{ translate: [0.3, 0.0, -1.0] }}
  - type: sphere
    center: [0.0, 2.0, -1.0]
    radius: 0.4
    material: {{ type: emissive, albedo: [4.0, 4.0, 4.0] }}
"""


def test_scene_assembly_matches_host_and_renders_the_same(ctx, mcrt, tmp_path):
    from mcrt_gb300 import scenes
    a = tmp_path / "a.obj"
    b = tmp_path / "b.obj"
    a.write_bytes(scenes.displaced_icosphere_obj(5, 2))
    b.write_bytes(C.EDGE_CASES["no_normals_polygons"] + C.EDGE_CASES["uv_keys"])
    path = tmp_path / "s.yaml"
    path.write_text(SCENE.format(a=a, b=b))
    host = mcrt.load_scene_yaml(str(path))
    ctx.mesh_reset()
    dscene = ctx.mesh_append_scene_yaml(str(path))
    v_d, t_d = ctx.mesh_read()
    assert same(v_d, t_d, host.vertices, host.triangles)
    assert len(dscene.vertices) < len(host.vertices)          # primitives only on the host side
    env = mcrt.gradient_env_map()
    cam = mcrt.compute_camera(96, 64, host.camera["look_from"], host.camera["look_at"], host.camera["vfov"])
    ctx.upload_scene(materials=host.materials, spheres=host.spheres, env=env, device_mesh=True)
    img_d = ctx.render(cam, 96, 64, 8, max_depth=6)
    ctx.upload_scene(materials=host.materials, spheres=host.spheres, vertices=host.vertices,
                     triangles=host.triangles, env=env)
    img_h = ctx.render(cam, 96, 64, 8, max_depth=6)
    assert np.array_equal(img_d["sum"], img_h["sum"]) and np.array_equal(img_d["rgba"], img_h["rgba"])


def test_headless_parses_meshes_on_the_device(mcrt, tmp_path):
    a = tmp_path / "a.obj"
    b = tmp_path / "b.obj"
    a.write_bytes(C.EDGE_CASES["shared_normals"])
    b.write_bytes(C.EDGE_CASES["negative_indices"])
    path = tmp_path / "s.yaml"
    path.write_text(SCENE.format(a=a, b=b))
    out = tmp_path / "o.png"
    mcrt.headless_run(str(path), str(out), 48, 32, 2)
    assert out.stat().st_size > 100
    b.write_bytes(b"v 1 2 3\n")
    with pytest.raises(mcrt.MCRTError) as e:
        mcrt.headless_run(str(path), str(out), 48, 32, 2)
    assert str(e.value).endswith(f"failed to load mesh '{b}': '{b}': no geometry found after parsing")


def test_appends_concatenate_in_call_order(ctx, oracle):
    t1, t2 = C.EDGE_CASES["comments"], C.EDGE_CASES["uv_keys"]
    v1, r1 = oracle.obj_load(t1, 2)
    v2, r2 = oracle.obj_load(t2, 5)
    quad_v = np.zeros(4, v1.dtype)
    quad_v["position"][:, 3] = 1.0
    quad_v["position"][:, 0] = [0, 1, 1, 0]
    quad_t = np.zeros(2, r1.dtype)
    quad_t["v"] = [(0, 1, 2), (0, 2, 3)]
    ctx.mesh_reset()
    ctx.mesh_append_obj(t1, 2)
    ctx.mesh_append(quad_v, quad_t)
    ctx.mesh_append_obj(t2, 5)
    v, t = ctx.mesh_read()
    n1 = len(v1)
    want_v = np.concatenate([v1, quad_v, v2])
    qt = quad_t.copy()
    qt["v"] += n1
    r2s = r2.copy()
    r2s["v"] += n1 + 4
    want_t = np.concatenate([r1, qt, r2s])
    assert same(v, t, want_v, want_t)


def test_icosphere_level8_matches_oracle(ctx, oracle):
    """The displaced icosphere of the closest-hit benchmark (1,310,720
    triangles, 116 MB of OBJ text) parsed on the device, bit for bit."""
    from mcrt_gb300 import scenes
    text = scenes.displaced_icosphere_obj(1234, 8)
    v_o, t_o = oracle.obj_load(text, 0)
    v_d, t_d = dev_load(ctx, text, 0)
    assert (len(v_d), len(t_d)) == (655362, 1310720)
    assert same(v_d, t_d, v_o, t_o)


def test_text_at_every_alignment(ctx, oracle, mcrt):
    """The text starting at every offset within a 16-byte group of the caller's
    buffer (the in-place first pass reads whole aligned groups and keeps only
    the text's bytes), and ending at every offset too."""
    import ctypes
    from mcrt_gb300 import _native as N
    text = C.EDGE_CASES["mixed_has_norm_fan"] + C.EDGE_CASES["uv_keys"] + b"\n# \xc3\xa9\n"
    v_o, t_o = oracle.obj_load(text, 4)
    for shift in range(16):
        for tail in (0, 5):
            data = text[:len(text) - tail] if tail else text
            v_want, t_want = (v_o, t_o) if not tail else oracle.obj_load(data, 4)
            buf = ctypes.create_string_buffer(b"\n" * 16 + data + b"f 1 2 3\n" * 4, len(data) + 64)
            addr = ctypes.addressof(buf) + 16 + shift - (ctypes.addressof(buf) + 16) % 16
            ctypes.memmove(addr, data, len(data))
            ctx.mesh_reset()
            nv, nt = ctypes.c_uint32(), ctypes.c_uint32()
            N.check(N.lib().mcrt_mesh_append_obj(ctx._h, ctypes.cast(addr, ctypes.c_char_p), len(data), 4, None,
                                                 None, ctypes.byref(nv), ctypes.byref(nt)), ctx._h)
            v_d, t_d = ctx.mesh_read()
            assert same(v_d, t_d, v_want, t_want), (shift, tail)


def test_voxel_world_faces_round_trip(ctx, text_path):
    """The voxel world's face mesh (256 x 128 x 256, ~4.9 M triangles) written as
    OBJ and parsed on the device gives the mesher's own triangles: the same
    corner positions and normals in the same order (positions are multiples of
    1/8: exact in 6 decimals)."""
    if text_path == "copy":
        pytest.skip("the 667 MB text runs once, with the in-place first pass")
    from mcrt_gb300 import scenes
    w = scenes.voxel_world(1234)
    ctx.world_generate(w["params"])
    nv, nt = ctx.world_mesh(w["block_material"], greedy=False)
    wv, wt = ctx.world_read_mesh()
    text = scenes.world_mesh_obj(wv, wt)
    v_d, t_d = dev_load(ctx, text, 0)
    assert (len(v_d), len(t_d)) == (nv, nt)
    # vertices are numbered by first reference (the loader's cache), so compare triangle corners
    assert np.array_equal(v_d["position"][t_d["v"]], wv["position"][wt["v"]])
    assert np.array_equal(v_d["normal"][t_d["v"]][..., :3], wv["normal"][wt["v"]][..., :3])
