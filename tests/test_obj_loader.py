"""The OBJ loader, load_obj (mesh.rs:474-642), on the CPU: the oracle's
str::parse::<f32> against exact rational rounding, and the library's host
loader (the scene YAML API's mesh objects, scene.rs:829-879) bit for bit
against the oracle on the edge-case corpus and on seeded irregular files."""
import ctypes
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import obj_cases as C  # noqa: E402

import mcrt_gb300 as M  # noqa: E402
from mcrt_gb300 import _native as N  # noqa: E402


def f32_bits(x):
    return int(np.array(x, np.float32).view(np.uint32))


def test_oracle_f32_parse_is_correctly_rounded(oracle):
    for s in C.HARD_DECIMALS:
        assert f32_bits(oracle.parse_f32(s.encode())) == C.exact_f32_bits(s), s
    rng = np.random.default_rng(7)
    for _ in range(2000):
        nd = int(rng.integers(1, 40))
        digits = "".join(str(d) for d in rng.integers(0, 10, nd))
        point = int(rng.integers(0, nd + 1))
        s = digits[:point] + "." + digits[point:] + f"e{int(rng.integers(-60, 45))}"
        if s.startswith(".") and point == nd:
            continue
        assert f32_bits(oracle.parse_f32(s.encode())) == C.exact_f32_bits(s), s


def test_oracle_f32_syntax(oracle):
    for bad in [b"", b".", b"e5", b"1e", b"1e+", b"--1", b"1.5f", b"0x10", b"1_0", b"nan(1)", b"infin", b" 1", b"1 "]:
        assert oracle.parse_f32(bad) is None, bad
        assert C.exact_f32_bits(bad.decode()) is None, bad
    for good in [b"1.", b".5", b"+.5", b"-0", b"INF", b"-Infinity", b"NaN", b"1E5", b"1e05"]:
        assert oracle.parse_f32(good) is not None, good


def host_load(tmp_path, text, name="m.obj"):
    p = tmp_path / name
    p.write_bytes(text)
    s = M.load_scene_yaml_str(f"objects:\n  - type: mesh\n    path: {p}\n    material: {{ type: lambertian }}\n")
    return s.vertices, s.triangles


@pytest.mark.parametrize("name", sorted(C.EDGE_CASES))
def test_host_loader_matches_oracle_edge_cases(oracle, tmp_path, name):
    text = C.EDGE_CASES[name]
    v_o, t_o = oracle.obj_load(text, 0)
    v_h, t_h = host_load(tmp_path, text)
    assert np.array_equal(C.canon(v_h), C.canon(v_o))
    assert np.array_equal(t_h.view(np.uint32), t_o.view(np.uint32))


@pytest.mark.parametrize("seed", range(12))
def test_host_loader_matches_oracle_random_files(oracle, tmp_path, seed):
    text = C.random_obj(seed)
    try:
        v_o, t_o = oracle.obj_load(text, 0)
    except oracle.ObjError:
        with pytest.raises(N.MCRTError):
            host_load(tmp_path, text)
        return
    v_h, t_h = host_load(tmp_path, text)
    assert np.array_equal(C.canon(v_h), C.canon(v_o))
    assert np.array_equal(t_h.view(np.uint32), t_o.view(np.uint32))


@pytest.mark.parametrize("chunk", range(4))
def test_host_loader_matches_oracle_mutated_files(oracle, tmp_path, chunk):
    """Seeded near-valid files (obj_cases.mutated_obj, 50 per chunk): the
    host loader gives the oracle's records, or fails with its message."""
    for seed in range(50 * chunk, 50 * chunk + 50):
        text = C.mutated_obj(seed)
        try:
            v_o, t_o = oracle.obj_load(text, 0)
        except oracle.ObjError as e:
            with pytest.raises(N.MCRTError) as eh:
                host_load(tmp_path, text)
            assert str(eh.value).endswith(str(e)), seed
            continue
        v_h, t_h = host_load(tmp_path, text)
        assert np.array_equal(C.canon(v_h), C.canon(v_o)), seed
        assert np.array_equal(t_h.view(np.uint32), t_o.view(np.uint32)), seed


@pytest.mark.parametrize("case", C.ERROR_CASES, ids=[c[0] for c in C.ERROR_CASES])
def test_host_loader_error_messages(oracle, tmp_path, case):
    name, text, msg = case
    with pytest.raises(oracle.ObjError) as eo:
        oracle.obj_load(text, 0)
    assert str(eo.value) == msg
    with pytest.raises(N.MCRTError) as eh:
        host_load(tmp_path, text, "bad.obj")
    p = str(tmp_path / "bad.obj")
    sep = " " if msg.startswith("is not") else ": "
    assert str(eh.value).endswith(f"failed to load mesh '{p}': '{p}'{sep}{msg}")
    assert eh.value.status == -10                                  # MCRT_ERR_MESH_LOAD


def test_deferred_load_keeps_primitives_only(tmp_path):
    p = tmp_path / "m.obj"
    p.write_bytes(C.EDGE_CASES["shared_normals"])
    yaml = (f"objects:\n  - type: plane\n    normal: [0, 1, 0]\n    half_extents: [1, 1]\n    material: {{ type: lambertian }}\n"
            f"  - type: mesh\n    path: {p}\n    material: {{ type: lambertian }}\n")
    h = ctypes.c_void_p()
    N.check(N.lib().mcrt_scene_load_yaml_str_ex(yaml.encode(), b"<t>", N.LOAD_DEFER_MESHES, ctypes.byref(h)))
    try:
        s = M._scene_from_handle(h)
    finally:
        N.lib().mcrt_scene_free(h)
    full = M.load_scene_yaml_str(yaml)
    assert len(s.vertices) == 4 and len(s.triangles) == 2          # the plane's quad only
    assert len(full.vertices) == 8 and len(full.triangles) == 4
    # a deferred load of a scene without geometry still gets the stub triangle (scene.rs:887-899)
    h = ctypes.c_void_p()
    N.check(N.lib().mcrt_scene_load_yaml_str_ex(b"objects: []\n", b"<t>", N.LOAD_DEFER_MESHES, ctypes.byref(h)))
    try:
        assert len(M._scene_from_handle(h).triangles) == 1
    finally:
        N.lib().mcrt_scene_free(h)


def test_obj_writer_round_trips_through_the_loader(oracle):
    """scenes.obj_text (the benchmark meshes' OBJ text): fixed-point
    coordinates to 6 decimals in space-padded fields, 1-based a//n face tokens;
    loaded back, the positions are the 6-decimal values and the triangles the
    mesh's own, vertices shared by (position, normal)."""
    from mcrt_gb300 import scenes
    rng = np.random.default_rng(3)
    P = rng.uniform(-50, 50, (200, 3)).astype(np.float32)
    Nn = rng.normal(size=(200, 3)).astype(np.float32)
    F = rng.integers(0, 200, (300, 3))
    text = scenes.obj_text(P, F, normals=Nn)
    v, t = oracle.obj_load(text, 0)
    assert len(t) == 300
    got = v["position"][t["v"]][..., :3]
    want = np.round(P[F].astype(np.float64), 6)
    assert np.allclose(got, want, atol=1e-5, rtol=0)
    text2 = scenes.obj_text(P, F[:, [0, 1, 2]])            # no normals: a fresh vertex per face token
    v2, t2 = oracle.obj_load(text2, 0)
    assert len(v2) == 900 and len(t2) == 300
    assert np.allclose(v2["position"][:, :3], want.reshape(-1, 3), atol=1e-5, rtol=0)
