"""CPU checks of the oracle's voxel-world restatement against the reference's
own mesher tests (world/mesher.rs:407-508) and the generator's invariants."""
import numpy as np
import pytest

from mcrt_gb300 import scenes

CY = 256          # the reference's CHUNK_Y (world/chunk.rs:16)


def _chunk():
    return np.zeros((16, CY, 16), np.uint8)


def _mesh(oracle, vox, greedy=True):
    return oracle.world_mesh(vox, np.zeros(256, np.uint32), greedy=greedy)


def test_air_chunk_produces_no_triangles(oracle):          # mesher.rs:430-436
    v, t = _mesh(oracle, _chunk())
    assert len(t) == 0 and len(v) == 0


def test_single_voxel_produces_12_triangles(oracle):       # mesher.rs:438-450
    c = _chunk()
    c[8, 8, 8] = 1
    v, t = _mesh(oracle, c)
    assert len(t) == 12 and len(v) == 24
    # every face sits on the voxel's boundary at VOXEL_SIZE 0.125, normals axis-aligned
    p = v["position"][:, :3]
    assert p.min() == 1.0 and p.max() == 9 * 0.125
    assert np.all(np.abs(v["normal"][:, :3]).sum(1) == 1.0)


def test_flat_slab_top_face_is_merged(oracle):             # mesher.rs:452-474
    c = _chunk()
    c[0:2, 0, 0:2] = 1
    _, t = _mesh(oracle, c)
    assert len(t) < 24
    assert len(t) == 12            # six merged 2x2 / 2x1 faces
    _, tf = _mesh(oracle, c, greedy=False)
    assert len(tf) == 2 * (4 + 4 + 8)


def test_adjacent_blocks_cull_shared_face(oracle):         # mesher.rs:476-491
    c = _chunk()
    c[0, 0, 0] = 1
    c[1, 0, 0] = 1
    _, t = _mesh(oracle, c)
    assert len(t) < 24
    _, tf = _mesh(oracle, c, greedy=False)
    assert len(tf) == 20           # 10 exposed faces


def test_winding_as_the_reference_emits_it(oracle):
    """emit_quad (mesher.rs:343-366) orders the corners (u0,v0), (u0+h,v0),
    (u0+h,v0+w), (u0,v0+w) for every axis, so the geometric winding follows the
    stored normal on X and Z faces and is reversed on Y faces (u = X, v = Z)."""
    c = _chunk()
    c[3, 4, 5] = 2
    v, t = _mesh(oracle, c)
    p = v["position"][:, :3].astype(np.float64)
    for tri in t:
        a, b, d = p[tri["v"][0]], p[tri["v"][1]], p[tri["v"][2]]
        nrm = v["normal"][tri["v"][0], :3]
        s = np.dot(np.cross(b - a, d - a), nrm)
        assert (s < 0) if nrm[1] != 0 else (s > 0)


def test_chunks_see_their_neighbours(oracle):
    """A block on a chunk border hides the face it shares with the next chunk
    (neighbour sampling across chunks, mesher.rs:261-300), and the two-chunk mesh
    concatenates as merge_chunk_meshes does (vertex indices offset)."""
    g = np.zeros((32, 16, 16), np.uint8)
    g[15, 3, 3] = 1
    g[16, 3, 3] = 1
    v, t = oracle.world_mesh(g, np.zeros(256, np.uint32), greedy=True)
    assert len(t) == 20
    assert t["v"].max() == len(v) - 1
    assert np.all(np.diff(t["v"][::2, 0]) >= 0)


def test_material_map_and_origin(oracle):
    c = np.zeros((16, 8, 16), np.uint8)
    c[0, 0, 0] = 9
    mm = np.zeros(256, np.uint32)
    mm[9] = 6
    v, t = oracle.world_mesh(c, mm, greedy=True, chunk_x0=2, chunk_z0=-3)
    assert np.all(t["mat_idx"] == 6)
    p = v["position"][:, :3]
    # chunk_world_origin(2, -3) = (4, 0, -6) (chunk.rs:131-137, :190-195)
    assert p[:, 0].min() == 4.0 and p[:, 2].min() == -6.0


def test_generator_invariants(oracle):
    p = scenes.world_params(seed=5, nx=32, ny=64, nz=48)
    vox = oracle.world_generate(p)
    assert vox.shape == (32, 64, 48)
    assert set(np.unique(vox).tolist()) <= {0, 1, 2, 3, 4, 5, 8, 9, 10}
    assert np.all(vox[:, 0, :] != 0)                       # the floor is never carved
    assert np.array_equal(vox, oracle.world_generate(p))   # deterministic
    q = dict(p, seed=6)
    assert not np.array_equal(vox, oracle.world_generate(q))
    # chunk offsets continue the same world: the second half of a grid is the
    # grid generated from the next chunk coordinate
    a = oracle.world_generate(dict(p, nx=32, chunk_x0=0))
    b = oracle.world_generate(dict(p, nx=16, chunk_x0=1))
    assert np.array_equal(a[16:], b)


def test_voxel_world_workload_size(oracle):
    """The configured 256 x 128 x 256 world meshes to 4-6 M exposed-face triangles."""
    w = scenes.voxel_world()
    vox = oracle.world_generate(w["params"])
    _, t = oracle.world_mesh(vox, w["block_material"], greedy=False)
    assert 4_000_000 <= len(t) <= 6_000_000
