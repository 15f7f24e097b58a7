"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product never imports it.

``OracleScene`` builds the reference BVHs (src/bvh.rs:239, src/mesh.rs:82) from
the original primitive arrays with the oracle's restatement of the reference
builder, and traces / renders with the restatement of path_trace.wgsl.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_float, c_int, c_uint8, c_uint32, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

SPHERE = np.dtype([("center_r", "<f4", 4), ("mat_and_pad", "<u4", 4)])
NODE = np.dtype([("aabb_min", "<f4", 4), ("aabb_max", "<f4", 4), ("right_or_offset", "<u4"),
                 ("prim_count", "<u4"), ("pad", "<u4", 2)])
VERTEX = np.dtype([("position", "<f4", 4), ("normal", "<f4", 4), ("uv", "<f4", 4)])
TRIANGLE = np.dtype([("v", "<u4", 3), ("mat_idx", "<u4")])
RAY = np.dtype([("org", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
HIT = np.dtype([("t", "<f4"), ("prim", "<u4"), ("u", "<f4"), ("v", "<f4")])
CAMERA = np.dtype([("origin", "<f4", 4), ("lower_left", "<f4", 4), ("horizontal", "<f4", 4),
                   ("vertical", "<f4", 4), ("defocus_u", "<f4", 4), ("defocus_v", "<f4", 4),
                   ("frame_count", "<u4"), ("pad", "<u4", 3)])
NEE = 1   # ORC_RENDER_NEE


class _Scene(ctypes.Structure):
    _fields_ = [("spheres", c_void_p), ("n_spheres", c_uint32), ("sphere_ids", c_void_p),
                ("sphere_nodes", c_void_p), ("n_sphere_nodes", c_uint32),
                ("vertices", c_void_p), ("n_vertices", c_uint32),
                ("triangles", c_void_p), ("n_triangles", c_uint32), ("triangle_ids", c_void_p),
                ("mesh_nodes", c_void_p), ("n_mesh_nodes", c_uint32),
                ("materials", c_void_p),
                ("env_rgba", c_void_p), ("env_w", c_uint32), ("env_h", c_uint32),
                ("albedo", c_void_p), ("albedo_layers", c_uint32), ("albedo_size", c_uint32),
                ("sun_dir", c_float * 4), ("sun_irradiance", c_float * 4)]


def default_albedo_layers(size=512):
    """load_all_textures (texture.rs:235-256) without texture files: white, grey
    checker, magenta checker, magenta checker (build_checker_texture, :46-61)."""
    tile = max(size // 8, 1)
    y, x = np.mgrid[0:size, 0:size]
    sel = ((x // tile + y // tile) % 2 == 0)[..., None]
    def checker(a, b):
        return np.where(sel, np.array(a, np.uint8), np.array(b, np.uint8)).astype(np.uint8)
    out = np.zeros((4, size, size, 4), np.uint8)
    out[0] = 255
    out[1] = checker((220, 220, 220, 255), (50, 50, 50, 255))
    out[2] = checker((200, 0, 200, 255), (30, 30, 30, 255))
    out[3] = checker((200, 0, 200, 255), (30, 30, 30, 255))
    return out


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_build_sphere_bvh.restype = c_uint32
        L.orc_build_sphere_bvh.argtypes = [c_void_p, c_uint32, c_void_p, c_void_p, c_void_p]
        L.orc_build_mesh_bvh.restype = c_uint32
        L.orc_build_mesh_bvh.argtypes = [c_void_p, c_uint32, c_void_p, c_uint32, c_void_p, c_void_p, c_void_p]
        L.orc_trace.restype = None
        L.orc_trace.argtypes = [POINTER(_Scene), c_void_p, c_uint32, c_void_p, c_int, c_void_p, c_int]
        L.orc_render.restype = None
        L.orc_render.argtypes = [POINTER(_Scene), c_void_p, c_uint32, c_uint32, c_uint32, c_uint32, c_uint32,
                                 c_void_p, c_void_p, c_void_p, c_int]
        L.orc_render_rect.restype = None
        L.orc_render_rect.argtypes = [POINTER(_Scene), c_void_p, c_uint32, c_uint32, c_uint32, c_uint32, c_uint32,
                                      c_uint32, c_uint32, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p, c_int]
        L.orc_render_rect_stats.restype = None
        L.orc_render_rect_stats.argtypes = [POINTER(_Scene), c_void_p, c_uint32, c_uint32, c_uint32, c_uint32,
                                            c_uint32, c_uint32, c_uint32, c_uint32, c_uint32, c_void_p, c_void_p,
                                            c_void_p, c_int, c_void_p]
        L.orc_render_ex.restype = None
        L.orc_render_ex.argtypes = [POINTER(_Scene), c_void_p, c_uint32, c_uint32, c_uint32, c_uint32, c_uint32,
                                    c_uint32, c_uint32, c_uint32, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p,
                                    c_int, c_void_p]
        L.orc_adjoint.restype = None
        L.orc_adjoint.argtypes = [POINTER(_Scene), c_void_p, c_uint32, c_uint32, c_uint32, c_uint32, c_uint32,
                                  c_uint32, c_void_p, c_void_p, c_void_p, c_int]
        L.orc_denoise.restype = None
        L.orc_denoise.argtypes = [c_void_p, c_void_p, c_uint32, c_uint32, c_int, c_float, c_float, c_float, c_void_p]
        L.orc_tonemap_rgba8.restype = None
        L.orc_tonemap_rgba8.argtypes = [c_void_p, c_uint32, c_void_p]
        L.orc_compare_images.restype = None
        L.orc_compare_images.argtypes = [c_void_p, c_void_p, c_uint32, c_uint32, c_void_p]
        L.orc_math_eval.restype = None
        L.orc_math_eval.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_uint32]
        L.orc_pcg_hash.restype = c_uint32
        L.orc_pcg_hash.argtypes = [c_uint32]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(c_void_p)


def build_sphere_bvh(spheres):
    spheres = np.ascontiguousarray(spheres, SPHERE)
    n = len(spheres)
    nodes = np.zeros(max(2 * n, 1), NODE)
    ordered = np.zeros(n, SPHERE)
    ids = np.zeros(n, np.uint32)
    nn = lib().orc_build_sphere_bvh(_p(spheres), n, _p(nodes), _p(ordered), _p(ids))
    return nodes[:nn].copy(), ordered, ids


def build_mesh_bvh(vertices, triangles):
    vertices = np.ascontiguousarray(vertices, VERTEX)
    triangles = np.ascontiguousarray(triangles, TRIANGLE)
    n = len(triangles)
    nodes = np.zeros(max(2 * n, 1), NODE)
    ordered = np.zeros(n, TRIANGLE)
    ids = np.zeros(n, np.uint32)
    nn = lib().orc_build_mesh_bvh(_p(vertices), len(vertices), _p(triangles), n, _p(nodes), _p(ordered), _p(ids))
    return nodes[:nn].copy(), ordered, ids


class OracleScene:
    """A scene as the reference binds it, built by the oracle's reference builder."""

    def __init__(self, *, materials, spheres=None, vertices=None, triangles=None, env=None, albedo=None,
                 sun_dir=None, sun_irradiance=None):
        self.spheres_in = np.zeros(0, SPHERE) if spheres is None else np.ascontiguousarray(spheres, SPHERE)
        self.vertices = np.zeros(0, VERTEX) if vertices is None else np.ascontiguousarray(vertices, VERTEX)
        self.triangles_in = np.zeros(0, TRIANGLE) if triangles is None else np.ascontiguousarray(triangles, TRIANGLE)
        self.materials = np.ascontiguousarray(materials)
        self.sphere_nodes, self.spheres, self.sphere_ids = build_sphere_bvh(self.spheres_in)
        self.mesh_nodes, self.triangles, self.triangle_ids = build_mesh_bvh(self.vertices, self.triangles_in)
        self.env = None if env is None else np.ascontiguousarray(env, np.float32)
        s = _Scene()
        s.spheres, s.n_spheres, s.sphere_ids = _p(self.spheres), len(self.spheres), _p(self.sphere_ids)
        s.sphere_nodes, s.n_sphere_nodes = _p(self.sphere_nodes), len(self.sphere_nodes)
        s.vertices, s.n_vertices = _p(self.vertices), len(self.vertices)
        s.triangles, s.n_triangles, s.triangle_ids = _p(self.triangles), len(self.triangles), _p(self.triangle_ids)
        s.mesh_nodes, s.n_mesh_nodes = _p(self.mesh_nodes), len(self.mesh_nodes)
        s.materials = _p(self.materials)
        if self.env is not None:
            s.env_rgba, s.env_h, s.env_w = _p(self.env), self.env.shape[0], self.env.shape[1]
        self.albedo = np.ascontiguousarray(default_albedo_layers() if albedo is None else albedo, np.uint8)
        s.albedo, s.albedo_layers, s.albedo_size = _p(self.albedo), self.albedo.shape[0], self.albedo.shape[1]
        if sun_irradiance is not None:
            for k in range(3):
                s.sun_dir[k] = float(sun_dir[k])
                s.sun_irradiance[k] = float(sun_irradiance[k])
        self._s = s

    def reference_buffers(self):
        """The buffers the reference's build_scene_buffers would upload (ordered + BVHs + ids)."""
        return dict(spheres=self.spheres, sphere_bvh=self.sphere_nodes, sphere_order=self.sphere_ids,
                    vertices=self.vertices, triangles=self.triangles, mesh_bvh=self.mesh_nodes,
                    triangle_order=self.triangle_ids, materials=self.materials, env=self.env, albedo=self.albedo)

    def trace(self, rays, brute_force=False, threads=0, stats=False):
        rays = np.ascontiguousarray(rays, RAY)
        hits = np.zeros(len(rays), HIT)
        st = np.zeros(2 * len(rays), np.uint32) if stats else None
        lib().orc_trace(ctypes.byref(self._s), _p(rays), len(rays), _p(hits), 1 if brute_force else 0, _p(st),
                        threads)
        return (hits, st.reshape(-1, 2)) if stats else hits

    def render(self, camera, w, h, spp, first_frame=0, max_depth=8, threads=0, rect=None, stats=False, nee=False):
        cam = np.ascontiguousarray(camera)
        x0, y0, cw, ch = rect if rect else (0, 0, w, h)
        mean = np.zeros((ch, cw, 4), np.float32)
        acc = np.zeros((ch, cw, 3), np.float64)
        gbuf = np.zeros((ch, cw, 4), np.float32)
        st = np.zeros(3, np.uint64) if stats else None
        lib().orc_render_ex(ctypes.byref(self._s), _p(cam), w, h, x0, y0, cw, ch, spp, first_frame, max_depth,
                            NEE if nee else 0, _p(mean), _p(acc), _p(gbuf), threads, _p(st))
        out = dict(rgba=mean, sum=acc, gbuf=gbuf)
        if stats:
            out["stats"] = dict(rays=int(st[0]), nodes=int(st[1]), prims=int(st[2]))
        return out

    def dump_rays(self, camera, w, h, spp, rect=None, first_frame=0, max_depth=8, nee=False, bounces=4, threads=0):
        """The closest-hit queries of the rect's sampled paths, bounces 0 .. bounces-1:
        (rays, hits, bounce) of the queries the paths reach, in (pixel, frame, bounce) order."""
        L = lib()
        L.orc_dump_rays.restype = None
        L.orc_dump_rays.argtypes = [POINTER(_Scene), c_void_p] + [c_uint32] * 11 + [c_void_p, c_void_p, c_int]
        cam = np.ascontiguousarray(camera)
        x0, y0, cw, ch = rect if rect else (0, 0, w, h)
        n = cw * ch * spp * bounces
        rays = np.zeros(n, RAY)
        hits = np.zeros(n, HIT)
        L.orc_dump_rays(ctypes.byref(self._s), _p(cam), w, h, x0, y0, cw, ch, spp, first_frame, max_depth,
                        NEE if nee else 0, bounces, _p(rays), _p(hits), threads)
        bounce = np.tile(np.arange(bounces, dtype=np.uint32), cw * ch * spp)
        keep = rays["tmax"] > 0
        return rays[keep], hits[keep], bounce[keep]

    def render_cache_const(self, camera, w, h, spp, c3, spp_pass, train_stride, query_vertex, first_frame=0,
                           max_depth=8, nee=False, threads=0):
        """Render with paths stopped into a constant radiance cache (see oracle.h)."""
        L = lib()
        L.orc_render_cache_const.restype = None
        L.orc_render_cache_const.argtypes = [POINTER(_Scene), c_void_p, c_uint32, c_uint32, c_uint32, c_uint32,
                                             c_uint32, c_uint32, c_uint32, c_uint32, c_uint32, c_void_p, c_void_p,
                                             c_void_p, c_int]
        cam = np.ascontiguousarray(camera)
        c = np.ascontiguousarray(c3, np.float32)
        mean = np.zeros((h, w, 4), np.float32)
        acc = np.zeros((h, w, 3), np.float64)
        L.orc_render_cache_const(ctypes.byref(self._s), _p(cam), w, h, spp, first_frame, max_depth,
                                 NEE if nee else 0, spp_pass, train_stride, query_vertex, _p(c), _p(mean), _p(acc),
                                 threads)
        return dict(rgba=mean, sum=acc)

    def adjoint(self, camera, w, h, spp, d_image, first_frame=0, max_depth=8, nee=False, threads=0):
        """Brute-force (forward-mode) gradient of sum(d_image * image) with respect to
        the 64 x 4 material parameters (albedo rgb, roughness); also returns the f64 sums."""
        cam = np.ascontiguousarray(camera)
        d = np.ascontiguousarray(d_image, np.float32).reshape(h, w, 4)
        grad = np.zeros(256, np.float64)
        acc = np.zeros((h, w, 3), np.float64)
        lib().orc_adjoint(ctypes.byref(self._s), _p(cam), w, h, spp, first_frame, max_depth, NEE if nee else 0,
                          _p(d), _p(grad), _p(acc), threads)
        return grad.reshape(64, 4), acc


def compute_camera(width, height, look_from, look_at, vfov=60.0, aperture=0.0, focus_dist=None):
    """CameraUniform (structured CAMERA record) of camera.rs:76-127; focus_dist defaults to
    |look_from - look_at| in float32."""
    L = lib()
    L.orc_compute_camera.restype = None
    L.orc_compute_camera.argtypes = [c_uint32, c_uint32, c_void_p, c_void_p, c_float, c_float, c_float, c_void_p]
    lf = np.ascontiguousarray(look_from, np.float32)
    la = np.ascontiguousarray(look_at, np.float32)
    if focus_dist is None:
        d = lf - la
        focus_dist = float(np.sqrt(np.float32(d[0] * d[0] + d[1] * d[1]) + np.float32(d[2] * d[2])))
    out = np.zeros((), CAMERA)
    L.orc_compute_camera(width, height, _p(lf), _p(la), vfov, aperture, focus_dist, _p(out))
    return out


def denoise(rgba, gbuf, radius=3, sigma_s=2.0, sigma_d=0.5, normal_pow=8.0, sigma_color=0.0, sigma_normal=0.0):
    L = lib()
    L.orc_denoise_ex.restype = None
    L.orc_denoise_ex.argtypes = [c_void_p, c_void_p, c_uint32, c_uint32, c_int, c_float, c_float, c_float, c_float,
                                 c_float, c_void_p]
    rgba = np.ascontiguousarray(rgba, np.float32)
    gbuf = np.ascontiguousarray(gbuf, np.float32)
    h, w = rgba.shape[:2]
    out = np.zeros_like(rgba)
    L.orc_denoise_ex(_p(rgba), _p(gbuf), w, h, radius, sigma_s, sigma_d, normal_pow, sigma_color, sigma_normal,
                     _p(out))
    return out


def tonemap_rgba8(rgba):
    rgba = np.ascontiguousarray(rgba, np.float32)
    out = np.zeros(rgba.shape[:-1] + (4,), np.uint8)
    lib().orc_tonemap_rgba8(_p(rgba), rgba.size // 4, _p(out))
    return out


def compare_images(a, b):
    """regression.rs compare_images on RGBA8 arrays: (mse, psnr, max_delta)."""
    a = np.ascontiguousarray(a, np.uint8)
    b = np.ascontiguousarray(b, np.uint8)
    assert a.shape == b.shape
    out = np.zeros(3, np.float64)
    lib().orc_compare_images(_p(a), _p(b), a.shape[1], a.shape[0], _p(out))
    return float(out[0]), float(out[1]), float(out[2])


MATH_FNS = {"sin": 0, "cos": 1, "atan2": 2, "asin": 3, "exp": 4, "log": 5, "pow": 6, "tan": 7}


def math_eval(fn, x, y=None):
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(np.zeros_like(x) if y is None else y, np.float32)
    out = np.zeros_like(x)
    lib().orc_math_eval(MATH_FNS[fn], _p(x), _p(y), _p(out), x.size)
    return out


class _WorldParams(ctypes.Structure):
    _fields_ = [("nx", c_uint32), ("ny", c_uint32), ("nz", c_uint32), ("seed", c_uint32),
                ("chunk_x0", ctypes.c_int32), ("chunk_z0", ctypes.c_int32),
                ("height_base", c_float), ("height_amp", c_float), ("height_freq", c_float),
                ("height_octaves", c_uint32), ("lacunarity", c_float), ("gain", c_float),
                ("cave_freq", c_float), ("cave_octaves", c_uint32), ("cave_threshold", c_float),
                ("cave_contrast", c_float), ("cave_min_y", c_uint32), ("sea_level", c_float), ("sand_line", c_float)]


def world_generate(params):
    """The voxel grid (nx, ny, nz) uint8 of the world generator."""
    L = lib()
    L.orc_world_generate.restype = None
    L.orc_world_generate.argtypes = [POINTER(_WorldParams), c_void_p]
    p = _WorldParams(**params)
    vox = np.zeros((p.nx, p.ny, p.nz), np.uint8)
    L.orc_world_generate(ctypes.byref(p), _p(vox))
    return vox


def world_mesh(voxels, block_material, voxel_size=0.125, greedy=True, chunk_x0=0, chunk_z0=0):
    """The reference's greedy chunk mesher (or one quad per face) over a voxel grid:
    (vertices, triangles)."""
    L = lib()
    L.orc_world_mesh.restype = ctypes.c_uint64
    L.orc_world_mesh.argtypes = [c_void_p, c_uint32, c_uint32, c_uint32, ctypes.c_int32, ctypes.c_int32, c_int,
                                 c_void_p, c_float, c_void_p, c_void_p, ctypes.c_uint64]
    v = np.ascontiguousarray(voxels, np.uint8)
    nx, ny, nz = v.shape
    mm = np.zeros(256, np.uint32)
    bm = np.asarray(block_material, np.uint32).ravel()
    mm[:len(bm)] = bm
    q = L.orc_world_mesh(_p(v), nx, ny, nz, chunk_x0, chunk_z0, 1 if greedy else 0, _p(mm), voxel_size, None, None, 0)
    verts = np.zeros(4 * q, VERTEX)
    tris = np.zeros(2 * q, TRIANGLE)
    L.orc_world_mesh(_p(v), nx, ny, nz, chunk_x0, chunk_z0, 1 if greedy else 0, _p(mm), voxel_size, _p(verts),
                     _p(tris), q)
    return verts, tris


def _inv_extent(lo, hi):
    lo = np.asarray(lo, np.float32)
    ext = np.asarray(hi, np.float32) - lo
    return lo, np.where(ext > 0, np.float32(1.0) / ext, np.float32(0.0)).astype(np.float32)


def mlp_forward(params, lo, hi, queries):
    """Radiance-cache MLP predictions (n, 3) for (n, 12) queries."""
    L = lib()
    L.orc_mlp_forward.restype = None
    L.orc_mlp_forward.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_void_p]
    lo32, inv = _inv_extent(lo, hi)
    p = np.ascontiguousarray(params, np.float32)
    q = np.ascontiguousarray(queries, np.float32).reshape(-1, 12)
    out = np.zeros((len(q), 3), np.float32)
    L.orc_mlp_forward(_p(p), _p(lo32), _p(inv), _p(q), len(q), _p(out))
    return out


def mlp_grad(params, lo, hi, samples):
    """(gradient (float64, params), loss sum) of one training step on (n, 16) samples."""
    L = lib()
    L.orc_mlp_grad.restype = None
    L.orc_mlp_grad.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_void_p, c_void_p]
    lo32, inv = _inv_extent(lo, hi)
    p = np.ascontiguousarray(params, np.float32)
    s = np.ascontiguousarray(samples, np.float32).reshape(-1, 16)
    g = np.zeros(len(p), np.float64)
    loss = np.zeros(1, np.float64)
    L.orc_mlp_grad(_p(p), _p(lo32), _p(inv), _p(s), len(s), _p(g), _p(loss))
    return g, float(loss[0])


def mlp_encode(query, lo, hi):
    L = lib()
    L.orc_mlp_encode.restype = None
    L.orc_mlp_encode.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p]
    lo32, inv = _inv_extent(lo, hi)
    q = np.ascontiguousarray(query, np.float32)
    out = np.zeros(96, np.float32)
    L.orc_mlp_encode(_p(q), _p(lo32), _p(inv), _p(out))
    return out


def ggx_dg(alpha, mz, cos_o, cos_i):
    """(d(D G2)/d alpha, D G2) of the GGX lobe."""
    L = lib()
    L.orc_ggx_dg.restype = None
    L.orc_ggx_dg.argtypes = [c_double, c_double, c_double, c_double, c_void_p]
    out = np.zeros(2, np.float64)
    L.orc_ggx_dg(alpha, mz, cos_o, cos_i, _p(out))
    return float(out[0]), float(out[1])


def pcg_hash(v):
    return lib().orc_pcg_hash(v)


def tonemap_aces_rgba8(rgba):
    L = lib()
    L.orc_tonemap_aces_rgba8.restype = None
    L.orc_tonemap_aces_rgba8.argtypes = [c_void_p, c_uint32, c_void_p]
    rgba = np.ascontiguousarray(rgba, np.float32)
    out = np.zeros(rgba.shape[:-1] + (4,), np.uint8)
    L.orc_tonemap_aces_rgba8(_p(rgba), rgba.size // 4, _p(out))
    return out


VERTEX = np.dtype([("position", np.float32, 4), ("normal", np.float32, 4), ("uv", np.float32, 4)])
TRIANGLE = np.dtype([("v", np.uint32, 3), ("mat_idx", np.uint32)])


class ObjError(ValueError):
    """load_obj's error text after "'<path>' " or "'<path>': "."""


def obj_load(text, mat_idx=0):
    """load_obj (mesh.rs:474-642) on OBJ text (bytes): (vertices, triangles) as
    the reference's GpuVertex / GpuTriangle records, or ObjError."""
    L = lib()
    L.orc_obj_load.restype = c_void_p
    L.orc_obj_load.argtypes = [ctypes.c_char_p, ctypes.c_uint64, c_uint32, POINTER(c_uint32), POINTER(c_uint32),
                               ctypes.c_char_p, c_uint32]
    L.orc_obj_copy.restype = None
    L.orc_obj_copy.argtypes = [c_void_p, c_void_p, c_void_p]
    L.orc_obj_free.restype = None
    L.orc_obj_free.argtypes = [c_void_p]
    data = bytes(text)
    nv, nt = c_uint32(0), c_uint32(0)
    err = ctypes.create_string_buffer(512)
    h = L.orc_obj_load(data, len(data), mat_idx, ctypes.byref(nv), ctypes.byref(nt), err, 512)
    if not h:
        raise ObjError(err.value.decode())
    v = np.zeros(nv.value, VERTEX)
    t = np.zeros(nt.value, TRIANGLE)
    L.orc_obj_copy(h, _p(v), _p(t))
    L.orc_obj_free(h)
    return v, t


def parse_f32(token):
    """str::parse::<f32> of one token (bytes): the float, or None on a syntax error."""
    L = lib()
    L.orc_parse_f32.restype = ctypes.c_int
    L.orc_parse_f32.argtypes = [ctypes.c_char_p, c_uint32, c_void_p]
    out = np.zeros(1, np.float32)
    tok = bytes(token)
    return out[0] if L.orc_parse_f32(tok, len(tok), _p(out)) else None
