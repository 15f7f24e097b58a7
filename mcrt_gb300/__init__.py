"""mcrt_gb300 — GB300-native path-tracing hot path of mcrt behind a C ABI.

Python view of libmcrt_cuda.so (include/mcrt_cuda.h).  The CUDA library does
all of the work; this module only marshals numpy arrays.  It mirrors the
reference's interfaces for the path:

* ``load_scene_yaml`` / ``load_scene_yaml_str`` — scene.rs load_scene_from_yaml /
  load_scene_from_str (src/scene.rs:640-999);
* ``compute_camera`` — camera.rs compute_camera (src/camera.rs:76-127);
* ``load_env_map`` / ``gradient_env_map`` — texture.rs (src/texture.rs:158-220);
* ``Context.upload_scene`` — gpu_layout::build_scene_buffers (src/gpu_layout.rs:259-390);
* ``Context.render`` — the per-sample cs_main dispatches of headless::run
  (src/headless.rs:249-290, src/shaders/path_trace.wgsl:626-662);
* ``Context.denoise`` — cs_denoise (src/shaders/denoise.wgsl:52-120);
* ``headless_run`` — headless::run (src/headless.rs:112-386).
"""
from __future__ import annotations

import ctypes
from ctypes import c_double, c_float, c_uint32, c_uint64, c_void_p
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from ._native import (CAMERA, HIT, MATERIAL, MATERIAL_DATA, NODE, RAY, SPHERE, TRIANGLE, VERTEX, MCRTError,
                      check, lib, ptr)

__all__ = ["Context", "Scene", "load_scene_yaml", "load_scene_yaml_str", "compute_camera", "load_env_map",
           "gradient_env_map", "tonemap_rgba8", "write_png", "headless_run", "MCRTError", "SPHERE", "NODE",
           "VERTEX", "TRIANGLE", "MATERIAL", "MATERIAL_DATA", "CAMERA", "RAY", "HIT", "make_rays", "materials"]


def _arr(a, dtype):
    if a is None:
        return None
    a = np.ascontiguousarray(a)
    if a.dtype != dtype:
        raise TypeError(f"expected dtype {dtype}, got {a.dtype}")
    return a


@dataclass
class Scene:
    """LoadedScene (src/scene.rs:311-351) as numpy record arrays."""
    spheres: np.ndarray
    vertices: np.ndarray
    triangles: np.ndarray
    materials: np.ndarray          # MATERIAL_DATA, shape ()
    emissive_spheres: np.ndarray
    camera: dict | None = None     # look_from, look_at, vfov, aperture, focus_dist
    env_map_path: str | None = None
    material_names: list = field(default_factory=list)


def _scene_from_handle(h) -> Scene:
    L = lib()
    v = N.SceneView()
    check(L.mcrt_scene_view_get(h, ctypes.byref(v)))

    def grab(p, n, dt):
        if n == 0:
            return np.zeros(0, dt)
        buf = (ctypes.c_uint8 * (n * dt.itemsize)).from_address(p)
        return np.frombuffer(bytes(buf), dtype=dt).copy()

    mats = np.frombuffer(bytes((ctypes.c_uint8 * MATERIAL_DATA.itemsize).from_address(v.materials)),
                         dtype=MATERIAL_DATA)[0].copy()
    cam = None
    if v.has_camera:
        cam = dict(look_from=list(v.look_from), look_at=list(v.look_at), vfov=v.vfov, aperture=v.aperture,
                   focus_dist=v.focus_dist)
    names = [L.mcrt_scene_material_name(h, i).decode() for i in range(v.n_material_names)]
    return Scene(spheres=grab(v.spheres, v.n_spheres, SPHERE), vertices=grab(v.vertices, v.n_vertices, VERTEX),
                 triangles=grab(v.triangles, v.n_triangles, TRIANGLE), materials=mats,
                 emissive_spheres=grab(v.emissive_spheres, v.n_emissive_spheres, SPHERE), camera=cam,
                 env_map_path=v.env_map_path.decode() if v.env_map_path else None, material_names=names)


def load_scene_yaml(path: str) -> Scene:
    h = c_void_p()
    check(lib().mcrt_scene_load_yaml(path.encode(), ctypes.byref(h)))
    try:
        return _scene_from_handle(h)
    finally:
        lib().mcrt_scene_free(h)


def load_scene_yaml_str(text: str, source: str = "<inline>") -> Scene:
    h = c_void_p()
    check(lib().mcrt_scene_load_yaml_str(text.encode(), source.encode(), ctypes.byref(h)))
    try:
        return _scene_from_handle(h)
    finally:
        lib().mcrt_scene_free(h)


def compute_camera(width, height, look_from, look_at, vfov=60.0, aperture=0.0, focus_dist=None) -> np.ndarray:
    lf = (c_float * 3)(*look_from)
    la = (c_float * 3)(*look_at)
    if focus_dist is None:
        d = np.asarray(look_from, np.float32) - np.asarray(look_at, np.float32)
        focus_dist = float(np.sqrt(np.float32(d[0] * d[0] + d[1] * d[1]) + np.float32(d[2] * d[2])))
    out = np.zeros((), CAMERA)
    check(lib().mcrt_compute_camera(width, height, lf, la, vfov, aperture, focus_dist, ptr(out)))
    return out


def load_env_map(path: str | None) -> np.ndarray:
    out = np.zeros((N.ENV_H, N.ENV_W, 4), np.float32)
    check(lib().mcrt_load_env_map(path.encode() if path else None, ptr(out)))
    return out


def gradient_env_map() -> np.ndarray:
    out = np.zeros((N.ENV_H, N.ENV_W, 4), np.float32)
    check(lib().mcrt_gradient_env_map(ptr(out)))
    return out


def albedo_layers() -> np.ndarray:
    """The reference's default albedo texture array (4 x 512 x 512 RGBA8)."""
    out = np.zeros((4, 512, 512, 4), np.uint8)
    check(lib().mcrt_albedo_layers(ptr(out)))
    return out


def tonemap_rgba8(rgba: np.ndarray) -> np.ndarray:
    rgba = np.ascontiguousarray(rgba, np.float32)
    out = np.zeros(rgba.shape[:-1] + (4,), np.uint8)
    check(lib().mcrt_tonemap_rgba8(ptr(rgba), rgba.size // 4, ptr(out)))
    return out


def tonemap_aces_rgba8(rgba: np.ndarray) -> np.ndarray:
    rgba = np.ascontiguousarray(rgba, np.float32)
    out = np.zeros(rgba.shape[:-1] + (4,), np.uint8)
    check(lib().mcrt_tonemap_aces_rgba8(ptr(rgba), rgba.size // 4, ptr(out)))
    return out


def write_hdr(path: str, rgba: np.ndarray):
    rgba = np.ascontiguousarray(rgba, np.float32)
    h, w = rgba.shape[:2]
    check(lib().mcrt_write_hdr(path.encode(), ptr(rgba), w, h))


def write_png(path: str, rgba8: np.ndarray):
    rgba8 = np.ascontiguousarray(rgba8, np.uint8)
    h, w = rgba8.shape[:2]
    check(lib().mcrt_write_png(path.encode(), ptr(rgba8), w, h))


def headless_run(scene_path, output_path, width=None, height=None, spp=None, max_depth=0, nee=False):
    o = N.RenderOpts(max_depth=max_depth, flags=N.RENDER_NEE if nee else 0)
    check(lib().mcrt_headless_run(scene_path.encode(), output_path.encode(), width or 0, height or 0, spp or 0,
                                  ctypes.byref(o)))


def materials(entries) -> np.ndarray:
    """Build a GpuMaterialData from (type, albedo_rgb, w, ior_or_strength[, texture_layer]) tuples."""
    md = np.zeros((), MATERIAL_DATA)
    md["mat_count"] = len(entries)
    for i, e in enumerate(entries):
        t, alb, w, x = e[:4]
        md["materials"][i]["type_pad"][0] = t
        md["materials"][i]["type_pad"][1] = e[4] if len(e) > 4 else 0
        md["materials"][i]["albedo_fuzz"][:3] = alb
        md["materials"][i]["albedo_fuzz"][3] = w
        md["materials"][i]["ior_pad"][0] = x
    return md


def variant_info(variant: int) -> dict:
    """Closest-hit kernel variant: BVH width, block size, minimum resident blocks, stack depth, refill
    lanes, shared-memory top-tree records."""
    out = (c_uint32 * 6)()
    check(lib().mcrt_variant_info(variant, out))
    return dict(width=out[0], block=out[1], min_blocks=out[2], stack=out[3], refill=out[4], top=out[5])


def make_rays(org, dirs, tmin=1e-4, tmax=1e9) -> np.ndarray:
    org = np.asarray(org, np.float32).reshape(-1, 3)
    dirs = np.asarray(dirs, np.float32).reshape(-1, 3)
    r = np.zeros(len(dirs), RAY)
    r["org"] = org
    r["dir"] = dirs
    r["tmin"] = tmin
    r["tmax"] = tmax
    return r


class Context:
    """A CUDA context of the library: one device, one stream, one resident scene."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self._h = c_void_p()
        check(lib().mcrt_create(device, c_void_p(stream) if stream else None, ctypes.byref(self._h)))
        self._keep = []
        self._world_tris = 0

    def close(self):
        if self._h:
            lib().mcrt_destroy(self._h)
            self._h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, s):
        check(s, self._h)

    def upload_scene(self, *, materials, spheres=None, vertices=None, triangles=None, env=None, sphere_bvh=None,
                     sphere_order=None, mesh_bvh=None, triangle_order=None, albedo=None, sun_dir=None,
                     sun_irradiance=None, world_mesh=False, device_mesh=False):
        """world_mesh: take the triangles from the last world_mesh() call (no host geometry).
        device_mesh: take them from the device mesh (mesh_append*, no host geometry).
        sun_dir / sun_irradiance: a directional light sampled by next-event estimation."""
        sph = _arr(spheres, SPHERE)
        ver = _arr(vertices, VERTEX)
        tri = _arr(triangles, TRIANGLE)
        mats = _arr(materials, MATERIAL_DATA)
        def opt(a, dt):      # an empty prebuilt BVH / order means "none given"
            a = _arr(a, dt)
            return None if a is None or a.size == 0 else a
        sbvh = opt(sphere_bvh, NODE)
        mbvh = opt(mesh_bvh, NODE)
        sord = opt(sphere_order, np.uint32)
        tord = opt(triangle_order, np.uint32)
        envp = None if env is None else np.ascontiguousarray(env, np.float32)
        d = N.SceneDesc()
        d.spheres, d.n_spheres = ptr(sph), 0 if sph is None else len(sph)
        d.sphere_bvh, d.n_sphere_nodes = ptr(sbvh), 0 if sbvh is None else len(sbvh)
        d.sphere_order = ptr(sord)
        d.vertices, d.n_vertices = ptr(ver), 0 if ver is None else len(ver)
        d.triangles, d.n_triangles = ptr(tri), 0 if tri is None else len(tri)
        d.mesh_bvh, d.n_mesh_nodes = ptr(mbvh), 0 if mbvh is None else len(mbvh)
        d.triangle_order = ptr(tord)
        d.materials = ptr(mats)
        if envp is not None:
            d.env_rgba, d.env_h, d.env_w = ptr(envp), envp.shape[0], envp.shape[1]
        alb = None if albedo is None else np.ascontiguousarray(albedo, np.uint8)
        if alb is not None:
            d.albedo_rgba8, d.albedo_layers, d.albedo_size = ptr(alb), alb.shape[0], alb.shape[1]
        if sun_irradiance is not None:
            for k in range(3):
                d.sun_dir[k] = float(sun_dir[k])
                d.sun_irradiance[k] = float(sun_irradiance[k])
        if world_mesh:
            d.flags |= N.SCENE_WORLD_MESH
        if device_mesh:
            d.flags |= N.SCENE_DEVICE_MESH
        self._check(lib().mcrt_upload_scene(self._h, ctypes.byref(d)))
        self.n_triangles = (self._world_tris if world_mesh else self.mesh_counts()[1] if device_mesh
                            else d.n_triangles)

    # ---------------------------------------------------------------- scene ingestion on the device
    def mesh_reset(self):
        """Empty the device mesh."""
        self._check(lib().mcrt_mesh_reset(self._h))

    def mesh_append(self, vertices, triangles):
        """Append host records (triangle indices relative to these vertices)."""
        ver = _arr(vertices, VERTEX)
        tri = _arr(triangles, TRIANGLE)
        self._check(lib().mcrt_mesh_append(self._h, ptr(ver), 0 if ver is None else len(ver), ptr(tri),
                                           0 if tri is None else len(tri)))

    def mesh_append_obj(self, text, mat_idx=0, translate=None, rotate=None, scale=None, source=None):
        """Parse OBJ text (bytes or str) on the device (load_obj, mesh.rs:474-642) and append
        it with the mesh object's transform (scene.rs:838-861); returns this call's
        (n_vertices, n_triangles)."""
        data = text.encode() if isinstance(text, str) else bytes(text)
        xf = None
        if translate is not None or rotate is not None or scale is not None:
            xf = N.MeshTransform()
            if translate is not None:
                xf.has_translate = 1
                xf.translate[:] = [float(x) for x in translate]
            if rotate is not None:
                xf.has_rotate = 1
                xf.rotate_deg[:] = [float(x) for x in rotate]
            if scale is not None:
                xf.has_scale = 1
                xf.scale = float(scale)
        nv, nt = c_uint32(), c_uint32()
        self._check(lib().mcrt_mesh_append_obj(self._h, data, len(data), mat_idx,
                                               None if xf is None else ctypes.byref(xf),
                                               None if source is None else source.encode(), ctypes.byref(nv),
                                               ctypes.byref(nt)))
        return nv.value, nt.value

    def mesh_obj_stats(self):
        """The last mesh_append_obj: dict of the text copy and kernel times (ms) and the
        text bytes, lines, face tokens and kernel launches."""
        ms = (c_float * 2)()
        cnt = (c_uint64 * 4)()
        self._check(lib().mcrt_mesh_obj_stats(self._h, ms, cnt))
        return dict(h2d_ms=ms[0], kernel_ms=ms[1], bytes=cnt[0], lines=cnt[1], tokens=cnt[2], launches=cnt[3])

    def mesh_counts(self):
        nv, nt = c_uint32(), c_uint32()
        self._check(lib().mcrt_mesh_read(self._h, None, 0, None, 0, ctypes.byref(nv), ctypes.byref(nt)))
        return nv.value, nt.value

    def mesh_read(self):
        """The device mesh as (vertices, triangles) host records."""
        nv, nt = self.mesh_counts()
        v = np.zeros(nv, VERTEX)
        t = np.zeros(nt, TRIANGLE)
        self._check(lib().mcrt_mesh_read(self._h, ptr(v), nv, ptr(t), nt, None, None))
        return v, t

    def mesh_append_scene_yaml(self, path):
        """Load a scene YAML with its mesh objects left unparsed and append its geometry
        to the device mesh in object order (OBJ text parsed on the device); returns the
        host Scene (spheres, materials, camera; its vertices hold the primitives only)."""
        h = c_void_p()
        check(lib().mcrt_scene_load_yaml_ex(path.encode(), N.LOAD_DEFER_MESHES, ctypes.byref(h)))
        try:
            self._check(lib().mcrt_mesh_append_scene(self._h, h))
            return _scene_from_handle(h)
        finally:
            lib().mcrt_scene_free(h)

    # ---------------------------------------------------------------- voxel world
    def world_generate(self, params, read_back=False):
        """Generate the voxel grid on the GPU from a dict of mcrt_world_params fields;
        returns the grid (nx, ny, nz) uint8 when read_back."""
        p = N.WorldParams(**params)
        vox = np.zeros((p.nx, p.ny, p.nz), np.uint8) if read_back else None
        self._check(lib().mcrt_world_generate(self._h, ctypes.byref(p), ptr(vox)))
        return vox

    def world_upload(self, voxels, chunk_x0=0, chunk_z0=0):
        v = np.ascontiguousarray(voxels, np.uint8)
        nx, ny, nz = v.shape
        self._check(lib().mcrt_world_upload(self._h, ptr(v), nx, ny, nz, chunk_x0, chunk_z0))

    def world_mesh(self, block_material, voxel_size=0.125, greedy=True):
        """Mesh the device voxel grid; returns (n_vertices, n_triangles)."""
        mm = np.zeros(256, np.uint32)
        bm = np.asarray(block_material, np.uint32).ravel()
        mm[:len(bm)] = bm
        nv, nt = c_uint32(), c_uint32()
        self._check(lib().mcrt_world_mesh(self._h, N.MESH_GREEDY if greedy else N.MESH_FACES, ptr(mm),
                                          float(voxel_size), ctypes.byref(nv), ctypes.byref(nt)))
        self._world_tris = nt.value
        return nv.value, nt.value

    def world_read_mesh(self):
        nt = self._world_tris
        nv = 2 * nt
        v = np.zeros(nv, VERTEX)
        t = np.zeros(nt, TRIANGLE)
        self._check(lib().mcrt_world_read_mesh(self._h, ptr(v), nv, ptr(t), nt))
        return v, t

    def update_vertices(self, vertices):
        ver = _arr(vertices, VERTEX)
        self._check(lib().mcrt_update_vertices(self._h, ptr(ver), len(ver)))

    def rebuild_bvh(self):
        self._check(lib().mcrt_rebuild_bvh(self._h))

    def mesh_bvh(self):
        n = c_uint32()
        self._check(lib().mcrt_get_mesh_bvh(self._h, None, 0, ctypes.byref(n), None))
        nodes = np.zeros(n.value, NODE)
        order = np.zeros(self.n_triangles, np.uint32)
        self._check(lib().mcrt_get_mesh_bvh(self._h, ptr(nodes), n.value, ctypes.byref(n), ptr(order)))
        return nodes, order

    def trace_closest(self, rays, reference_layout=False) -> np.ndarray:
        rays = _arr(rays, RAY)
        hits = np.zeros(len(rays), HIT)
        self._check(lib().mcrt_trace_closest(self._h, ptr(rays), len(rays), ptr(hits),
                                             N.TRACE_REFERENCE_LAYOUT if reference_layout else 0))
        return hits

    def render(self, camera, width, height, spp, first_frame=0, max_depth=0, nee=False, spp_per_pass=0,
               keep=False, outputs=("rgba", "sum", "gbuf"), graph=False, cache=False, out_rgba=None, variant=None,
               count=False):
        """Render; outputs names the host arrays to return.  out_rgba: a caller-owned (height, width, 4)
        float32 C-contiguous array (pinned host memory for the fastest copy) that receives the image.
        variant: a closest-hit kernel variant (0..7) instead of the context's autotuned one.
        count: the closest-hit kernels count their node and triangle record fetches (timings())."""
        cam = _arr(camera, CAMERA)
        o = N.RenderOpts(max_depth=max_depth, flags=(N.RENDER_NEE if nee else 0) |
                         (N.RENDER_KEEP_ACCUM if keep else 0) | (N.RENDER_GRAPH if graph else 0) |
                         (N.RENDER_CACHE if cache else 0) | (N.RENDER_COUNT if count else 0),
                         spp_per_pass=spp_per_pass, variant=0 if variant is None else variant + 1)
        if out_rgba is not None:
            if (out_rgba.dtype != np.float32 or out_rgba.shape != (height, width, 4)
                    or not out_rgba.flags["C_CONTIGUOUS"]):
                raise TypeError("out_rgba must be a C-contiguous float32 array of shape (height, width, 4)")
            rgba = out_rgba
        else:
            rgba = np.zeros((height, width, 4), np.float32) if "rgba" in outputs else None
        acc = np.zeros((height, width, 3), np.float64) if "sum" in outputs else None
        gb = np.zeros((height, width, 4), np.float32) if "gbuf" in outputs else None
        self._check(lib().mcrt_render(self._h, ptr(cam), width, height, spp, first_frame, ctypes.byref(o),
                                      ptr(rgba), ptr(acc), ptr(gb)))
        self._last_hw = (height, width)
        return dict(rgba=rgba, sum=acc, gbuf=gb)

    def read_accum(self):
        """The last render's accumulation: the running mean (h, w, 4) and the f64 sums (h, w, 3); after
        render_views, one row holding every view's pixels in view order."""
        h, w = self._last_hw
        mean = np.zeros((h, w, 4), np.float32)
        acc = np.zeros((h, w, 3), np.float64)
        self._check(lib().mcrt_read_accum(self._h, ptr(mean), ptr(acc), None))
        return mean, acc

    def render_views(self, views, spp, first_frame=0, max_depth=0, nee=False, spp_per_pass=0, graph=False,
                     read_back=True, keep=False, cache=False):
        """Trace several cameras of uneven sizes together.  views: list of (camera, width, height);
        returns the views' running means (list of (h, w, 4) arrays) when read_back.  keep continues
        the previous call's accumulation; cache terminates paths into the radiance cache."""
        vv = np.zeros(len(views), N.VIEW)
        for k, (cam, w, h) in enumerate(views):
            vv[k]["cam"] = _arr(cam, CAMERA)
            vv[k]["width"], vv[k]["height"] = w, h
        o = N.RenderOpts(max_depth=max_depth, flags=(N.RENDER_NEE if nee else 0) | (N.RENDER_GRAPH if graph else 0) |
                         (N.RENDER_KEEP_ACCUM if keep else 0) | (N.RENDER_CACHE if cache else 0),
                         spp_per_pass=spp_per_pass)
        outs = [np.zeros((h, w, 4), np.float32) for (_, w, h) in views] if read_back else []
        ptrs = (c_void_p * len(views))(*[o_.ctypes.data for o_ in outs]) if read_back else None
        self._check(lib().mcrt_render_views(self._h, ptr(vv), len(views), spp, first_frame, ctypes.byref(o),
                                            ctypes.cast(ptrs, c_void_p) if read_back else None))
        total = int(sum(w * h for (_, w, h) in views))
        self._last_hw = (1, total)
        return outs

    # ---------------------------------------------------------------- radiance cache
    def cache_config(self, query_vertex=1, train_stride=64, train_steps=4, train_batch=1 << 14, lr=1e-3, lo=None,
                     hi=None, max_bias=0.0):
        """Rendering with the cache (render(..., cache=True)); lo / hi None: the scene's bounds.
        max_bias > 0: render as the plain tracer (training on) while the judged bias exceeds it."""
        p = N.CacheParams(query_vertex=query_vertex, train_stride=train_stride, train_steps=train_steps,
                          train_batch=train_batch, lr=lr, max_bias=max_bias)
        if lo is not None:
            for k in range(3):
                p.lo[k], p.hi[k] = float(lo[k]), float(hi[k])
        self._check(lib().mcrt_cache_config(self._h, ctypes.byref(p)))

    def cache_stats(self):
        """The bias judge of the last cached render: relative bias per channel
        (sum of prediction - target over sum of target, on the training paths'
        samples), samples judged, and whether paths stopped into the cache."""
        out = (c_double * 5)()
        self._check(lib().mcrt_cache_stats(self._h, out))
        return {"bias": [out[0], out[1], out[2]], "samples": int(out[3]), "stopped": bool(out[4])}

    def cache_bench(self, n=1 << 20, reps=10):
        """(inference ms, training-step ms) on n synthetic queries / samples (device time)."""
        out = (c_float * 2)()
        self._check(lib().mcrt_cache_bench(self._h, n, reps, out))
        return out[0], out[1]

    def cache_init(self, seed=0):
        self._check(lib().mcrt_cache_init(self._h, seed))

    def cache_params(self) -> np.ndarray:
        p = np.zeros(lib().mcrt_cache_param_count(), np.float32)
        self._check(lib().mcrt_cache_get_params(self._h, ptr(p)))
        return p

    def cache_set_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == lib().mcrt_cache_param_count()
        self._check(lib().mcrt_cache_set_params(self._h, ptr(p)))

    def cache_set_bounds(self, lo, hi):
        lo = np.ascontiguousarray(lo, np.float32)
        hi = np.ascontiguousarray(hi, np.float32)
        self._check(lib().mcrt_cache_set_bounds(self._h, ptr(lo), ptr(hi)))

    def cache_infer(self, queries) -> np.ndarray:
        """Predictions (n, 3) for (n, 12) queries: position, outgoing direction, normal, albedo."""
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 12)
        out = np.zeros((len(q), 3), np.float32)
        self._check(lib().mcrt_cache_infer(self._h, ptr(q), len(q), ptr(out)))
        return out

    def cache_train(self, samples, steps=1, batch=0, lr=1e-3, want_grad=False):
        """Adam steps on (n, 16) samples (query, target, weight); returns (loss per step,
        gradient of the first step or None).  steps=0: gradient only."""
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 16)
        loss = np.zeros(max(steps, 1), np.float32)
        grad = np.zeros(lib().mcrt_cache_param_count(), np.float32) if want_grad else None
        self._check(lib().mcrt_cache_train(self._h, ptr(s), len(s), steps, batch, float(lr), ptr(loss), ptr(grad)))
        return loss, grad

    def update_materials(self, materials):
        """Replace the material table (same emissive slots) without re-uploading geometry."""
        md = _arr(materials, MATERIAL_DATA)
        self._check(lib().mcrt_update_materials(self._h, ptr(md)))

    def adjoint(self, camera, width, height, spp, d_image, first_frame=0, max_depth=0, nee=False,
                with_image=False):
        """Path-replay backpropagation: gradient of sum(d_image * image) with respect to the
        material parameters, as a (64, 4) array (albedo r, g, b, roughness per slot).
        d_image: (height, width, 3 or 4) = dLoss/d(image)."""
        cam = _arr(camera, CAMERA)
        d = np.zeros((height, width, 4), np.float32)
        di = np.asarray(d_image, np.float32).reshape(height, width, -1)
        d[..., :di.shape[-1]] = di
        o = N.RenderOpts(max_depth=max_depth, flags=N.RENDER_NEE if nee else 0)
        grad = np.zeros(256, np.float64)
        rgba = np.zeros((height, width, 4), np.float32) if with_image else None
        self._check(lib().mcrt_adjoint(self._h, ptr(cam), width, height, spp, first_frame, ctypes.byref(o), ptr(d),
                                       ptr(grad), ptr(rgba)))
        self._last_hw = (height, width)
        return (grad.reshape(64, 4), rgba) if with_image else grad.reshape(64, 4)

    def autotune(self, camera, width, height, spp, max_depth=0, nee=False):
        """Pick the fastest closest-hit kernel variant for this scene; returns (variant, extend ms per variant)."""
        cam = _arr(camera, CAMERA)
        o = N.RenderOpts(max_depth=max_depth, flags=N.RENDER_NEE if nee else 0)
        v = c_uint32()
        ms = (c_float * 8)()
        self._check(lib().mcrt_autotune(self._h, ptr(cam), width, height, spp, ctypes.byref(o), ctypes.byref(v), ms))
        self._last_hw = (height, width)
        return v.value, [ms[i] for i in range(8)]

    def image_rgba8(self, aces=False) -> np.ndarray:
        """Tone-map the last render on the GPU (Reinhard + gamma 2.2, or ACES + sRGB)."""
        n = ctypes.c_uint32()
        out = np.zeros((self._last_hw[0], self._last_hw[1], 4), np.uint8)
        self._check(lib().mcrt_read_image_rgba8(self._h, 1 if aces else 0, ptr(out)))
        return out

    def timings(self):
        ms = (c_float * 6)()
        cnt = (c_uint64 * 8)()
        self._check(lib().mcrt_last_timings(self._h, ms, cnt))
        keys = ["total", "extend", "shade", "shadow", "resolve", "bvh_build"]
        d = {f"{k}_ms": ms[i] for i, k in enumerate(keys)}
        d["rays"] = cnt[0]
        d["shadow_rays"] = cnt[1]
        d["render_launches"] = cnt[2]
        d["build_launches"] = cnt[3]
        d["extend_launches"] = cnt[4]
        d["stackless_rays"] = cnt[5]
        d["node_fetches"] = cnt[6]
        d["triangle_fetches"] = cnt[7]
        return d

    def copy_bandwidth(self, nbytes, reps=20):
        """GB/s (read + write) of the library's float4 copy kernel over two nbytes buffers."""
        g = c_float()
        self._check(lib().mcrt_copy_bandwidth(self._h, int(nbytes), int(reps), ctypes.byref(g)))
        return g.value

    def denoise_accum(self, radius=3, sigma_s=2.0, sigma_d=0.5, normal_pow=8.0, sigma_color=0.0, sigma_normal=0.0,
                      read_back=True):
        """Denoise the device accumulation of the last render with its G-buffer."""
        h, w = self._last_hw
        p = N.DenoiseParams(radius=radius, sigma_s=sigma_s, sigma_d=sigma_d, normal_pow=normal_pow,
                            sigma_color=sigma_color, sigma_normal=sigma_normal)
        out = np.zeros((h, w, 4), np.float32) if read_back else None
        self._check(lib().mcrt_denoise_accum(self._h, ctypes.byref(p), ptr(out)))
        return out

    def denoise(self, rgba, gbuf, radius=3, sigma_s=2.0, sigma_d=0.5, normal_pow=8.0, sigma_color=0.0,
                sigma_normal=0.0):
        rgba = np.ascontiguousarray(rgba, np.float32)
        gbuf = np.ascontiguousarray(gbuf, np.float32)
        h, w = rgba.shape[:2]
        p = N.DenoiseParams(radius=radius, sigma_s=sigma_s, sigma_d=sigma_d, normal_pow=normal_pow,
                            sigma_color=sigma_color, sigma_normal=sigma_normal)
        out = np.zeros_like(rgba)
        self._check(lib().mcrt_denoise(self._h, ptr(rgba), ptr(gbuf), w, h, ctypes.byref(p), ptr(out)))
        return out
