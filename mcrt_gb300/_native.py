"""ctypes binding of libmcrt_cuda.so (include/mcrt_cuda.h).

The record dtypes are byte-identical to the reference's #[repr(C)] types:
GpuSphere (src/scene.rs:24-29), GpuBvhNode (src/bvh.rs:56-68), GpuVertex
(src/mesh.rs:26-34), GpuTriangle (src/mesh.rs:41-46), GpuMaterial /
GpuMaterialData (src/material.rs:37-63), CameraUniform (src/camera.rs:37-53).

The library is built in-tree by ``__graft_entry__.build()``; importing this
module without it raises, there is no fallback.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_uint32, c_uint64, c_uint8, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmcrt_cuda.so")
CLI_PATH = os.path.join(HERE, "mcrt_headless")

SPHERE = np.dtype([("center_r", "<f4", 4), ("mat_and_pad", "<u4", 4)])
NODE = np.dtype([("aabb_min", "<f4", 4), ("aabb_max", "<f4", 4), ("right_or_offset", "<u4"),
                 ("prim_count", "<u4"), ("pad", "<u4", 2)])
VERTEX = np.dtype([("position", "<f4", 4), ("normal", "<f4", 4), ("uv", "<f4", 4)])
TRIANGLE = np.dtype([("v", "<u4", 3), ("mat_idx", "<u4")])
MATERIAL = np.dtype([("type_pad", "<u4", 4), ("albedo_fuzz", "<f4", 4), ("ior_pad", "<f4", 4)])
MATERIAL_DATA = np.dtype([("mat_count", "<u4"), ("n_emissive", "<u4"), ("pad", "<u4", 2),
                          ("materials", MATERIAL, 64)])
CAMERA = np.dtype([("origin", "<f4", 4), ("lower_left", "<f4", 4), ("horizontal", "<f4", 4),
                   ("vertical", "<f4", 4), ("defocus_u", "<f4", 4), ("defocus_v", "<f4", 4),
                   ("frame_count", "<u4"), ("pad", "<u4", 3)])
RAY = np.dtype([("org", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
HIT = np.dtype([("t", "<f4"), ("prim", "<u4"), ("u", "<f4"), ("v", "<f4")])

assert SPHERE.itemsize == 32 and NODE.itemsize == 48 and VERTEX.itemsize == 48
assert TRIANGLE.itemsize == 16 and MATERIAL.itemsize == 48 and MATERIAL_DATA.itemsize == 3088
assert CAMERA.itemsize == 112 and RAY.itemsize == 32 and HIT.itemsize == 16

MAT_LAMBERTIAN, MAT_METAL, MAT_DIELECTRIC, MAT_EMISSIVE, MAT_GGX = 0, 1, 2, 3, 4
BACKFACE_CULL_FLAG = 0x80000000
HIT_MISS = 0xFFFFFFFF
HIT_SPHERE = 0x80000000
TRACE_REFERENCE_LAYOUT = 1
RENDER_NEE, RENDER_GBUFFER, RENDER_KEEP_ACCUM, RENDER_GRAPH = 1, 2, 4, 8
VIEW = np.dtype([("cam", CAMERA), ("width", "<u4"), ("height", "<u4"), ("_pad", "<u4", 2)])   # mcrt_view
ENV_W, ENV_H = 1024, 512

STATUS = {0: "OK", -1: "INVALID_ARG", -2: "OOM", -3: "CUDA", -4: "TIMEOUT", -5: "STACK_OVERFLOW",
          -6: "NO_SCENE", -7: "PARSE", -8: "IO", -9: "UNKNOWN_MATERIAL", -10: "MESH_LOAD",
          -11: "TOO_MANY_MATERIALS", -12: "UNSUPPORTED"}


class SceneDesc(ctypes.Structure):
    _fields_ = [("spheres", c_void_p), ("n_spheres", c_uint32),
                ("sphere_bvh", c_void_p), ("n_sphere_nodes", c_uint32),
                ("sphere_order", c_void_p),
                ("vertices", c_void_p), ("n_vertices", c_uint32),
                ("triangles", c_void_p), ("n_triangles", c_uint32),
                ("mesh_bvh", c_void_p), ("n_mesh_nodes", c_uint32),
                ("triangle_order", c_void_p),
                ("materials", c_void_p),
                ("env_rgba", c_void_p), ("env_w", c_uint32), ("env_h", c_uint32),
                ("albedo_rgba8", c_void_p), ("albedo_layers", c_uint32), ("albedo_size", c_uint32),
                ("flags", c_uint32), ("sun_dir", c_float * 4), ("sun_irradiance", c_float * 4)]


class CacheParams(ctypes.Structure):
    _fields_ = [("query_vertex", c_uint32), ("train_stride", c_uint32), ("train_steps", c_uint32),
                ("train_batch", c_uint32), ("lr", c_float), ("lo", c_float * 3), ("hi", c_float * 3),
                ("max_bias", c_float)]


RENDER_CACHE = 16
RENDER_COUNT = 32
SCENE_WORLD_MESH = 1
SCENE_DEVICE_MESH = 2
LOAD_DEFER_MESHES = 1
MESH_GREEDY, MESH_FACES = 0, 1


class WorldParams(ctypes.Structure):
    _fields_ = [("nx", c_uint32), ("ny", c_uint32), ("nz", c_uint32), ("seed", c_uint32),
                ("chunk_x0", c_int32), ("chunk_z0", c_int32),
                ("height_base", c_float), ("height_amp", c_float), ("height_freq", c_float),
                ("height_octaves", c_uint32), ("lacunarity", c_float), ("gain", c_float),
                ("cave_freq", c_float), ("cave_octaves", c_uint32), ("cave_threshold", c_float),
                ("cave_contrast", c_float), ("cave_min_y", c_uint32), ("sea_level", c_float), ("sand_line", c_float)]


class MeshTransform(ctypes.Structure):
    _fields_ = [("has_translate", c_uint32), ("has_rotate", c_uint32), ("has_scale", c_uint32),
                ("translate", c_float * 3), ("rotate_deg", c_float * 3), ("scale", c_float)]


class RenderOpts(ctypes.Structure):
    _fields_ = [("max_depth", c_uint32), ("flags", c_uint32), ("spp_per_pass", c_uint32), ("variant", c_uint32)]


class DenoiseParams(ctypes.Structure):
    _fields_ = [("radius", c_int32), ("sigma_s", c_float), ("sigma_d", c_float), ("normal_pow", c_float),
                ("sigma_color", c_float), ("sigma_normal", c_float), ("pad", c_uint32 * 2)]


class SceneView(ctypes.Structure):
    _fields_ = [("spheres", c_void_p), ("n_spheres", c_uint32),
                ("vertices", c_void_p), ("n_vertices", c_uint32),
                ("triangles", c_void_p), ("n_triangles", c_uint32),
                ("emissive_spheres", c_void_p), ("n_emissive_spheres", c_uint32),
                ("materials", c_void_p),
                ("has_camera", c_int32),
                ("look_from", c_float * 3), ("look_at", c_float * 3), ("vfov", c_float), ("aperture", c_float),
                ("focus_dist", c_float),
                ("env_map_path", c_char_p),
                ("n_material_names", c_uint32)]


# (name, restype, argtypes) for every entry point declared in include/mcrt_cuda.h
SIGNATURES = [
    ("mcrt_create", c_int, [c_int, c_void_p, POINTER(c_void_p)]),
    ("mcrt_destroy", None, [c_void_p]),
    ("mcrt_last_error", c_char_p, [c_void_p]),
    ("mcrt_version", c_char_p, []),
    ("mcrt_upload_scene", c_int, [c_void_p, POINTER(SceneDesc)]),
    ("mcrt_update_vertices", c_int, [c_void_p, c_void_p, c_uint32]),
    ("mcrt_rebuild_bvh", c_int, [c_void_p]),
    ("mcrt_get_mesh_bvh", c_int, [c_void_p, c_void_p, c_uint32, POINTER(c_uint32), c_void_p]),
    ("mcrt_trace_closest", c_int, [c_void_p, c_void_p, c_uint32, c_void_p, c_uint32]),
    ("mcrt_render", c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_uint32, c_uint32, POINTER(RenderOpts),
                            c_void_p, c_void_p, c_void_p]),
    ("mcrt_render_noalloc", c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_uint32, c_uint32,
                                    POINTER(RenderOpts), c_void_p]),
    ("mcrt_read_accum", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("mcrt_update_materials", c_int, [c_void_p, c_void_p]),
    ("mcrt_mlp_gemm_probe", c_int, [c_int, c_void_p, c_void_p, c_uint32, c_uint32, c_uint32, c_void_p]),
    ("mcrt_cache_param_count", c_uint32, []),
    ("mcrt_cache_config", c_int, [c_void_p, POINTER(CacheParams)]),
    ("mcrt_cache_stats", c_int, [c_void_p, c_void_p]),
    ("mcrt_cache_bench", c_int, [c_void_p, c_uint32, c_uint32, c_void_p]),
    ("mcrt_cache_init", c_int, [c_void_p, c_uint32]),
    ("mcrt_cache_set_params", c_int, [c_void_p, c_void_p]),
    ("mcrt_cache_get_params", c_int, [c_void_p, c_void_p]),
    ("mcrt_cache_set_bounds", c_int, [c_void_p, c_void_p, c_void_p]),
    ("mcrt_cache_infer", c_int, [c_void_p, c_void_p, c_uint32, c_void_p]),
    ("mcrt_cache_train", c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_uint32, c_float, c_void_p, c_void_p]),
    ("mcrt_render_views", c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_uint32, POINTER(RenderOpts), c_void_p]),
    ("mcrt_variant_info", c_int, [c_uint32, c_void_p]),
    ("mcrt_denoise_accum", c_int, [c_void_p, POINTER(DenoiseParams), c_void_p]),
    ("mcrt_world_generate", c_int, [c_void_p, POINTER(WorldParams), c_void_p]),
    ("mcrt_world_upload", c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_uint32, c_int32, c_int32]),
    ("mcrt_world_mesh", c_int, [c_void_p, c_uint32, c_void_p, c_float, POINTER(c_uint32), POINTER(c_uint32)]),
    ("mcrt_world_read_mesh", c_int, [c_void_p, c_void_p, c_uint32, c_void_p, c_uint32]),
    ("mcrt_mesh_reset", c_int, [c_void_p]),
    ("mcrt_mesh_append", c_int, [c_void_p, c_void_p, c_uint32, c_void_p, c_uint32]),
    ("mcrt_mesh_append_obj", c_int, [c_void_p, c_char_p, c_uint64, c_uint32, POINTER(MeshTransform), c_char_p,
                                     POINTER(c_uint32), POINTER(c_uint32)]),
    ("mcrt_mesh_read", c_int, [c_void_p, c_void_p, c_uint32, c_void_p, c_uint32, POINTER(c_uint32),
                               POINTER(c_uint32)]),
    ("mcrt_mesh_append_scene", c_int, [c_void_p, c_void_p]),
    ("mcrt_mesh_obj_stats", c_int, [c_void_p, POINTER(c_float), POINTER(c_uint64)]),
    ("mcrt_adjoint", c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_uint32, c_uint32, POINTER(RenderOpts),
                             c_void_p, c_void_p, c_void_p]),
    ("mcrt_autotune", c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_uint32, POINTER(RenderOpts),
                              POINTER(c_uint32), POINTER(c_float)]),
    ("mcrt_read_image_rgba8", c_int, [c_void_p, c_uint32, c_void_p]),
    ("mcrt_tonemap_aces_rgba8", c_int, [c_void_p, c_uint32, c_void_p]),
    ("mcrt_write_hdr", c_int, [c_char_p, c_void_p, c_uint32, c_uint32]),
    ("mcrt_last_timings", c_int, [c_void_p, POINTER(c_float), POINTER(c_uint64)]),
    ("mcrt_copy_bandwidth", c_int, [c_void_p, c_uint64, c_uint32, POINTER(c_float)]),
    ("mcrt_denoise", c_int, [c_void_p, c_void_p, c_void_p, c_uint32, c_uint32, POINTER(DenoiseParams), c_void_p]),
    ("mcrt_scene_load_yaml", c_int, [c_char_p, POINTER(c_void_p)]),
    ("mcrt_scene_load_yaml_str", c_int, [c_char_p, c_char_p, POINTER(c_void_p)]),
    ("mcrt_scene_load_yaml_ex", c_int, [c_char_p, c_uint32, POINTER(c_void_p)]),
    ("mcrt_scene_load_yaml_str_ex", c_int, [c_char_p, c_char_p, c_uint32, POINTER(c_void_p)]),
    ("mcrt_scene_free", None, [c_void_p]),
    ("mcrt_scene_view_get", c_int, [c_void_p, POINTER(SceneView)]),
    ("mcrt_scene_material_name", c_char_p, [c_void_p, c_uint32]),
    ("mcrt_compute_camera", c_int, [c_uint32, c_uint32, POINTER(c_float), POINTER(c_float), c_float, c_float,
                                    c_float, c_void_p]),
    ("mcrt_load_env_map", c_int, [c_char_p, c_void_p]),
    ("mcrt_gradient_env_map", c_int, [c_void_p]),
    ("mcrt_albedo_layers", c_int, [c_void_p]),
    ("mcrt_tonemap_rgba8", c_int, [c_void_p, c_uint32, c_void_p]),
    ("mcrt_write_png", c_int, [c_char_p, c_void_p, c_uint32, c_uint32]),
    ("mcrt_headless_run", c_int, [c_char_p, c_char_p, c_uint32, c_uint32, c_uint32, POINTER(RenderOpts)]),
]

_lib = None


def lib() -> ctypes.CDLL:
    """Load the in-tree CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class MCRTError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


def ptr(a):
    return None if a is None else a.ctypes.data_as(c_void_p)


def check(status: int, ctx=None):
    if status != 0:
        msg = lib().mcrt_last_error(ctx)
        raise MCRTError(status, msg.decode() if msg else "")
