"""ctypes bindings of include/mcrt_gb300.h.

The library is the in-tree ``mcrt_gb300/_lib/libmcrt_gb300.so`` built by
``mcrt_gb300.build``.  There is no fallback: if the library cannot be loaded every
call raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libmcrt_gb300.so")

c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_float = ctypes.c_float
c_void_p = ctypes.c_void_p

MCRT_OK = 0
ERRORS = {
    -1: "invalid argument", -2: "CUDA error", -3: "out of memory", -4: "queue overflow",
    -5: "stack overflow", -6: "internal error", -7: "I/O error",
}

TRAVERSE_FAST = 0
TRAVERSE_REF = 1
PTR_HOST = 0
PTR_DEVICE = 1
PROFILE_STAGES = 1
PROFILE_COUNT = 2
VARIANT_STACK32 = 1
VARIANT_REGCAP = 2
VARIANT_EXPLICIT = 4
VARIANT_GRIDSTRIDE = 8
FILM_HDR = 0
FILM_PPM = 1
TONEMAP_GAMMA = 0
TONEMAP_REINHARD = 1
SCHEDULE_STREAM = 0
SCHEDULE_WAVES = 1
SCHEDULE_PATHS = 2  # the plain GPU path tracer: one thread per path
BUILD_SAH = 0
BUILD_EXTERNAL = 1
BUILD_SAH_SPLIT = 2
MAT_CONSISTENT = 0x100


class Material(ctypes.Structure):
    _fields_ = [("type", c_int32), ("color", c_float * 3), ("roughness", c_float), ("ior", c_float),
                ("albedo_param", c_int32), ("emission_param", c_int32)]


class BvhTree(ctypes.Structure):
    _fields_ = [("num_nodes", c_int32), ("num_refs", c_int32), ("node_box", c_void_p), ("node_info", c_void_p),
                ("ref_prim", c_void_p), ("ref_box", c_void_p)]


class SceneDesc(ctypes.Structure):
    _fields_ = [("num_triangles", c_int64), ("vertices", c_void_p), ("normals", c_void_p),
                ("material_ids", c_void_p), ("num_materials", c_int32), ("materials", ctypes.POINTER(Material)),
                ("env_width", c_int32), ("env_height", c_int32), ("env_rgb", c_void_p), ("builder", c_int32),
                ("leaf_size", c_int32), ("external_tree", ctypes.POINTER(BvhTree)), ("vertex_alpha", c_void_p)]


class Ray(ctypes.Structure):
    _fields_ = [("org", c_float * 3), ("tmin", c_float), ("dir", c_float * 3), ("tmax", c_float)]


class Hit(ctypes.Structure):
    _fields_ = [("t", c_float), ("u", c_float), ("v", c_float), ("prim", c_int32)]


class Camera(ctypes.Structure):
    _fields_ = [("origin", c_float * 3), ("target", c_float * 3), ("up", c_float * 3), ("fov_y", c_float),
                ("width", c_int32), ("height", c_int32)]


class RenderParams(ctypes.Structure):
    _fields_ = [("spp", c_int32), ("max_depth", c_int32), ("rr_depth", c_int32), ("seed", ctypes.c_uint64),
                ("traverse", c_int32), ("ptr_mode", c_int32), ("path_chunk", c_int64), ("block_size", c_int32),
                ("use_graph", c_int32), ("profile", c_int32), ("variant", c_int32), ("schedule", c_int32),
                ("reserved", c_int32)]


class RenderStats(ctypes.Structure):
    _fields_ = [("paths", c_int64), ("extension_rays", c_int64), ("shadow_rays", c_int64), ("waves", c_int32),
                ("kernel_launches", c_int32), ("device_ms", c_float), ("stage_ms", c_float * 4),
                ("extend_launches", c_int32), ("ext_nodes", c_int64), ("ext_tris", c_int64), ("nee_nodes", c_int64),
                ("nee_tris", c_int64), ("h2d_bytes", c_int64), ("d2h_bytes", c_int64), ("node_bytes", c_int32),
                ("reserved0", c_int32)]


TUNE_MAX = 16


class TuneReport(ctypes.Structure):
    _fields_ = [("num_candidates", c_int32), ("chosen", c_int32), ("probe_paths", c_int64),
                ("path_chunk", c_int64 * TUNE_MAX), ("variant", c_int32 * TUNE_MAX), ("ms", c_float * TUNE_MAX)]


EXPORTS = {
    "mcrt_get_abi_version": (c_int32, []),
    "mcrt_last_error": (ctypes.c_char_p, []),
    "mcrt_scene_create": (c_int32, [ctypes.POINTER(SceneDesc), ctypes.POINTER(c_void_p)]),
    "mcrt_scene_destroy": (c_int32, [c_void_p]),
    "mcrt_scene_set_materials": (c_int32, [c_void_p, c_int32, ctypes.POINTER(Material), c_void_p]),
    "mcrt_scene_info": (c_int32, [c_void_p, ctypes.POINTER(c_int64), ctypes.POINTER(c_int64),
                                  ctypes.POINTER(c_int64), ctypes.POINTER(c_int64)]),
    "mcrt_trace_closest": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_int32, c_int32, c_void_p]),
    "mcrt_trace_any": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_int32, c_int32, c_void_p]),
    "mcrt_render": (c_int32, [c_void_p, ctypes.POINTER(Camera), ctypes.POINTER(RenderParams), c_void_p,
                              ctypes.POINTER(RenderStats), c_void_p]),
    "mcrt_render_adjoint": (c_int32, [c_void_p, ctypes.POINTER(Camera), ctypes.POINTER(RenderParams), c_void_p,
                                      c_void_p, c_int32, c_void_p, c_int32, ctypes.POINTER(RenderStats), c_void_p]),
    "mcrt_render_noalloc": (c_int32, [c_void_p, ctypes.POINTER(Camera), ctypes.POINTER(RenderParams), c_void_p,
                                      ctypes.POINTER(RenderStats), c_void_p]),
    "mcrt_render_adjoint_batch": (c_int32, [c_int32, ctypes.POINTER(c_void_p), ctypes.POINTER(Camera),
                                            ctypes.POINTER(RenderParams), ctypes.POINTER(c_void_p), c_void_p, c_int32,
                                            c_void_p, c_int32, ctypes.POINTER(RenderStats), c_void_p]),
    "mcrt_render_batch": (c_int32, [c_int32, ctypes.POINTER(c_void_p), ctypes.POINTER(Camera),
                                    ctypes.POINTER(RenderParams), ctypes.POINTER(c_void_p),
                                    ctypes.POINTER(RenderStats), c_void_p]),
    "mcrt_vertex_alpha": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p]),
    "mcrt_build_bvh": (c_int32, [c_void_p, c_int64, c_int32, ctypes.POINTER(c_int32), ctypes.POINTER(c_int32),
                                 c_void_p, c_void_p, c_void_p, c_void_p]),
    "mcrt_build_bvh_split": (c_int32, [c_void_p, c_int64, c_int32, ctypes.POINTER(c_int32),
                                       ctypes.POINTER(c_int32), c_void_p, c_void_p, c_void_p, c_void_p]),
    "mcrt_scene_desc_hash": (c_int32, [ctypes.POINTER(SceneDesc), ctypes.POINTER(ctypes.c_uint64)]),
    "mcrt_mesh_load_obj": (c_int32, [ctypes.c_char_p, c_void_p, ctypes.POINTER(c_int64), c_void_p, c_void_p,
                                     c_void_p]),
    "mcrt_envmap_load_bin": (c_int32, [ctypes.c_char_p, ctypes.POINTER(c_int32), ctypes.POINTER(c_int32), c_void_p]),
    "mcrt_scene_save": (c_int32, [c_void_p, ctypes.c_char_p]),
    "mcrt_scene_load": (c_int32, [ctypes.c_char_p, ctypes.c_uint64, ctypes.POINTER(c_void_p)]),
    "mcrt_film_encode": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_void_p, c_int64, ctypes.POINTER(c_int64),
                                   c_int32, c_void_p]),
    "mcrt_film_tonemap": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_float, c_int32, c_void_p]),
    "mcrt_probe_l2_read": (c_int32, [c_int64, c_int32, ctypes.POINTER(c_float), c_void_p]),
    "mcrt_autotune": (c_int32, [c_int32, ctypes.POINTER(c_void_p), ctypes.POINTER(Camera),
                                ctypes.POINTER(RenderParams), ctypes.POINTER(RenderParams),
                                ctypes.POINTER(TuneReport), c_void_p]),
}

_lib = None


class McrtError(RuntimeError):
    pass


def load(path: str = LIB_PATH):
    """Loads the native library (building it first if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            from .native_build import build
            build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in EXPORTS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(rc: int, what: str = "") -> None:
    if rc != MCRT_OK:
        msg = load().mcrt_last_error().decode(errors="replace")
        raise McrtError(f"{what}: {ERRORS.get(rc, rc)}: {msg}")
