"""Loader for the oracle libraries -- test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module, and only as the checker.  Two libraries live here:

* ``oracle/_build/liborc.so``: the CPU restatement of the reference path tracer
  (``pt_oracle.cpp``), built from this directory by :func:`build_restatement`.
* ``oracle/_ref/libmcrt_ref.so``: the reference renderer's own C++ sources compiled
  by ``oracle/Makefile`` from the staged copy ``baseline/_ref`` (``oracle/stage_reference.py``).
  Only present where those sources are; :func:`load_reference` returns None otherwise.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
ORC_SO = os.path.join(BUILD_DIR, "liborc.so")
REF_SO = os.path.join(HERE, "_ref", "libmcrt_ref.so")

P = ctypes.c_void_p
I = ctypes.c_int
F = ctypes.c_float
LL = ctypes.c_longlong


def build_restatement(force: bool = False) -> str:
    """Compile pt_oracle.cpp (g++, no FMA contraction so x86 and aarch64 agree)."""
    src = os.path.join(HERE, "pt_oracle.cpp")
    if not force and os.path.exists(ORC_SO) and os.path.getmtime(ORC_SO) >= os.path.getmtime(src):
        return ORC_SO
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = ORC_SO + ".tmp"
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
                    src, "-o", tmp], check=True)
    os.replace(tmp, ORC_SO)
    return ORC_SO


def build_reference() -> str | None:
    """Compile the reference sources into oracle/_ref when they are present here (staged
    into baseline/_ref from a checkout, or already staged)."""
    from oracle.stage_reference import stage
    src = stage()
    if src is None:
        return None
    subprocess.run(["make", "-s", "-C", HERE, f"REF={src}", f"-j{os.cpu_count() or 4}"], check=True)
    return REF_SO


SEAM_SO = os.path.join(HERE, "_ref", "libmcrt_ref_gb300.so")


def build_seam() -> str | None:
    """The reference build with the library behind its seams (SceneBVH backend and the
    integrator-seam converter linked against libmcrt_gb300.so): oracle/_ref/libmcrt_ref_gb300.so.
    Needs the reference sources and the built library; None where either is missing."""
    from oracle.stage_reference import source_dir
    src = source_dir()
    lib = os.path.join(os.path.dirname(HERE), "mcrt_gb300", "_lib", "libmcrt_gb300.so")
    if src is None or not os.path.exists(lib):
        return None
    subprocess.run(["make", "-s", "-C", HERE, f"REF={src}", f"-j{os.cpu_count() or 4}", "seam"], check=True)
    return SEAM_SO


_orc = None
_ref = None


def load_restatement():
    global _orc
    if _orc is None:
        lib = ctypes.CDLL(build_restatement())
        lib.orc_scene_create.restype = P
        lib.orc_scene_create.argtypes = [I, P, P, P, I, P, P, I, P, I, I]
        lib.orc_scene_destroy.argtypes = [P]
        lib.orc_scene_set_tree.argtypes = [P, P, P, I, P, P, I]
        lib.orc_render.restype = LL
        lib.orc_render.argtypes = [P, P, P, ctypes.c_ulonglong, I, I, I, P, P, P, P, I, P, I, P]
        lib.orc_last_extension_rays.restype = LL
        lib.orc_last_extension_rays.argtypes = []
        lib.orc_trace.argtypes = [P, P, LL, I, P, P]
        lib.orc_linear_trace.argtypes = [P, P, LL, P, P, I]
        lib.orc_material_sample.argtypes = [I, P, F, F, P, P, F, F, P, P, P]
        lib.orc_material_evaluate.argtypes = [I, P, F, F, P, P, P, P, P]
        lib.orc_fresnel.restype = F
        lib.orc_fresnel.argtypes = [F, F]
        lib.orc_onb_to_world.argtypes = [P, P, P]
        lib.orc_sample_hemisphere_cosine.argtypes = [F, F, P]
        lib.orc_camera_ray.argtypes = [P, I, I, F, F, P, P]
        lib.orc_discrete_sample.restype = I
        lib.orc_discrete_sample.argtypes = [P, I, F, P]
        lib.orc_envmap_create.restype = P
        lib.orc_envmap_create.argtypes = [P, I, I]
        lib.orc_envmap_destroy.argtypes = [P]
        lib.orc_envmap_sample.argtypes = [P, F, F, F, F, P, P, P]
        lib.orc_envmap_pdf.restype = F
        lib.orc_envmap_pdf.argtypes = [P, P]
        lib.orc_envmap_radiance.argtypes = [P, P, P]
        lib.orc_envmap_sample_texel.argtypes = [P, F, F, P, P]
        lib.orc_pcg32.argtypes = [ctypes.c_ulonglong, ctypes.c_uint, ctypes.c_uint, I, P]
        lib.orc_film_hdr.restype = LL
        lib.orc_film_hdr.argtypes = [I, I, P, P, LL]
        lib.orc_film_ppm.restype = LL
        lib.orc_film_ppm.argtypes = [I, I, P, P, LL]
        lib.orc_film_tonemap.argtypes = [I, I, P, I, F]
        lib.orc_scene_set_alpha.argtypes = [P, P]
        lib.orc_consistent_normal.argtypes = [P, P, P, P, F, F, P]
        _orc = lib
    return _orc


def load_reference():
    """The reference's compiled sources, or None where they are not available."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            try:
                if build_reference() is None:
                    return None
            except (OSError, subprocess.CalledProcessError):
                return None
        lib = ctypes.CDLL(REF_SO)
        lib.ref_bvh_create.restype = P
        lib.ref_bvh_create.argtypes = [P, I, I]
        lib.ref_bvh_destroy.argtypes = [P]
        lib.ref_bvh_intersect.argtypes = [P, P, LL, P, P, P, P, I]
        lib.ref_scenebvh_intersect.restype = I
        lib.ref_scenebvh_intersect.argtypes = [P, P, LL, P, P, P]
        lib.ref_scenebvh_occluded.restype = I
        lib.ref_scenebvh_occluded.argtypes = [P, P, LL, P, P]
        lib.ref_bvh_dump_sizes.argtypes = [P, P, P]
        lib.ref_bvh_dump.argtypes = [P, P, P, P, P]
        lib.ref_material_sample.argtypes = [I, P, P, P, F, F, P, P, P, P]
        lib.ref_material_evaluate.argtypes = [I, P, P, P, P, P, P]
        lib.ref_fresnel.restype = F
        lib.ref_fresnel.argtypes = [F, F]
        lib.ref_onb_to_world.argtypes = [P, P, P]
        lib.ref_sample_hemisphere_cosine.argtypes = [F, F, P]
        lib.ref_camera_ray.argtypes = [P, P, I, I, F, F, F, P, P]
        lib.ref_discrete_sample.restype = I
        lib.ref_discrete_sample.argtypes = [P, I, F, P]
        lib.ref_triangle_sample_point.argtypes = [P, F, F, P, P]
        lib.ref_triangle_normal_area.argtypes = [P, P, P]
        lib.ref_envmap_load.restype = P
        lib.ref_envmap_load.argtypes = [ctypes.c_char_p]
        lib.ref_envmap_destroy.argtypes = [P]
        lib.ref_envmap_sample.argtypes = [P, F, F, P, P, P]
        lib.ref_envmap_pdf.restype = F
        lib.ref_envmap_pdf.argtypes = [P, P]
        lib.ref_envmap_radiance.argtypes = [P, P, P]
        lib.ref_render_pt.restype = I
        lib.ref_render_pt.argtypes = [P, P, P, I, P, P, I, ctypes.c_char_p, P, I, I, I, I, I, I, P, P, P, P]
        lib.ref_pt_scene_create.restype = P
        lib.ref_pt_scene_create.argtypes = [P, P, P, I, P, P, I, ctypes.c_char_p, P, I, I]
        lib.ref_pt_render.restype = I
        lib.ref_pt_render.argtypes = [P, I, I, I, I, I, I, P, P, P, P]
        lib.ref_pt_scene_destroy.argtypes = [P]
        lib.ref_load_obj.restype = I
        lib.ref_load_obj.argtypes = [ctypes.c_char_p, P, P, P, P]
        lib.ref_cornell_export.restype = I
        lib.ref_cornell_export.argtypes = [P, P, P, P]
        lib.ref_cornell_paths.restype = I
        lib.ref_cornell_paths.argtypes = [I, I, I, P, P]
        lib.ref_render_cornell.restype = I
        lib.ref_render_cornell.argtypes = [I, I, I, I, I, I, P, P, P, P]
        lib.ref_film_dump.argtypes = [I, I, P, ctypes.c_char_p, I]
        lib.ref_consistent_normal.argtypes = [P, P, P, P, F, F, P, P, P]
        lib.ref_mesh_alpha.argtypes = [P, I, P, I, P, P]
        lib.ref_film_tonemap.argtypes = [I, I, P, I, F]
        _ref = lib
    return _ref


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def film_encode(rgb: np.ndarray, hdr: bool) -> bytes:
    """The oracle's FrameBuffer::dumpHDR / dumpPPM bytes of an [h][w][3] image (row 0 the
    bottom row)."""
    lib = load_restatement()
    img = np.ascontiguousarray(rgb, np.float32)
    h, w = img.shape[:2]
    fn = lib.orc_film_hdr if hdr else lib.orc_film_ppm
    n = fn(w, h, ptr(img), None, 0)
    out = np.zeros(n, np.uint8)
    fn(w, h, ptr(img), ptr(out), n)
    return out.tobytes()


def film_tonemap(rgb: np.ndarray, reinhard: bool, gamma: float = 2.2) -> np.ndarray:
    """The oracle's FrameBuffer::tonemapReinhard / tonemapGamma(gamma) of an image."""
    lib = load_restatement()
    img = np.array(rgb, np.float32, copy=True, order="C")
    lib.orc_film_tonemap(img.shape[1], img.shape[0], ptr(img), 1 if reinhard else 0, gamma)
    return img


class OracleScene:
    """A scene held by the CPU restatement (precision 32 or 64)."""

    def __init__(self, scene, precision: int = 64):
        lib = load_restatement()
        self.lib = lib
        self.scene = scene
        v = np.ascontiguousarray(scene.vertices, np.float32)
        n = None if scene.normals is None else np.ascontiguousarray(scene.normals, np.float32)
        mid = np.ascontiguousarray(scene.material_ids, np.int32)
        mt = np.ascontiguousarray(scene.material_types, np.int32)
        mp = np.ascontiguousarray(scene.material_params_array(), np.float32)
        env = None if scene.envmap is None else np.ascontiguousarray(scene.envmap, np.float32)
        ew, eh = (0, 0) if env is None else (env.shape[1], env.shape[0])
        self._keep = (v, n, mid, mt, mp, env)
        self.h = lib.orc_scene_create(precision, ptr(v), ptr(n), ptr(mid), len(mid), ptr(mt), ptr(mp), len(mt),
                                      ptr(env), ew, eh)
        alpha = getattr(scene, "vertex_alpha", None)
        if alpha is not None:
            self._alpha = np.ascontiguousarray(alpha, np.float32)
            lib.orc_scene_set_alpha(self.h, ptr(self._alpha))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_scene_destroy(self.h)
            self.h = None

    def set_reference_tree(self, tree: dict):
        """Traverse `tree` (node_box, node_info, ref_prim, ref_box as dumped from the
        reference SplitBVH) with the reference's visit order and arithmetic."""
        nb = np.ascontiguousarray(tree["node_box"], np.float32)
        ni = np.ascontiguousarray(tree["node_info"], np.int32)
        rp = np.ascontiguousarray(tree["ref_prim"], np.int32)
        rb = np.ascontiguousarray(tree["ref_box"], np.float32)
        self._tree = (nb, ni, rp, rb)
        self.lib.orc_scene_set_tree(self.h, ptr(nb), ptr(ni), ni.shape[0], ptr(rp), ptr(rb), rp.shape[0])
        return self

    def render(self, camera, width, height, spp, max_depth, rr_depth=-1, seed=0, rows=None, threads=None,
               keep_paths=False, dLdI=None, n_albedo=0, n_emission=0, ref_stream=0):
        """Returns dict(mean, var_of_mean, rays, extension_rays, paths?, g_albedo?, g_emission?)."""
        r0, r1 = (0, height) if rows is None else rows
        threads = threads or os.cpu_count() or 1
        cam = np.ascontiguousarray(camera, np.float32)
        ip = np.array([width, height, spp, max_depth, rr_depth, ref_stream], np.int32)
        s = np.zeros((height, width, 3), np.float64)
        s2 = np.zeros((height, width, 3), np.float64)
        paths = np.zeros((height, width, spp, 3), np.float32) if keep_paths else None
        dl = None if dLdI is None else np.ascontiguousarray(dLdI, np.float32)
        ga = np.zeros((max(n_albedo, 0), 3), np.float64)
        ge = np.zeros((max(n_emission, 0), 3), np.float64)
        rays = self.lib.orc_render(self.h, ptr(cam), ptr(ip), seed & ((1 << 64) - 1), r0, r1, threads, ptr(s),
                                   ptr(s2), ptr(paths), ptr(dl), n_albedo, ptr(ga), n_emission, ptr(ge))
        mean = s / spp
        var = np.maximum(s2 / spp - mean * mean, 0.0) / max(spp - 1, 1)
        out = {"mean": mean, "var_of_mean": var, "rays": int(rays),
               "extension_rays": int(self.lib.orc_last_extension_rays())}
        if keep_paths:
            out["paths"] = paths
        if dl is not None:
            out["g_albedo"] = ga
            out["g_emission"] = ge
        return out

    def linear_trace(self, rays: np.ndarray, threads: int | None = None):
        """Closest hits of (n, 8) rays by testing every triangle (float scenes): the
        reference's DebugMesh linear scan.  Returns (t, prim); misses have t = inf, prim -1."""
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        t = np.empty(n, np.float32)
        p = np.empty(n, np.int32)
        self.lib.orc_linear_trace(self.h, ptr(rays), n, ptr(t), ptr(p), threads or os.cpu_count() or 1)
        return t, p

    def trace(self, rays: np.ndarray, any_hit: bool = False):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        t = np.zeros(n, np.float32)
        p = np.zeros(n, np.int32)
        self.lib.orc_trace(self.h, ptr(rays), n, 1 if any_hit else 0, ptr(t), ptr(p))
        return t, p
