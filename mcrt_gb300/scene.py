"""Host-side scene description and the GPU scene handle.

``SceneDesc`` mirrors what the reference's scene API accumulates before
``Scene::finalize`` (src/core/scene.h:28-103): a triangle soup with per-triangle
material ids (``Scene::add`` + ``todo_addMaterial``, scene.cpp:109-112,
material.cpp:135-139), optional vertex normals (``Scene::loadModel``), an
environment map (``Scene::setEnvmap``) and cameras (``Scene::setCamera``).
``GpuScene`` is the finalized, device-resident scene: the drop-in for the
reference's ``SceneBVH`` (intersect / occluded) and for ``DemoSimple::run``
(render), through the C ABI of include/mcrt_gb300.h.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

# MaterialType (src/core/material.h:7) plus the GGX conductor
LGHT, DIFF, SPEC, REFR, GLSY, GGX = 0, 1, 2, 3, 4, 8
CONSISTENT = 0x100  # OR'd into a type: shade with the consistent normal (TriangleObject::consistentNormal)


@dataclass
class Material:
    """Material(color, emission, type) (material.cpp:5-27) with the extension parameters."""
    type: int
    color: tuple = (1.0, 1.0, 1.0)
    roughness: float = 1.0     # GGX alpha (reference default m_roughness = 1)
    ior: float = 1.33          # reference: fixed 1.33 (material.h:51)
    albedo_param: int = -1     # adjoint parameter group (DIFF albedo)
    emission_param: int = -1   # adjoint parameter group (LGHT radiance)


@dataclass
class CameraDesc:
    """Scene::setCamera(origin, target, width, height, fov_y) (scene.cpp:224-232)."""
    origin: tuple
    target: tuple
    width: int
    height: int
    fov_y: float
    up: tuple = (0.0, 1.0, 0.0)

    def as_array(self) -> np.ndarray:
        return np.array(list(self.origin) + list(self.target) + list(self.up) + [self.fov_y], np.float32)

    def to_c(self) -> N.Camera:
        c = N.Camera()
        c.origin[:] = [float(v) for v in self.origin]
        c.target[:] = [float(v) for v in self.target]
        c.up[:] = [float(v) for v in self.up]
        c.fov_y = float(self.fov_y)
        c.width = int(self.width)
        c.height = int(self.height)
        return c


@dataclass
class SceneDesc:
    vertices: np.ndarray                 # (n, 9) float32: a, b, c
    material_ids: np.ndarray             # (n,) int32
    materials: list                      # list[Material]
    normals: np.ndarray | None = None    # (n, 9) float32: na, nb, nc
    envmap: np.ndarray | None = None     # (H, W, 3) float32, top row first
    vertex_alpha: np.ndarray | None = None  # (n, 3) float32 consistent-normal alphas (None: derived)
    name: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def num_triangles(self) -> int:
        return int(self.vertices.shape[0])

    @property
    def material_types(self) -> np.ndarray:
        return np.array([m.type for m in self.materials], np.int32)

    def material_params_array(self) -> np.ndarray:
        """(m, 8) float32: r, g, b, roughness, ior, albedo_param, emission_param, 0."""
        out = np.zeros((len(self.materials), 8), np.float32)
        for i, m in enumerate(self.materials):
            out[i, 0:3] = m.color
            out[i, 3] = m.roughness
            out[i, 4] = m.ior
            out[i, 5] = m.albedo_param
            out[i, 6] = m.emission_param
        return out

    def c_materials(self):
        arr = (N.Material * len(self.materials))()
        for i, m in enumerate(self.materials):
            arr[i].type = int(m.type)
            arr[i].color[:] = [float(c) for c in m.color]
            arr[i].roughness = float(m.roughness)
            arr[i].ior = float(m.ior)
            arr[i].albedo_param = int(m.albedo_param)
            arr[i].emission_param = int(m.emission_param)
        return arr


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _stream_ptr():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _c_desc(desc: SceneDesc, builder: str = "sah", external_tree: dict | None = None, leaf_size: int = 0):
    """The C description of a scene and the arrays it points into (keep them alive)."""
    v = np.ascontiguousarray(desc.vertices, np.float32).reshape(-1, 9)
    mid = np.ascontiguousarray(desc.material_ids, np.int32)
    nrm = None if desc.normals is None else np.ascontiguousarray(desc.normals, np.float32).reshape(-1, 9)
    env = None if desc.envmap is None else np.ascontiguousarray(desc.envmap, np.float32)
    mats = desc.c_materials()
    d = N.SceneDesc()
    d.num_triangles = v.shape[0]
    d.vertices = v.ctypes.data
    d.normals = None if nrm is None else nrm.ctypes.data
    d.material_ids = mid.ctypes.data
    d.num_materials = len(desc.materials)
    d.materials = mats
    if env is not None:
        d.env_height, d.env_width = env.shape[0], env.shape[1]
        d.env_rgb = env.ctypes.data
    d.leaf_size = int(leaf_size)
    alpha = None if desc.vertex_alpha is None else np.ascontiguousarray(desc.vertex_alpha, np.float32).reshape(-1, 3)
    d.vertex_alpha = None if alpha is None else alpha.ctypes.data
    keep = [v, mid, nrm, env, mats, alpha]
    if builder == "external":
        t = external_tree
        nb = np.ascontiguousarray(t["node_box"], np.float32)
        ni = np.ascontiguousarray(t["node_info"], np.int32)
        rp = np.ascontiguousarray(t["ref_prim"], np.int32)
        rb = np.ascontiguousarray(t["ref_box"], np.float32)
        tree = N.BvhTree(ni.shape[0], rp.shape[0], nb.ctypes.data, ni.ctypes.data, rp.ctypes.data, rb.ctypes.data)
        d.builder = N.BUILD_EXTERNAL
        d.external_tree = ctypes.pointer(tree)
        keep += [nb, ni, rp, rb, tree]
    elif builder == "sah_split":
        d.builder = N.BUILD_SAH_SPLIT
    elif builder == "sah":
        d.builder = N.BUILD_SAH
    else:
        raise ValueError(f"unknown builder {builder!r} (sah, sah_split, external)")
    return d, keep


def vertex_alpha(vertices, normals) -> np.ndarray:
    """mcrt_vertex_alpha: per-corner consistent-normal alphas (n, 3) of a triangle soup."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 9)
    nrm = np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
    out = np.zeros((v.shape[0], 3), np.float32)
    N.check(N.load().mcrt_vertex_alpha(v.ctypes.data, nrm.ctypes.data, v.shape[0], out.ctypes.data),
            "mcrt_vertex_alpha")
    return out


def load_obj(path: str, transform=None):
    """mcrt_mesh_load_obj: the triangles Scene::loadModel(path, transform, mat) adds
    (scene.cpp:368-408) -- vertices (n, 9), vertex normals (n, 9) and consistent-normal
    alphas (n, 3) of Mesh::genNormals.  transform: a 4x4 matrix acting on column vectors
    (as glm::mat4 in the reference), or None."""
    lib = N.load()
    t = None if transform is None else np.ascontiguousarray(np.asarray(transform, np.float32).T).ravel()
    tp = None if t is None else t.ctypes.data
    n = ctypes.c_int64(0)
    N.check(lib.mcrt_mesh_load_obj(path.encode(), tp, ctypes.byref(n), None, None, None), "mcrt_mesh_load_obj")
    v = np.zeros((n.value, 9), np.float32)
    nrm = np.zeros((n.value, 9), np.float32)
    alpha = np.zeros((n.value, 3), np.float32)
    N.check(lib.mcrt_mesh_load_obj(path.encode(), tp, ctypes.byref(n), v.ctypes.data, nrm.ctypes.data,
                                   alpha.ctypes.data), "mcrt_mesh_load_obj")
    return v, nrm, alpha


def load_envmap_bin(path: str) -> np.ndarray:
    """mcrt_envmap_load_bin: the (height, width, 3) float32 map EnvmapLoader reads from a
    .bin file (envmap.cpp:98-119), top row first -- SceneDesc's envmap layout."""
    lib = N.load()
    w, h = ctypes.c_int32(0), ctypes.c_int32(0)
    N.check(lib.mcrt_envmap_load_bin(path.encode(), ctypes.byref(w), ctypes.byref(h), None), "mcrt_envmap_load_bin")
    img = np.zeros((h.value, w.value, 3), np.float32)
    N.check(lib.mcrt_envmap_load_bin(path.encode(), ctypes.byref(w), ctypes.byref(h), img.ctypes.data),
            "mcrt_envmap_load_bin")
    return img


def build_bvh(vertices, leaf_size: int = 0, split: bool = False) -> dict:
    """mcrt_build_bvh (split: mcrt_build_bvh_split, with spatial splits): the library's
    binned-SAH tree of (n, 9) triangle vertices, in the form of a reference SplitBVH dump
    (node_box, node_info, ref_prim, ref_box; root 0)."""
    lib = N.load()
    fn = lib.mcrt_build_bvh_split if split else lib.mcrt_build_bvh
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 9)
    nn, nr = ctypes.c_int32(), ctypes.c_int32()
    N.check(fn(v.ctypes.data, v.shape[0], int(leaf_size), ctypes.byref(nn), ctypes.byref(nr),
               None, None, None, None), "mcrt_build_bvh")
    nb = np.zeros((nn.value, 6), np.float32)
    ni = np.zeros((nn.value, 6), np.int32)
    rp = np.zeros(nr.value, np.int32)
    rb = np.zeros((nr.value, 6), np.float32)
    N.check(fn(v.ctypes.data, v.shape[0], int(leaf_size), ctypes.byref(nn), ctypes.byref(nr),
               nb.ctypes.data, ni.ctypes.data, rp.ctypes.data, rb.ctypes.data), "mcrt_build_bvh")
    return {"node_box": nb, "node_info": ni, "ref_prim": rp, "ref_box": rb}


def sah_cost(tree: dict, c_node: float = 1.0, c_tri: float = 1.0, root: int = 0) -> float:
    """SAH cost of a binary tree in mcrt_bvh_tree form: sum over inner nodes of
    c_node * area / root area plus over leaves of c_tri * references * area / root area
    (areas as AABB::surfaceAreaCost, aabb.cpp:276-282)."""
    nb = np.asarray(tree["node_box"], np.float64).reshape(-1, 6)
    ni = np.asarray(tree["node_info"]).reshape(-1, 6)
    e = nb[:, 3:] - nb[:, :3]
    area = e[:, 0] * e[:, 1] + e[:, 1] * e[:, 2] + e[:, 0] * e[:, 2]
    leaf = ni[:, 0] != 0
    return float((c_node * area[~leaf].sum() + c_tri * (area[leaf] * ni[leaf, 5]).sum()) / area[root])


def desc_hash(desc: SceneDesc, builder: str = "sah", external_tree: dict | None = None, leaf_size: int = 0) -> int:
    """mcrt_scene_desc_hash: the key a scene cache file is written under."""
    d, keep = _c_desc(desc, builder, external_tree, leaf_size)
    h = ctypes.c_uint64()
    N.check(N.load().mcrt_scene_desc_hash(ctypes.byref(d), ctypes.byref(h)), "mcrt_scene_desc_hash")
    del keep
    return int(h.value)


class GpuScene:
    """A finalized scene on the GPU (owns its device memory)."""

    def __init__(self, desc: SceneDesc, builder: str = "sah", external_tree: dict | None = None,
                 leaf_size: int = 0):
        lib = N.load()
        self._lib = lib
        self.desc = desc
        d, keep = _c_desc(desc, builder, external_tree, leaf_size)
        h = ctypes.c_void_p()
        N.check(lib.mcrt_scene_create(ctypes.byref(d), ctypes.byref(h)), "mcrt_scene_create")
        self.handle = h
        del keep

    def close(self):
        if getattr(self, "handle", None):
            self._lib.mcrt_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- scene cache files ------------------------------------------------------------
    def save(self, path: str) -> None:
        """mcrt_scene_save: the prepared device scene, for GpuScene.load."""
        N.check(self._lib.mcrt_scene_save(self.handle, str(path).encode()), "mcrt_scene_save")

    @classmethod
    def load(cls, path: str, desc: SceneDesc | None = None, **kw) -> "GpuScene":
        """mcrt_scene_load; with `desc`, the file must have been written for that
        description (McrtError otherwise)."""
        lib = N.load()
        self = cls.__new__(cls)
        self._lib = lib
        self.desc = desc
        self._keep = []
        h = ctypes.c_void_p()
        want = 0 if desc is None else desc_hash(desc, **kw)
        N.check(lib.mcrt_scene_load(str(path).encode(), ctypes.c_uint64(want), ctypes.byref(h)), "mcrt_scene_load")
        self.handle = h
        return self

    @classmethod
    def cached(cls, desc: SceneDesc, path: str, **kw) -> "GpuScene":
        """Loads `path` when it holds this description's scene, else builds and writes it."""
        import os
        if os.path.exists(path):
            try:
                return cls.load(path, desc, **kw)
            except N.McrtError:
                pass
        sc = cls(desc, **kw)
        sc.save(path)
        return sc

    def info(self) -> dict:
        a, b, c, d = N.c_int64(), N.c_int64(), N.c_int64(), N.c_int64()
        N.check(self._lib.mcrt_scene_info(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                          ctypes.byref(d)), "mcrt_scene_info")
        return {"fast_nodes": a.value, "ref_nodes": b.value, "refs": c.value, "device_bytes": d.value}

    # -- SceneBVH::intersect / occluded ------------------------------------------------
    def trace_closest(self, rays, traverse: int = N.TRAVERSE_FAST):
        """rays: (n, 8) float32 {ox, oy, oz, tmin, dx, dy, dz, tmax}; numpy or CUDA tensor.
        Returns (n, 4) float32 {t, u, v, prim-bits} (prim = view(int32)[:, 3])."""
        if _is_torch(rays):
            import torch
            n = rays.shape[0]
            out = torch.empty((n, 4), dtype=torch.float32, device=rays.device)
            N.check(self._lib.mcrt_trace_closest(self.handle, rays.data_ptr(), n, out.data_ptr(), traverse,
                                                 N.PTR_DEVICE, _stream_ptr()), "mcrt_trace_closest")
            return out
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        out = np.zeros((r.shape[0], 4), np.float32)
        N.check(self._lib.mcrt_trace_closest(self.handle, r.ctypes.data, r.shape[0], out.ctypes.data, traverse,
                                             N.PTR_HOST, None), "mcrt_trace_closest")
        return out

    def trace_any(self, rays, traverse: int = N.TRAVERSE_FAST):
        if _is_torch(rays):
            import torch
            n = rays.shape[0]
            out = torch.empty((n,), dtype=torch.int32, device=rays.device)
            N.check(self._lib.mcrt_trace_any(self.handle, rays.data_ptr(), n, out.data_ptr(), traverse,
                                             N.PTR_DEVICE, _stream_ptr()), "mcrt_trace_any")
            return out
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        out = np.zeros((r.shape[0],), np.int32)
        N.check(self._lib.mcrt_trace_any(self.handle, r.ctypes.data, r.shape[0], out.ctypes.data, traverse,
                                         N.PTR_HOST, None), "mcrt_trace_any")
        return out

    # -- rayTrace + DemoSimple::run -----------------------------------------------------
    def render(self, camera: CameraDesc, spp: int, max_depth: int, rr_depth: int = -1, seed: int = 0,
               traverse: int = N.TRAVERSE_FAST, out=None, path_chunk: int = 0, use_graph: bool = False,
               profile: int = 0, variant: int = 0, schedule: int = N.SCHEDULE_STREAM):
        """Returns (image (H, W, 3) float32, stats dict).  `out` may be a CUDA tensor."""
        p = make_params(spp, max_depth, rr_depth, seed, traverse, path_chunk, use_graph, profile, variant, schedule)
        cam = camera.to_c()
        st = N.RenderStats()
        if out is not None and _is_torch(out):
            p.ptr_mode = N.PTR_DEVICE
            N.check(self._lib.mcrt_render(self.handle, ctypes.byref(cam), ctypes.byref(p), out.data_ptr(),
                                          ctypes.byref(st), _stream_ptr()), "mcrt_render")
            img = out
        else:
            img = np.zeros((camera.height, camera.width, 3), np.float32) if out is None else out
            p.ptr_mode = N.PTR_HOST
            N.check(self._lib.mcrt_render(self.handle, ctypes.byref(cam), ctypes.byref(p), img.ctypes.data,
                                          ctypes.byref(st), None), "mcrt_render")
        return img, stats_dict(st)

    def render_adjoint(self, camera: CameraDesc, spp: int, max_depth: int, dL_dimage, n_albedo: int,
                       n_emission: int, rr_depth: int = -1, seed: int = 0, traverse: int = N.TRAVERSE_FAST,
                       d_albedo=None, d_emission=None, schedule: int = N.SCHEDULE_STREAM, path_chunk: int = 0):
        """Path-replay adjoint; returns (d_albedo (n,3), d_emission (m,3), stats).
        Gradients are ADDED into d_albedo / d_emission when given.  schedule STREAM replays
        the paths through the wavefront queues; WAVES and PATHS replay each path in one
        thread."""
        p = make_params(spp, max_depth, rr_depth, seed, traverse, path_chunk, False, schedule=schedule)
        cam = camera.to_c()
        st = N.RenderStats()
        if _is_torch(dL_dimage):
            import torch
            dev = dL_dimage.device
            ga = torch.zeros((max(n_albedo, 1), 3), dtype=torch.float32, device=dev) if d_albedo is None else d_albedo
            ge = torch.zeros((max(n_emission, 1), 3), dtype=torch.float32, device=dev) if d_emission is None \
                else d_emission
            p.ptr_mode = N.PTR_DEVICE
            N.check(self._lib.mcrt_render_adjoint(self.handle, ctypes.byref(cam), ctypes.byref(p),
                                                  dL_dimage.contiguous().data_ptr(), ga.data_ptr(), n_albedo,
                                                  ge.data_ptr(), n_emission, ctypes.byref(st), _stream_ptr()),
                    "mcrt_render_adjoint")
            return ga[:n_albedo], ge[:n_emission], stats_dict(st)
        dl = np.ascontiguousarray(dL_dimage, np.float32)
        ga = np.zeros((max(n_albedo, 1), 3), np.float32) if d_albedo is None else d_albedo
        ge = np.zeros((max(n_emission, 1), 3), np.float32) if d_emission is None else d_emission
        p.ptr_mode = N.PTR_HOST
        N.check(self._lib.mcrt_render_adjoint(self.handle, ctypes.byref(cam), ctypes.byref(p), dl.ctypes.data,
                                              ga.ctypes.data, n_albedo, ge.ctypes.data, n_emission,
                                              ctypes.byref(st), None), "mcrt_render_adjoint")
        return ga[:n_albedo], ge[:n_emission], stats_dict(st)

    def set_materials(self, materials: list):
        """mcrt_scene_set_materials: new colours and parameters for the scene's materials
        (the emitter set and consistent normals stay as built; McrtError otherwise, and the
        scene keeps its materials)."""
        old = self.desc.materials
        self.desc.materials = list(materials)
        try:
            arr = self.desc.c_materials()
            N.check(self._lib.mcrt_scene_set_materials(self.handle, len(materials), arr, None),
                    "mcrt_scene_set_materials")
        except Exception:
            self.desc.materials = old
            raise


def make_params(spp, max_depth, rr_depth=-1, seed=0, traverse=N.TRAVERSE_FAST, path_chunk=0, use_graph=False,
                profile=0, variant=0, schedule=0):
    p = N.RenderParams()
    p.spp = int(spp)
    p.max_depth = int(max_depth)
    p.rr_depth = int(rr_depth)
    p.seed = int(seed) & ((1 << 64) - 1)
    p.traverse = int(traverse)
    p.path_chunk = int(path_chunk)
    p.use_graph = 1 if use_graph else 0
    p.profile = int(profile)
    p.variant = int(variant)
    p.schedule = int(schedule)
    return p


def stats_dict(st: N.RenderStats) -> dict:
    return {"paths": st.paths, "extension_rays": st.extension_rays, "shadow_rays": st.shadow_rays,
            "rays": st.extension_rays + st.shadow_rays, "waves": st.waves, "kernel_launches": st.kernel_launches,
            "device_ms": st.device_ms, "stage_ms": list(st.stage_ms), "extend_launches": st.extend_launches,
            "ext_nodes": st.ext_nodes, "ext_tris": st.ext_tris, "nee_nodes": st.nee_nodes, "nee_tris": st.nee_tris,
            "h2d_bytes": st.h2d_bytes, "d2h_bytes": st.d2h_bytes, "node_bytes": st.node_bytes}


def render_batch(scenes: list, cameras: list, params: list, outs: list | None = None):
    """One wavefront over many (scene, camera, params) jobs.  params: dicts for make_params.
    outs: optional CUDA tensors (device mode) -- otherwise numpy images are returned."""
    lib = N.load()
    n = len(scenes)
    hs = (ctypes.c_void_p * n)(*[s.handle.value for s in scenes])
    cs = (N.Camera * n)(*[c.to_c() for c in cameras])
    ps = (N.RenderParams * n)(*[make_params(**p) for p in params])
    device = outs is not None and _is_torch(outs[0])
    if outs is None:
        outs = [np.zeros((c.height, c.width, 3), np.float32) for c in cameras]
    ptrs = (ctypes.c_void_p * n)(*[(o.data_ptr() if device else o.ctypes.data) for o in outs])
    for k in range(n):
        ps[k].ptr_mode = N.PTR_DEVICE if device else N.PTR_HOST
    st = N.RenderStats()
    N.check(lib.mcrt_render_batch(n, hs, cs, ps, ptrs, ctypes.byref(st), _stream_ptr() if device else None),
            "mcrt_render_batch")
    return outs, stats_dict(st)


def autotune(scenes: list, cameras: list, params: list):
    """mcrt_autotune over (scene, camera, params) jobs.  Returns (tuned params dicts with
    path_chunk and variant set, report dict with every timed candidate)."""
    lib = N.load()
    n = len(scenes)
    hs = (ctypes.c_void_p * n)(*[s.handle.value for s in scenes])
    cs = (N.Camera * n)(*[c.to_c() for c in cameras])
    ps = (N.RenderParams * n)(*[make_params(**p) for p in params])
    out = (N.RenderParams * n)()
    rep = N.TuneReport()
    N.check(lib.mcrt_autotune(n, hs, cs, ps, out, ctypes.byref(rep), None), "mcrt_autotune")
    tuned = [dict(p, path_chunk=int(out[k].path_chunk), variant=int(out[k].variant)) for k, p in enumerate(params)]
    k = rep.num_candidates
    report = {"probe_paths": int(rep.probe_paths), "chosen": int(rep.chosen),
              "candidates": [{"path_chunk": int(rep.path_chunk[i]), "variant": int(rep.variant[i]),
                              "ms": round(float(rep.ms[i]), 3)} for i in range(k)]}
    return tuned, report


def render_adjoint_batch(scenes: list, cameras: list, params: list, dL_dimages: list, n_albedo: int,
                         n_emission: int):
    """Adjoint of render_batch: all jobs' paths replayed in one launch, gradients summed.
    dL_dimages: numpy arrays (host mode) or CUDA tensors (device mode).
    Returns (d_albedo (n_albedo, 3), d_emission (n_emission, 3), stats)."""
    lib = N.load()
    n = len(scenes)
    hs = (ctypes.c_void_p * n)(*[s.handle.value for s in scenes])
    cs = (N.Camera * n)(*[c.to_c() for c in cameras])
    ps = (N.RenderParams * n)(*[make_params(**p) for p in params])
    device = _is_torch(dL_dimages[0])
    for k in range(n):
        ps[k].ptr_mode = N.PTR_DEVICE if device else N.PTR_HOST
    if device:
        import torch
        dls = [d.contiguous() for d in dL_dimages]
        ptrs = (ctypes.c_void_p * n)(*[d.data_ptr() for d in dls])
        dev = dls[0].device
        ga = torch.zeros((max(n_albedo, 1), 3), dtype=torch.float32, device=dev)
        ge = torch.zeros((max(n_emission, 1), 3), dtype=torch.float32, device=dev)
        gap, gep, stream = ga.data_ptr(), ge.data_ptr(), _stream_ptr()
    else:
        dls = [np.ascontiguousarray(d, np.float32) for d in dL_dimages]
        ptrs = (ctypes.c_void_p * n)(*[d.ctypes.data for d in dls])
        ga = np.zeros((max(n_albedo, 1), 3), np.float32)
        ge = np.zeros((max(n_emission, 1), 3), np.float32)
        gap, gep, stream = ga.ctypes.data, ge.ctypes.data, None
    st = N.RenderStats()
    N.check(lib.mcrt_render_adjoint_batch(n, hs, cs, ps, ptrs, gap, n_albedo, gep, n_emission, ctypes.byref(st),
                                          stream), "mcrt_render_adjoint_batch")
    return ga[:n_albedo], ge[:n_emission], stats_dict(st)
