"""MCRT's scene-building calls on this library: the Python form of `Scene`, `Material`,
`TriangleObject` and the material library as `demo_pt.cpp` uses them, so a scene written
against MCRT's API builds a `GpuScene` with the same calls.

    mat = todo_addMaterial(Material((0.73, 0.73, 0.73), 0.0, DIFF))
    scene = Scene()
    scene.add(TriangleObject(a, b, c), mat)             # or with vertex normals
    scene.loadModel("mesh.obj", transform, Material(color, 0.0, SPEC))
    scene.setCamera(origin, target, width, height, fov_y)
    scene.setEnvmap("envmap.bin")
    gpu = scene.finalize()                                # the GpuScene (BVH built, uploaded)
    img, stats = gpu.render(scene.camera(), spp=16, max_depth=10)

Reference interfaces: `Scene::add` / `loadModel` / `setCamera` / `setEnvmap` / `finalize`
(src/core/scene.cpp:109-112, 368-408, 224-232, 206-222, 129-194), `Material(c, e, t)` and
`todo_addMaterial` / `todo_getMaterial` (src/core/material.cpp:5-27, 130-139),
`TriangleObject(a, b, c[, na, nb, nc])` with `setMaterialID` (src/core/triangle.h:11-58).
Errors raise `McrtError` (the reference asserts or exits).  Unlike the reference's global
`mat_lib`, the material library here belongs to the caller's process but is only read when
a scene is finalized.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _native as N
from .scene import DIFF, GLSY, LGHT, REFR, SPEC, CameraDesc, GpuScene
from .scene import Material as LibMaterial
from .scene import SceneDesc, load_envmap_bin, load_obj

__all__ = ["Material", "TriangleObject", "Scene", "todo_addMaterial", "todo_getMaterial",
           "LGHT", "DIFF", "SPEC", "REFR", "GLSY"]


@dataclass
class Material:
    """Material(color, emission, type) (material.cpp:5-27); `ior` and `roughness` keep the
    reference's defaults (1.33, 1.0)."""
    color: tuple
    emission: float = 0.0
    type: int = DIFF
    ior: float = 1.33
    roughness: float = 1.0


_mat_lib: list = []


def todo_addMaterial(mat: Material) -> int:
    """Adds a material to the library and returns its id (material.cpp:135-139)."""
    _mat_lib.append(mat)
    return len(_mat_lib) - 1


def todo_getMaterial(mat_id: int) -> Material:
    if not 0 <= mat_id < len(_mat_lib):
        raise N.McrtError(f"todo_getMaterial: no material {mat_id}")
    return _mat_lib[mat_id]


@dataclass
class TriangleObject:
    """TriangleObject(a, b, c) or (a, b, c, na, nb, nc): without normals the face normal is
    used, as the reference's constructor does (triangle.cpp)."""
    a: tuple
    b: tuple
    c: tuple
    na: tuple | None = None
    nb: tuple | None = None
    nc: tuple | None = None
    material_id: int = 0

    def setMaterialID(self, mat_id: int) -> None:
        self.material_id = int(mat_id)

    def materialID(self) -> int:
        return self.material_id


class Scene:
    """Scene (scene.h:28-102): triangles, a camera and an environment map; finalize()
    builds the BVH and uploads everything, returning the GpuScene."""

    def __init__(self):
        self._verts: list = []    # (k, 9) arrays
        self._normals: list = []  # (k, 9) arrays
        self._given: list = []    # whether each part came with vertex normals
        self._mids: list = []     # (k,) arrays of material-library ids
        self._camera: CameraDesc | None = None
        self._envmap: np.ndarray | None = None

    def add(self, tri: TriangleObject, mat_id: int | None = None) -> None:
        """Scene::add (scene.cpp:109-112); `mat_id` is a shortcut for setMaterialID."""
        if mat_id is not None:
            tri.setMaterialID(mat_id)
        v = np.array([*tri.a, *tri.b, *tri.c], np.float32).reshape(1, 9)
        if tri.na is None:
            a, b, c = v[0, 0:3].astype(np.float32), v[0, 3:6].astype(np.float32), v[0, 6:9].astype(np.float32)
            n = np.cross(a - c, b - c).astype(np.float32)  # the reference's face normal (cross(a-c, b-c))
            n = (n * (np.float32(1.0) / np.sqrt(np.float32(np.dot(n, n))))).astype(np.float32)
            nrm = np.tile(n, 3).reshape(1, 9)
        else:
            nrm = np.array([*tri.na, *tri.nb, *tri.nc], np.float32).reshape(1, 9)
        self._verts.append(v)
        self._normals.append(nrm)
        self._given.append(tri.na is not None)
        self._mids.append(np.array([tri.material_id], np.int32))

    def loadModel(self, filename: str, transform, mat: Material) -> None:
        """Scene::loadModel (scene.cpp:368-408): the OBJ's triangles, transformed, with
        Mesh::genNormals' vertex normals, all with a new library material `mat`."""
        mat_id = todo_addMaterial(mat)
        v, n, _ = load_obj(filename, transform)
        self._verts.append(v)
        self._normals.append(n)
        self._given.append(True)
        self._mids.append(np.full(v.shape[0], mat_id, np.int32))

    def setCamera(self, origin, target, width: int, height: int, fov_y: float) -> None:
        """Scene::setCamera (scene.cpp:224-232), up = (0, 1, 0)."""
        self._camera = CameraDesc(origin=tuple(float(x) for x in origin), target=tuple(float(x) for x in target),
                                  width=int(width), height=int(height), fov_y=float(fov_y))

    def camera(self) -> CameraDesc:
        if self._camera is None:
            raise N.McrtError("Scene::camera: setCamera was not called")
        return self._camera

    def setEnvmap(self, filename: str) -> None:
        """Scene::setEnvmap (scene.cpp:206-222): an EnvmapLoader .bin file."""
        self._envmap = load_envmap_bin(filename)

    def numTrangles(self) -> int:  # the reference's spelling (scene.h:84)
        return int(sum(v.shape[0] for v in self._verts))

    def desc(self) -> SceneDesc:
        """The library's description of the scene: one library material per library id used."""
        if not self._verts:
            raise N.McrtError("Scene::finalize: the scene has no triangles")
        mids = np.concatenate(self._mids)
        used = np.unique(mids)
        remap = {int(m): k for k, m in enumerate(used)}
        mats = []
        for m in used:
            src = todo_getMaterial(int(m))
            mats.append(LibMaterial(int(src.type), tuple(float(x) for x in src.color), roughness=float(src.roughness),
                                    ior=float(src.ior)))
        # no vertex normals anywhere: the library computes the face normals itself (as the
        # reference's constructor does); otherwise the face normals of the parts without
        # normals are taken from add()
        normals = np.concatenate(self._normals) if any(self._given) else None
        return SceneDesc(np.concatenate(self._verts), np.array([remap[int(m)] for m in mids], np.int32), mats,
                         normals=normals, envmap=self._envmap)

    def finalize(self, **kw) -> GpuScene:
        """Scene::finalize (scene.cpp:129-194): builds the BVH, the emitter and environment
        sampling tables and uploads the scene; keyword arguments go to GpuScene."""
        return GpuScene(self.desc(), **kw)
