"""mcrt_gb300: GB300-native (sm_103a) wavefront path tracer behind MCRT's scene API.

Public surface:
  SceneDesc, Material, CameraDesc      host-side scene description (scene.py)
  GpuScene                             device scene: trace_closest / trace_any / render /
                                       render_adjoint / set_materials
  render_batch                         many scenes/cameras/spp budgets in one wavefront
  render_adjoint_batch                 the adjoint of render_batch in one launch
  autotune                             launch configuration (queue capacity, kernel variant)
                                       timed on a reduced-spp probe of the jobs
  load_obj, load_envmap_bin            the reference's scene inputs (Scene::loadModel's OBJ
                                       triangles and normals, EnvmapLoader's .bin maps)
  mcrt_scene                           MCRT's own scene-building calls (Scene::add, loadModel,
                                       setCamera, setEnvmap, finalize; Material, todo_addMaterial)
  film                                 FrameBuffer's .hdr / .ppm writers and tone mappers on the GPU
  build()                              compile the in-tree native library
The native library (mcrt_gb300/_lib/libmcrt_gb300.so, C ABI in include/mcrt_gb300.h)
is required: there is no CPU fallback.
"""
from . import film, mcrt_scene, scenes
from ._native import (PTR_DEVICE, PTR_HOST, TRAVERSE_FAST, TRAVERSE_REF, McrtError, load)
from .native_build import build
from .scene import (DIFF, GGX, GLSY, LGHT, REFR, SPEC, CameraDesc, GpuScene, Material, SceneDesc, autotune,
                    load_envmap_bin, load_obj, make_params, render_adjoint_batch, render_batch)

__all__ = ["SceneDesc", "Material", "CameraDesc", "GpuScene", "render_batch", "render_adjoint_batch", "autotune",
           "build", "load", "load_obj", "load_envmap_bin",
           "scenes", "film", "mcrt_scene",
           "McrtError", "TRAVERSE_FAST", "TRAVERSE_REF", "PTR_HOST", "PTR_DEVICE", "make_params",
           "LGHT", "DIFF", "SPEC", "REFR", "GLSY", "GGX"]
