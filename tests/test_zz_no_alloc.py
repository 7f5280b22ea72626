"""mcrt_render_noalloc: the render for callers that cannot call cudaMalloc or cudaFree
while they render (a plug-in confined to its host application's memory pool, a render loop
that must not let an allocation synchronise the device, a process held to a memory budget
fixed at start-up).  It must give the same image as mcrt_render on device buffers, bit for
bit, call after call, although its scratch is one fixed device array that every call
reuses.

This file is collected last (tests/test_zz_*) so that a run stopping at the first
failure has run every other test before it; it also passes on its own in a fresh
process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _render_noalloc(lib, N, scene, cam, params, out):
    st = N.RenderStats()
    rc = lib.mcrt_render_noalloc(scene.handle, ctypes.byref(cam), ctypes.byref(params), out.data_ptr(),
                                 ctypes.byref(st), None)
    return rc, st


def test_noalloc_render_matches_render_twice(cuda_device):
    import torch
    from mcrt_gb300 import GpuScene, scenes
    from mcrt_gb300 import _native as N
    from mcrt_gb300.scene import make_params
    lib = N.load()
    desc = scenes.cfg0_scene()
    cam = scenes.cfg0_camera(96, 80)
    sc = GpuScene(desc)
    c_cam = cam.to_c()
    # 96 x 80 px x 24 spp = 184,320 paths: three waves of the fixed 65,536-slot scratch
    for seed in (3, 4):
        p = make_params(24, 8, 3, seed)
        p.ptr_mode = N.PTR_DEVICE
        want = torch.zeros((80, 96, 3), dtype=torch.float32, device=cuda_device)
        st_ref = N.RenderStats()
        N.check(lib.mcrt_render(sc.handle, ctypes.byref(c_cam), ctypes.byref(p), want.data_ptr(),
                                ctypes.byref(st_ref), None), "mcrt_render")
        got = torch.full((80, 96, 3), -1.0, dtype=torch.float32, device=cuda_device)
        rc, st = _render_noalloc(lib, N, sc, c_cam, p, got)
        N.check(rc, "mcrt_render_noalloc")
        assert torch.cuda.current_device() == cuda_device.index
        assert st.waves == 3
        assert st.paths == st_ref.paths and st.extension_rays == st_ref.extension_rays
        np.testing.assert_array_equal(got.cpu().numpy(), want.cpu().numpy())


def test_noalloc_rejects_requests_beyond_its_scratch(cuda_device):
    import torch
    from mcrt_gb300 import GpuScene, scenes
    from mcrt_gb300 import _native as N
    from mcrt_gb300.scene import make_params
    lib = N.load()
    sc = GpuScene(scenes.cfg0_scene())
    out = torch.zeros((16, 16, 3), dtype=torch.float32, device=cuda_device)
    c_cam = scenes.cfg0_camera(16, 16).to_c()
    p = make_params(70000, 4)
    p.ptr_mode = N.PTR_DEVICE
    rc, _ = _render_noalloc(lib, N, sc, c_cam, p, out)
    assert rc == -1 and b"exceeds" in lib.mcrt_last_error()
    p = make_params(4, 4)
    p.ptr_mode = N.PTR_HOST
    rc, _ = _render_noalloc(lib, N, sc, c_cam, p, out)
    assert rc == -1 and b"device" in lib.mcrt_last_error()
