"""The reference's own renderer with this library behind its two seams, on the GPU.

oracle/_ref/libmcrt_ref_gb300.so is the reference build with scenebvh.cpp replaced by the
drop-in SceneBVH backend (mcrt_gb300/integration/scenebvh_gb300.cpp) and the
integrator-seam converter (render_gb300.cpp) linked in.  Both are compared with the
reference's own image of its Cornell box (demo_pt.cpp rayTrace with the SplitBVH backend,
tests/golden/ref_image_cornell.npz):

  * SceneBVH seam: demo_pt.cpp's rayTrace, unchanged, with every ray query answered by the
    GPU (the backend in its reference-tree mode, MCRT_SCENEBVH_TREE=splitbvh: the same
    SplitBVH, bit-identical hits);
  * integrator seam: the finalized reference Scene converted by gb300_scene_from_mcrt and
    rendered by mcrt_render through gb300_render_into.

The seam build defines the reference's symbols again, so it is loaded in a child process
of its own, never beside oracle/_ref/libmcrt_ref.so."""
import ctypes
import multiprocessing as mp
import os

import numpy as np
import pytest

from conftest import ROOT, golden

pytestmark = pytest.mark.gpu

SEAM_SO = os.path.join(ROOT, "oracle", "_ref", "libmcrt_ref_gb300.so")


def _child(scenebvh_batches, scenebvh_spp, integrator_spp):
    """Runs in a spawned process: both seams on the reference Cornell box."""
    os.environ["MCRT_SCENEBVH_TREE"] = "splitbvh"
    import time
    fx = np.load(os.path.join(ROOT, "tests", "golden", "ref_image_cornell.npz"))
    lib = ctypes.CDLL(SEAM_SO)
    P, I = ctypes.c_void_p, ctypes.c_int
    lib.ref_pt_scene_create.restype = P
    lib.ref_pt_scene_create.argtypes = [P, P, P, I, P, P, I, ctypes.c_char_p, P, I, I]
    lib.ref_pt_render.argtypes = [P, I, I, I, I, I, I, P, P, P, P]
    lib.ref_pt_scene_destroy.argtypes = [P]
    lib.seam_render_gb300.argtypes = [P, ctypes.c_char_p, P, I, I, I, I, I, ctypes.c_ulonglong, I, P, P]
    verts = np.ascontiguousarray(fx["verts"], np.float32)
    n = verts.shape[0]
    mid = np.arange(n, dtype=np.int32)
    types = np.ascontiguousarray(fx["mat_types"], np.int32)
    colors = np.ascontiguousarray(fx["mat_colors"], np.float32)
    cam7 = np.ascontiguousarray(fx["camera"], np.float32)
    res = fx["batch_means"].shape[1]
    h = lib.ref_pt_scene_create(verts.ctypes.data, None, mid.ctypes.data, n, types.ctypes.data, colors.ctypes.data,
                                n, b"", cam7.ctypes.data, res, res)
    batches = []
    ni, no, sec = ctypes.c_longlong(0), ctypes.c_longlong(0), ctypes.c_double(0.0)
    t0 = time.time()
    for _ in range(scenebvh_batches):
        out = np.zeros((res, res, 3), np.float32)
        lib.ref_pt_render(h, res, res, scenebvh_spp, os.cpu_count() or 1, 0, res, out.ctypes.data, ctypes.byref(ni),
                          ctypes.byref(no), ctypes.byref(sec))
        batches.append(out)
    t_scenebvh = time.time() - t0
    img = np.zeros((res, res, 3), np.float32)
    rays = ctypes.c_longlong(0)
    rc = lib.seam_render_gb300(h, None, cam7.ctypes.data, res, res, integrator_spp, 10, -1, 17, 0, img.ctypes.data,
                               ctypes.byref(rays))
    lib.ref_pt_scene_destroy(h)
    return np.stack(batches), t_scenebvh, rc, img, int(rays.value)


def _z_tests(mean, spp_total, name, max_frac=0.01, mean_z=True):
    """Per-pixel and image-mean z-tests of an image of `spp_total` samples per pixel
    against the reference's batch means, with the per-sample variance of the reference.
    At low spp the mirror and glass caustics make single pixels heavy-tailed, so a caller
    may allow more pixels beyond 4 sigma; the image-mean test is exact at any spp."""
    fx = golden("ref_image_cornell.npz")
    ref_b = fx["batch_means"].astype(np.float64)
    k = int(fx["spp_per_batch"])
    ref_mean = ref_b.mean(axis=0)
    var_sample = ref_b.var(axis=0, ddof=1) * k  # per-sample variance of each pixel
    var_ref_mean = var_sample / (k * ref_b.shape[0])
    var_mean = var_sample / spp_total
    z = (mean - ref_mean) / np.sqrt(var_mean + var_ref_mean + 1e-12)
    assert np.mean(np.abs(z) > 4) < max_frac, f"{name}: {np.mean(np.abs(z) > 4):.3f} of pixels beyond 4 sigma"
    if not mean_z:
        return
    npx = mean.shape[0] * mean.shape[1]
    for c in range(3):
        d = mean[..., c].mean() - ref_mean[..., c].mean()
        se = np.sqrt((var_mean[..., c] + var_ref_mean[..., c]).sum()) / npx
        assert abs(d / se) < 4.0, f"{name}: channel {c}: image-mean z = {d / se:.2f}"


@pytest.fixture(scope="module")
def seam_run(cuda_device):
    if not os.path.exists(SEAM_SO):
        from oracle import oracle as O
        if O.build_reference() is None or O.build_seam() is None:
            pytest.fail("the seam build needs the reference sources (a checkout or baseline/_ref)")
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        # a bounded wait: a child that dies (an abort in the backend) must fail the test,
        # not leave the pool waiting for a result that never comes
        try:
            return pool.apply_async(_child, (8, 16, 1024)).get(timeout=900)
        except mp.TimeoutError:
            pytest.fail("the seam child process did not finish within 900 s (it may have died)")


def test_scenebvh_seam_runs_reference_ray_trace_on_the_gpu(seam_run):
    """demo_pt.cpp's rayTrace unchanged, its SceneBVH queries on the GPU (reference tree,
    reference traversal order and arithmetic): the reference's image, statistically."""
    batches, seconds, _, _, _ = seam_run
    print(f"SceneBVH seam: {batches.shape[0]} x 16 spp at {batches.shape[1]}^2 in {seconds:.1f} s")
    # the reference's rayTrace draws from its global, unseeded random stream, so every run
    # is a new sample: at 128 spp the caustic pixels put 1.1-2.4 % of pixels beyond 4 sigma
    # from run to run (the queries themselves are bit-identical to the SplitBVH backend's);
    # the image-mean test carries the accuracy
    _z_tests(batches.astype(np.float64).mean(axis=0), batches.shape[0] * 16, "SceneBVH seam", max_frac=0.04)


def test_integrator_seam_renders_the_reference_scene(seam_run):
    """The finalized reference Scene converted with gb300_scene_from_mcrt and rendered by
    mcrt_render (1,024 spp, depth 10, no roulette): the reference's image, statistically;
    the library's own tree, so the 2 % image-mean bound of the own-tree Cornell test holds
    too."""
    _, _, rc, img, rays = seam_run
    assert rc == 0
    assert rays > 0
    fx = golden("ref_image_cornell.npz")
    ref_mean = fx["batch_means"].astype(np.float64).mean(axis=0)
    for c in range(3):
        assert abs(img[..., c].mean() - ref_mean[..., c].mean()) < 0.02 * ref_mean[..., c].mean()
    # the pixel test at 1,024 spp: mirror and glass caustics are heavy-tailed, and on the
    # library's tree a few floor pixels beside the boxes resolve coplanar faces differently
    _z_tests(img.astype(np.float64), 1024, "integrator seam", max_frac=0.02, mean_z=False)
