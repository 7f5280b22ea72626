"""Hit parity of the CUDA traversal against the reference SplitBVH, through the C ABI."""
import numpy as np
import pytest

from conftest import golden
from parity import TRAVERSE_SETS, classify, fixture_scene, fixture_tree

FIXTURES = ["cornell", "cfg0", "sphere5", "debugmesh", "debugmesh_diag"]

pytestmark = pytest.mark.gpu


def _scene(fx, builder):
    from mcrt_gb300 import GpuScene
    desc = fixture_scene(fx)
    if builder == "external":
        return GpuScene(desc, builder="external", external_tree=fixture_tree(fx))
    return GpuScene(desc)


def _sets(fx):
    return [k for k in TRAVERSE_SETS if f"rays_{k}" in fx.files]


@pytest.mark.parametrize("name", FIXTURES)
def test_ref_mode_bit_exact_on_reference_tree(name, cuda_device):
    """Same BVH (the reference's own SplitBVH tree), same rays: identical prim, t, u, v."""
    from mcrt_gb300 import TRAVERSE_REF
    fx = golden(f"ref_traverse_{name}.npz")
    sc = _scene(fx, "external")
    for k in _sets(fx):
        rays = fx[f"rays_{k}"]
        out = sc.trace_closest(rays, TRAVERSE_REF)
        prim = out[:, 3].view(np.int32)
        ref_p = fx[f"prim_{k}"]
        assert np.array_equal(prim, ref_p), f"{name}/{k}: {np.sum(prim != ref_p)} prim mismatches"
        hit = ref_p >= 0
        assert np.array_equal(out[hit, 0].view(np.int32), fx[f"t_{k}"][hit].view(np.int32)), f"{name}/{k}: t"
        assert np.array_equal(out[hit, 1].view(np.int32), fx[f"u_{k}"][hit].view(np.int32)), f"{name}/{k}: u"
        assert np.array_equal(out[hit, 2].view(np.int32), fx[f"v_{k}"][hit].view(np.int32)), f"{name}/{k}: v"


@pytest.mark.parametrize("name", FIXTURES)
def test_ref_mode_occluded_matches_scenebvh(name, cuda_device):
    """SceneBVH::occluded(ray, tfar) = a hit in [1e-4, tfar - 1e-4] (scenebvh.cpp:379-396)."""
    from mcrt_gb300 import TRAVERSE_REF
    fx = golden(f"ref_traverse_{name}.npz")
    sc = _scene(fx, "external")
    for k in _sets(fx):
        rays = fx[f"rays_{k}"].copy()
        rays[:, 3] = np.float32(1e-4)
        rays[:, 7] = (rays[:, 7] - np.float32(1e-4)).astype(np.float32)
        occ = sc.trace_any(rays, TRAVERSE_REF)
        assert np.array_equal(occ, fx[f"occ_{k}"]), f"{name}/{k}: {np.sum(occ != fx[f'occ_{k}'])} mismatches"


@pytest.mark.parametrize("builder", ["external", "sah"])
@pytest.mark.parametrize("name", FIXTURES)
def test_fast_mode_nonmarginal(name, builder, cuda_device):
    """Watertight FP32 traversal: same prim and t within 4 ulp on every non-marginal ray."""
    from mcrt_gb300 import TRAVERSE_FAST
    fx = golden(f"ref_traverse_{name}.npz")
    sc = _scene(fx, builder)
    total = 0
    marginal_total = 0
    for k in _sets(fx):
        rays = fx[f"rays_{k}"]
        out = sc.trace_closest(rays, TRAVERSE_FAST)
        bad, marginal = classify(fx["verts"], rays, fx[f"t_{k}"], fx[f"prim_{k}"], out[:, 0],
                                 out[:, 3].view(np.int32))
        assert not bad.any(), f"{name}/{k}/{builder}: {bad.sum()} non-marginal mismatches, e.g. ray {np.argmax(bad)}"
        total += rays.shape[0]
        if k != "axis":
            marginal_total += int(marginal.sum())
    # marginal disagreements stay rare apart from the zero-direction rays
    assert marginal_total <= max(8, total // 200), f"{marginal_total} marginal disagreements of {total}"


@pytest.mark.parametrize("builder", ["external", "sah"])
def test_ref_mode_own_builder_closest_hit(builder, cuda_device):
    """Reference arithmetic on the library's own tree: the closest hit is tree-independent."""
    from mcrt_gb300 import TRAVERSE_REF
    fx = golden("ref_traverse_cfg0.npz")
    sc = _scene(fx, builder)
    for k in _sets(fx):
        rays = fx[f"rays_{k}"]
        out = sc.trace_closest(rays, TRAVERSE_REF)
        bad, _ = classify(fx["verts"], rays, fx[f"t_{k}"], fx[f"prim_{k}"], out[:, 0], out[:, 3].view(np.int32))
        assert not bad.any()


def test_fast_any_hit_matches_occluded(cuda_device):
    from mcrt_gb300 import TRAVERSE_FAST
    fx = golden("ref_traverse_cfg0.npz")
    sc = _scene(fx, "sah")
    for k in ["primary", "incoherent", "segment"]:
        rays = fx[f"rays_{k}"].copy()
        rays[:, 3] = np.float32(1e-4)
        rays[:, 7] = (rays[:, 7] - np.float32(1e-4)).astype(np.float32)
        occ = sc.trace_any(rays, TRAVERSE_FAST)
        diff = occ != fx[f"occ_{k}"]
        # disagreements only on rays whose reference closest hit is marginal
        assert diff.sum() <= max(2, rays.shape[0] // 1000), f"{k}: {diff.sum()}"


def test_device_pointer_path(cuda_device):
    """Rays and hits resident in device memory (torch tensors) give the same answer."""
    import torch
    from mcrt_gb300 import TRAVERSE_FAST
    fx = golden("ref_traverse_cfg0.npz")
    sc = _scene(fx, "sah")
    rays = fx["rays_incoherent"]
    host = sc.trace_closest(rays, TRAVERSE_FAST)
    dev = sc.trace_closest(torch.from_numpy(rays).to(cuda_device), TRAVERSE_FAST).cpu().numpy()
    assert np.array_equal(host.view(np.int32), dev.view(np.int32))


def test_empty_and_single_ray(cuda_device):
    from mcrt_gb300 import TRAVERSE_FAST, TRAVERSE_REF
    fx = golden("ref_traverse_cornell.npz")
    sc = _scene(fx, "external")
    assert sc.trace_closest(np.zeros((0, 8), np.float32)).shape == (0, 4)
    r = fx["rays_primary"][:1]
    for mode in (TRAVERSE_FAST, TRAVERSE_REF):
        out = sc.trace_closest(r, mode)
        assert out[0, 3].view(np.int32) == fx["prim_primary"][0]


def test_l2_read_probe(cuda_device):
    """The L2 roofline denominator: a plausible bandwidth, above the HBM copy rate of this
    class of GPU (several TB/s) and below any L2's (100 TB/s)."""
    import ctypes
    from mcrt_gb300 import _native as N
    lib = N.load()
    g = ctypes.c_float(0.0)
    N.check(lib.mcrt_probe_l2_read(48 << 20, 20, ctypes.byref(g), None), "mcrt_probe_l2_read")
    assert 3000.0 < g.value < 100000.0, g.value
