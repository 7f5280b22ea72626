"""The path-replay adjoint: against the FP64 CPU adjoint of the oracle (same seeds) and
against central finite differences with common random numbers (step 1e-3)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RES, SPP, DEPTH = 32, 16, 6


def _setup(seed=3, groups=256):
    from mcrt_gb300 import GpuScene, scenes
    desc, albedo, emission = scenes.cfg3_scene(param_seed=seed, groups=groups)
    cam = scenes.cfg0_camera(RES, RES)
    return desc, cam, albedo, emission, GpuScene(desc)


def _loss_and_grad_image(img, target):
    d = img - target
    return float(np.sum(d.astype(np.float64) ** 2)), (2.0 * d).astype(np.float32)


def test_adjoint_matches_fp64_oracle_adjoint(cuda_device):
    from oracle.oracle import OracleScene
    desc, cam, albedo, emission, sc = _setup()
    rng = np.random.default_rng(0)
    dl = rng.normal(size=(RES, RES, 3)).astype(np.float32)
    ga, ge, st = sc.render_adjoint(cam, SPP, DEPTH, dl, albedo.shape[0], 1, seed=11)
    ref = OracleScene(desc, 64).render(cam.as_array(), RES, RES, SPP, DEPTH, -1, seed=11, dLdI=dl,
                                       n_albedo=albedo.shape[0], n_emission=1)
    for got, want, name in ((ga, ref["g_albedo"], "albedo"), (ge, ref["g_emission"], "emission")):
        err = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert err < 2e-2, f"{name}: relative L2 error {err:.3e}"
    assert st["paths"] == RES * RES * SPP


def test_adjoint_vs_central_finite_differences(cuda_device):
    """Directional derivatives of an L2 image loss: adjoint vs (L(p + h v) - L(p - h v)) / 2h,
    h = 1e-3, common random numbers.

    The loss sums over the pixels whose value responds to the sphere albedos by more than
    2 % (the sphere and its near surroundings).  Elsewhere a 1e-3 albedo step changes a
    pixel by less than one float32 ulp of its value, and the rounding of the two float32
    images would make the finite difference itself off by ~2 %."""
    desc, cam, albedo, emission, sc = _setup()
    from mcrt_gb300 import scenes
    target_desc, _, _ = scenes.cfg3_scene(param_seed=99)
    from mcrt_gb300 import GpuScene
    target, _ = GpuScene(target_desc).render(cam, spp=SPP, max_depth=DEPTH, seed=5)
    target = target.astype(np.float64)

    def render_at(a, e):
        sc.set_materials(scenes.cfg3_with_params(a, e).materials)
        img, _ = sc.render(cam, spp=SPP, max_depth=DEPTH, seed=11)
        return img.astype(np.float64)

    lo = render_at(np.clip(albedo - 0.05, 0.01, 1.0).astype(np.float32), emission)
    hi = render_at(np.clip(albedo + 0.05, 0.0, 1.0).astype(np.float32), emission)
    mask = (np.abs(hi - lo) / (np.abs(lo) + 1e-3) > 0.02).astype(np.float64)
    assert 0.02 < mask.mean() < 0.9

    def loss_at(a, e):
        d = render_at(a, e) - target
        return float(np.sum(mask * d * d)), (2.0 * mask * d).astype(np.float32)

    L0, dl = loss_at(albedo, emission)
    ga, ge, _ = sc.render_adjoint(cam, SPP, DEPTH, dl, albedo.shape[0], 1, seed=11)
    rng = np.random.default_rng(1)
    h = 1e-3
    for trial in range(3):
        va = rng.normal(size=albedo.shape).astype(np.float32)
        ve = rng.normal(size=emission.shape).astype(np.float32) * (0.0 if trial < 2 else 1.0)
        Lp, _ = loss_at(albedo + h * va, emission + h * ve)
        Lm, _ = loss_at(albedo - h * va, emission - h * ve)
        fd = (Lp - Lm) / (2 * h)
        an = float(np.sum(ga * va) + np.sum(ge * ve))
        assert abs(an - fd) <= 0.02 * abs(fd) + 1e-6, f"trial {trial}: adjoint {an:.6g} vs FD {fd:.6g}"
    sc.set_materials(scenes.cfg3_with_params(albedo, emission).materials)


def test_torch_autograd_function(cuda_device):
    import torch
    from mcrt_gb300.autograd import DiffRender
    desc, cam, albedo, emission, sc = _setup()
    r = DiffRender(sc, cam, spp=8, max_depth=DEPTH, seed=2)
    a = torch.tensor(albedo, device=cuda_device, requires_grad=True)
    e = torch.tensor(emission, device=cuda_device, requires_grad=True)
    img = r(a, e)
    w = torch.randn_like(img)
    (img * w).sum().backward()
    ga, ge, _ = sc.render_adjoint(cam, 8, DEPTH, w, albedo.shape[0], 1, seed=2)
    np.testing.assert_allclose(a.grad.cpu().numpy(), ga.cpu().numpy(), rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(e.grad.cpu().numpy(), ge.cpu().numpy(), rtol=1e-4, atol=1e-6)


def test_torch_autograd_backward_uses_its_own_forward_parameters(cuda_device):
    """forward(a1), forward(a2), then backward of the first: the gradient is the adjoint at
    a1 (the scene holds a2 when that backward runs), and the scene keeps a2 afterwards."""
    import torch
    from mcrt_gb300 import scenes
    from mcrt_gb300.autograd import DiffRender
    desc, cam, albedo, emission, sc = _setup()
    r = DiffRender(sc, cam, spp=8, max_depth=DEPTH, seed=2)
    a1 = torch.tensor(albedo, device=cuda_device, requires_grad=True)
    e1 = torch.tensor(emission, device=cuda_device, requires_grad=True)
    a2 = torch.tensor(np.clip(albedo * 0.6 + 0.2, 0.05, 0.95), device=cuda_device, requires_grad=True)
    e2 = torch.tensor(emission * 1.5, device=cuda_device, requires_grad=True)
    img1 = r(a1, e1)
    img2 = r(a2, e2)
    w = torch.randn_like(img1)
    (img1 * w).sum().backward()
    # the scene was put back to the second forward's parameters after that backward
    after, _ = sc.render(cam, spp=8, max_depth=DEPTH, seed=2)
    np.testing.assert_array_equal(after, img2.detach().cpu().numpy())
    sc.set_materials(scenes.cfg3_with_params(albedo, emission).materials)
    ga, ge, _ = sc.render_adjoint(cam, 8, DEPTH, w, albedo.shape[0], 1, seed=2)
    np.testing.assert_allclose(a1.grad.cpu().numpy(), ga.cpu().numpy(), rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(e1.grad.cpu().numpy(), ge.cpu().numpy(), rtol=1e-4, atol=1e-6)


def test_adjoint_forward_time_ratio(cuda_device):
    """Forward + adjoint stays within 3x the forward time (same image, same spp)."""
    import time
    desc, cam, albedo, emission, sc = _setup()
    from mcrt_gb300 import scenes
    big = scenes.cfg0_camera(128, 128)
    dl = np.ones((128, 128, 3), np.float32)
    sc.render(big, spp=SPP, max_depth=DEPTH, seed=1)
    t0 = time.perf_counter()
    _, fst = sc.render(big, spp=SPP, max_depth=DEPTH, seed=1)
    tf = time.perf_counter() - t0
    sc.render_adjoint(big, SPP, DEPTH, dl, albedo.shape[0], 1, seed=1)
    t0 = time.perf_counter()
    sc.render_adjoint(big, SPP, DEPTH, dl, albedo.shape[0], 1, seed=1)
    ta = time.perf_counter() - t0
    assert (tf + ta) / tf <= 3.0, f"forward {tf * 1e3:.1f} ms, adjoint {ta * 1e3:.1f} ms"


def test_batched_adjoint_equals_sum_of_single_adjoints(cuda_device):
    """Several views of one scene in one adjoint launch: the summed gradient."""
    from mcrt_gb300 import CameraDesc, render_adjoint_batch
    desc, cam, albedo, emission, sc = _setup()
    cams = [cam, CameraDesc(origin=(0.4, 0.2, 3.3), target=(0.0, -0.3, 0.0), width=24, height=20, fov_y=45.0)]
    rng = np.random.default_rng(4)
    dls = [rng.normal(size=(c.height, c.width, 3)).astype(np.float32) for c in cams]
    params = [dict(spp=8, max_depth=DEPTH, seed=21), dict(spp=4, max_depth=DEPTH, seed=22)]
    gab, geb, st = render_adjoint_batch([sc, sc], cams, params, dls, albedo.shape[0], 1)
    ga = np.zeros_like(gab)
    ge = np.zeros_like(geb)
    for c, p, d in zip(cams, params, dls):
        a, e, _ = sc.render_adjoint(c, p["spp"], p["max_depth"], d, albedo.shape[0], 1, seed=p["seed"])
        ga += a
        ge += e
    np.testing.assert_allclose(gab, ga, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(geb, ge, rtol=1e-4, atol=1e-5)
    assert st["paths"] == 32 * 32 * 8 + 24 * 20 * 4


@pytest.mark.parametrize("path_chunk,groups", [(0, 256), (512, 256), (0, 2560)])
def test_wavefront_adjoint_equals_per_path_replay(path_chunk, groups, cuda_device):
    """The wavefront replay (queues, vertex log, split albedo term) and the one-thread-per-
    path replay compute the same derivative; they differ only in float summation order.
    256 albedo groups are summed per block in shared memory, 2560 (30 KB) straight into
    the global vector."""
    desc, cam, albedo, emission, sc = _setup(groups=groups)
    rng = np.random.default_rng(8)
    dl = rng.normal(size=(RES, RES, 3)).astype(np.float32)
    ga_w, ge_w, st_w = sc.render_adjoint(cam, SPP, DEPTH, dl, albedo.shape[0], 1, seed=4, schedule=0,
                                         path_chunk=path_chunk)
    ga_m, ge_m, st_m = sc.render_adjoint(cam, SPP, DEPTH, dl, albedo.shape[0], 1, seed=4, schedule=1)
    for got, want, name in ((ga_w, ga_m, "albedo"), (ge_w, ge_m, "emission")):
        err = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert err < 1e-4, f"{name}: relative L2 difference {err:.3e}"
    assert st_w["extension_rays"] + st_w["shadow_rays"] == st_m["extension_rays"]
    if path_chunk:
        assert st_w["waves"] > 8


def test_deep_adjoint_uses_per_path_replay(cuda_device):
    """Depths beyond the wavefront vertex log replay each path in one thread."""
    desc, cam, albedo, emission, sc = _setup()
    dl = np.ones((RES, RES, 3), np.float32)
    ga, ge, st = sc.render_adjoint(cam, 2, 20, dl, albedo.shape[0], 1, seed=4)
    assert st["waves"] == 1 and np.all(np.isfinite(ga)) and np.abs(ga).sum() > 0
