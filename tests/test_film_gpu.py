"""Film outputs on the GPU against the reference's FrameBuffer (golden bytes and floats
generated from the compiled reference, tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_film.npz")


def _images():
    g = np.load(GOLD)
    k = 0
    while f"img{k}" in g:
        yield k, g
        k += 1


def test_hdr_and_ppm_bytes_match_reference(cuda_device):
    from mcrt_gb300 import film
    for k, g in _images():
        img = np.ascontiguousarray(g[f"img{k}"])
        assert film.encode(img, "hdr") == g[f"hdr{k}"].tobytes(), f"image {k}: hdr"
        assert film.encode(img, "ppm") == g[f"ppm{k}"].tobytes(), f"image {k}: ppm"


def test_device_tensor_encode_matches_host(cuda_device):
    import torch
    from mcrt_gb300 import film
    for k, g in _images():
        img = np.ascontiguousarray(g[f"img{k}"])
        t = torch.tensor(img, device=cuda_device)
        assert film.encode(t, "hdr") == g[f"hdr{k}"].tobytes()


def test_reinhard_bit_exact(cuda_device):
    from mcrt_gb300 import film
    for k, g in _images():
        img = np.array(g[f"img{k}"], np.float32, copy=True)
        film.tonemap(img, "reinhard")
        np.testing.assert_array_equal(img, g[f"reinhard{k}"])


def test_gamma_within_two_ulp(cuda_device):
    """tonemapGamma evaluates powf per pixel: CUDA's powf against the C library's."""
    from mcrt_gb300 import film
    for k, g in _images():
        img = np.array(g[f"img{k}"], np.float32, copy=True)
        film.tonemap(img, "gamma", 2.2)
        want = g[f"gamma{k}"]
        ulp = np.abs(img.view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64))
        assert ulp.max() <= 2, f"image {k}: {ulp.max()} ulp"


def test_rendered_frame_to_hdr_and_ppm(cuda_device, tmp_path):
    """A rendered frame written through the device path: the file is the oracle's bytes of
    the same image."""
    import torch
    from mcrt_gb300 import GpuScene, film, scenes
    from oracle.oracle import film_encode
    desc = scenes.cfg0_scene()
    cam = scenes.cfg0_camera(64, 48)
    out = torch.empty((48, 64, 3), device=cuda_device)
    GpuScene(desc).render(cam, spp=4, max_depth=4, seed=1, out=out)
    host = out.cpu().numpy()
    path = tmp_path / "frame.hdr"
    film.write(str(path), out)
    assert path.read_bytes() == film_encode(host, True)
    film.tonemap(out, "reinhard")
    film.tonemap(out, "gamma", 2.2)
    ppm = film.encode(out, "ppm")
    assert ppm[:2] == b"P6" and len(ppm) == len(b"P6\n64 48\n255\n") + 64 * 48 * 3
