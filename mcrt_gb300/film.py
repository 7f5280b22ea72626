"""Film outputs of FrameBuffer (src/core/film.cpp) on the GPU: the Radiance ``.hdr`` and
binary ``.ppm`` writers (byte for byte) and the gamma / Reinhard tone mappers, for images
in mcrt_render's layout ([height][width][3] float32, row 0 the bottom row).  Images may be
numpy arrays (copied in and out inside the call) or CUDA tensors (device mode, torch's
current stream)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N


def _args(img):
    from .scene import _is_torch, _stream_ptr
    if _is_torch(img):
        if not img.is_contiguous():
            raise ValueError("image tensor must be contiguous")
        return img.data_ptr(), N.PTR_DEVICE, _stream_ptr()
    if not (img.flags["C_CONTIGUOUS"] and img.dtype == np.float32):
        raise ValueError("image array must be C-contiguous float32")
    return img.ctypes.data, N.PTR_HOST, None


def encode(img, fmt: str = "hdr") -> bytes:
    """The bytes FrameBuffer::dumpHDR ("hdr") or dumpPPM ("ppm") writes for this image."""
    lib = N.load()
    h, w = int(img.shape[0]), int(img.shape[1])
    f = N.FILM_HDR if fmt == "hdr" else N.FILM_PPM
    ptr, mode, stream = _args(img)
    size = ctypes.c_int64()
    N.check(lib.mcrt_film_encode(ptr, w, h, f, None, 0, ctypes.byref(size), mode, stream), "mcrt_film_encode")
    if mode == N.PTR_DEVICE:
        import torch
        out = torch.empty(size.value, dtype=torch.uint8, device=img.device)
        N.check(lib.mcrt_film_encode(ptr, w, h, f, out.data_ptr(), size.value, ctypes.byref(size), mode, stream),
                "mcrt_film_encode")
        return out.cpu().numpy().tobytes()
    out = np.zeros(size.value, np.uint8)
    N.check(lib.mcrt_film_encode(ptr, w, h, f, out.ctypes.data, size.value, ctypes.byref(size), mode, stream),
            "mcrt_film_encode")
    return out.tobytes()


def write(path: str, img, fmt: str | None = None) -> None:
    """Writes the image as FrameBuffer::dumpHDR / dumpPPM would (format from the suffix)."""
    fmt = fmt or ("ppm" if path.lower().endswith(".ppm") else "hdr")
    with open(path, "wb") as f:
        f.write(encode(img, fmt))


def tonemap(img, op: str = "reinhard", gamma: float = 2.2):
    """FrameBuffer::tonemapReinhard() or tonemapGamma(gamma), in place; returns img."""
    lib = N.load()
    h, w = int(img.shape[0]), int(img.shape[1])
    ptr, mode, stream = _args(img)
    o = N.TONEMAP_REINHARD if op == "reinhard" else N.TONEMAP_GAMMA
    N.check(lib.mcrt_film_tonemap(ptr, w, h, o, float(gamma), mode, stream), "mcrt_film_tonemap")
    return img
