"""The eight-child compressed tree of the FAST traversal, checked on the CPU.

tests/native/wide_host.cu runs the device traversal code (trace_wide is host+device) on
the host over the library's eight-child tree, built from the library's SAH tree or from
the reference's own SplitBVH tree.  Its closest hits must be the reference's primitives
with t within 4 ulp on every non-marginal ray of the hit fixtures (the rule of the GPU
tests, t recomputed by the same refine_hit), and its any-hit answers must agree with
SceneBVH::occluded.  A wrong child index, an inward-rounded quantised box or a lost stack
entry shows up here before any GPU runs the layout."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden
from parity import TRAVERSE_SETS, classify, fixture_tree

FIXTURES = ["cornell", "cfg0", "sphere5", "debugmesh", "debugmesh_diag"]


@pytest.fixture(scope="session")
def harness(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("wide") / "libwide_host.so")
    csrc = os.path.join(ROOT, "mcrt_gb300", "csrc")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    subprocess.run([os.path.join(cuda, "bin", "nvcc"), "-gencode=arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
                    "-shared", "-Xcompiler", "-fPIC,-ffp-contract=off,-pthread",
                    os.path.join(ROOT, "tests", "native", "wide_host.cu"), os.path.join(csrc, "bvh_build.cpp"),
                    os.path.join(csrc, "flatten.cpp"), os.path.join(csrc, "wide_build.cpp"), "-o", out], check=True,
                   capture_output=True)
    lib = ctypes.CDLL(out)
    P, LL, I = ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int
    lib.wide_host_error.restype = ctypes.c_char_p
    lib.wide_host_trace.argtypes = [P, LL, I, P, P, I, P, P, I, P, LL, I, P, P, P]
    return lib


def _trace(lib, verts, rays, any_hit=False, tree=None, leaf=2):
    n = rays.shape[0]
    t = np.zeros(n, np.float32)
    p = np.zeros(n, np.int32)
    st = np.zeros(5, np.int64)
    v = np.ascontiguousarray(verts, np.float32)
    r = np.ascontiguousarray(rays, np.float32)
    keep = []
    if tree is None:
        args = (None, None, 0, None, None, 0)
    else:
        keep = [np.ascontiguousarray(tree["node_box"], np.float32), np.ascontiguousarray(tree["node_info"], np.int32),
                np.ascontiguousarray(tree["ref_prim"], np.int32), np.ascontiguousarray(tree["ref_box"], np.float32)]
        args = (keep[0].ctypes.data, keep[1].ctypes.data, keep[1].shape[0], keep[2].ctypes.data, keep[3].ctypes.data,
                keep[2].shape[0])
    rc = lib.wide_host_trace(v.ctypes.data, v.shape[0], leaf, *args, r.ctypes.data, n, 1 if any_hit else 0,
                             t.ctypes.data, p.ctypes.data, st.ctypes.data)
    assert rc == 0, lib.wide_host_error().decode()
    return t, p, st


def _check(verts, rays, ref_t, ref_p, t, p, what):
    bad, _ = classify(verts, rays, ref_t, ref_p, t, p)
    assert not bad.any(), f"{what}: {bad.sum()} non-marginal mismatches, e.g. ray {np.argmax(bad)}"


@pytest.mark.parametrize("builder", ["sah", "external", "sah_split"])
@pytest.mark.parametrize("name", FIXTURES)
def test_wide_tree_closest_and_any_hit_on_the_host(name, builder, harness):
    """sah: the library's builder; external: the reference's SplitBVH tree; sah_split: the
    library's spatial-split builder, whose clipped reference boxes must still contain the
    parts of the triangles they stand for (a box clipped too tightly loses hits here)."""
    fx = golden(f"ref_traverse_{name}.npz")
    tree = None
    if builder == "external":
        tree = fixture_tree(fx)
    elif builder == "sah_split":
        from mcrt_gb300.scene import build_bvh
        tree = build_bvh(fx["verts"], leaf_size=2, split=True)
    for k in TRAVERSE_SETS:
        if f"rays_{k}" not in fx.files:
            continue
        rays = fx[f"rays_{k}"]
        t, p, st = _trace(harness, fx["verts"], rays, tree=tree)
        _check(fx["verts"], rays, fx[f"t_{k}"], fx[f"prim_{k}"], t, p, f"{name}/{builder}/{k}")
        if k == "axis":  # the reference misses every ray with a zero direction component
            continue
        r2 = rays.copy()
        r2[:, 3] = np.float32(1e-4)
        r2[:, 7] = (r2[:, 7] - np.float32(1e-4)).astype(np.float32)
        _, occ, _ = _trace(harness, fx["verts"], r2, any_hit=True, tree=tree)
        diff = (occ != fx[f"occ_{k}"]).sum()
        assert diff <= max(2, rays.shape[0] // 1000), f"{name}/{builder}/{k}: {diff} occluded answers differ"
        assert st[3] <= st[4], "the eight-child tree is never deeper than the binary one"


def test_wide_tree_at_1_3m_triangles_on_the_host(harness):
    """The large configuration's 1,310,722 triangles: 8,192 rays of each class."""
    import hashlib
    from mcrt_gb300 import scenes
    fx = golden("ref_traverse_cfg1.npz")
    verts = np.ascontiguousarray(scenes.cfg1_scene().vertices, np.float32)
    assert hashlib.sha256(verts.tobytes()).hexdigest() == str(fx["verts_sha256"])
    for k in ["primary", "bounce", "incoherent", "segment"]:
        rays = fx[f"rays_{k}"][:8192]
        t, p, st = _trace(harness, verts, rays)
        _check(verts, rays, fx[f"t_{k}"][:8192], fx[f"prim_{k}"][:8192], t, p, f"cfg1/{k}")
    # a wide node replaces about three binary levels
    assert st[3] * 2 <= st[4], (st[3], st[4])
