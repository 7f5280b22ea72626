"""Shared parity helpers: fixture scenes and the hit-parity rule.

Hit parity (closest hit of the same rays on the same triangles):
  * MCRT_TRAVERSE_REF must reproduce the reference bit for bit (prim, t, u, v) on
    every ray, including the reference's own quirks (rays with a zero direction
    component miss, |det| < 1e-6 rejected).
  * MCRT_TRAVERSE_FAST (watertight test) must give the reference's prim and a t
    within 4 ulp on every non-marginal ray.  A disagreement is marginal when, for
    either of the two triangles involved, |det_MT| lies within 2^-8 of the 1e-6
    rejection threshold, a barycentric coordinate is within 2^-20 of an edge, the
    ray origin lies within 8 ulp (of its largest coordinate) of the triangle's plane
    (a self-intersection, where t is rounding noise), the two hits lie within 4 ulp
    of each other (a tie), or the ray has a zero direction component (the
    reference's inv_dir = 0 slab test, ray.cpp:39-42).
"""
from __future__ import annotations

import numpy as np

from mcrt_gb300.scene import DIFF, Material, SceneDesc

TRAVERSE_SETS = ["primary", "bounce", "incoherent", "segment", "axis"]


def fixture_scene(fx) -> SceneDesc:
    v = fx["verts"]
    return SceneDesc(v, np.zeros(v.shape[0], np.int32), [Material(DIFF, (0.5, 0.5, 0.5))])


def fixture_tree(fx) -> dict:
    return dict(node_box=fx["tree_node_box"], node_info=fx["tree_node_info"], ref_prim=fx["tree_ref_prim"],
                ref_box=fx["tree_ref_box"])


def ulp_diff(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    ai = a.astype(np.float32).view(np.int32).astype(np.int64)
    bi = b.astype(np.float32).view(np.int32).astype(np.int64)
    ai = np.where(ai < 0, -(ai & 0x7FFFFFFF), ai)
    bi = np.where(bi < 0, -(bi & 0x7FFFFFFF), bi)
    return np.abs(ai - bi)


def mt_terms(verts: np.ndarray, prim: np.ndarray, rays: np.ndarray):
    """|det|, min barycentric and t of Moller-Trumbore in double for (ray, prim) pairs."""
    tri = verts.reshape(-1, 3, 3)[np.maximum(prim, 0)].astype(np.float64)
    o = rays[:, 0:3].astype(np.float64)
    d = rays[:, 4:7].astype(np.float64)
    e1 = tri[:, 1] - tri[:, 0]
    e2 = tri[:, 2] - tri[:, 0]
    pv = np.cross(d, e2)
    det = np.sum(e1 * pv, axis=1)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / det
        tv = o - tri[:, 0]
        u = np.sum(tv * pv, axis=1) * inv
        qv = np.cross(tv, e1)
        v = np.sum(d * qv, axis=1) * inv
        t = np.sum(e2 * qv, axis=1) * inv
        bmin = np.minimum(np.minimum(u, v), 1.0 - u - v)  # NaN where det = 0 (never marginal)
    return np.abs(det), bmin, t


def plane_distance(verts, prim, rays):
    tri = verts.reshape(-1, 3, 3)[np.maximum(prim, 0)].astype(np.float64)
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-300)
    return np.abs(np.sum((rays[:, 0:3].astype(np.float64) - tri[:, 0]) * n, axis=1))


def classify(verts, rays, ref_t, ref_p, got_t, got_p):
    """Returns (unexplained disagreement mask, marginal disagreement mask)."""
    same = (ref_p == got_p) & ((ref_p < 0) | (ulp_diff(ref_t, got_t) <= 4))
    marginal = np.zeros(rays.shape[0], bool)
    marginal |= np.any(rays[:, 4:7] == 0.0, axis=1)
    lo, hi = 1e-6 * (1 - 2.0 ** -8), 1e-6 * (1 + 2.0 ** -8)
    oulp = np.spacing(np.max(np.abs(rays[:, 0:3]), axis=1).astype(np.float32)).astype(np.float64)
    for p in (ref_p, got_p):
        det, bmin, _ = mt_terms(verts, p, rays)
        m = (p >= 0) & (((det >= lo) & (det <= hi)) | (np.abs(bmin) < 2.0 ** -20))
        m |= (p >= 0) & (plane_distance(verts, p, rays) <= 8 * oulp)
        marginal |= m
    both = (ref_p >= 0) & (got_p >= 0)
    marginal |= both & (ulp_diff(ref_t, got_t) <= 4)
    bad = ~same & ~marginal
    return bad, marginal & ~same
