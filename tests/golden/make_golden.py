"""Generates the golden fixtures in tests/golden/ from the reference renderer itself.

Run where the reference sources are (the reference is compiled by oracle/Makefile into
oracle/_ref/libmcrt_ref.so; it does not exist on GPU machines, so the fixtures are
committed):

    python tests/golden/make_golden.py

Fixtures (all seeded):
  ref_traverse_<name>.npz  triangles, the reference SplitBVH tree (splitbvh.cpp:1410-1625,
                           dumped node by node), ray sets and the reference's closest hits
                           (SplitBVH::intersect, splitbvh.cpp:1627-1642) and SceneBVH::occluded
                           answers (scenebvh.cpp:379-396)
  ref_functions.npz        per-function input/output vectors of the reference's BSDFs,
                           Fresnel, orthonormal frame, cosine warp, camera, discrete
                           sampler, triangle sampling and environment map
  ref_image_cornell.npz    the reference path tracer (demo_pt.cpp rayTrace, depth 10, no RR)
                           on its own Cornell box: per-pixel means of independent batches
  ref_paths_cornell.npz    the same path tracer single-threaded from the start of its global
                           random stream: every sample's radiance, for a draw-by-draw replay
  ref_obj.npz              an OBJ file (a displaced level-2 icosphere written here, with
                           comments and other records the reader skips), a transform, and
                           what the reference's Scene::loadModel makes of it: triangles,
                           vertex normals and Mesh::genNormals' alphas per corner
                               python tests/golden/make_golden.py --only-obj
  ref_traverse_cfg1.npz    hit parity at full scale: the displaced level-8 icosphere + ground
                           (1,310,722 T, scenes.cfg1_scene(); only its SHA-256 is stored, the
                           triangles are regenerated where the test runs), 65,536 rays in each
                           of the primary / bounce / incoherent / segment classes and the
                           reference SplitBVH's closest hits (prim, t) and occluded answers.
                           Its reference tree takes about 60-110 s to build:
                               python tests/golden/make_golden.py --only-cfg1
"""
from __future__ import annotations

import ctypes
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from mcrt_gb300 import scenes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
ptr = O.ptr


def ref_tree(ref, verts):
    n = verts.shape[0]
    h = ref.ref_bvh_create(ptr(verts), n, 1)
    nn, nr = ctypes.c_int(), ctypes.c_int()
    ref.ref_bvh_dump_sizes(h, ctypes.byref(nn), ctypes.byref(nr))
    node_box = np.zeros((nn.value, 6), np.float32)
    node_info = np.zeros((nn.value, 6), np.int32)
    ref_prim = np.zeros(nr.value, np.int32)
    ref_box = np.zeros((nr.value, 6), np.float32)
    ref.ref_bvh_dump(h, ptr(node_box), ptr(node_info), ptr(ref_prim), ptr(ref_box))
    return h, dict(node_box=node_box, node_info=node_info, ref_prim=ref_prim, ref_box=ref_box)


def ref_hits(ref, h, rays):
    n = rays.shape[0]
    t = np.zeros(n, np.float32)
    p = np.zeros(n, np.int32)
    u = np.zeros(n, np.float32)
    v = np.zeros(n, np.float32)
    ref.ref_bvh_intersect(h, ptr(rays), n, ptr(t), ptr(p), ptr(u), ptr(v), os.cpu_count() or 1)
    return t, p, u, v


def ref_occluded(ref, h, rays, tfar):
    occ = np.zeros(rays.shape[0], np.int32)
    rc = ref.ref_scenebvh_occluded(h, ptr(rays), rays.shape[0], ptr(tfar), ptr(occ))
    assert rc == 0
    return occ


def make_rays(o, d, tmin=1e-4, tmax=np.inf):
    r = np.zeros((o.shape[0], 8), np.float32)
    r[:, 0:3] = o
    r[:, 3] = tmin
    r[:, 4:7] = d
    r[:, 7] = tmax
    return r


def unit(v):
    v = np.asarray(v, np.float64)
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def camera_rays(ref, cam, w, h, rng, jitter=True):
    o = np.zeros(3, np.float32)
    d = np.zeros(3, np.float32)
    cam = np.asarray(cam, np.float32)
    out_o, out_d = [], []
    for y in range(h):
        for x in range(w):
            jx, jy = (rng.uniform(-1, 1, 2) if jitter else (0.0, 0.0))
            ref.ref_camera_ray(ptr(cam[0:3]), ptr(cam[3:6]), w, h, float(cam[9] if cam.size > 7 else cam[6]),
                               float((x + 0.5 + jx) / w), float((y + 0.5 + jy) / h), ptr(o), ptr(d))
            out_o.append(o.copy())
            out_d.append(d.copy())
    return np.array(out_o), np.array(out_d)


def traverse_fixture(ref, name, desc_verts, normals, cam, rng, n_random=8192, random_box=(-1.0, 1.0), res=48):
    verts = np.ascontiguousarray(desc_verts, np.float32)
    h, tree = ref_tree(ref, verts)
    sets = {}
    if cam is not None:
        o, d = camera_rays(ref, cam, res, res, rng)
        sets["primary"] = make_rays(o, d)
        t, p, u, v = ref_hits(ref, h, sets["primary"])
        hit = p >= 0
        ph = (o + d * t[:, None])[hit]
        nrm = normals.reshape(-1, 3, 3)[p[hit]].mean(axis=1) if normals is not None else None
        if nrm is None:
            tri = verts.reshape(-1, 3, 3)[p[hit]]
            nrm = np.cross(tri[:, 0] - tri[:, 2], tri[:, 1] - tri[:, 2])
        nrm = unit(nrm)
        # cosine-distributed bounce directions about the (interpolated) normal, flipped toward the viewer
        flip = np.sign(np.sum(-d[hit] * nrm, axis=1, keepdims=True))
        flip[flip == 0] = 1
        nrm = nrm * flip
        a = rng.normal(size=nrm.shape)
        bd = unit(nrm + unit(a))
        sets["bounce"] = make_rays(ph, bd)
    lo, hi = random_box
    o = rng.uniform(lo, hi, (n_random, 3)).astype(np.float32)
    d = unit(rng.uniform(-0.5, 0.5, (n_random, 3)))
    sets["incoherent"] = make_rays(o, d)
    # finite segments (shadow-ray like): tmax = distance to a random target point
    o2 = rng.uniform(lo, hi, (n_random // 2, 3)).astype(np.float32)
    tg = rng.uniform(lo, hi, (n_random // 2, 3)).astype(np.float32)
    seg = tg - o2
    dist = np.linalg.norm(seg, axis=1).astype(np.float32)
    sets["segment"] = make_rays(o2, unit(seg), tmax=dist)
    # axis-aligned directions: zero direction components take the reference's
    # inv_dir = 0 path (ray.cpp:39-42)
    na = 512
    o3 = rng.uniform(lo, hi, (na, 3)).astype(np.float32)
    d3 = np.zeros((na, 3), np.float32)
    ax = rng.integers(0, 3, na)
    d3[np.arange(na), ax] = rng.choice([-1.0, 1.0], na)
    sets["axis"] = make_rays(o3, d3)
    out = dict(verts=verts, **{f"tree_{k}": v for k, v in tree.items()})
    for k, r in sets.items():
        t, p, u, v = ref_hits(ref, h, r)
        out[f"rays_{k}"] = r
        out[f"t_{k}"] = t
        out[f"prim_{k}"] = p
        out[f"u_{k}"] = u
        out[f"v_{k}"] = v
        tfar = np.where(np.isfinite(r[:, 7]), r[:, 7], np.inf).astype(np.float32)
        # SceneBVH::occluded(ray, tfar) uses [1e-4, tfar - 1e-4]
        out[f"occ_{k}"] = ref_occluded(ref, h, r, tfar)
        print(f"{name}/{k}: {r.shape[0]} rays, hit {np.mean(p >= 0):.3f}")
    ref.ref_bvh_destroy(h)
    np.savez_compressed(os.path.join(OUT, f"ref_traverse_{name}.npz"), **out)


def obj_fixture(ref):
    rng = np.random.default_rng(7)
    v, f = scenes.icosphere(2)
    v = v * (1.0 + 0.2 * rng.uniform(-1, 1, (v.shape[0], 1)))
    lines = ["# displaced level-2 icosphere", "o sphere"]
    lines += [f"v {x:.7g} {y:.7g} {z:.7g}" for x, y, z in v]
    lines += ["vn 0 1 0", "vt 0.5 0.5", "s off"]
    lines += [f"f {a + 1} {b + 1} {c + 1}" for a, b, c in f]
    # no newline after the last record: Mesh::Mesh reads tokens while !eof(), and a final
    # newline makes it read one more face from the exhausted stream (indices 0 - 1, a face
    # outside the vertex array); without it the reference reads exactly the file's faces
    text = "\n".join(lines).encode()
    # translate, rotate about y, scale (a column-major glm::mat4, as Scene::loadModel gets it)
    c, s_ = np.cos(0.3), np.sin(0.3)
    m = np.array([[2 * c, 0, 2 * s_, 0.25], [0, 2, 0, -0.5], [-2 * s_, 0, 2 * c, 1.0], [0, 0, 0, 1]], np.float32)
    t16 = np.ascontiguousarray(m.T).ravel()
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "mesh.obj")
        with open(path, "wb") as fh:
            fh.write(text)
        n = ref.ref_load_obj(path.encode(), ptr(t16), None, None, None)
        verts = np.zeros((n, 9), np.float32)
        nrm = np.zeros((n, 9), np.float32)
        alpha = np.zeros((n, 3), np.float32)
        ref.ref_load_obj(path.encode(), ptr(t16), ptr(verts), ptr(nrm), ptr(alpha))
    np.savez_compressed(os.path.join(OUT, "ref_obj.npz"), obj=np.frombuffer(text, np.uint8), transform=m,
                        verts=verts, normals=nrm, alpha=alpha)
    print(f"obj: {n} triangles")


def geometry_sha256(verts) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(verts, np.float32).tobytes()).hexdigest()


def cfg1_traverse_fixture(ref, n=65536, seed=20261204):
    """Hit parity on the 1.31 M-triangle geometry of the large configuration, where the
    reference's absolute |det| < 1e-6 cull bites (edges of ~4.7e-3 on a unit sphere)."""
    rng = np.random.default_rng(seed)
    desc = scenes.cfg1_scene()
    verts = np.ascontiguousarray(desc.vertices, np.float32)
    h, _ = ref_tree(ref, verts)  # the tree itself is not stored (about 100 MB)
    sets = {}
    # primary: the large configuration's camera at random film positions
    cam = scenes.cfg1_camera(1024, 1024).as_array()
    m = rng.uniform(0, 1, (n, 2)).astype(np.float32)
    o, d = np.zeros(3, np.float32), np.zeros(3, np.float32)
    po, pd = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
    for i in range(n):
        ref.ref_camera_ray(ptr(cam[0:3]), ptr(cam[3:6]), 1024, 1024, float(cam[9]), float(m[i, 0]),
                           float(m[i, 1]), ptr(o), ptr(d))
        po[i], pd[i] = o, d
    sets["primary"] = make_rays(po, pd)
    t, p, _, _ = ref_hits(ref, h, sets["primary"])
    hit = np.nonzero(p >= 0)[0]
    # bounce: cosine-distributed about the interpolated normal (flipped to the viewer) at
    # primary hit points, resampled to n rays
    pick = rng.choice(hit, n)
    ph = (po[pick] + pd[pick] * t[pick, None]).astype(np.float32)
    nrm = unit(desc.normals.reshape(-1, 3, 3)[p[pick]].mean(axis=1))
    flip = np.sign(np.sum(-pd[pick] * nrm, axis=1, keepdims=True))
    flip[flip == 0] = 1
    nrm = nrm * flip
    sets["bounce"] = make_rays(ph, unit(nrm + unit(rng.normal(size=nrm.shape))))
    # incoherent: origins uniform in [-2, 2]^3, directions uniform on the sphere (the
    # random-ray measurement of the reference SplitBVH)
    sets["incoherent"] = make_rays(rng.uniform(-2, 2, (n, 3)).astype(np.float32), unit(rng.normal(size=(n, 3))))
    # segment: finite rays between random points around the sphere (next-event-like)
    o2 = rng.uniform(-1.3, 1.3, (n, 3)).astype(np.float32)
    seg = rng.uniform(-1.3, 1.3, (n, 3)).astype(np.float32) - o2
    sets["segment"] = make_rays(o2, unit(seg), tmax=np.linalg.norm(seg, axis=1).astype(np.float32))
    out = dict(verts_sha256=np.array(geometry_sha256(verts)), num_triangles=np.array(verts.shape[0]))
    for k, r in sets.items():
        t, p, _, _ = ref_hits(ref, h, r)
        out[f"rays_{k}"], out[f"t_{k}"], out[f"prim_{k}"] = r, t, p
        tfar = np.where(np.isfinite(r[:, 7]), r[:, 7], np.inf).astype(np.float32)
        out[f"occ_{k}"] = ref_occluded(ref, h, r, tfar).astype(np.int8)
        print(f"cfg1/{k}: {r.shape[0]} rays, hit {np.mean(p >= 0):.3f}")
    ref.ref_bvh_destroy(h)
    np.savez_compressed(os.path.join(OUT, "ref_traverse_cfg1.npz"), **out)


def functions_fixture(ref, rng):
    out = {}
    n = 2000
    types = [1, 2, 3, 4]  # DIFF, SPEC, REFR, GLSY (the reference's BSDFs)
    wi = unit(rng.normal(size=(n, 3)))
    nl = unit(rng.normal(size=(n, 3)))
    r = rng.uniform(size=(n, 2)).astype(np.float32)
    col = rng.uniform(0.05, 1.0, (n, 3)).astype(np.float32)
    for ty in types:
        wo = np.zeros((n, 3), np.float32)
        w = np.zeros((n, 3), np.float32)
        pdf = np.zeros(n, np.float32)
        cw = np.zeros(n, np.float32)
        f = np.zeros((n, 3), np.float32)
        epdf = np.zeros(n, np.float32)
        wo2 = unit(rng.normal(size=(n, 3)))
        for i in range(n):
            a, b = ctypes.c_float(), ctypes.c_float()
            ref.ref_material_sample(ty, ptr(col[i]), ptr(wi[i]), ptr(nl[i]), float(r[i, 0]), float(r[i, 1]),
                                    ptr(wo[i]), ptr(w[i]), ctypes.byref(a), ctypes.byref(b))
            pdf[i], cw[i] = a.value, b.value
            ref.ref_material_evaluate(ty, ptr(col[i]), ptr(wi[i]), ptr(nl[i]), ptr(wo2[i]), ptr(f[i]),
                                      ctypes.byref(a))
            epdf[i] = a.value
        out[f"mat{ty}_wo"], out[f"mat{ty}_weight"], out[f"mat{ty}_pdf"] = wo, w, pdf
        out[f"mat{ty}_eval_wo"], out[f"mat{ty}_eval_f"], out[f"mat{ty}_eval_pdf"] = wo2, f, epdf
    out["mat_wi"], out["mat_nl"], out["mat_r"], out["mat_color"] = wi, nl, r, col
    # Fresnel
    c = rng.uniform(-1, 1, n).astype(np.float32)
    ior = rng.uniform(1.0, 2.5, n).astype(np.float32)
    out["fresnel_cos"], out["fresnel_ior"] = c, ior
    out["fresnel"] = np.array([ref.ref_fresnel(float(a), float(b)) for a, b in zip(c, ior)], np.float32)
    # frame + cosine warp
    cc = rng.normal(size=(n, 3)).astype(np.float32)
    out["onb_n"], out["onb_c"] = nl, cc
    tw = np.zeros((n, 3), np.float32)
    for i in range(n):
        ref.ref_onb_to_world(ptr(nl[i]), ptr(cc[i]), ptr(tw[i]))
    out["onb_world"] = tw
    hs = np.zeros((n, 3), np.float32)
    for i in range(n):
        ref.ref_sample_hemisphere_cosine(float(r[i, 0]), float(r[i, 1]), ptr(hs[i]))
    out["cosine_hemisphere"] = hs
    # camera
    cam = np.array([0.3, 0.2, 3.5, 0.0, -0.1, 0.0, 0, 1, 0, 40.0], np.float32)
    m = rng.uniform(0, 1, (n, 2)).astype(np.float32)
    co = np.zeros((n, 3), np.float32)
    cd = np.zeros((n, 3), np.float32)
    for i in range(n):
        ref.ref_camera_ray(ptr(cam[0:3]), ptr(cam[3:6]), 320, 240, float(cam[9]), float(m[i, 0]), float(m[i, 1]),
                           ptr(co[i]), ptr(cd[i]))
    out["camera"], out["camera_m"], out["camera_o"], out["camera_d"] = cam, m, co, cd
    # discrete sampler
    wts = rng.uniform(0, 1, 37).astype(np.float32)
    wts[5] = 0.0
    rr = rng.uniform(0, 1, n).astype(np.float32)
    pd = ctypes.c_float()
    idx = []
    pds = []
    for x in rr:
        idx.append(ref.ref_discrete_sample(ptr(wts), wts.size, float(x), ctypes.byref(pd)))
        pds.append(pd.value)
    out["discrete_w"], out["discrete_r"] = wts, rr
    out["discrete_idx"], out["discrete_pdf"] = np.array(idx, np.int32), np.array(pds, np.float32)
    # triangle sampling / normal / area
    tri = rng.uniform(-1, 1, (n, 9)).astype(np.float32)
    pts = np.zeros((n, 3), np.float32)
    uv = np.zeros((n, 2), np.float32)
    fn = np.zeros((n, 3), np.float32)
    ar = np.zeros(n, np.float32)
    for i in range(n):
        ref.ref_triangle_sample_point(ptr(tri[i]), float(r[i, 0]), float(r[i, 1]), ptr(pts[i]), ptr(uv[i]))
        a = ctypes.c_float()
        ref.ref_triangle_normal_area(ptr(tri[i]), ptr(fn[i]), ctypes.byref(a))
        ar[i] = a.value
    out["tri"], out["tri_point"], out["tri_uv"], out["tri_normal"], out["tri_area"] = tri, pts, uv, fn, ar
    # environment map: small procedural map through the reference loader
    env = scenes.sky_envmap(64, 32, sun_diameter_deg=6.0, sun_radiance=50.0)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "env.bin")
        scenes.write_envmap_bin(path, env)
        eh = ref.ref_envmap_load(path.encode())
        dirs = unit(rng.normal(size=(n, 3)))
        epdf = np.array([ref.ref_envmap_pdf(eh, ptr(dd)) for dd in dirs], np.float32)
        erad = np.zeros((n, 3), np.float32)
        for i in range(n):
            ref.ref_envmap_radiance(eh, ptr(dirs[i]), ptr(erad[i]))
        sdir = np.zeros((n, 3), np.float32)
        srad = np.zeros((n, 3), np.float32)
        spdf = np.zeros(n, np.float32)
        for i in range(n):
            p_ = ctypes.c_float()
            ref.ref_envmap_sample(eh, float(r[i, 0]), float(r[i, 1]), ptr(sdir[i]), ptr(srad[i]), ctypes.byref(p_))
            spdf[i] = p_.value
        ref.ref_envmap_destroy(eh)
    out["env"], out["env_dirs"], out["env_pdf"], out["env_rad"] = env, dirs, epdf, erad
    out["env_sample_dir"], out["env_sample_rad"], out["env_sample_pdf"] = sdir, srad, spdf
    np.savez_compressed(os.path.join(OUT, "ref_functions.npz"), **out)
    print("functions:", len(out), "arrays")


def cornell_image_fixture(ref, res=32, spp=256, batches=16):
    n = ref.ref_cornell_export(None, None, None, None)
    verts = np.zeros((n, 9), np.float32)
    mt = np.zeros(n, np.int32)
    mc = np.zeros((n, 3), np.float32)
    cam = np.zeros(7, np.float32)
    ref.ref_cornell_export(ptr(verts), ptr(mt), ptr(mc), ptr(cam))
    imgs = []
    rays = 0
    secs = 0.0
    for _ in range(batches):
        img = np.zeros((res, res, 3), np.float32)
        ni, no, sec = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_double()
        ref.ref_render_cornell(res, res, spp, os.cpu_count() or 1, 0, res, ptr(img), ctypes.byref(ni),
                               ctypes.byref(no), ctypes.byref(sec))
        imgs.append(img)
        rays += ni.value + no.value
        secs += sec.value
    imgs = np.array(imgs)
    np.savez_compressed(os.path.join(OUT, "ref_image_cornell.npz"), verts=verts, mat_types=mt, mat_colors=mc,
                        camera=cam, batch_means=imgs, spp_per_batch=spp, rays=rays, seconds=secs)
    print(f"cornell image: {batches}x{spp} spp at {res}^2, {rays / max(secs, 1e-9) / 1e6:.2f} Mrays/s")


def cornell_paths_fixture(ref, res=16, spp=8):
    """Per-sample radiance of the reference's rayTrace on its Cornell box, rendered
    single-threaded from the start of the global randf() stream (must run first in the
    process), with the number of randf() draws consumed after each sample."""
    paths = np.zeros((res, res, spp, 3), np.float32)
    draws = np.zeros(res * res * spp, np.int64)
    ref.ref_cornell_paths(res, res, spp, ptr(paths), ptr(draws))
    np.savez_compressed(os.path.join(OUT, "ref_paths_cornell.npz"), paths=paths, draws=draws, res=res, spp=spp)
    print(f"cornell paths: {res}x{res}x{spp} samples, {draws[-1]} draws")


def film_images(rng):
    """Test images for the film writers: radiance over many octaves, exact zeros, values
    below the RGBE cut-off, exact powers of two, values above 1 for the PPM clamp; one
    image wider than 255 pixels (two-byte scanline width, several 127-byte runs)."""
    imgs = []
    for (h, w) in ((23, 37), (5, 300), (1, 1), (3, 127), (2, 128)):
        a = np.exp(rng.uniform(-9.0, 7.0, (h, w, 3))).astype(np.float32)
        a[rng.uniform(size=(h, w)) < 0.08] = 0.0
        a[rng.uniform(size=(h, w)) < 0.04] = 1e-33
        a[rng.uniform(size=(h, w, 3)) < 0.05] = 2.0 ** rng.integers(-6, 7, 1)[0]
        imgs.append(a)
    return imgs


def film_fixture(ref):
    """FrameBuffer::dumpHDR / dumpPPM bytes and tonemapGamma / tonemapReinhard outputs of
    the reference (film.cpp) for seeded images."""
    import tempfile
    rng = np.random.default_rng(33)
    out = {}
    for k, img in enumerate(film_images(rng)):
        h, w = img.shape[:2]
        out[f"img{k}"] = img
        with tempfile.TemporaryDirectory() as d:
            for hdr, ext in ((1, "hdr"), (0, "ppm")):
                path = os.path.join(d, f"f.{ext}")
                ref.ref_film_dump(w, h, ptr(img), path.encode(), hdr)
                out[f"{ext}{k}"] = np.frombuffer(open(path, "rb").read(), np.uint8)
        for mode, name in ((0, "gamma"), (1, "reinhard")):
            t = np.array(img, np.float32, copy=True)
            ref.ref_film_tonemap(w, h, ptr(t), mode, 2.2)
            out[f"{name}{k}"] = t
    np.savez_compressed(os.path.join(OUT, "ref_film.npz"), **out)


def consistent_fixture(ref):
    """TriangleObject::consistentNormal on random triangles / directions / barycentrics,
    and Mesh::genNormals' vertex normals and alphas of an indexed displaced icosphere."""
    rng = np.random.default_rng(44)
    n = 2000
    abc = rng.normal(size=(n, 9)).astype(np.float32)
    nabc = rng.normal(size=(n, 3, 3))
    nabc /= np.linalg.norm(nabc, axis=2, keepdims=True)
    nabc = nabc.reshape(n, 9).astype(np.float32)
    alpha = rng.uniform(0.0, 1.2, (n, 3)).astype(np.float32)
    u = rng.uniform(0, 1, n).astype(np.float32)
    v = (rng.uniform(0, 1, n) * (1 - u)).astype(np.float32)
    wi = rng.normal(size=(n, 3))
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    # keep wi on the side of the interpolated normal (as a view direction is)
    nint = (1 - u - v)[:, None] * nabc[:, 0:3] + u[:, None] * nabc[:, 3:6] + v[:, None] * nabc[:, 6:9]
    wi = np.where((np.sum(wi * nint, axis=1) < 0)[:, None], -wi, wi).astype(np.float32)
    out = np.zeros((n, 7), np.float32)
    for i in range(n):
        nc, rf, cs = np.zeros(3, np.float32), np.zeros(3, np.float32), np.zeros(1, np.float32)
        ref.ref_consistent_normal(ptr(abc[i]), ptr(nabc[i]), ptr(alpha[i]), ptr(wi[i]), float(u[i]), float(v[i]),
                                  ptr(nc), ptr(rf), ptr(cs))
        out[i, 0:3], out[i, 3:6], out[i, 6] = nc, rf, cs[0]
    verts, faces = scenes.icosphere(2)
    verts = (verts * (1.0 + 0.15 * rng.uniform(-1, 1, (verts.shape[0], 1)))).astype(np.float32)
    faces = faces.astype(np.int32)
    vn = np.zeros_like(verts)
    va = np.zeros(verts.shape[0], np.float32)
    ref.ref_mesh_alpha(ptr(verts), verts.shape[0], ptr(faces), faces.shape[0], ptr(vn), ptr(va))
    np.savez_compressed(os.path.join(OUT, "ref_consistent.npz"), abc=abc, nabc=nabc, alpha=alpha, u=u, v=v, wi=wi,
                        out=out, mesh_verts=verts, mesh_faces=faces, mesh_normals=vn, mesh_alpha=va)


def main():
    ref = O.load_reference()
    if ref is None:
        raise SystemExit("reference sources not available: cannot regenerate fixtures")
    if "--only-film" in sys.argv:
        film_fixture(ref)
        return
    if "--only-consistent" in sys.argv:
        consistent_fixture(ref)
        return
    if "--only-obj" in sys.argv:
        obj_fixture(ref)
        return
    if "--only-cfg1" in sys.argv:
        cfg1_traverse_fixture(ref)
        return
    film_fixture(ref)
    consistent_fixture(ref)
    cornell_paths_fixture(ref)  # first: the global random stream starts at its seed here
    rng = np.random.default_rng(20261203)
    # the reference's own Cornell box (demo_pt.cpp:83-414)
    n = ref.ref_cornell_export(None, None, None, None)
    cv = np.zeros((n, 9), np.float32)
    mt = np.zeros(n, np.int32)
    mc = np.zeros((n, 3), np.float32)
    cam7 = np.zeros(7, np.float32)
    ref.ref_cornell_export(ptr(cv), ptr(mt), ptr(mc), ptr(cam7))
    cam = np.concatenate([cam7[:6], [0, 1, 0], cam7[6:]]).astype(np.float32)
    traverse_fixture(ref, "cornell", cv, None, cam, rng, n_random=4096, random_box=(0.0, 56.0), res=32)
    # cfg0 scene (Cornell shell + level-4 icosphere)
    s0 = scenes.cfg0_scene()
    cam0 = scenes.cfg0_camera(48, 48).as_array()
    traverse_fixture(ref, "cfg0", s0.vertices, s0.normals, cam0, rng, n_random=8192)
    # displaced level-5 sphere (20,480 T): small triangles, grazing |det| culls
    v5, n5 = scenes.displaced_sphere(5, 1.0, 0.1, 7)
    cam5 = np.array([0.0, 0.4, 3.0, 0.0, 0.0, 0.0, 0, 1, 0, 45.0], np.float32)
    traverse_fixture(ref, "sphere5", v5, n5, cam5, rng, n_random=8192, random_box=(-1.5, 1.5))
    # split-BVH benchmark mesh (debug_mesh.cpp:761-778): vector3f(randf()*2-1) broadcasts
    # one number to x, y and z, so every triangle is collinear and nothing is hit
    # (100 of them here: the spatial splits of collinear triangles multiply references)
    diag = np.repeat(rng.uniform(-1, 1, (100, 3, 1)), 3, axis=2).reshape(100, 9).astype(np.float32)
    traverse_fixture(ref, "debugmesh_diag", diag, None, None, rng, n_random=2048)
    # the same benchmark with independent coordinates (rays as demo_splitbvh.cpp:200-238)
    rnd = rng.uniform(-1, 1, (1000, 9)).astype(np.float32)
    traverse_fixture(ref, "debugmesh", rnd, None, None, rng, n_random=16384)
    functions_fixture(ref, rng)
    cornell_image_fixture(ref)
    obj_fixture(ref)


if __name__ == "__main__":
    main()
