"""Procedural scenes for the five benchmark configurations (seeded, no external data).

  cfg0  Cornell box of 5 wall quads (10 T, Lambert 0.73 / red 0.65,0.05,0.05 /
        green 0.12,0.45,0.15), a 2-T ceiling emitter of radiance (17,12,4) and a
        level-4 icosphere (5,120 T, r = 0.3, Lambert 0.8); 256^2, 16 spp, depth 8, RR from 3
  cfg1  level-8 icosphere (1,310,720 T) radially displaced by seeded 3-octave value noise
        (amplitude 0.1) on a 2-T ground plane; 1,024-T patches of 40 % Lambert /
        30 % GGX (roughness U[0.05, 0.5]) / 30 % dielectric (IOR 1.5); procedural
        1024x512 environment map (sky gradient + 0.5 deg sun disc of radiance 1e4);
        1024^2, 64 spp, depth 16
  cfg2  64 scenes: displaced icospheres of log-uniform 1k..500k T inside a Cornell shell,
        resolutions {128,256,512,1024}^2, spp 1..64, depth 4..16
  cfg3  cfg0 with the sphere split into 256 albedo groups + the emitter radiance as
        parameters; 512^2, 32 spp, depth 6
  cfg4  cfg1 geometry and environment map seen from 32 cameras on a Fibonacci sphere of
        radius 3; 4,096 Lambert patch albedos as parameters; 256^2, 16 spp, depth 8

Box extents, emitter size and cameras are not fixed by the configuration text; the
values chosen here are the ones every renderer (GPU, oracle, reference) is fed.
The environment map uses the reference's direction convention (envmap.cpp:414-459):
texel (u, v) -> (sin(v pi) sin(2 pi u), cos(v pi), -sin(v pi) cos(2 pi u)).
"""
from __future__ import annotations

import math

import numpy as np

from .scene import DIFF, GGX, LGHT, REFR, CameraDesc, Material, SceneDesc

CORNELL_CAMERA = dict(origin=(0.0, 0.0, 3.5), target=(0.0, 0.0, 0.0), fov_y=40.0)


# ---------------------------------------------------------------------------
# meshes
# ---------------------------------------------------------------------------
def icosphere(level: int):
    """Unit icosphere with hierarchical face order: the children of face f at level
    L are faces 4f..4f+3 at level L+1, so runs of 4^k faces are spatial patches."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        nv = v.shape[0]
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        e = np.stack([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)], 1).reshape(-1, 2)
        e.sort(axis=1)
        key = e[:, 0] * nv + e[:, 1]
        uk, inv = np.unique(key, return_inverse=True)
        i0, i1 = uk // nv, uk % nv
        mid = v[i0] + v[i1]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid])
        m = (inv + nv).reshape(-1, 3)
        ab, bc, ca = m[:, 0], m[:, 1], m[:, 2]
        f = np.stack([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1), np.stack([c, ca, bc], 1),
                      np.stack([ab, bc, ca], 1)], 1).reshape(-1, 3)
    return v, f


def _value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """3-D lattice value noise in [-1, 1] with smoothstep trilinear interpolation."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(256)
    vals = rng.uniform(-1.0, 1.0, 256)

    def h(ix, iy, iz):
        return vals[perm[(perm[(perm[ix & 255] + iy) & 255] + iz) & 255]]

    fl = np.floor(p)
    i = fl.astype(np.int64)
    fr = p - fl
    w = fr * fr * (3.0 - 2.0 * fr)
    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                wx = w[:, 0] if dx else 1.0 - w[:, 0]
                wy = w[:, 1] if dy else 1.0 - w[:, 1]
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out = out + wx * wy * wz * h(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz)
    return out


def displaced_sphere(level: int, radius: float, amplitude: float, seed: int, center=(0.0, 0.0, 0.0)):
    """Icosphere displaced radially by 3-octave value noise; returns (verts (n,9), normals (n,9))."""
    v, f = icosphere(level)
    n = np.zeros(v.shape[0])
    if amplitude != 0.0:
        wsum = 0.0
        for k in range(3):
            wgt = 0.5 ** k
            n += wgt * _value_noise(v * (2.0 * 2 ** k) + 17.0 * k, seed + k)
            wsum += wgt
        n /= wsum
    pos = v * (radius * (1.0 + amplitude * n))[:, None] + np.asarray(center)[None, :]
    if amplitude == 0.0:
        vn = v.copy()
    else:
        # area-weighted vertex normals (as Mesh::genNormals, mesh.cpp:66-118)
        fa, fb, fc = pos[f[:, 0]], pos[f[:, 1]], pos[f[:, 2]]
        fn = np.cross(fb - fa, fc - fa)
        vn = np.zeros_like(pos)
        for k in range(3):
            np.add.at(vn, f[:, k], fn)
        vn /= np.linalg.norm(vn, axis=1, keepdims=True)
    verts = pos[f].reshape(-1, 9).astype(np.float32)
    norms = vn[f].reshape(-1, 9).astype(np.float32)
    return verts, norms


def _quad(p0, p1, p2, p3, normal):
    """Two triangles (p0,p1,p2), (p0,p2,p3) wound so that TriangleObject's face normal
    normalize(cross(a - c, b - c)) (triangle.cpp:71) equals `normal`."""
    tris = []
    for a, b, c in ((p0, p1, p2), (p0, p2, p3)):
        a, b, c = np.asarray(a, np.float64), np.asarray(b, np.float64), np.asarray(c, np.float64)
        if np.dot(np.cross(a - c, b - c), normal) < 0:
            b, c = c, b
        tris.append(np.concatenate([a, b, c]))
    verts = np.array(tris, np.float32)
    norms = np.tile(np.asarray(normal, np.float32), (2, 3))
    return verts, norms


def cornell_shell(emitter_radiance=(17.0, 12.0, 4.0)):
    """5 wall quads of the box [-1, 1]^3 open at +z, normals facing inward, plus the
    0.5 x 0.5 ceiling emitter just below the ceiling, facing down."""
    grey, red, green = (0.73, 0.73, 0.73), (0.65, 0.05, 0.05), (0.12, 0.45, 0.15)
    quads = [
        ((-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1), (0, 1, 0), grey),     # floor
        ((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1), (0, -1, 0), grey),       # ceiling
        ((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (0, 0, 1), grey),    # back
        ((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1), (1, 0, 0), red),     # left
        ((1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1), (-1, 0, 0), green),      # right
    ]
    verts, norms, colors = [], [], []
    for p0, p1, p2, p3, nrm, col in quads:
        v, n = _quad(p0, p1, p2, p3, nrm)
        verts.append(v)
        norms.append(n)
        colors += [col, col]
    y = 0.999
    v, n = _quad((-0.25, y, -0.25), (0.25, y, -0.25), (0.25, y, 0.25), (-0.25, y, 0.25), (0, -1, 0))
    verts.append(v)
    norms.append(n)
    return np.concatenate(verts), np.concatenate(norms), colors, emitter_radiance


def _assemble(parts):
    """parts: list of (verts, norms, material_index_per_tri)."""
    v = np.concatenate([p[0] for p in parts]).astype(np.float32)
    n = np.concatenate([p[1] for p in parts]).astype(np.float32)
    m = np.concatenate([p[2] for p in parts]).astype(np.int32)
    return v, n, m


# ---------------------------------------------------------------------------
# environment map
# ---------------------------------------------------------------------------
def sky_envmap(width=1024, height=512, sun_elevation_deg=40.0, sun_azimuth_deg=60.0, sun_radiance=1e4,
               sun_diameter_deg=0.5):
    """Vertical sky gradient + sun disc; (H, W, 3) float32, top row first."""
    u = (np.arange(width) + 0.5) / width
    v = (np.arange(height) + 0.5) / height
    phi = v[:, None] * math.pi
    theta = u[None, :] * 2 * math.pi
    dy = np.cos(phi) * np.ones_like(theta)
    horizon = np.array([0.95, 0.85, 0.75])
    zenith = np.array([0.20, 0.40, 0.95])
    ground = np.array([0.25, 0.22, 0.20])
    s = np.sqrt(np.clip(dy, 0.0, 1.0))[..., None]
    sky = horizon * (1 - s) + zenith * s
    gnd = ground * (0.6 + 0.4 * np.clip(1.0 + dy, 0.0, 1.0))[..., None]
    img = np.where((dy >= 0)[..., None], sky, gnd)
    # sun: per-texel coverage of the disc by 16x16 supersampling near the sun direction
    el, az = math.radians(sun_elevation_deg), math.radians(sun_azimuth_deg)
    ps = math.pi / 2 - el
    sun = np.array([math.sin(ps) * math.sin(az), math.cos(ps), -math.sin(ps) * math.cos(az)])
    cos_r = math.cos(math.radians(sun_diameter_deg / 2))
    vc = int(ps / math.pi * height)
    uc = int(az / (2 * math.pi) * width)
    k = 4
    for m in range(max(0, vc - k), min(height, vc + k + 1)):
        for nn in range(uc - k, uc + k + 1):
            n_ = nn % width
            ss = (np.arange(16) + 0.5) / 16
            uu = (n_ + ss[None, :]) / width
            vv = (m + ss[:, None]) / height
            ph, th = vv * math.pi, uu * 2 * math.pi
            d = np.stack([np.sin(ph) * np.sin(th), np.cos(ph) * np.ones_like(th), -np.sin(ph) * np.cos(th)], -1)
            cov = float(np.mean(d @ sun >= cos_r))
            if cov > 0:
                img[m, n_] = img[m, n_] * (1 - cov) + sun_radiance * cov
    return img.astype(np.float32)


def write_envmap_bin(path: str, img: np.ndarray) -> None:
    """The reference's .bin format: {int32 width, int32 height} + row-major RGB float32
    (envmap.cpp:98-119)."""
    h, w, _ = img.shape
    with open(path, "wb") as f:
        np.array([w, h], np.int32).tofile(f)
        np.ascontiguousarray(img, np.float32).tofile(f)


# ---------------------------------------------------------------------------
# configurations
# ---------------------------------------------------------------------------
def cfg0_scene(sphere_level: int = 4) -> SceneDesc:
    wv, wn, colors, erad = cornell_shell()
    mats = [Material(DIFF, c) for c in colors] + [Material(LGHT, erad)]
    wm = np.concatenate([np.arange(10), [10, 10]])  # 10 wall triangles, 2 emitter triangles
    sv, sn = displaced_sphere(sphere_level, 0.3, 0.0, 0, center=(0.0, -0.7, 0.0))
    mats.append(Material(DIFF, (0.8, 0.8, 0.8)))
    sm = np.full(sv.shape[0], len(mats) - 1)
    v, n, m = _assemble([(wv, wn, wm), (sv, sn, sm)])
    return SceneDesc(v, m, mats, normals=n, name="cfg0")


def cfg0_camera(width=256, height=256) -> CameraDesc:
    return CameraDesc(width=width, height=height, **CORNELL_CAMERA)


CFG0 = dict(width=256, height=256, spp=16, max_depth=8, rr_depth=3)


def _patch_materials(n_patches: int, rng) -> list:
    mats = []
    kinds = rng.uniform(size=n_patches)
    for k in range(n_patches):
        if kinds[k] < 0.4:
            mats.append(Material(DIFF, tuple(rng.uniform(0.2, 0.9, 3))))
        elif kinds[k] < 0.7:
            mats.append(Material(GGX, tuple(rng.uniform(0.5, 1.0, 3)), roughness=float(rng.uniform(0.05, 0.5))))
        else:
            mats.append(Material(REFR, (1.0, 1.0, 1.0), ior=1.5))
    return mats


def cfg1_scene(level: int = 8, seed: int = 1, env_size=(1024, 512), patch_tris: int = 1024) -> SceneDesc:
    rng = np.random.default_rng(seed)
    sv, sn = displaced_sphere(level, 1.0, 0.1, seed)
    n_faces = sv.shape[0]
    patch_tris = min(patch_tris, n_faces)
    n_patches = (n_faces + patch_tris - 1) // patch_tris
    mats = _patch_materials(n_patches, rng)
    sm = np.arange(n_faces) // patch_tris
    gy = -1.15
    gv, gn = _quad((-20, gy, -20), (20, gy, -20), (20, gy, 20), (-20, gy, 20), (0, 1, 0))
    mats.append(Material(DIFF, (0.5, 0.5, 0.5)))
    gm = np.full(2, len(mats) - 1)
    v, n, m = _assemble([(sv, sn, sm), (gv, gn, gm)])
    env = sky_envmap(env_size[0], env_size[1])
    return SceneDesc(v, m, mats, normals=n, envmap=env, name="cfg1")


def cfg1_camera(width=1024, height=1024) -> CameraDesc:
    return CameraDesc(origin=(0.0, 0.9, 3.6), target=(0.0, -0.1, 0.0), width=width, height=height, fov_y=40.0)


CFG1 = dict(width=1024, height=1024, spp=64, max_depth=16, rr_depth=-1)


def cfg2_jobs(n_scenes: int = 64, seed: int = 2, max_level: int = 7):
    """Returns a list of (SceneDesc, CameraDesc, params dict)."""
    rng = np.random.default_rng(seed)
    jobs = []
    levels = np.arange(3, max_level + 1)
    for k in range(n_scenes):
        target = math.exp(rng.uniform(math.log(1e3), math.log(5e5)))
        lv = int(levels[np.argmin(np.abs(np.log(20 * 4.0 ** levels) - math.log(target)))])
        res = int(rng.choice([128, 256, 512, 1024]))
        spp = int(rng.integers(1, 65))
        depth = int(rng.integers(4, 17))
        wv, wn, colors, erad = cornell_shell()
        mats = [Material(DIFF, c) for c in colors] + [Material(LGHT, erad)]
        wm = np.concatenate([np.arange(10), [10, 10]])
        sv, sn = displaced_sphere(lv, 0.45, 0.1, seed * 1000 + k, center=(0.0, -0.45, 0.0))
        n_faces = sv.shape[0]
        patch = max(16, min(1024, n_faces // 64))
        n_patches = (n_faces + patch - 1) // patch
        pm = _patch_materials(n_patches, rng)
        sm = len(mats) + np.arange(n_faces) // patch
        mats += pm
        v, n, m = _assemble([(wv, wn, wm), (sv, sn, sm)])
        desc = SceneDesc(v, m, mats, normals=n, name=f"cfg2_{k}")
        cam = CameraDesc(width=res, height=res, **CORNELL_CAMERA)
        jobs.append((desc, cam, dict(spp=spp, max_depth=depth, rr_depth=-1, seed=1000 + k)))
    return jobs


def cfg3_scene(param_seed: int = 3, groups: int = 256):
    """Returns (SceneDesc, albedo params (groups, 3), emission params (1, 3))."""
    rng = np.random.default_rng(param_seed)
    albedo = rng.uniform(0.1, 0.9, (groups, 3)).astype(np.float32)
    emission = np.array([[17.0, 12.0, 4.0]], np.float32)
    return cfg3_with_params(albedo, emission), albedo, emission


def cfg3_with_params(albedo: np.ndarray, emission: np.ndarray, sphere_level: int = 4) -> SceneDesc:
    groups = albedo.shape[0]
    wv, wn, colors, _ = cornell_shell(tuple(float(x) for x in emission[0]))
    mats = [Material(DIFF, c) for c in colors] + [Material(LGHT, tuple(float(x) for x in emission[0]),
                                                           emission_param=0)]
    wm = np.concatenate([np.arange(10), [10, 10]])
    sv, sn = displaced_sphere(sphere_level, 0.3, 0.0, 0, center=(0.0, -0.7, 0.0))
    per = sv.shape[0] // groups
    base = len(mats)
    for g in range(groups):
        mats.append(Material(DIFF, tuple(float(x) for x in albedo[g]), albedo_param=g))
    sm = base + np.minimum(np.arange(sv.shape[0]) // per, groups - 1)
    v, n, m = _assemble([(wv, wn, wm), (sv, sn, sm)])
    return SceneDesc(v, m, mats, normals=n, name="cfg3")


CFG3 = dict(width=512, height=512, spp=32, max_depth=6, rr_depth=-1)


def fibonacci_cameras(n=32, radius=3.0, width=256, height=256, fov_y=40.0):
    cams = []
    ga = math.pi * (3.0 - math.sqrt(5.0))
    for i in range(n):
        y = 1.0 - 2.0 * (i + 0.5) / n
        r = math.sqrt(max(0.0, 1.0 - y * y))
        th = ga * i
        o = (radius * r * math.cos(th), radius * y, radius * r * math.sin(th))
        up = (0.0, 1.0, 0.0) if abs(y) < 0.99 else (1.0, 0.0, 0.0)
        cams.append(CameraDesc(origin=o, target=(0.0, 0.0, 0.0), width=width, height=height, fov_y=fov_y, up=up))
    return cams


def cfg4_scene(level: int = 8, seed: int = 4, n_params: int = 4096, env_size=(1024, 512)):
    """Returns (SceneDesc, albedo params (n_params, 3))."""
    rng = np.random.default_rng(seed)
    sv, sn = displaced_sphere(level, 1.0, 0.1, 1)
    n_faces = sv.shape[0]
    per = max(1, n_faces // n_params)
    albedo = rng.uniform(0.1, 0.9, (n_params, 3)).astype(np.float32)
    mats = [Material(DIFF, tuple(float(x) for x in albedo[g]), albedo_param=g) for g in range(n_params)]
    sm = np.minimum(np.arange(n_faces) // per, n_params - 1)
    gy = -1.15
    gv, gn = _quad((-20, gy, -20), (20, gy, -20), (20, gy, 20), (-20, gy, 20), (0, 1, 0))
    mats.append(Material(DIFF, (0.5, 0.5, 0.5)))
    gm = np.full(2, len(mats) - 1)
    v, n, m = _assemble([(sv, sn, sm), (gv, gn, gm)])
    env = sky_envmap(env_size[0], env_size[1])
    return SceneDesc(v, m, mats, normals=n, envmap=env, name="cfg4"), albedo


CFG4 = dict(width=256, height=256, spp=16, max_depth=8, rr_depth=-1, views=32)
