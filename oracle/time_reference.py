"""Times the reference's own CPU path tracer next to the oracle's float port, on one host.

The reference side is `demo_pt.cpp`'s own `rayTrace` in `DemoSimple::run`'s pixel loop
(`oracle/_ref`, entry `ref_render_pt`): the scene is built through the reference API
(`todo_addMaterial`, `TriangleObject`, `Scene::add/setCamera/setEnvmap/finalize`, which
builds its SplitBVH), and rays are counted by the link-time wrappers around
`SceneBVH::intersect/occluded`.  Materials the reference cannot express are substituted
as the reference would have to: GGX conductor -> GLSY (Phong), the dielectric keeps the
reference's fixed IOR 1.33, depth is the reference's fixed 10 with no Russian roulette.

The port side is the oracle's float restatement of the estimator as this library
specifies it (`OracleScene(..., 32)`), on the same rows, at the configuration's depth and
Russian-roulette setting.  Both run OpenMP over pixels on the same number of threads.

This is test infrastructure: it needs `oracle/_ref`, which is built only where the
reference sources are present (a checkout, or the staged copy in `baseline/_ref`).
`bench.py --impl reference` uses `ReferenceTracer` for its timed CPU baseline.

    python -m oracle.time_reference --workload cfg1 --rows 448 480 --spp 16
"""
import argparse
import json
import os
import sys
import tempfile
import time

import ctypes
import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from mcrt_gb300 import scenes  # noqa: E402
from oracle.oracle import OracleScene, load_reference, ptr  # noqa: E402

GGX, GLSY = 8, 4


def reference_materials(desc):
    types = np.array([(m.type & 0xFF) for m in desc.materials], np.int32)
    types[types == GGX] = GLSY
    colors = np.ascontiguousarray([[m.color[0], m.color[1], m.color[2]] for m in desc.materials], np.float32)
    return types, colors


class ReferenceTracer:
    """demo_pt.cpp's own rayTrace over a scene built through the reference API (the
    SplitBVH build runs here, once); render() times a band of rows."""

    def __init__(self, desc, cam):
        lib = load_reference()
        if lib is None:
            raise RuntimeError("oracle/_ref is not built here (the reference sources are absent)")
        self.lib, self.cam = lib, cam
        v = np.ascontiguousarray(desc.vertices, np.float32)
        n = None if desc.normals is None else np.ascontiguousarray(desc.normals, np.float32)
        mid = np.ascontiguousarray(desc.material_ids, np.int32)
        types, colors = reference_materials(desc)
        c7 = np.array(list(cam.origin) + list(cam.target) + [cam.fov_y], np.float32)
        t0 = time.perf_counter()
        with tempfile.TemporaryDirectory() as tmp:
            env_path = b""
            if desc.envmap is not None:
                p = os.path.join(tmp, "env.bin")
                scenes.write_envmap_bin(p, desc.envmap)
                env_path = p.encode()
            self.h = lib.ref_pt_scene_create(ptr(v), ptr(n), ptr(mid), len(mid), ptr(types), ptr(colors),
                                             len(types), env_path, ptr(c7), cam.width, cam.height)
        self.build_s = time.perf_counter() - t0
        self.out = np.zeros((cam.height, cam.width, 3), np.float32)

    def render(self, spp, rows, threads):
        ni, no, sec = ctypes.c_longlong(0), ctypes.c_longlong(0), ctypes.c_double(0.0)
        self.lib.ref_pt_render(self.h, self.cam.width, self.cam.height, spp, threads, rows[0], rows[1],
                               ptr(self.out), ctypes.byref(ni), ctypes.byref(no), ctypes.byref(sec))
        return {"rays": ni.value + no.value, "seconds": sec.value, "band": self.out[rows[0]:rows[1]]}

    def close(self):
        if self.h:
            self.lib.ref_pt_scene_destroy(self.h)
            self.h = None


def time_reference(desc, cam, spp, rows, threads):
    tr = ReferenceTracer(desc, cam)
    try:
        r = tr.render(spp, rows, threads)
    finally:
        tr.close()
    return {"rays": r["rays"], "render_s": round(r["seconds"], 3), "scene_build_s": round(tr.build_s, 2),
            "mrays_per_s": round(r["rays"] / r["seconds"] / 1e6, 3), "image_mean": float(r["band"].mean())}


def time_port(desc, cam, spp, max_depth, rr_depth, rows, threads):
    sc = OracleScene(desc, 32)
    t0 = time.perf_counter()
    r = sc.render(cam.as_array(), cam.width, cam.height, spp, max_depth, rr_depth, seed=11, rows=tuple(rows),
                  threads=threads)
    dt = time.perf_counter() - t0
    mean = r["mean"]
    band = mean[rows[0]:rows[1]] if mean.shape[0] == cam.height else mean
    return {"rays": r["rays"], "render_s": round(dt, 3), "mrays_per_s": round(r["rays"] / dt / 1e6, 3),
            "image_mean": float(band.mean())}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="cfg1", choices=["cfg0", "cfg1"])
    ap.add_argument("--rows", type=int, nargs=2, default=None)
    ap.add_argument("--spp", type=int, default=0)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    if args.workload == "cfg0":
        desc, cam, spp, depth, rr = scenes.cfg0_scene(), scenes.cfg0_camera(256, 256), 16, 8, 3
    else:
        desc, cam, spp, depth, rr = scenes.cfg1_scene(), scenes.cfg1_camera(1024, 1024), 64, 16, -1
    spp = args.spp or spp
    rows = args.rows or [cam.height // 2 - 16, cam.height // 2 + 16]
    ref = time_reference(desc, cam, spp, rows, args.threads)
    port = time_port(desc, cam, spp, depth, rr, rows, args.threads)
    print(json.dumps({"workload": args.workload, "triangles": int(len(desc.material_ids)), "rows": rows,
                      "width": cam.width, "spp": spp, "threads": args.threads,
                      "reference_rayTrace": ref, "port": port,
                      "port_over_reference": round(port["mrays_per_s"] / ref["mrays_per_s"], 3)}))


if __name__ == "__main__":
    main()
