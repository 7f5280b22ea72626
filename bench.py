#!/usr/bin/env python
"""Benchmark: the path tracer on the large plain configuration.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload cfg1|cfg0]

One step = one complete render of the workload (default cfg1: displaced level-8
icosphere, 1,310,722 triangles, procedural 1024x512 environment map with a sun,
Lambert/GGX/dielectric patches, 1024x1024 pixels, 64 spp, depth 16) with the scene
resident on the GPU.  Metric: Mrays/s (every extension and next-event ray traced),
with samples/s beside it.  Under torchrun (N > 1) every rank renders its own replica
(the path tracer does not shard across GPUs here): weak scaling, value = rays of all
ranks / max time.

--impl reference times the reference's own CPU path tracer on this machine's cores
instead: demo_pt.cpp's rayTrace in DemoSimple::run's pixel loop, compiled from the
reference's sources (oracle/_ref), on a band of rows of the same frame per step, with the
scene and its SplitBVH built once before the timed steps.  Where the reference sources
are not present it times the oracle's float port of the same estimator and says so
(cpu_baseline.kind "port").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s & samples/s per GB300 at fixed FP64-oracle RMSE; adjoint/forward ratio"
UNIT = "Mrays/s"


def workload(name: str):
    from mcrt_gb300 import scenes
    if name == "cfg0":
        desc = scenes.cfg0_scene()
        cam = scenes.cfg0_camera(256, 256)
        p = dict(spp=16, max_depth=8, rr_depth=3)
        text = "cfg0: Cornell box + level-4 icosphere (5,132 T), 256x256, 16 spp, depth 8, RR from 3"
    else:
        desc = scenes.cfg1_scene()
        cam = scenes.cfg1_camera(1024, 1024)
        p = dict(spp=64, max_depth=16, rr_depth=-1)
        text = ("cfg1: displaced level-8 icosphere + ground (1,310,722 T), 1024x512 envmap with 0.5 deg sun, "
                "40/30/30 Lambert/GGX/dielectric patches, 1024x1024, 64 spp, depth 16")
    return desc, cam, p, text


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        # raw samples go to MCRT_CLOCKS_DIR (default: the temp directory); the JSON line
        # carries their summary
        self.path = os.path.join(os.environ.get("MCRT_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"mcrt_clocks_{os.getpid()}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) per extension ray of
# k_extend on the large configuration, from a capture of three full-queue launches of a
# reduced case (2,097,152-ray queue, same scene and frame: 337.9 MB per launch); the bench
# scales it by the extension rays of an average launch of the measured configuration.  An
# upper bound for larger launches, whose rays share more of the tree lines fetched.  Keyed
# by the node size of the traversal (64: two-child nodes).
K_EXTEND_DRAM_BYTES_PER_RAY = {64: 161.1}


# rows of the cfg0 / cfg1 frames the CPU port renders for cpu_baseline and --impl reference
CPU_BASELINE_ROWS = {"cfg0": (64, 192), "cfg1": (384, 640)}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def l2_read_peak():
    """L2 read bandwidth of this GPU, measured live by the library's probe kernel
    (mcrt_probe_l2_read: a 48 MB L2-resident buffer read 100 times in one launch), best of 3.
    The traversal kernels' node and triangle reads mostly hit L2, so their algorithmic
    bandwidth is also quoted against this figure."""
    import ctypes
    from mcrt_gb300 import _native as N
    lib = N.load()
    best = 0.0
    for _ in range(3):
        g = ctypes.c_float(0.0)
        N.check(lib.mcrt_probe_l2_read(48 << 20, 100, ctypes.byref(g), None), "mcrt_probe_l2_read")
        best = max(best, g.value)
    return best


def cpu_port_sample(desc, cam, p, rows, seed=7, osc=None):
    """The oracle's float port of the estimator on all host cores, over a band of rows."""
    from oracle.oracle import OracleScene
    t0 = time.time()
    osc = osc or OracleScene(desc, 32)
    build_s = time.time() - t0
    r0, r1 = rows
    t0 = time.time()
    out = osc.render(cam.as_array(), cam.width, cam.height, p["spp"], p["max_depth"], p["rr_depth"], seed=seed,
                     rows=(r0, r1), threads=os.cpu_count())
    dt = time.time() - t0
    return out["rays"], (r1 - r0) * cam.width * p["spp"], dt, build_s


# rows of the frame the reference's own rayTrace renders per step of --impl reference (the
# middle of the cfg1 frame: sphere, ground and sky; about 1-2 s of CPU work per step)
REFERENCE_ROWS = {"cfg0": (96, 160), "cfg1": (504, 520)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    desc, cam, p, text = workload(args.workload)
    cores = os.cpu_count() or 1
    tracer, why = None, None
    try:
        from oracle.time_reference import ReferenceTracer
        tracer = ReferenceTracer(desc, cam)  # scene + SplitBVH built once, outside the timed steps
    except (RuntimeError, OSError) as e:
        why = str(e)
    times, rays_total, paths_total = [], 0, 0
    if tracer is not None:
        # demo_pt.cpp's rayTrace as it is: fixed depth 10, no Russian roulette, GGX -> Phong,
        # IOR 1.33 (the reference cannot express the configuration's own estimator)
        r0, r1 = REFERENCE_ROWS.get(args.workload, REFERENCE_ROWS["cfg1"])
        for step in range(args.warmup + args.steps):
            r = tracer.render(p["spp"], (r0, r1), cores)
            if step >= args.warmup:
                times.append(r["seconds"])
                rays_total += r["rays"]
                paths_total += (r1 - r0) * cam.width * p["spp"]
        build_s = tracer.build_s
        tracer.close()
        kind = "reference"
        sample = (f"{args.workload} rows {r0}-{r1} x {cam.width} px x {p['spp']} spp per step: demo_pt.cpp "
                  f"rayTrace (depth 10, no RR, GGX as Phong, IOR 1.33), SplitBVH built once in {build_s:.0f} s "
                  f"(not timed), {cores} OpenMP threads; rays counted at SceneBVH::intersect/occluded")
    else:
        from oracle.oracle import OracleScene
        r0, r1 = CPU_BASELINE_ROWS.get(args.workload, CPU_BASELINE_ROWS["cfg1"])
        osc = OracleScene(desc, 32)
        for step in range(args.warmup + args.steps):
            rays, paths, dt, _ = cpu_port_sample(desc, cam, p, (r0, r1), seed=step, osc=osc)
            if step >= args.warmup:
                times.append(dt)
                rays_total += rays
                paths_total += paths
        kind = "port"
        sample = (f"{args.workload} rows {r0}-{r1} x {cam.width} px x {p['spp']} spp per step (float port of the "
                  f"estimator, {cores} threads; the reference's own tracer is unavailable here: {why})")
    value = rays_total / sum(times) / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sum(times) / len(times), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (procedural scene, seeded)", "config": {"workload": text},
            "msamples_per_s": round(paths_total / sum(times) / 1e6, 4),
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def incoherent_trace_leg(sc, dev, n=2_000_000, reps=5):
    """Closest hits of random incoherent rays through mcrt_trace_closest (device buffers):
    origins uniform in [-2, 2]^3, directions uniform on the sphere -- the random-ray
    measurement of the reference SplitBVH (0.923 Mrays/s on 1 thread, 7.77 on 8, at
    1,310,720 triangles on an 8-core x86 host).  Not the headline: the wavefront's own
    traversal kernels are timed above."""
    import numpy as np
    import torch
    g = torch.Generator().manual_seed(20261204)
    rays = torch.zeros((n, 8), dtype=torch.float32)
    rays[:, 0:3] = torch.rand((n, 3), generator=g) * 4.0 - 2.0
    d = torch.randn((n, 3), generator=g, dtype=torch.float64)
    rays[:, 4:7] = (d / d.norm(dim=1, keepdim=True)).float()
    rays[:, 3] = 1e-4
    rays[:, 7] = float("inf")
    rays = rays.to(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    hits = sc.trace_closest(rays)  # warm-up
    ms = []
    for _ in range(reps):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        hits = sc.trace_closest(rays)
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    hit_rate = float((hits[:, 3].view(torch.int32) >= 0).float().mean())
    best = float(np.median(ms))
    return {"mrays_s": round(n / (best / 1e3) / 1e6, 1), "rays": n, "hit_rate": round(hit_rate, 4),
            "ms": round(best, 3), "recipe": "origins U[-2,2]^3, directions uniform on the sphere, tmin 1e-4, "
                                            "closest hit (FAST traversal, library tree), L2 flushed before each call",
            "reference_splitbvh_mrays_s": {"1_thread": 0.923, "8_threads": 7.77,
                                           "where": "8-core x86 host, reference built from source, 2 M rays"}}


def fp64_error(desc, cam, p, rows, band, fp64_spp=512):
    """Per-channel RMSE of the first timed render against the FP64 oracle (a band of rows
    rendered at high spp on the host cores), computed outside the timed region."""
    import numpy as np
    from oracle.oracle import OracleScene
    t0 = time.time()
    ref = OracleScene(desc, 64).render(cam.as_array(), cam.width, cam.height, fp64_spp, p["max_depth"],
                                       p["rr_depth"], seed=77, rows=tuple(rows), threads=os.cpu_count())
    rmean, rvar = ref["mean"], ref["var_of_mean"]
    if rmean.shape[0] != rows[1] - rows[0]:
        rmean, rvar = rmean[rows[0]:rows[1]], rvar[rows[0]:rows[1]]
    g = band.astype(np.float64)
    rmse = [float(np.sqrt(np.mean((g[..., c] - rmean[..., c]) ** 2))) for c in range(3)]
    noise = [float(np.sqrt(np.mean(rvar[..., c]))) for c in range(3)]
    return {"rmse": [round(x, 5) for x in rmse], "fp64_noise_rms": [round(x, 5) for x in noise],
            "rows": list(rows), "width": cam.width, "gpu_spp": p["spp"], "fp64_spp": fp64_spp,
            "render": "the first timed render", "fp64_seconds": round(time.time() - t0, 1),
            "note": "the CPU baseline renders the same estimator at the same spp, so both are at this error"}


def _timed(fn, reps=1):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        r = fn()
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / reps, r


def bench_cfg2(args):
    """64 procedural scenes of uneven size: one batched wavefront against the same renders
    issued scene by scene (streaming per scene, and the wave schedule per scene).
    --cfg2-part batched|sequential|waves|paths runs one of them alone (launch lists); `paths`
    is the plain GPU path tracer (MCRT_SCHEDULE_PATHS: one thread per path) scene by scene;
    --no-autotune keeps the library's default launch configuration."""
    import torch
    from mcrt_gb300 import GpuScene, autotune, render_batch, scenes
    jobs = scenes.cfg2_jobs(64)
    t0 = time.time()
    gs = [GpuScene(d) for d, _, _ in jobs]
    setup_s = time.time() - t0
    part = args.cfg2_part
    load_s = cache_mb = None
    if part == "all":
        # the same 64 scenes from scene cache files (mcrt_scene_save / mcrt_scene_load)
        with tempfile.TemporaryDirectory() as tmp:
            paths = [os.path.join(tmp, f"s{k}.mcrt") for k in range(len(gs))]
            for g, pth in zip(gs, paths):
                g.save(pth)
            t0 = time.time()
            loaded = [GpuScene.load(pth, d) for pth, (d, _, _) in zip(paths, jobs)]
            load_s = time.time() - t0
            cache_mb = sum(os.path.getsize(pth) for pth in paths) / 1e6
            for g in loaded:
                g.close()
    cams = [c for _, c, _ in jobs]
    params = [dict(p, use_graph=True, schedule=args.schedule_id) for _, _, p in jobs]
    outs = [torch.empty((c.height, c.width, 3), device="cuda") for c in cams]
    tune, tune_s = None, 0.0
    if part in ("all", "batched") and not args.no_autotune:
        t0 = time.time()
        params, tune = autotune(gs, cams, params)  # queue capacity and kernel variant for the batch
        tune_s = time.time() - t0

    def sequential():
        tot = 0
        for s, c, (_, _, p), o in zip(gs, cams, jobs, outs):
            _, st = s.render(c, out=o, schedule=args.schedule_id, **p)
            tot += st["rays"]
        return tot

    def sequential_waves():
        for s, c, (_, _, p), o in zip(gs, cams, jobs, outs):
            s.render(c, out=o, schedule=1, **p)

    def sequential_paths():  # the plain GPU path tracer: one thread per path, scene by scene
        for s, c, (_, _, p), o in zip(gs, cams, jobs, outs):
            s.render(c, out=o, schedule=2, **p)

    line = {"workload": "cfg2: 64 scenes, displaced icospheres 1k-500k T in Cornell shells, res {128..1024}^2, "
                        "spp 1..64, depth 4..16", "part": part, "schedule": args.schedule,
            "scene_setup_s": round(setup_s, 1),
            "triangles": int(sum(d.num_triangles for d, _, _ in jobs))}
    if part in ("all", "batched"):
        render_batch(gs, cams, params, outs)  # warm-up
        tb, (_, stb) = _timed(lambda: render_batch(gs, cams, params, outs), reps=args.steps)
        line.update({"paths": stb["paths"], "rays": stb["rays"], "batched_ms": round(tb * 1e3, 2),
                     "batched_mrays_s": round(stb["rays"] / tb / 1e6, 1),
                     "batched_msamples_s": round(stb["paths"] / tb / 1e6, 1), "waves": stb["waves"]})
        if tune is not None:
            line["autotune"] = {"seconds": round(tune_s, 2), "probe_paths": tune["probe_paths"],
                                "chosen": tune["candidates"][tune["chosen"]], "candidates": len(tune["candidates"])}
    if part in ("all", "sequential"):
        sequential()
        ts, seq_rays = _timed(sequential, reps=args.steps)
        line.update({"sequential_ms": round(ts * 1e3, 2), "sequential_mrays_s": round(seq_rays / ts / 1e6, 1)})
    if part in ("all", "waves"):
        sequential_waves()
        tw, _ = _timed(sequential_waves, reps=args.steps)
        line["sequential_waves_ms"] = round(tw * 1e3, 2)
    if part in ("all", "paths"):
        sequential_paths()
        tp, _ = _timed(sequential_paths, reps=args.steps)
        line["sequential_paths_ms"] = round(tp * 1e3, 2)
    if part == "all":
        line.update({"speedup_batched_vs_sequential": round(line["sequential_ms"] / line["batched_ms"], 3),
                     "speedup_batched_vs_sequential_waves": round(line["sequential_waves_ms"] / line["batched_ms"], 3),
                     "speedup_batched_vs_plain_paths": round(line["sequential_paths_ms"] / line["batched_ms"], 3),
                     "scene_cache_load_s": round(load_s, 2), "scene_cache_mb": round(cache_mb, 1)})
    print(json.dumps(line), flush=True)


def bench_cfg3(args):
    """Differentiable Cornell box (256 albedo groups + emission), 512^2, 32 spp, depth 6:
    forward time, forward+adjoint time."""
    import torch
    from mcrt_gb300 import GpuScene, scenes
    desc, albedo, emission = scenes.cfg3_scene()
    cam = scenes.cfg0_camera(512, 512)
    sc = GpuScene(desc)
    out = torch.empty((512, 512, 3), device="cuda")
    kw = dict(spp=32, max_depth=6, seed=3, schedule=args.schedule_id)
    dl = torch.randn((512, 512, 3), device="cuda")
    sc.render(cam, out=out, **kw)
    sc.render_adjoint(cam, 32, 6, dl, albedo.shape[0], 1, seed=3)
    tf, (_, stf) = _timed(lambda: sc.render(cam, out=out, **kw), reps=args.steps)
    ta, (_, _, sta) = _timed(lambda: sc.render_adjoint(cam, 32, 6, dl, albedo.shape[0], 1, seed=3), reps=args.steps)
    line = {"workload": "cfg3: Cornell + 256 albedo groups + emission, 512x512, 32 spp, depth 6",
            "forward_ms": round(tf * 1e3, 2), "adjoint_ms": round(ta * 1e3, 2),
            "forward_plus_adjoint_over_forward": round((tf + ta) / tf, 3),
            "forward_mrays_s": round(stf["rays"] / tf / 1e6, 1), "paths": stf["paths"], "schedule": args.schedule}
    print(json.dumps(line), flush=True)


def adjoint_ratio_leg(reps=3):
    """The metric's adjoint/forward ratio on its own workload (cfg3: the Cornell box with 256
    albedo groups + emission, 512^2, 32 spp, depth 6): wall time of forward + path-replay
    adjoint over the forward, best of `reps` (the gradient's accuracy is a test)."""
    import torch
    from mcrt_gb300 import GpuScene, scenes
    desc, albedo, emission = scenes.cfg3_scene()
    cam = scenes.cfg0_camera(512, 512)
    sc = GpuScene(desc)
    out = torch.empty((512, 512, 3), device="cuda")
    dl = torch.randn((512, 512, 3), device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
    fwd = lambda: sc.render(cam, out=out, spp=32, max_depth=6, seed=3)  # noqa: E731
    adj = lambda: sc.render_adjoint(cam, 32, 6, dl, albedo.shape[0], 1, seed=3)  # noqa: E731
    fwd()
    adj()
    tf = min(_timed(fwd)[0] for _ in range(reps))
    ta = min(_timed(adj)[0] for _ in range(reps))
    sc.close()
    return {"workload": "cfg3: Cornell box + 256 albedo groups + emission, 512x512, 32 spp, depth 6",
            "forward_ms": round(tf * 1e3, 2), "adjoint_ms": round(ta * 1e3, 2),
            "forward_plus_adjoint_over_forward": round((tf + ta) / tf, 3), "target": "<= 3"}


def bench_cfg4(args):
    """32 views of the 1.3 M-triangle scene, 256^2, 16 spp, depth 8, 4,096 albedo
    parameters: batched forward + batched adjoint vs 32 sequential forward + adjoint."""
    import torch
    from mcrt_gb300 import GpuScene, render_adjoint_batch, render_batch, scenes
    desc, albedo = scenes.cfg4_scene()
    sc = GpuScene(desc)
    cams = scenes.fibonacci_cameras(32)
    p = dict(spp=16, max_depth=8, rr_depth=-1)
    params = [dict(p, seed=100 + k, use_graph=True, schedule=args.schedule_id) for k in range(32)]
    outs = [torch.empty((256, 256, 3), device="cuda") for _ in cams]
    dls = [torch.randn((256, 256, 3), device="cuda") for _ in cams]
    n = albedo.shape[0]

    def batched():
        render_batch([sc] * 32, cams, params, outs)
        return render_adjoint_batch([sc] * 32, cams, [dict(p, seed=100 + k) for k in range(32)], dls, n, 0)

    def sequential():
        for k, c in enumerate(cams):
            sc.render(c, out=outs[k], seed=100 + k, schedule=args.schedule_id, **p)
            sc.render_adjoint(c, p["spp"], p["max_depth"], dls[k], n, 0, seed=100 + k)

    batched()
    sequential()
    tb, _ = _timed(batched, reps=args.steps)
    ts, _ = _timed(sequential, reps=args.steps)
    tfb, _ = _timed(lambda: render_batch([sc] * 32, cams, params, outs), reps=args.steps)
    line = {"workload": "cfg4: 32 Fibonacci views of the 1.3 M-T scene, 256x256, 16 spp, depth 8, 4096 albedos",
            "batched_forward_adjoint_ms": round(tb * 1e3, 2), "sequential_forward_adjoint_ms": round(ts * 1e3, 2),
            "speedup": round(ts / tb, 3), "batched_forward_ms": round(tfb * 1e3, 2),
            "forward_plus_adjoint_over_forward": round(tb / tfb, 3), "schedule": args.schedule}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg1", choices=["cfg1", "cfg0", "cfg2", "cfg3", "cfg4"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--traverse", default="fast", choices=["fast", "ref"])
    ap.add_argument("--res", type=int, default=0, help="override the resolution (profiling small cases)")
    ap.add_argument("--spp", type=int, default=0, help="override spp (profiling small cases)")
    ap.add_argument("--schedule", default="stream", choices=["stream", "waves"],
                    help="stream: slots refilled with new paths as paths end; waves: fixed waves")
    ap.add_argument("--path-chunk", type=int, default=0, help="path slots in flight (0: library default)")
    ap.add_argument("--variant", type=int, default=0, help="traversal kernel variant bits (0: default policy)")
    ap.add_argument("--autotune", action="store_true", help="pick path_chunk / variant with mcrt_autotune first")
    ap.add_argument("--cfg2-part", default="all", choices=["all", "batched", "sequential", "waves", "paths"],
                    help="cfg2: run the batched render, the per-scene renders or the per-scene wave renders alone")
    ap.add_argument("--no-autotune", action="store_true", help="cfg2: the library's default launch configuration")
    ap.add_argument("--quick", action="store_true",
                    help="only the timed renders, stage split and counts (profiling small cases)")
    ap.add_argument("--fp64-rows", type=int, nargs=2, default=None,
                    help="rows of the first timed render compared with the FP64 oracle (default: cfg1 496-512)")
    ap.add_argument("--leaf-size", type=int, default=0,
                    help="largest BVH leaf of the scene build (1..15; 0: the library default, 2)")
    args = ap.parse_args()
    args.schedule_id = 0 if args.schedule == "stream" else 1
    if args.fp64_rows is None and args.workload == "cfg1" and not args.res and not args.quick:
        args.fp64_rows = [496, 512]
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload in ("cfg2", "cfg3", "cfg4"):
        {"cfg2": bench_cfg2, "cfg3": bench_cfg3, "cfg4": bench_cfg4}[args.workload](args)
        return

    import numpy as np
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        import torch.distributed as td
        td.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import mcrt_gb300
    from mcrt_gb300 import GpuScene, TRAVERSE_FAST, TRAVERSE_REF
    from mcrt_gb300._native import PROFILE_COUNT, PROFILE_STAGES
    from mcrt_gb300.replicas import aggregate

    mcrt_gb300.load()
    desc, cam, p, text = workload(args.workload)
    if args.res:
        cam.width = cam.height = args.res
        text += f" [reduced: {args.res}x{args.res}]"
    if args.spp:
        p["spp"] = args.spp
        text += f" [reduced: {args.spp} spp]"
    t0 = time.time()
    sc = GpuScene(desc, leaf_size=args.leaf_size)
    setup_s = time.time() - t0
    traverse = TRAVERSE_FAST if args.traverse == "fast" else TRAVERSE_REF
    out = torch.empty((cam.height, cam.width, 3), dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2
    kw = dict(spp=p["spp"], max_depth=p["max_depth"], rr_depth=p["rr_depth"], traverse=traverse,
              schedule=args.schedule_id, path_chunk=args.path_chunk, variant=args.variant)
    tune = None
    if args.autotune:
        from mcrt_gb300 import autotune
        (tuned,), tune = autotune([sc], [cam], [kw])
        kw.update(path_chunk=tuned["path_chunk"], variant=tuned["variant"])
        args.path_chunk, args.variant = tuned["path_chunk"], tuned["variant"]

    def barrier():
        if dist:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for w in range(args.warmup):
        sc.render(cam, seed=100 + w, out=out, **kw)
    # timed region: one production render per step (no per-stage events), L2 flushed
    # between steps
    step_ms, rays, paths = [], 0, 0
    st_last = None
    first_band = None
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            barrier()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            _, st = sc.render(cam, seed=k, out=out, **kw)
            e1.record()
            barrier()
            step_ms.append(e0.elapsed_time(e1))
            rays += st["rays"]
            paths += st["paths"]
            st_last = st
            if k == 0 and args.fp64_rows:
                first_band = out[args.fp64_rows[0]:args.fp64_rows[1]].cpu().numpy()
    clocks = clk.summary()
    total_ms = sum(step_ms)
    total_ms, rays, paths = aggregate(total_ms, rays, paths, dev)
    value = rays / (total_ms / 1e3) / 1e6
    msamples = paths / (total_ms / 1e3) / 1e6

    # per-stage CUDA events (one pair per launch) in separate, untimed renders of the same
    # seeds: the stage split and each traversal kernel's average launch time
    n_staged = max(1, min(args.steps, 5))
    stage_ms = [0.0, 0.0, 0.0, 0.0]
    extend_launches = 0
    for k in range(n_staged):
        flush.zero_()
        _, st = sc.render(cam, seed=k, out=out, profile=PROFILE_STAGES, **kw)
        stage_ms = [a + b for a, b in zip(stage_ms, st["stage_ms"])]
        extend_launches += st["extend_launches"]
    stage_ms = [x / n_staged for x in stage_ms]
    extend_launches /= n_staged
    staged_frame_ms = sum(stage_ms)

    # algorithmic bytes of the two traversal kernels: a counting render of the same seeds.
    # k_extend per extension ray: one node fetch per node visited (96 B for the eight-child
    # nodes of the FAST traversal, the sectors a visit touches), 48 B per triangle tested,
    # 32 B ray + 16 B hit; k_connect per next-event ray: nodes/triangles as above, 64 B ray +
    # payload + meta in, 16 B result out.  Both kernels launch once per iteration.
    _, sc_cnt = sc.render(cam, seed=0, out=out, profile=PROFILE_COUNT, **kw)
    nb = sc_cnt["node_bytes"]
    # the same counts by bounce class: a depth-0 counting render of the same seeds traces
    # the camera rays alone (and their vertices' next-event rays); the rest of the
    # extension rays are the secondary ones
    _, sc_prim = sc.render(cam, seed=0, out=out, profile=PROFILE_COUNT, **dict(kw, max_depth=0))

    def per_ray(nodes, tris, rays):
        return {"rays": int(rays), "nodes_per_ray": round(nodes / max(rays, 1), 2),
                "tris_per_ray": round(tris / max(rays, 1), 2),
                "bytes_per_ray": round((nb * nodes + 48 * tris) / max(rays, 1) + 48, 1)}
    per_class = {
        "primary": per_ray(sc_prim["ext_nodes"], sc_prim["ext_tris"], sc_prim["extension_rays"]),
        "secondary": per_ray(sc_cnt["ext_nodes"] - sc_prim["ext_nodes"], sc_cnt["ext_tris"] - sc_prim["ext_tris"],
                             sc_cnt["extension_rays"] - sc_prim["extension_rays"]),
        "next_event": {**per_ray(sc_cnt["nee_nodes"], sc_cnt["nee_tris"], sc_cnt["shadow_rays"]),
                       "bytes_per_ray": round((nb * sc_cnt["nee_nodes"] + 48 * sc_cnt["nee_tris"])
                                              / max(sc_cnt["shadow_rays"], 1) + 80, 1)},
        "note": "counting build (MCRT_PROFILE_COUNT), same seeds as the timed steps; bytes per ray as the "
                "roofline's algorithmic bytes (ray in + hit or result out included)",
    }
    ext_bytes = nb * sc_cnt["ext_nodes"] + 48 * sc_cnt["ext_tris"] + (32 + 16) * sc_cnt["extension_rays"]
    nee_bytes = nb * sc_cnt["nee_nodes"] + 48 * sc_cnt["nee_tris"] + (64 + 16) * sc_cnt["shadow_rays"]
    launches_per_render = max(extend_launches, 1)
    kernels = {
        "k_extend (closest-hit traversal of extension rays)": (ext_bytes, stage_ms[1], sc_cnt["extension_rays"],
                                                                sc_cnt["ext_nodes"], sc_cnt["ext_tris"]),
        "k_connect (next-event rays: any-hit / bounded closest-hit)": (nee_bytes, stage_ms[3], sc_cnt["shadow_rays"],
                                                                        sc_cnt["nee_nodes"], sc_cnt["nee_tris"]),
    }
    dom = max(kernels, key=lambda k: kernels[k][1])
    bytes_per_render, kern_ms, kern_rays, kern_nodes, kern_tris = kernels[dom]
    per_launch_bytes = bytes_per_render / launches_per_render
    avg_launch_ms = kern_ms / launches_per_render
    achieved = per_launch_bytes / (avg_launch_ms / 1e3) / 1e9 if avg_launch_ms > 0 else 0.0
    peak, peak_kind = measured_peak_hbm()
    l2_peak = l2_read_peak()
    other = [k for k in kernels if k != dom][0]
    traffic = None
    if dom.startswith("k_extend") and args.workload == "cfg1" and nb in K_EXTEND_DRAM_BYTES_PER_RAY:
        traffic = K_EXTEND_DRAM_BYTES_PER_RAY[nb] * kern_rays / launches_per_render
    ob, oms = kernels[other][0], kernels[other][1]
    other_achieved = (ob / launches_per_render) / (oms / launches_per_render / 1e3) / 1e9 if oms > 0 else 0.0

    # e2e: the C-ABI call with host buffers (image copied back inside the call, into pinned
    # host memory)
    host_img = torch.zeros((cam.height, cam.width, 3), dtype=torch.float32, pin_memory=True).numpy()
    e2e_ms, e2e_rays, h2d, d2h = [], 0, 0, 0
    for k in range(max(1, args.steps)):
        flush.zero_()
        barrier()
        t0 = time.perf_counter()
        _, st = sc.render(cam, seed=k, out=host_img, **kw)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
        e2e_rays += st["rays"]
        h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
    e2e_value = e2e_rays / (sum(e2e_ms) / 1e3) / 1e6 * (world if dist else 1)

    # launches of our kernels inside the timed region
    launches = st_last["kernel_launches"] * args.steps

    trace_leg = adjoint = plain = None
    if rank == 0 and not args.quick:
        trace_leg = incoherent_trace_leg(sc, dev)
        adjoint = adjoint_ratio_leg()
        # the same frame with the plain GPU path tracer (one thread per path, no queues):
        # what the wavefront buys on this workload
        pkw = dict(kw, schedule=2)
        sc.render(cam, seed=0, out=out, **pkw)
        tp, (_, stp) = _timed(lambda: sc.render(cam, seed=1, out=out, **pkw), reps=2)
        plain = {"ms_per_frame": round(tp * 1e3, 2), "mrays_s": round(stp["rays"] / tp / 1e6, 1),
                 "wavefront_speedup": round(tp * 1e3 / (total_ms / args.steps), 3),
                 "what": "MCRT_SCHEDULE_PATHS: one thread runs each path start to end, same paths and rays"}

    cpu = None
    fp64 = None
    if rank == 0 and not args.quick:
        if not args.no_cpu_baseline:
            rows = CPU_BASELINE_ROWS[args.workload]
            c_rays, c_paths, c_dt, c_build = cpu_port_sample(desc, cam, p, rows)
            cpu = {"value": round(c_rays / c_dt / 1e6, 3), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                   "sample": f"{args.workload} rows {rows[0]}-{rows[1]} x {cam.width} px x {p['spp']} spp "
                             f"({c_paths} paths, {c_dt:.1f} s; float port of the estimator)"}
        if first_band is not None:
            fp64 = fp64_error(desc, cam, p, args.fp64_rows, first_band)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (procedural scene, seeded)",
            "config": {"workload": text, "traversal": args.traverse, "l2": "flushed between steps (256 MB write)",
                       "parallelism": f"replicas x{world}", "schedule": args.schedule,
                       "path_slots": args.path_chunk or "default (67108864, clamped to the paths)",
                       "variant": args.variant, "leaf_size": args.leaf_size or 2, "autotuned": tune is not None,
                       "waves_or_iterations_per_step": st_last["waves"], "scene_setup_s": round(setup_s, 2),
                       "scene_device_bytes": sc.info()["device_bytes"], "fast_nodes": sc.info()["fast_nodes"]},
            "msamples_per_s": round(msamples, 3),
            "rays_per_path": round(rays / max(paths, 1), 3),
            "fp64_oracle": fp64,
            "roofline": {"bound": "l2", "kernel": dom, "achieved": round(achieved, 1), "peak": round(l2_peak, 1),
                         "unit": "GB/s", "frac": round(achieved / l2_peak, 4) if l2_peak > 0 else None,
                         "peak_source": "mcrt_probe_l2_read in this run: 48 MB L2-resident buffer read 100 times "
                                        "per launch, best of 3 (the traversal's node and triangle reads are served "
                                        "by L2; ncu shows DRAM a few % busy)",
                         "limiter": "dependent-load latency and SIMT divergence (ncu: long-scoreboard stalls, "
                                    "about 10 of 32 lanes active per instruction)",
                         "traffic": None if traffic is None else int(traffic),
                         "traffic_unit": "DRAM bytes per launch: ncu read + write per extension ray of a "
                                         "2 M-ray-queue case (161.1 B) times this configuration's rays per launch "
                                         "(an upper bound: larger launches share more tree lines)",
                         "algorithmic_bytes_per_launch": int(per_launch_bytes),
                         "avg_launch_ms": round(avg_launch_ms, 4),
                         "hbm": {"peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                                 "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
                         "bytes_per_ray": round(bytes_per_render / max(kern_rays, 1), 1),
                         "node_bytes": nb,
                         "nodes_per_ray": round(kern_nodes / max(kern_rays, 1), 2),
                         "tris_per_ray": round(kern_tris / max(kern_rays, 1), 2),
                         "per_bounce_class": per_class,
                         "share_of_step": round(kern_ms / max(staged_frame_ms, 1e-9), 3),
                         "timing": f"CUDA events around every launch, {n_staged} untimed renders of the same seeds",
                         "second_kernel": {"kernel": other, "achieved": round(other_achieved, 1),
                                           "frac": round(other_achieved / l2_peak, 4) if l2_peak > 0 else None,
                                           "frac_hbm": round(other_achieved / peak, 4),
                                           "share_of_step": round(oms / max(staged_frame_ms, 1e-9), 3)}},
            "stage_ms_per_step": {"begin+regen": round(stage_ms[0], 2), "extend": round(stage_ms[1], 2),
                                  "shade": round(stage_ms[2], 2), "connect": round(stage_ms[3], 2),
                                  "note": "untimed renders with an event pair around every launch"},
            "trace_incoherent": trace_leg,
            "adjoint_over_forward": adjoint,
            "plain_path_tracer": plain,
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    if dist:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
