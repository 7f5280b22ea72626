"""Error of every configuration's GPU render against the FP64 oracle.

For each configuration the GPU renders the full frame at the configuration's own spp
(eight independent seeds, for the per-pixel variance of one render); the FP64 oracle
renders a band of rows of the same frame at high spp.  Reported per configuration: the
per-channel RMSE of one GPU render against the FP64 reference, the relative error of the
band mean, and the fraction of pixels beyond 4 sigma; asserted: the Monte Carlo
confidence band (pixel z-test and band-mean z-test).

Set MCRT_FP64_REPORT=<path> to write the measured table as JSON."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases():
    from mcrt_gb300 import scenes
    cfg2 = scenes.cfg2_jobs(64)
    # the cfg2 scene with the median path count
    order = sorted(range(len(cfg2)), key=lambda k: cfg2[k][1].width * cfg2[k][1].height * cfg2[k][2]["spp"])
    d2, c2, p2 = cfg2[order[len(order) // 2]]
    d3, _, _ = scenes.cfg3_scene()
    d4, _ = scenes.cfg4_scene()
    c4 = scenes.fibonacci_cameras(32)[5]
    return [
        ("cfg0", scenes.cfg0_scene(), scenes.cfg0_camera(256, 256), dict(spp=16, max_depth=8, rr_depth=3), 1024,
         (112, 144)),
        ("cfg1", scenes.cfg1_scene(), scenes.cfg1_camera(1024, 1024), dict(spp=64, max_depth=16, rr_depth=-1), 512,
         (496, 512)),
        ("cfg2", d2, c2, dict(spp=p2["spp"], max_depth=p2["max_depth"], rr_depth=p2["rr_depth"]), 512,
         (c2.height // 2 - 8, c2.height // 2 + 8)),
        ("cfg3", d3, scenes.cfg0_camera(512, 512), dict(spp=32, max_depth=6, rr_depth=-1), 512, (240, 264)),
        ("cfg4", d4, c4, dict(spp=16, max_depth=8, rr_depth=-1), 512, (120, 136)),
    ]


@pytest.fixture(scope="module")
def report():
    rows = {}
    yield rows
    path = os.environ.get("MCRT_FP64_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(rows, f, indent=1)


@pytest.mark.parametrize("case", range(5))
def test_error_against_fp64_oracle(case, report, cuda_device):
    from mcrt_gb300 import GpuScene
    from oracle.oracle import OracleScene
    name, desc, cam, p, ref_spp, (r0, r1) = _cases()[case]
    sc = GpuScene(desc)
    renders = np.stack([sc.render(cam, seed=500 + b, **p)[0][r0:r1] for b in range(8)]).astype(np.float64)
    one = renders[0]
    var_one = np.var(renders, axis=0, ddof=1)  # variance of one render at the configuration's spp
    ref = OracleScene(desc, 64).render(cam.as_array(), cam.width, cam.height, ref_spp, p["max_depth"], p["rr_depth"],
                                       seed=77, rows=(r0, r1), threads=os.cpu_count())
    rmean, rvar = ref["mean"], ref["var_of_mean"]
    if rmean.shape[0] != r1 - r0:
        rmean, rvar = rmean[r0:r1], rvar[r0:r1]
    # pixel z-test of the 8-render mean against the reference
    g = renders.mean(axis=0)
    z = (g - rmean) / np.sqrt(var_one / len(renders) + rvar + 1e-12)
    frac4 = float(np.mean(np.abs(z) > 4))
    rmse = [float(np.sqrt(np.mean((one[..., c] - rmean[..., c]) ** 2))) for c in range(3)]
    mean_rel, zmean = [], []
    for c in range(3):
        m = rmean[..., c].mean()
        d = g[..., c].mean() - m
        sd = np.sqrt((var_one[..., c].sum() / len(renders) + rvar[..., c].sum())) / g[..., c].size
        mean_rel.append(float(d / m) if m > 0 else 0.0)
        zmean.append(float(d / sd) if sd > 0 else 0.0)
    report[name] = {"gpu_spp": p["spp"], "fp64_spp": ref_spp, "rows": [r0, r1], "width": cam.width,
                    "rmse_one_render": rmse, "band_mean_rel_err": mean_rel, "band_mean_z": zmean,
                    "frac_pixels_beyond_4sigma": frac4}
    assert frac4 < 0.02, f"{name}: {frac4:.4f} of pixels beyond 4 sigma"
    assert max(abs(x) for x in zmean) < 5, f"{name}: band-mean z {zmean}"
