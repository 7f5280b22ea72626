"""The default ray queue (64 M slots, about 49 GB) halves itself when the device has not
the memory for it.  A child process (a fresh CUDA context, so no earlier render's working
block is reused) fills the device up to about 20 GB free, renders a 67 M-path frame with
the default queue, and must get the image that an explicitly small queue renders: the
queue size never changes a path's arithmetic."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

_CHILD = r"""
import json
import numpy as np
import torch
from mcrt_gb300 import GpuScene, scenes
desc = scenes.cfg1_scene(level=5, env_size=(256, 128), patch_tris=64)
cam = scenes.cfg1_camera(1024, 1024)
kw = dict(spp=64, max_depth=4, seed=3)  # 67,108,864 paths
sc = GpuScene(desc)
free0 = free = torch.cuda.mem_get_info()[0]
hog = []
for _ in range(64):  # leave about 20 GB free, in blocks of at most 16 GB
    n = min(16 << 30, free - (20 << 30))
    if n < (1 << 30):
        break
    hog.append(torch.empty(n, dtype=torch.uint8, device="cuda"))
    free = torch.cuda.mem_get_info()[0]
img, st = sc.render(cam, **kw)  # the default queue cannot be allocated whole
hog.clear()
torch.cuda.empty_cache()
full, st_full = sc.render(cam, path_chunk=1 << 26, **kw)  # the whole default, now that it fits
small, st_small = sc.render(cam, path_chunk=1 << 22, **kw)
print(json.dumps({"iterations": st["waves"], "iterations_full_queue": st_full["waves"],
                  "equal": bool(np.array_equal(img, small) and np.array_equal(img, full)),
                  "rays": st["rays"], "rays_small": st_small["rays"], "free_gb": free0 / 2**30}))
"""


def test_default_queue_halves_when_memory_is_short(cuda_device):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _CHILD], cwd=root, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["equal"] and out["rays"] == out["rays_small"]
    # the halved queue needs more admission rounds than the whole 64 M-slot default
    assert out["iterations"] > out["iterations_full_queue"], out
