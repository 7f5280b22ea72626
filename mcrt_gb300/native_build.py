"""Builds the in-tree native library ``mcrt_gb300/_lib/libmcrt_gb300.so``.

CUDA sources are compiled for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``);
host C++ is compiled with ``-ffp-contract=off`` so the float tables it builds follow
the reference's operation order on x86 and aarch64 alike.  Translation units are
compiled in parallel; the library links the CUDA runtime statically and has no
torch dependency.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIB_DIR, "libmcrt_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["kernels.cu", "noalloc.cu", "film.cu", "probe.cu"]
CPP_SOURCES = ["bvh_build.cpp", "flatten.cpp", "scene_prep.cpp", "autotune.cpp", "scene_cache.cpp", "ingest.cpp",
               "wide_build.cpp", "sbvh_build.cpp"]
HEADERS = ["layout.h", "host.h", "device.cuh", "estimator.cuh", "wavefront.h"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build mcrt_gb300")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(LIB_DIR, exist_ok=True)
    # MCRT_NVCC_DEFINES: extra -D options for all sources (e.g. -DMCRT_FAST_WIDE=1 builds the
    # eight-child FAST traversal); a change of them rebuilds everything
    defines = os.environ.get("MCRT_NVCC_DEFINES", "").split()
    if any(not d.startswith("-D") for d in defines):
        raise ValueError("MCRT_NVCC_DEFINES takes -D options only")
    stamp = os.path.join(LIB_DIR, "defines.txt")
    old = open(stamp).read() if os.path.exists(stamp) else ""
    if old != " ".join(defines):
        force = True
        with open(stamp, "w") as f:
            f.write(" ".join(defines))
    include = os.path.join(os.path.dirname(HERE), "include", "mcrt_gb300.h")
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [include]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(LIB_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         "-Xptxas", "-warn-spills"] + defines + ["-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(LIB_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-pthread",
                         f"-I{cuda}/include"] + defines + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)

    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        run([nvcc, ARCH, "-shared", "-o", tmp] + objs + ["-Xcompiler", "-fPIC", "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
