"""Stages the reference's C++ sources for the reference builds -- test infrastructure.

The reference builds (``oracle/Makefile`` -> ``oracle/_ref/libmcrt_ref.so``) compile the
reference renderer's own sources: ``src/core`` (with ``acceleration``), the path-tracing
example ``src/examples/pt/demo_pt.cpp`` and the vendored ``glm``, ``nanolog`` and
``nanort`` headers/sources it includes.  They are compiled from ``baseline/_ref/src`` at
the repository root, a git-ignored copy of exactly those subtrees.  The copy is made
here from a checkout of the reference (``$MCRT_REFERENCE_DIR``, else the development
container's read-only checkout below) and travels with the working tree to machines
that have no checkout (the GPU machines), so the reference can be built and timed there
too.  Nothing under ``baseline/_ref`` is committed.

    python -m oracle.stage_reference          # copy (only changed files)
"""
from __future__ import annotations

import os
import shutil

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
STAGE_DIR = os.path.join(ROOT, "baseline", "_ref")
# the development container's checkout of the reference (read-only)
_CHECKOUT_DEFAULT = "/root/reference"
SUBTREES = ["src/core", "src/examples/pt", "src/thirdparty/glm/include", "src/thirdparty/nanolog",
            "src/thirdparty/nanort"]


def checkout_dir() -> str | None:
    """The reference checkout to stage from, or None where there is none."""
    for c in (os.environ.get("MCRT_REFERENCE_DIR"), _CHECKOUT_DEFAULT):
        if c and os.path.isdir(os.path.join(c, "src", "core")):
            return c
    return None


def source_dir() -> str | None:
    """The tree the reference builds compile from (``baseline/_ref``), or None."""
    return STAGE_DIR if os.path.isdir(os.path.join(STAGE_DIR, "src", "core")) else None


def stage() -> str | None:
    """Copies the reference subtrees into baseline/_ref (files whose size or mtime changed)
    and returns the staged tree; without a checkout, returns what is staged already."""
    src = checkout_dir()
    if src is None:
        return source_dir()
    for sub in SUBTREES:
        top = os.path.join(src, sub)
        for dirpath, _, files in os.walk(top):
            rel = os.path.relpath(dirpath, src)
            dst_dir = os.path.join(STAGE_DIR, rel)
            os.makedirs(dst_dir, exist_ok=True)
            for f in files:
                s, d = os.path.join(dirpath, f), os.path.join(dst_dir, f)
                st = os.stat(s)
                if os.path.exists(d):
                    dt = os.stat(d)
                    if dt.st_size == st.st_size and int(dt.st_mtime) == int(st.st_mtime):
                        continue
                shutil.copy2(s, d)
    return source_dir()


if __name__ == "__main__":
    print(stage() or "no reference checkout and nothing staged")
