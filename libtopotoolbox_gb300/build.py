"""Build the native CUDA library libtt_cuda.so in-tree.

Each translation unit under ``csrc/`` is compiled for sm_103a in parallel and
linked into ``libtopotoolbox_gb300/libtt_cuda.so``.  Object files go to
``libtopotoolbox_gb300/_build/`` (git-ignored).  A unit is rebuilt only when
its source or the shared headers are newer than its object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libtt_cuda.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-Xcompiler", "-fvisibility=hidden"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtt_cuda")


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _headers():
    return sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "tt_cuda.h"]


def build(verbose: bool = False, force: bool = False, extra_flags=()) -> Path:
    nvcc = nvcc_path()
    BUILD.mkdir(exist_ok=True)
    hdr_time = max(p.stat().st_mtime for p in _headers())
    jobs = []
    objs = []
    for src in _sources():
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr_time):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, "-I", str(ROOT / "include"),
                   "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}:\n{r.stdout}\n{r.stderr}")
        return r

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if jobs or force or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        run(cmd)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":  # pragma: no cover
    import sys

    print(build(verbose=True, force="--force" in sys.argv))
