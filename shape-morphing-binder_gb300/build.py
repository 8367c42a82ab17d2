"""Build libmpm.so (the CUDA engine) in-tree with nvcc for sm_103a.

Usage: python shape-morphing-binder_gb300/build.py [--force] [--debug]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
LIB = HERE / "diffmpm_bindings" / "libmpm.so"
SOURCES = ["mpm_kernels.cu", "mpm_engine.cu", "mpm_noalloc.cu", "mpm_sort.cu", "mpm_geometry.cu", "mpm_checks.cu",
           "gs_rasterizer.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def flags(debug: bool = False):
    f = ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-I", str(INCLUDE),
         "--expt-relaxed-constexpr", "-Xptxas", "-v" if os.environ.get("MPM_PTXAS_V") else "-O3"]
    if debug:
        f += ["-DMPM_DEBUG"]
    # extra compile flags (tuning experiments), e.g. MPM_NVCC_FLAGS="-DMPM_P2G_MIN_BLOCKS=2"
    f += os.environ.get("MPM_NVCC_FLAGS", "").split()
    return f


def _inputs():
    return [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + \
        [INCLUDE / "mpm.h", INCLUDE / "gsplat.h", Path(__file__)]


def up_to_date() -> bool:
    if not LIB.exists() or os.environ.get("MPM_NVCC_FLAGS"):
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _inputs())


def build(force: bool = False, debug: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    objdir = HERE / "_build"
    objdir.mkdir(exist_ok=True)
    base = flags(debug)
    jobs = []
    for s in SOURCES:
        obj = objdir / (s + ".o")
        jobs.append([nvcc(), *base, "-c", str(CSRC / s), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(run, jobs))
    if verbose:
        for o in outs:
            sys.stderr.write(o)
    link = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *[str(objdir / (s + ".o")) for s in SOURCES], "-lcudart"]
    run(link)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--debug", action="store_true")
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args()
    print(build(a.force, a.debug, a.v))
