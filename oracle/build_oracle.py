"""Build recipe for the test oracle (test infrastructure only).

* ``oracle/liboracle.so`` -- the FP64 CPU restatement in ``mpm_oracle.c``
  (gcc + OpenMP).  Built on every machine that runs the tests.
* ``oracle/_ref/libref32.so`` / ``libref64.so`` -- the reference's own
  DiffMPMLib3D sources compiled together with ``ref_driver.cpp``.  Built only
  where the reference tree is named by the ``REF_DIR`` environment variable
  (the checkout's root, holding ``DiffMPMLib3D/`` and ``include/``); without
  it they are skipped and the tests that need them skip too.  The sources
  are read where they lie; the FP64 variant and the ``private:`` ->
  ``public:`` edit (so ``ref_driver.cpp`` can set CompGraph's dt, drag and
  smoothing) are applied to temporary copies outside this repository.  Only
  the two shared libraries are written into ``oracle/_ref/``.
* ``oracle/_ref/gs_*.cubin`` -- the reference's Gaussian rasterizer kernels
  (``build_ref_gauss``), from the same checkout.

Usage: ``REF_DIR=<reference checkout> python oracle/build_oracle.py [--no-ref] [--force]``
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT_REF = HERE / "_ref"


def ref_dir() -> Path | None:
    """The reference checkout named by $REF_DIR, or None."""
    d = os.environ.get("REF_DIR")
    return Path(d) if d else None


REF_SOURCES = [
    "ForwardSimulation.cpp", "BackPropagation.cpp", "Elasticity.cpp", "PointCloud.cpp",
    "Grid.cpp", "GridNode.cpp", "MaterialPoint.cpp", "CompGraph.cpp", "Tensor3x3x3x3.cpp",
    "GeometryLoading.cpp",  # mesh -> lattice sampling (libigl signed distance, header-only)
]
CXXFLAGS = ["-std=c++17", "-O2", "-fopenmp", "-fPIC", "-fno-fast-math", "-ffp-contract=off",
            "-DNDEBUG", "-DEIGEN_NO_DEBUG", "-D_USE_MATH_DEFINES", "-w"]


def _newer(out: Path, inputs) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(Path(i).stat().st_mtime <= t for i in inputs)


def build_oracle(force: bool = False) -> Path:
    src = HERE / "mpm_oracle.c"
    out = HERE / "liboracle.so"
    if force or not _newer(out, [src]):
        cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c99", "-ffp-contract=off",
               str(src), "-o", str(out), "-lm"]
        subprocess.check_call(cmd)
    return out


_FLOAT_LIT = re.compile(r"\b((?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?)f\b")


def _widen(text: str) -> str:
    """float -> double, Eigen *f types -> *d, strip float literal suffixes."""
    text = re.sub(r"\bVector3f\b", "Vector3d", text)
    text = re.sub(r"\bMatrix3f\b", "Matrix3d", text)
    text = re.sub(r"\bMatrixXf\b", "MatrixXd", text)
    text = re.sub(r"\bVectorXf\b", "VectorXd", text)
    text = re.sub(r"\bfloat\b", "double", text)
    return _FLOAT_LIT.sub(r"\1", text)


def _stage(tmp: Path, widen: bool, ref: Path) -> Path:
    """Copy DiffMPMLib3D into tmp with the mechanical edits applied."""
    dst = tmp / ("src64" if widen else "src32")
    dst.mkdir(parents=True, exist_ok=True)
    for f in (ref / "DiffMPMLib3D").iterdir():
        if f.suffix not in (".h", ".cpp"):
            continue
        text = f.read_text(encoding="utf-8", errors="replace")
        if f.name == "CompGraph.h":
            text = text.replace("private:", "public:")
        if widen:
            text = _widen(text)
        (dst / f.name).write_text(text, encoding="utf-8")
    return dst


def _compile(args):
    cmd, = args
    subprocess.check_call(cmd)


def build_ref(force: bool = False) -> list[Path]:
    ref = ref_dir()
    if ref is None or not (ref / "DiffMPMLib3D" / "ForwardSimulation.cpp").exists():
        return []
    OUT_REF.mkdir(exist_ok=True)
    outs = []
    inputs = [HERE / "ref_driver.cpp", Path(__file__)] + [ref / "DiffMPMLib3D" / s for s in REF_SOURCES]
    todo = []
    for widen, name in ((False, "libref32.so"), (True, "libref64.so")):
        out = OUT_REF / name
        outs.append(out)
        if force or not _newer(out, inputs):
            todo.append((widen, out))
    if not todo:
        return outs
    tmp = Path(tempfile.mkdtemp(prefix="mpm_ref_"))
    try:
        jobs, links = [], []
        for widen, out in todo:
            src = _stage(tmp, widen, ref)
            inc = ["-I", str(src), "-I", str(ref / "include"), "-I", str(ref / "include" / "qrsvd")]
            objs = []
            for s in REF_SOURCES + ["ref_driver.cpp"]:
                cpp = (HERE / s) if s == "ref_driver.cpp" else (src / s)
                obj = tmp / f"{'64' if widen else '32'}_{s}.o"
                objs.append(obj)
                jobs.append(["g++", *CXXFLAGS, *inc, "-c", str(cpp), "-o", str(obj)])
            links.append(["g++", "-shared", "-fopenmp", *map(str, objs), "-o", str(out)])
        with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
            list(ex.map(_compile, [(j,) for j in jobs]))
        for cmd in links:
            subprocess.check_call(cmd)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return outs


GAUSS_SUBDIR = Path("gaussian-splatting") / "submodules" / "diff-gaussian-rasterization"
GAUSS_UNITS = {"gs_forward.cubin": "forward.cu", "gs_backward.cubin": "backward.cu",
               "gs_impl.cubin": "rasterizer_impl.cu"}


def build_ref_gauss(force: bool = False) -> list[Path]:
    """The reference's differentiable Gaussian rasterizer
    (``cuda_rasterizer/{forward,backward,rasterizer_impl}.cu``) compiled as
    sm_103a device code (cubins) into ``oracle/_ref/``, from the sources
    where they lie (``-include cstdint``: rasterizer_impl.h uses uint32_t
    without including it; its own build gets it through torch's headers).
    Device code does not depend on the host's architecture, so the cubins
    run on the GPU host, driven by ``tests/golden/make_gauss_golden.py``."""
    ref = ref_dir()
    if ref is None:
        return []
    src = ref / GAUSS_SUBDIR
    if not (src / "cuda_rasterizer" / "forward.cu").exists():
        return []
    OUT_REF.mkdir(exist_ok=True)
    nvcc = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    headers = list((src / "cuda_rasterizer").glob("*.h"))
    outs, jobs = [], []
    for name, unit in GAUSS_UNITS.items():
        out = OUT_REF / name
        outs.append(out)
        cu = src / "cuda_rasterizer" / unit
        if force or not _newer(out, [cu, Path(__file__), *headers]):
            jobs.append([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                         "-include", "cstdint", "-I", str(src / "third_party" / "glm"),
                         "-I", str(src / "cuda_rasterizer"), "-w", str(cu), "-o", str(out)])
    with cf.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(_compile, [(j,) for j in jobs]))
    return outs


def build_ref_module(widen: bool = False, force: bool = False) -> Path | None:
    """The reference's own Python module, ``diffmpm_bindings`` (bind/bind.cpp
    and the DiffMPMLib3D sources, without its optional torch support),
    compiled with g++ and pybind11: float as shipped into
    ``oracle/_ref/pymod32/``, or with float widened to double (bind.cpp
    included, on temporary copies) into ``oracle/_ref/pymod64/``.  Only
    tests/golden/run_py_sequence.py imports it, to record what the reference
    returns for run.py's call sequence."""
    ref = ref_dir()
    if ref is None or not (ref / "bind" / "bind.cpp").exists():
        return None
    try:
        import pybind11
    except ImportError:
        return None
    import sysconfig
    out_dir = OUT_REF / ("pymod64" if widen else "pymod32")
    out = out_dir / ("diffmpm_bindings" + sysconfig.get_config_var("EXT_SUFFIX"))
    inputs = [ref / "DiffMPMLib3D" / s for s in REF_SOURCES] + [ref / "bind" / "bind.cpp", Path(__file__)]
    if not force and _newer(out, inputs):
        return out
    out_dir.mkdir(parents=True, exist_ok=True)
    tmp = Path(tempfile.mkdtemp(prefix="mpm_refmod_"))
    try:
        src = _stage(tmp, widen, ref)
        bind = (ref / "bind" / "bind.cpp").read_text(encoding="utf-8", errors="replace")
        (src / "bind.cpp").write_text(_widen(bind) if widen else bind, encoding="utf-8")
        inc = ["-I", str(src), "-I", str(ref / "include"), "-I", str(ref / "include" / "qrsvd"),
               "-I", pybind11.get_include(), "-I", sysconfig.get_paths()["include"]]
        objs, jobs = [], []
        for name in REF_SOURCES + ["bind.cpp"]:
            obj = tmp / (name + ".o")
            objs.append(obj)
            jobs.append((["g++", *CXXFLAGS, "-fvisibility=hidden", *inc, "-c", str(src / name), "-o", str(obj)],))
        with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
            list(ex.map(_compile, jobs))
        subprocess.check_call(["g++", "-shared", "-fopenmp", *map(str, objs), "-o", str(out)])
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--no-ref", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build_oracle(a.force))
    if not a.no_ref:
        for p in build_ref(a.force) + build_ref_gauss(a.force):
            print(p)
    return 0


if __name__ == "__main__":
    sys.exit(main())
