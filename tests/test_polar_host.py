"""The FP32 polar factor of the stress (Newton-Schulz for nearly orthogonal F,
scaled Newton otherwise, the FP64 SVD guard near inversion), compiled from
csrc/mpm_math.cuh for the host and checked against the FP64 Jacobi-SVD
factor on seeded random F (tests/polar_host.cu).  No GPU needed: nvcc
compiles the host side only.  The device build of the same code is covered
by the GPU parity tests."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "shape-morphing-binder_gb300" / "csrc"


def test_polar_factor_matches_fp64_svd(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not found")
    exe = tmp_path / "polar_host"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-x", "cu", "-I", str(CSRC), "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "polar_host.cu"), "-o", str(exe)], check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
