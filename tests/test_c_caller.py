"""libmpm.so from plain C: tests/c_caller.c is compiled with gcc against
include/mpm.h (as C99, so the header is C-compatible) and linked to the
library, then run.  The host mode needs no GPU; the sim mode runs a small
forward and backward pass through the C ABI alone."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def c_caller(tmp_path_factory):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    from diffmpm_bindings import _lib  # builds nothing; fails loudly if libmpm.so is missing
    libdir = _lib.LIB_PATH.parent
    exe = tmp_path_factory.mktemp("c_caller") / "c_caller"
    cmd = [gcc, "-std=c99", "-O1", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(ROOT / "tests" / "c_caller.c"),
           "-o", str(exe), "-L", str(libdir), "-lmpm", "-lm", f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _run(exe, mode):
    r = subprocess.run([str(exe), mode], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_c_caller_host(c_caller):
    assert "host ok" in _run(c_caller, "host")


@pytest.mark.gpu
def test_c_caller_simulation(c_caller):
    assert "sim ok" in _run(c_caller, "sim")
