"""libmpm.so loads and exports every entry point include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b((?:mpm|gs)_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert len(names) >= 40
    assert "mpm_compgraph_forward" in names and "mpm_compgraph_backward" in names


def test_library_exports_all_declared_symbols(dm):
    lib = ctypes.CDLL(str(dm._lib.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header(dm):
    bound = set(dm._lib.exported_symbols())
    assert set(declared_functions()) <= bound, set(declared_functions()) - bound


def test_build_targets_sm103a():
    text = (ROOT / "shape-morphing-binder_gb300" / "build.py").read_text()
    assert "arch=compute_103a,code=sm_103a" in text


def test_host_only_calls(dm):
    lib = dm._lib.lib
    p = dm._lib.MpmParams()
    lib.mpm_default_params(ctypes.byref(p))
    assert abs(p.dt - 1.0 / 120.0) < 1e-15 and p.drag == 0.5 and p.smoothing == 0.1
    o = dm._lib.MpmOptions()
    lib.mpm_default_options(ctypes.byref(o))
    assert o.precision == 0 and o.adjoint == 0 and o.checkpoint_every == 1
    lam, mu = ctypes.c_double(), ctypes.c_double()
    assert lib.mpm_lame(1e4, 0.3, ctypes.byref(lam), ctypes.byref(mu)) == 0
    assert abs(lam.value - 1e4 * 0.3 / (1.3 * 0.4)) < 1e-9
    assert lib.mpm_set_tile_nodes(-1) == dm._lib.MPM_ERR_ARG
    assert b"tile" in lib.mpm_last_error()
    assert lib.mpm_compgraph_forward(None, 0, 0) == dm._lib.MPM_ERR_ARG
