"""Test configuration: the `gpu` marker and import paths.

`-m "not gpu"` runs the oracle, golden-vector, host-logic and ABI tests on
CPU; `-m gpu` runs the CUDA parity tests (they call libmpm.so through its C
ABI via diffmpm_bindings and compare with the FP64 oracle).
"""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT / "oracle", ROOT / "shape-morphing-binder_gb300", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))
os.environ.setdefault("MPM_QUIET", "1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    import build_oracle
    build_oracle.build_oracle()
    import oracle as O
    return O.Oracle()


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(ROOT / "tests" / "golden" / "reference_small.npz"))


@pytest.fixture(scope="session")
def golden_opt():
    return dict(np.load(ROOT / "tests" / "golden" / "reference_optimize.npz"))


@pytest.fixture(scope="session")
def dm():
    import diffmpm_bindings
    diffmpm_bindings._lib.lib.mpm_set_verbose(0)
    return diffmpm_bindings
