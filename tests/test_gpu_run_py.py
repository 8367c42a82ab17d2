"""run.py's physics-only call sequence through this package, against the
reference's own pybind11 module making the identical calls.

tests/golden/run_py_sequence.py holds the sequence (build_opt_input ->
load_point_cloud_from_obj x2 -> Grid x2 -> calculate_point_cloud_volumes x2
-> CompGraph -> get_positions_from_pc -> two episodes of run_optimization
with promote_last_as_initial between them; run.py:318-387,1276-1364) and
recorded what the reference module returns for it, float as shipped and
widened to double (tests/golden/reference_run_py.npz).  Here the same
function runs on diffmpm_bindings, held to the double build: the FP64
engine to 1e-9 on the losses (its arrays come back as float32 through the
API, as the reference's do, so to that rounding); the FP32 engine as close
as the reference's own float build is (after three Adam passes the float
build's controls are 3e-4 to 8e-4 from the double build's).
"""
import sys
from pathlib import Path

import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_run_py_physics_sequence_matches_reference(dm, tmp_path, prec):
    sys.path.insert(0, str(GOLDEN))
    import run_py_sequence as seq
    gold = dict(np.load(GOLDEN / "reference_run_py.npz"))
    bits = 64 if prec == "fp64" else 32
    dm.set_default_precision(prec)
    try:
        rec = seq.physics_episodes(dm, seq.CONFIG, tmp_path)
    finally:
        dm.set_default_precision("fp32")
    ref = {k[len(f"ref{bits}_"):]: v for k, v in gold.items() if k.startswith(f"ref{bits}_")}
    r64 = {k[len("ref64_"):]: v for k, v in gold.items() if k.startswith("ref64_")}
    r32 = {k[len("ref32_"):]: v for k, v in gold.items() if k.startswith("ref32_")}
    # the mesh -> particle sampling keeps the same lattice points, in the same
    # order, with the same masses
    assert rec["n_input"] == int(ref["n_input"]) and rec["n_target"] == int(ref["n_target"])
    assert np.array_equal(rec["input_x"], ref["input_x"])
    assert rel_err(rec["input_m"], ref["input_m"]) == 0.0
    lossrel = lambda a, b: abs(float(a) - float(b)) / abs(float(b))  # noqa: E731
    for ep in range(seq.CONFIG["optimization"]["num_animations"]):
        assert rec[f"ep{ep}_layers"] == int(ref[f"ep{ep}_layers"])
        e_loss = lossrel(rec[f"ep{ep}_loss"], r64[f"ep{ep}_loss"])
        e_dfc = rel_err(rec[f"ep{ep}_dFc"], r64[f"ep{ep}_dFc"])
        e_x = rel_err(rec[f"ep{ep}_xT"], r64[f"ep{ep}_xT"])
        print(f"{prec} episode {ep} vs the double build: loss {e_loss:.2e}, control dFc {e_dfc:.2e}, x_T {e_x:.2e}")
        if prec == "fp64":
            # get_positions / get_def_grads_morph return float32 arrays, as
            # the reference's bindings do (py::array_t<float>), also from the
            # FP64 engine: arrays agree to that rounding, the loss to 1e-9
            assert e_loss < 1e-9 and e_dfc < 2e-7 and e_x < 2e-7, (ep, e_loss, e_dfc, e_x)
        else:
            # FP32: as close to the double build as the reference's own float
            # build is (its distance, doubled, or 1e-4 / 1e-5 if larger)
            f_loss = lossrel(r32[f"ep{ep}_loss"], r64[f"ep{ep}_loss"])
            f_dfc = rel_err(r32[f"ep{ep}_dFc"], r64[f"ep{ep}_dFc"])
            f_x = rel_err(r32[f"ep{ep}_xT"], r64[f"ep{ep}_xT"])
            print(f"  reference float build vs double: loss {f_loss:.2e}, control dFc {f_dfc:.2e}, x_T {f_x:.2e}")
            assert e_loss < max(1e-4, 2 * f_loss) and e_dfc < max(1e-4, 2 * f_dfc) and e_x < max(1e-5, 2 * f_x), \
                (ep, e_loss, e_dfc, e_x)
