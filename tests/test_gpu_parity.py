"""CUDA path (libmpm.so through diffmpm_bindings) against the FP64 oracle and
the reference golden vectors.

Tolerances: the plain FP64 engine must agree with the FP64 oracle to 1e-9
relative (atomic summation order is the only difference).  The FP32 engine
is held to tolerances below the reference's own FP32 noise floor on the same
inputs (tests/golden: its float build differs from its double build by up to
~1e-4 in C): x 1e-6, F 1e-6, v 5e-6 and C 1e-5 relative to the field's max
magnitude, gradients 1e-5 in norm for one step (measured on a GB300: fields
<= 8e-7, one-step gradients <= 6e-7, so each bound keeps a margin of 10x or
more against the atomics' order).  The precision target for gradients is
1e-4.
"""
import numpy as np
import pytest

import oracle as O
from helpers import (get_grads, golden_grid, golden_params, golden_state, layer_state, make_graph, norm_err,
                     rel_err, set_grads)

pytestmark = pytest.mark.gpu

FWD_TOL = {"fp64": dict(x=1e-9, v=1e-9, C=1e-9, F=1e-9), "fp32": dict(x=1e-6, v=5e-6, C=1e-5, F=1e-6)}
BWD_TOL = {"fp64": 1e-9, "fp32": 1e-5}


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_forward_step(dm, orc, golden, prec):
    s, g, prm = golden_state(golden), golden_grid(golden), golden_params(golden)
    cg, keep = make_graph(dm, s, g, prm, precision=prec)
    cg.compute_forward_pass(0, 0)
    got = layer_state(cg, 1)
    want, _ = orc.forward_step(g, prm, s)
    for k in ("x", "v", "C", "F"):
        e = rel_err(got[k], getattr(want, k))
        print(f"{prec} fwd {k} rel {e:.3e}")
        assert e < FWD_TOL[prec][k], (k, e)
        assert rel_err(got[k], golden[f"fwd64_{k}"]) < max(FWD_TOL[prec][k], 1e-8), k


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("adjoint", ["reference", "exact"])
def test_backward_step(dm, orc, golden, prec, adjoint):
    s, g = golden_state(golden), golden_grid(golden)
    prm = golden_params(golden, exact=adjoint == "exact")
    cg, keep = make_graph(dm, s, g, prm, precision=prec, adjoint=adjoint)
    cg.compute_forward_pass(0, 0)
    g1 = O.Grads(golden["bwd_gx1"], golden["bwd_gv1"], golden["bwd_gF1"], golden["bwd_gC1"])
    set_grads(cg, 1, g1)
    cg.compute_backward_pass(0)
    got = get_grads(cg, 0)
    # the oracle runs the adjoint on the engine's own forward (layer 1 + grid)
    s1, step = orc.forward_step(g, prm, s)
    want = orc.backward_step(g, prm, s, s1.C, step, g1, want_ft=True)
    for k in ("x", "v", "F", "C"):
        e = norm_err(got[k], getattr(want, k))
        print(f"{prec} {adjoint} bwd g{k} norm-rel {e:.3e}")
        assert e < BWD_TOL[prec], (k, e)
    if adjoint == "reference":
        for k in ("x", "v", "F", "C"):
            assert norm_err(got[k], golden[f"bwd64_g{k}"]) < max(BWD_TOL[prec], 1e-8) * 10, k
    ctl = cg.get_grad(0, "dFc", np.float64)
    assert norm_err(ctl, want.Ft) < BWD_TOL[prec]


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("adjoint", ["reference", "exact"])
def test_mass_loss(dm, orc, golden, prec, adjoint):
    s, g = golden_state(golden), golden_grid(golden)
    prm = golden_params(golden, exact=adjoint == "exact")
    cg, keep = make_graph(dm, s, g, prm, precision=prec, adjoint=adjoint, layers=1,
                          target_mass=golden["loss_target"])
    loss = cg.end_layer_mass_loss()
    want, d = orc.mass_loss(g, prm, s.x, s.m, golden["loss_target"])
    assert abs(loss - want) <= (1e-6 if prec == "fp32" else 1e-9) * abs(want)
    gx = cg.get_grad(0, "x", np.float64)
    e = norm_err(gx, d["gx"])
    print(f"{prec} {adjoint} loss {loss:.9g} vs {want:.9g}; dLdx norm-rel {e:.3e}")
    assert e < (2e-5 if prec == "fp32" else 1e-9)  # measured 1.3e-6
    for k in ("v", "F", "C"):
        assert np.abs(cg.get_grad(0, k)).max() == 0.0


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_adam(dm, orc, golden, prec):
    s, g, prm = golden_state(golden), golden_grid(golden), golden_params(golden)
    cg, keep = make_graph(dm, s, g, prm, precision=prec, layers=2)
    n = s.n
    dFc, mom, vec, vmax = s.dFc.copy(), np.zeros((n, 3, 3)), np.zeros((n, 3, 3)), np.zeros((n, 3, 3))
    pc = cg.get_point_cloud(0)
    for t in (1, 2, 3):
        gF = golden["adam_gF"] * t
        pc.set("grad_F", gF)
        gn = cg.grad_norm(0)
        assert abs(gn - orc.grad_norm(gF)) <= 1e-6 * gn
        cg.adam_step(0, 0.05, gn, timestep=t)
        orc.adam(gF, dFc, mom, vec, vmax, 0.05, orc.grad_norm(gF), timestep=t)
    got = pc.get("dFc", np.float64)
    assert rel_err(got, dFc) < (1e-6 if prec == "fp32" else 1e-12)
    assert rel_err(got, golden["adam64_dFc"]) < (1e-6 if prec == "fp32" else 1e-9)


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_volumes_and_p2g(dm, orc, golden, prec):
    s, g = golden_state(golden), golden_grid(golden)
    dt = np.float64 if prec == "fp64" else np.float32
    pc = dm.PointCloud.from_arrays(s.x.astype(dt), v=s.v.astype(dt), C_=s.C.astype(dt), m=s.m.astype(dt),
                                   precision=prec)
    grid = dm.Grid(*g.dims, g.dx, g.min, precision=prec)
    dm.calculate_point_cloud_volumes(pc, grid)
    tol = 1e-5 if prec == "fp32" else 1e-10
    assert rel_err(pc.get("vol", np.float64), golden["vol64"]) < tol
    assert rel_err(grid.get_node_masses(np.float64), golden["vol64_gm"]) < tol
    assert rel_err(grid.get_node_momenta(np.float64), golden["vol64_gp"]) < 10 * tol
    # p2g accumulates onto the un-reset grid
    dm.p2g(pc, grid)
    assert rel_err(grid.get_node_masses(np.float64), 2 * golden["vol64_gm"]) < tol


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_rollout_against_reference_golden(dm, golden, prec):
    """5-step full tape through CompGraph, reference adjoint, vs the reference."""
    s, g = golden_state(golden), golden_grid(golden)
    n = s.n
    s0 = O.State(s.x, s.v, np.zeros((n, 3, 3)), np.tile(np.eye(3), (n, 1, 1)), s.m, s.vol, s.lam, s.mu, s.dFc)
    prm = O.Params(dt=1e-3, drag=0.5, smoothing=0.1)
    T = int(golden["roll_T"])
    cg, keep = make_graph(dm, s0, g, prm, precision=prec, layers=T + 1)
    cg.compute_forward_pass(0, 0)
    xT = cg.get_point_cloud(T).get("x", np.float64)
    assert rel_err(xT, golden["roll64_xT"]) < (1e-6 if prec == "fp32" else 1e-10)
    last = cg.get_point_cloud(T)
    last.set("grad_x", golden["roll_seed"])
    for k in ("v", "F", "C"):
        last.set("grad_" + k, np.zeros((n, 3) if k == "v" else (n, 3, 3)))
    cg.compute_backward_pass(0)
    got = get_grads(cg, 0)
    for k in ("x", "v"):
        e = norm_err(got[k], golden[f"roll64_g{k}"])
        print(f"{prec} roll g{k} {e:.3e}")
        assert e < (1e-5 if prec == "fp32" else 1e-8), k  # measured <= 4.1e-7
