"""The FP64 oracle against golden vectors recorded from the reference's own
sources (tests/golden/reference_small.npz, made by tests/golden/make_golden.py
from DiffMPMLib3D compiled with float widened to double)."""
from pathlib import Path

import numpy as np

import oracle as O
from helpers import golden_grid, golden_params, golden_state, rel_err

TOL = 1e-9


def test_forward_step_matches_reference(orc, golden):
    s, g, prm = golden_state(golden), golden_grid(golden), golden_params(golden)
    s1, gs = orc.forward_step(g, prm, s)
    for k in ("x", "v", "C", "F"):
        assert rel_err(getattr(s1, k), golden[f"fwd64_{k}"]) < TOL, k
    assert rel_err(gs["m"], golden["fwd64_gm"]) < TOL
    assert rel_err(gs["v"], golden["fwd64_gv"]) < TOL


def test_backward_step_matches_reference(orc, golden):
    s, g, prm = golden_state(golden), golden_grid(golden), golden_params(golden)
    g1 = O.Grads(golden["bwd_gx1"], golden["bwd_gv1"], golden["bwd_gF1"], golden["bwd_gC1"])
    step = dict(m=golden["bwd_gm"], v=golden["bwd_gv"])
    gb = orc.backward_step(g, prm, s, golden["bwd_C1"], step, g1)
    for k in ("x", "v", "F", "C"):
        assert rel_err(getattr(gb, k), golden[f"bwd64_g{k}"]) < TOL, k


def test_mass_loss_matches_reference(orc, golden):
    g, prm = golden_grid(golden), golden_params(golden)
    loss, d = orc.mass_loss(g, prm, golden["fwd64_x"], golden["m"], golden["loss_target"])
    assert abs(loss - golden["loss64"]) <= 1e-12 * max(1.0, abs(golden["loss64"]))
    assert rel_err(d["gx"], golden["loss64_gx"]) < TOL
    assert rel_err(d["dLdm"], golden["loss64_dLdm"]) < TOL


def test_adam_matches_reference(orc, golden):
    n = len(golden["m"])
    dFc, mom, vec, vmax = golden["dFc"].copy(), np.zeros((n, 3, 3)), np.zeros((n, 3, 3)), np.zeros((n, 3, 3))
    for t in (1, 2, 3):
        gF = golden["adam_gF"] * t
        orc.adam(gF, dFc, mom, vec, vmax, 0.05, orc.grad_norm(gF), timestep=t)
    assert rel_err(dFc, golden["adam64_dFc"]) < TOL
    assert rel_err(vmax, golden["adam64_vmax"]) < TOL


def test_volumes_match_reference(orc, golden):
    s, g = golden_state(golden), golden_grid(golden)
    gm, gp = np.zeros(g.n_nodes), np.zeros((g.n_nodes, 3))
    vol = orc.volumes(g, s.x, s.v, s.C, s.m, gm, gp)
    assert rel_err(vol, golden["vol64"]) < TOL
    assert rel_err(gm, golden["vol64_gm"]) < TOL
    assert rel_err(gp, golden["vol64_gp"]) < TOL


def test_constitutive_matches_reference(orc, golden):
    for F, dF, P, H in zip(golden["cons_F"], golden["cons_dF"], golden["cons_P64"], golden["cons_H64"]):
        assert rel_err(orc.pk(F, 5769.23, 3846.15), P) < 1e-8
        assert rel_err(orc.pk_vjp(F, 5769.23, 3846.15, dF), H) < 1e-7


def test_rollout_matches_reference(orc, golden):
    s, g = golden_state(golden), golden_grid(golden)
    n = s.n
    s0 = O.State(s.x, s.v, np.zeros((n, 3, 3)), np.tile(np.eye(3), (n, 1, 1)), s.m, s.vol, s.lam, s.mu, s.dFc)
    prm = O.Params(dt=1e-3, drag=0.5, smoothing=0.1)
    xT, gr = orc.rollout(g, prm, s0, int(golden["roll_T"]), golden["roll_seed"])
    assert rel_err(xT, golden["roll64_xT"]) < TOL
    for k in ("x", "v"):
        assert rel_err(getattr(gr, k), golden[f"roll64_g{k}"]) < 1e-8, k
    # dL/dF and dL/dC are ~1e-15 here; the reference's own OpenMP atomics make
    # it differ from run to run by ~1e-6 relative at that magnitude
    for k in ("F", "C"):
        assert rel_err(getattr(gr, k), golden[f"roll64_g{k}"]) < 1e-4, k


def test_float_reference_noise_floor(golden):
    """The reference's own float build differs from its double build by the
    FP32 noise floor; this bounds the tolerances the GPU tests use."""
    assert rel_err(golden["fwd32_x"], golden["fwd64_x"]) < 1e-6
    assert rel_err(golden["fwd32_C"], golden["fwd64_C"]) < 2e-3
    assert rel_err(golden["roll32_xT"], golden["roll64_xT"]) < 1e-6


def test_optimizer_matches_reference(orc, golden_opt):
    """OptimizeDefGradControlSequence (CompGraph.cpp:213-368): the oracle's
    restatement reproduces the reference's recorded run (3 passes, line
    search with rejections) -- every layer's control, the final positions and
    the initial/final loss."""
    from helpers import golden_opt_case
    s, g, tgt, prm, kw = golden_opt_case(golden_opt)
    hist, layers = orc.run_optimization(g, prm, s, tgt, **kw)
    assert abs(hist[0] - golden_opt["opt64_initial_loss"]) <= 1e-5 * hist[0]  # printed with 6 digits
    assert abs(hist[-1] - golden_opt["opt64_loss"]) <= 1e-12 * hist[-1]
    assert hist[-1] < hist[0]
    want = golden_opt["opt64_dFc"]
    for l, lay in enumerate(layers):
        assert rel_err(lay.dFc, want[l]) < 1e-10 if np.abs(want[l]).max() > 0 else np.abs(lay.dFc).max() == 0
    assert rel_err(layers[-1].x, golden_opt["opt64_xT"]) < 1e-13


def test_mesh_sampling_oracle_matches_reference():
    """The inside test of GeometryLoading.cpp:57-77 (libigl signed distance,
    winding-number sign) restated by the oracle's winding numbers keeps the
    same lattice points as the reference on a convex and a non-convex mesh
    (every 4th lattice point, to keep the CPU suite short)."""
    from diffmpm_bindings.geometry import lattice
    from geometry_oracle import winding_numbers
    g = dict(np.load(__import__("pathlib").Path(__file__).parent / "golden" / "reference_mesh_sampling.npz"))
    for name in ("ellipsoid", "torus"):
        V, F, dx, ref = g[f"{name}_V"], g[f"{name}_F"], float(g[f"{name}_dx"]), g[f"{name}_points"]
        pts = lattice(V, dx)
        sub = pts[::4]
        keep = np.abs(winding_numbers(sub, V, F)) >= 0.5
        ref_set = {tuple(p) for p in ref.astype(np.float32).tolist()}
        want = np.array([tuple(p) in ref_set for p in sub.tolist()])
        assert (keep == want).all(), name


def test_single_timestep_optimiser_matches_reference(orc):
    """OptimizeSingleTimestep as run.py's E2E path calls it (layers, a forward
    pass, stored render gradients, then four calls at layers 2, 0, 2, 4):
    the oracle's restatement against the reference's double build, call by
    call -- every layer's dFc, the last positions and the end-layer loss."""
    gs = dict(np.load(Path(__file__).resolve().parent / "golden" / "reference_single.npz"))
    n = len(gs["m"])
    s = O.State(gs["x"], gs["v"], np.zeros((n, 3, 3)), np.tile(np.eye(3), (n, 1, 1)), gs["m"], gs["vol"],
                gs["lam"], gs["mu"])
    g = O.Grid(tuple(int(d) for d in gs["dims"]), float(gs["dx"]))
    prm = O.Params(dt=float(gs["dt"]), drag=float(gs["drag"]), smoothing=float(gs["smoothing"]))
    og = O.OracleGraph(orc, g, prm, s, gs["target"])
    O.OracleGraph.adam_step = 0  # the reference's counter in a fresh process
    og.set_up(int(gs["layers"]))
    og.forward(0)
    og.set_render_gradients(gs["render_dLdF"].astype(np.float64), gs["render_dLdx"].astype(np.float64))
    for c, (t, gd, alpha, ls) in enumerate(gs["calls"]):
        og.optimize_single_timestep(int(t), int(gd), 0, float(alpha), int(ls))
        dfc = np.stack([lay.dFc for lay in og.layers])
        assert rel_err(dfc, gs["single64_dFc"][c]) < 1e-11, c
        assert rel_err(og.layers[-1].x, gs["single64_xT"][c]) < 1e-13, c
        assert abs(og.loss() - gs["single64_loss"][c]) < 1e-12 * abs(gs["single64_loss"][c]), c
    assert O.OracleGraph.adam_step == int((gs["single64_ls"] >= 0).sum())
