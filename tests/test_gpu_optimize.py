"""The control-sequence optimiser on the GPU (OptimizeDefGradControlSequence,
CompGraph.cpp:213-368; run_optimization in bind.cpp:165-172) against the
reference's recorded run (tests/golden/reference_optimize.npz) and the
oracle's restatement of it: the loss curve (every loss evaluated: initial,
before each gradient step, each line-search trial, final), every layer's
control dFc and the final positions.

FP64 engine: to 1e-9.  FP32 engine (default and deterministic scatters):
the same curve, same accept/reject decisions, within 1e-4 relative -- the
reference's own float build lands 3e-5 from its double build here."""
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from helpers import golden_opt_case, make_graph, rel_err

pytestmark = pytest.mark.gpu


def _run(dm, golden_opt, precision, deterministic=False, passes=None):
    s, g, tgt, prm, kw = golden_opt_case(golden_opt)
    cg, keep = make_graph(dm, s, g, prm, precision=precision, layers=1, target_mass=tgt,
                          deterministic=deterministic)
    opt = dm.OptInput()
    opt.num_timesteps, opt.control_stride = kw["num_steps"], kw["control_stride"]
    opt.max_gd_iters, opt.max_ls_iters = kw["max_gd_iters"], kw["max_ls_iters"]
    opt.dt, opt.drag, opt.smoothing_factor = prm.dt, prm.drag, prm.smoothing
    opt.initial_alpha, opt.gd_tol = kw["initial_alpha"], kw["gd_tol"]
    if precision == "fp64":
        # OptInput's float fields round to float32 like the reference's struct;
        # the recorded run used the double values
        for k, v in (("dt", prm.dt), ("drag", prm.drag), ("smoothing_factor", prm.smoothing),
                     ("initial_alpha", kw["initial_alpha"]), ("gd_tol", kw["gd_tol"])):
            object.__setattr__(opt, k, float(v))
    cg.run_optimization(opt, passes=passes)
    L = cg.get_num_layers()
    dfc = np.stack([cg.get_point_cloud(i).get("dFc", np.float64) for i in range(L)])
    xT = cg.get_point_cloud(L - 1).get("x", np.float64)
    return cg.loss_history(), dfc, xT


@pytest.fixture(scope="module")
def oracle_curve(orc, golden_opt):
    s, g, tgt, prm, kw = golden_opt_case(golden_opt)
    hist, layers = orc.run_optimization(g, prm, s, tgt, **kw)
    return hist, np.stack([lay.dFc for lay in layers]), layers[-1].x


def test_fp64_optimizer_matches_reference(dm, golden_opt, oracle_curve):
    hist, dfc, xT = _run(dm, golden_opt, "fp64")
    want_hist, _, _ = oracle_curve
    assert len(hist) == len(want_hist)
    assert np.abs(hist - want_hist).max() <= 1e-9 * want_hist.max()
    assert abs(hist[-1] - golden_opt["opt64_loss"]) <= 1e-9 * hist[-1]
    assert rel_err(dfc, golden_opt["opt64_dFc"]) < 1e-8
    assert rel_err(xT, golden_opt["opt64_xT"]) < 1e-10


@pytest.mark.parametrize("deterministic", [False, True])
def test_fp32_optimizer_curve(dm, golden_opt, oracle_curve, deterministic):
    hist, dfc, xT = _run(dm, golden_opt, "fp32", deterministic=deterministic)
    want_hist, want_dfc, want_x = oracle_curve
    assert len(hist) == len(want_hist)
    assert np.abs(hist - want_hist).max() <= 1e-4 * want_hist.max()
    assert rel_err(dfc, want_dfc) < 2e-3
    assert rel_err(xT, want_x) < 1e-5
    # the reference's float build on the same run, for scale
    ref32 = rel_err(golden_opt["opt32_dFc"], golden_opt["opt64_dFc"])
    print(f"fp32 det={deterministic}: dFc err {rel_err(dfc, want_dfc):.2e} (reference float build {ref32:.2e})")


def test_more_passes(dm, golden_opt):
    h3, _, _ = _run(dm, golden_opt, "fp32", deterministic=True)
    h5, _, _ = _run(dm, golden_opt, "fp32", deterministic=True, passes=5)
    assert len(h5) > len(h3)
    assert np.array_equal(h5[:len(h3) - 1], h3[:-1])  # same first three passes (bitwise: deterministic)
    assert h5[-1] <= h3[-1]


def test_control_episode_twin_loss_curve(dm, orc):
    """A down-scaled twin of the 500k-particle control-optimisation episode (sphere -> spherical-harmonic
    target, deterministic scatters, FP64 Adam moments): the FP32 engine's loss
    curve against the FP64 oracle's, evaluation by evaluation."""
    import oracle as O
    from diffmpm_bindings import workloads as W
    w = W.morph500k(n=3000, G=20, episode=1, amp=0.06)
    n = w.n
    s = O.State(w.x, w.v, np.zeros((n, 3, 3)), w.F, w.m, w.vol, w.lam, w.mu)
    g = O.Grid(w.dims, w.dx)
    tgt = np.zeros(g.n_nodes)
    orc.p2g_accumulate(g, w.target, w.v, np.zeros((n, 3, 3)), w.m, tgt, np.zeros((g.n_nodes, 3)))
    prm = O.Params(dt=w.dt, drag=0.0, smoothing=0.0)
    kw = dict(num_steps=16, control_stride=5, max_gd_iters=1, max_ls_iters=4, initial_alpha=1e-2, gd_tol=1e-4)
    want, _ = orc.run_optimization(g, prm, s, tgt, passes=2, **kw)
    cg, keep = make_graph(dm, s, g, prm, layers=1, target_mass=tgt, deterministic=True, checkpoint_every=5)
    opt = dm.OptInput()
    opt.num_timesteps, opt.control_stride = kw["num_steps"], kw["control_stride"]
    opt.max_gd_iters, opt.max_ls_iters = kw["max_gd_iters"], kw["max_ls_iters"]
    for k, v in (("dt", prm.dt), ("drag", 0.0), ("smoothing_factor", 0.0), ("initial_alpha", 1e-2),
                 ("gd_tol", 1e-4)):
        object.__setattr__(opt, k, float(v))
    cg.run_optimization(opt, passes=2)
    got = cg.loss_history()
    print("twin curve", got[0], got[-1], len(got))
    assert len(got) == len(want)
    assert np.abs(got - want).max() <= 1e-4 * want.max()
    assert got[-1] < got[0]


def _single(dm, precision):
    """run.py's E2E physics path on the GPU with the fixture's inputs: layers,
    a forward pass, stored render gradients, then the fixture's calls of
    optimize_single_timestep.  Per call: every layer's dFc, the last
    positions, the end-layer loss and the losses the call evaluated."""
    gs = dict(np.load(Path(__file__).resolve().parent / "golden" / "reference_single.npz"))
    n = len(gs["m"])
    s = O.State(gs["x"], gs["v"], np.zeros((n, 3, 3)), np.tile(np.eye(3), (n, 1, 1)), gs["m"], gs["vol"],
                gs["lam"], gs["mu"])
    g = O.Grid(tuple(int(d) for d in gs["dims"]), float(gs["dx"]))
    prm = O.Params(dt=float(gs["dt"]), drag=float(gs["drag"]), smoothing=float(gs["smoothing"]))
    L = int(gs["layers"])
    cg, keep = make_graph(dm, s, g, prm, precision=precision, layers=1, target_mass=gs["target"])
    cg.set_up_comp_graph(L)
    cg.compute_forward_pass(0, 0)
    cg.set_render_gradients(gs["render_dLdF"], gs["render_dLdx"])
    dm.single_timestep_adam_step(set_to=0)  # as in a fresh reference process
    out = []
    for t, gd, alpha, ls in gs["calls"]:
        # the reference's double build takes alpha as a double: bypass the
        # binding's float32 rounding of initial_alpha for the FP64 engine
        a = float(alpha) if precision == "fp64" else float(np.float32(alpha))
        dm._lib.check(dm._lib.lib.mpm_compgraph_optimize_single_timestep(cg._h, int(t), int(gd), 0, a, int(ls)))
        hist = cg.loss_history()
        dfc = np.stack([cg.get_point_cloud(i).get("dFc", np.float64) for i in range(L)])
        xT = cg.get_point_cloud(L - 1).get("x", np.float64)
        out.append((dfc, xT, cg.end_layer_mass_loss(), hist))
    return gs, out, dm.single_timestep_adam_step()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_single_timestep_optimizer_matches_reference(dm, orc, precision):
    """optimize_single_timestep (OptimizeSingleTimestep, CompGraph.cpp:369-465;
    bind.cpp:294-317), the call run.py's E2E mode makes (run.py:686), with
    render gradients injected at every backward (CompGraph.cpp:148-197),
    against the reference's recorded calls and the oracle's restatement of
    them, loss by loss.  FP64 engine to 1e-9; FP32 engine within 1e-4 with
    the same accept/reject decisions (the reference's float build is ~1e-6
    from its double build on these losses)."""
    gs, out, adam_steps = _single(dm, precision)
    n = len(gs["m"])
    s = O.State(gs["x"], gs["v"], np.zeros((n, 3, 3)), np.tile(np.eye(3), (n, 1, 1)), gs["m"], gs["vol"],
                gs["lam"], gs["mu"])
    og = O.OracleGraph(orc, O.Grid(tuple(int(d) for d in gs["dims"]), float(gs["dx"])),
                       O.Params(dt=float(gs["dt"]), drag=float(gs["drag"]), smoothing=float(gs["smoothing"])),
                       s, gs["target"])
    O.OracleGraph.adam_step = 0
    og.set_up(int(gs["layers"]))
    og.forward(0)
    og.set_render_gradients(gs["render_dLdF"].astype(np.float64), gs["render_dLdx"].astype(np.float64))
    tol = 1e-9 if precision == "fp64" else 1e-4
    for c, ((dfc, xT, loss, hist), (t, gd, alpha, ls)) in enumerate(zip(out, gs["calls"])):
        og.history = []
        og.optimize_single_timestep(int(t), int(gd), 0, float(alpha), int(ls))
        want_hist = np.asarray(og.history)
        assert len(hist) == len(want_hist), (c, hist, want_hist)
        e_hist = float(np.abs(hist - want_hist).max() / np.abs(want_hist).max())
        e_dfc = rel_err(dfc, gs["single64_dFc"][c])
        e_loss = abs(loss - gs["single64_loss"][c]) / abs(gs["single64_loss"][c])
        print(f"{precision} call {c}: losses {e_hist:.2e}, dFc {e_dfc:.2e}, end loss {e_loss:.2e}")
        assert e_hist < tol and e_dfc < tol and e_loss < tol, (c, e_hist, e_dfc, e_loss)
        assert rel_err(xT, gs["single64_xT"][c]) < (1e-11 if precision == "fp64" else 1e-6)
    assert adam_steps == O.OracleGraph.adam_step == int((gs["single64_ls"] >= 0).sum())
