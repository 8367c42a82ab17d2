"""The control-sequence optimiser on the GPU (OptimizeDefGradControlSequence,
CompGraph.cpp:213-368; run_optimization in bind.cpp:165-172) against the
reference's recorded run (tests/golden/reference_optimize.npz) and the
oracle's restatement of it: the loss curve (every loss evaluated: initial,
before each gradient step, each line-search trial, final), every layer's
control dFc and the final positions.

FP64 engine: to 1e-9.  FP32 engine (default and deterministic scatters):
the same curve, same accept/reject decisions, within 1e-4 relative -- the
reference's own float build lands 3e-5 from its double build here."""
import numpy as np
import pytest

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
