"""Deterministic scatters (mpm_options.deterministic, FP32): node sums in
64-bit fixed point.  The reference sums nodes under `omp atomic` /
`omp critical` (ForwardSimulation.cpp:26-80, BackPropagation.cpp:36-55), so
its results depend on thread timing; here the deterministic mode must give
bit-identical results run to run, a checkpointed backward must recompute
the forward bit for bit (so it equals the full tape exactly), and accuracy
against the FP64 oracle must stay what the default FP32 path reaches."""
import numpy as np
import pytest

import oracle as O
from helpers import get_grads, make_graph, norm_err, oracle_rollout, rel_err

pytestmark = pytest.mark.gpu


def _case(seed=0, G=14):
    from diffmpm_bindings import workloads as W
    w = W.sphere32(seed=seed, G=G, rho=60.0)
    rng = np.random.default_rng(seed)
    n = w.n
    s0 = O.State(w.x, w.v, 0.05 * rng.normal(size=(n, 3, 3)), np.eye(3) + 0.02 * rng.normal(size=(n, 3, 3)),
                 w.m, w.vol, w.lam, w.mu, 0.01 * rng.normal(size=(n, 3, 3)))
    return s0, O.Grid(w.dims, w.dx), rng


def _rollout(dm, s0, g, prm, T, seed_gx, **kw):
    cg, keep = make_graph(dm, s0, g, prm, precision="fp32", layers=T + 1, **kw)
    cg.compute_forward_pass(0, 0)
    n = s0.n
    last = cg.get_point_cloud(T)
    last.set("grad_x", seed_gx)
    last.set("grad_v", np.zeros((n, 3)))
    last.set("grad_F", np.zeros((n, 3, 3)))
    last.set("grad_C", np.zeros((n, 3, 3)))
    cg.compute_backward_pass(0)
    out = {"xT": last.get("x", np.float32)}
    for k, v in get_grads(cg, 0, np.float32).items():
        out["g" + k] = v
    out["gdFc"] = cg.get_grad(0, "dFc", np.float32)
    return out, cg, keep


def _same_bits(a, b):
    return all(np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)) for k in a)


@pytest.mark.parametrize("kernel,adjoint", [("cubic", "exact"), ("cubic", "reference"), ("quadratic", "exact")])
def test_deterministic_runs_are_bit_identical(dm, kernel, adjoint):
    s0, g, rng = _case(3)
    prm = O.Params(dt=1e-3, drag=0.2, smoothing=0.1, exact=adjoint == "exact")
    T = 6
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    a, cg, keep = _rollout(dm, s0, g, prm, T, seed_gx, kernel=kernel, adjoint=adjoint, deterministic=True)
    b, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, kernel=kernel, adjoint=adjoint, deterministic=True)
    assert _same_bits(a, b)
    # the same graph again (recorded CUDA graph replays)
    for _ in range(2):
        cg.compute_forward_pass(0, 0)
        cg.compute_backward_pass(0)
    c = {"xT": cg.get_point_cloud(T).get("x", np.float32)}
    for k, v in get_grads(cg, 0, np.float32).items():
        c["g" + k] = v
    c["gdFc"] = cg.get_grad(0, "dFc", np.float32)
    assert _same_bits(a, c)
    # and it is the same simulation as the default (float atomic) path
    d, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, kernel=kernel, adjoint=adjoint)
    assert rel_err(a["xT"], d["xT"]) < 1e-6
    for k in ("gx", "gv", "gF", "gdFc"):
        assert norm_err(a[k], d[k]) < 1e-4, k


def test_deterministic_checkpointing_recomputes_exactly(dm):
    s0, g, rng = _case(5)
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.05, exact=True)
    T = 9
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    full, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, adjoint="exact", deterministic=True)
    ck3, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, adjoint="exact", deterministic=True, checkpoint_every=3)
    assert _same_bits(full, ck3)


def test_deterministic_matches_oracle(dm, orc):
    s0, g, rng = _case(1)
    prm = O.Params(dt=1e-3, drag=0.3, smoothing=0.2, exact=True)
    T = 8
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    a, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, adjoint="exact", deterministic=True)
    xw, gw = oracle_rollout(orc, g, prm, s0, T, seed_gx)
    assert rel_err(a["xT"], xw) < 1e-6
    for k, want in (("gx", gw.x), ("gv", gw.v), ("gF", gw.F), ("gC", gw.C), ("gdFc", gw.Ft)):
        assert norm_err(a[k], want) < 2e-4, k


def test_deterministic_loss_and_optimisation(dm, orc):
    s0, g, rng = _case(2)
    tgt = np.zeros(g.n_nodes)
    orc.p2g_accumulate(g, s0.x + 0.02, s0.v, np.zeros((s0.n, 3, 3)), s0.m, tgt, np.zeros((g.n_nodes, 3)))
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.0)
    runs = []
    for _ in range(2):
        cg, keep = make_graph(dm, s0, g, prm, layers=5, target_mass=tgt, deterministic=True)
        for it in range(2):  # two Adam steps on the control of layer 0 (PointCloud.cpp:83-147)
            cg.compute_forward_pass(0, 0)
            l0 = cg.end_layer_mass_loss() if it == 0 else l0
            cg.compute_backward_pass(0)
            gn = cg.grad_norm(0)
            cg.adam_step(0, 0.5, gn, timestep=it + 1)
        cg.compute_forward_pass(0, 0)
        runs.append((l0, cg.end_layer_mass_loss(), cg.get_point_cloud(0).get("dFc", np.float32), gn))
    assert runs[0][0] == runs[1][0] and runs[0][1] == runs[1][1] and runs[0][3] == runs[1][3]
    assert runs[0][1] < runs[0][0]
    assert np.array_equal(runs[0][2].view(np.uint32), runs[1][2].view(np.uint32))
    cg, keep = make_graph(dm, s0, g, prm, layers=5, target_mass=tgt)
    cg.compute_forward_pass(0, 0)
    assert abs(cg.end_layer_mass_loss() - runs[0][0]) <= 1e-5 * abs(runs[0][0])


def test_deterministic_batch(dm):
    from test_gpu_batch import _instances, _pc, _run
    insts = _instances(seed=4, count=3)
    pcs = [_pc(dm, s, "fp32") for s, g, _ in insts]
    grids = [dm.Grid(*g.dims, g.dx, g.min) for s, g, _ in insts]
    out = []
    for det in (True, True, False):
        cg = dm.CompGraph.batch(pcs, grids, adjoint="exact", deterministic=det)
        n_total = len(cg.get_point_cloud(0))
        ranges = [cg.instance_range(i) for i in range(len(insts))]
        out.append(_run(cg, 4, [sd for _, _, sd in insts], ranges, n_total))
    (xa, ga), (xb, gb), (xc, gc) = out
    assert np.array_equal(xa, xb) and all(np.array_equal(ga[k], gb[k]) for k in ga)
    assert rel_err(xa, xc) < 1e-6
    assert all(norm_err(ga[k], gc[k]) < 1e-4 for k in ga)


def test_deterministic_overflow_is_reported(dm):
    s0, g, _ = _case(0, G=10)
    s0.v[:] = 1e9  # momentum far outside the fixed-point range: reported, not wrapped
    prm = O.Params(dt=1e-3, drag=0.0, smoothing=0.0)
    cg, keep = make_graph(dm, s0, g, prm, layers=2, deterministic=True)
    with pytest.raises(RuntimeError, match="fixed-point"):
        cg.compute_forward_pass(0, 0)
    # the flag is cleared: a sane state runs again on the same graph
    cg.get_point_cloud(0).set("v", np.zeros((s0.n, 3)))
    cg.compute_forward_pass(0, 0)


def test_deterministic_rejected_for_fp64(dm):
    s0, g, _ = _case(0, G=8)
    prm = O.Params(dt=1e-3)
    with pytest.raises(RuntimeError, match="FP32"):
        make_graph(dm, s0, g, prm, precision="fp64", deterministic=True)


def test_deterministic_launch_count(dm):
    s0, g, _ = _case(6, G=10)
    prm = O.Params(dt=1e-3)
    T = 4
    cg, keep = make_graph(dm, s0, g, prm, layers=T + 1, deterministic=True)
    lib = dm._lib.lib
    for _ in range(3):
        cg.compute_forward_pass(0, 0)
    n0 = lib.mpm_launch_count()
    cg.compute_forward_pass(0, 0)  # a replay counts what it replays
    assert lib.mpm_launch_count() - n0 == 3 * T + 1  # + the mass-scale kernel


def test_checkpoint_tail_kept_from_the_forward_pass(dm):
    """The backward pass takes the last checkpoint segment (states, grids,
    trust scales) from the forward pass instead of recomputing it, unless a
    state write came in between.  Either way the gradients are the same bits."""
    s0, g, rng = _case(7)
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.05, exact=True)
    T, k = 9, 3
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    cg, keep = make_graph(dm, s0, g, prm, precision="fp32", adjoint="exact", layers=T + 1, checkpoint_every=k,
                          deterministic=True)

    def backward():
        cg.get_point_cloud(T).set("grad_x", seed_gx)
        f0, b0 = dm.step_count()
        cg.compute_backward_pass(0)
        f1, b1 = dm.step_count()
        assert b1 - b0 == T
        return f1 - f0, {key: cg.get_grad(0, key, np.float32) for key in ("x", "v", "F", "dFc")}

    cg.compute_forward_pass(0, 0)
    fwd_kept, g_kept = backward()
    assert fwd_kept == T - k  # segments [0,3] and [3,6] recomputed, [6,9] kept
    cg.compute_forward_pass(0, 0)
    cg.get_point_cloud(0).set("v", s0.v)  # the same values: a state write all the same
    fwd_redo, g_redo = backward()
    assert fwd_redo == T
    for key in g_kept:
        assert np.array_equal(g_kept[key], g_redo[key]), key
    # two backward passes after one forward: the first keeps the tail, then
    # overwrites the scratch with segments [3,6] and [0,3]; the second recomputes
    cg.compute_forward_pass(0, 0)
    assert backward()[0] == T - k
    fwd_again, g_again = backward()
    assert fwd_again == T
    for key in g_kept:
        assert np.array_equal(g_kept[key], g_again[key]), key
