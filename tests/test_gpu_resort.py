"""The re-sort of a graph's particles by grid cell.  The reference keeps its
particles in input order; here a graph orders them by (instance, cell) at
set-up (and on request) for the scatter/gather kernels, keeps the
permutation and maps every get/set through it.  What a caller sees must not
change: the same arrays in the same order, the same results as without the
re-sort (within FP32 summation-order noise), and the same optimiser runs."""
import numpy as np
import pytest

import oracle as O
from helpers import get_grads, make_graph, norm_err, oracle_rollout, rel_err

pytestmark = pytest.mark.gpu


def _shuffled(seed=0, G=14):
    from diffmpm_bindings import workloads as W
    w = W.sphere32(seed=seed, G=G, rho=60.0)
    rng = np.random.default_rng(seed)
    n = w.n
    p = rng.permutation(n)
    s0 = O.State(w.x[p], w.v[p], 0.05 * rng.normal(size=(n, 3, 3)), np.eye(3) + 0.02 * rng.normal(size=(n, 3, 3)),
                 w.m[p], w.vol[p], w.lam[p], w.mu[p], 0.01 * rng.normal(size=(n, 3, 3)))
    return s0, O.Grid(w.dims, w.dx), rng


def _rollout(dm, s0, g, prm, T, seed_gx, resort, **kw):
    cg, keep = make_graph(dm, s0, g, prm, layers=T + 1, adjoint="exact", resort=resort, **kw)
    cg.compute_forward_pass(0, 0)
    n = s0.n
    last = cg.get_point_cloud(T)
    last.set("grad_x", seed_gx)
    last.set("grad_v", np.zeros((n, 3)))
    last.set("grad_F", np.zeros((n, 3, 3)))
    last.set("grad_C", np.zeros((n, 3, 3)))
    cg.compute_backward_pass(0)
    out = {"xT": last.get("x", np.float64)}
    out.update({"g" + k: v for k, v in get_grads(cg, 0).items()})
    out["gdFc"] = cg.get_grad(0, "dFc", np.float64)
    return out, cg, keep


@pytest.mark.parametrize("checkpoint_every", [1, 3])
def test_resort_is_invisible(dm, orc, checkpoint_every):
    s0, g, rng = _shuffled(1)
    prm = O.Params(dt=1e-3, drag=0.2, smoothing=0.1, exact=True)
    T = 6
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    a, cg, _ = _rollout(dm, s0, g, prm, T, seed_gx, True, checkpoint_every=checkpoint_every)
    b, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, False, checkpoint_every=checkpoint_every)
    assert rel_err(a["xT"], b["xT"]) < 1e-6
    for k in ("gx", "gv", "gF", "gC", "gdFc"):
        assert norm_err(a[k], b[k]) < 1e-4, k
    # the caller's arrays come back in the caller's order
    pc0 = cg.get_point_cloud(0)
    assert np.array_equal(pc0.get("x", np.float32), s0.x.astype(np.float32))
    assert np.array_equal(pc0.get("m", np.float32), s0.m.astype(np.float32))
    xw, gw = oracle_rollout(orc, g, prm, s0, T, seed_gx)
    assert rel_err(a["xT"], xw) < 1e-6
    assert norm_err(a["gdFc"], gw.Ft) < 2e-4


def test_explicit_resort_moves_every_plane(dm):
    s0, g, rng = _shuffled(2)
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.0, exact=True)
    T = 4
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    a, cg, keep = _rollout(dm, s0, g, prm, T, seed_gx, False)
    before = [{k: cg.get_point_cloud(i).get(k, np.float32) for k in ("x", "v", "C", "F", "dFc", "m", "grad_x",
                                                                     "grad_F")} for i in range(T + 1)]
    cg.resort()
    after = [{k: cg.get_point_cloud(i).get(k, np.float32) for k in before[0]} for i in range(T + 1)]
    for i in range(T + 1):
        for k in before[0]:
            assert np.array_equal(before[i][k], after[i][k]), (i, k)
    # and the graph keeps working in the new order
    cg.compute_forward_pass(0, 0)
    cg.compute_backward_pass(0)
    assert rel_err(cg.get_point_cloud(T).get("x", np.float64), a["xT"]) < 1e-6
    assert norm_err(cg.get_grad(0, "dFc", np.float64), a["gdFc"]) < 1e-4


def test_resort_batch_keeps_instances(dm):
    from test_gpu_batch import _instances, _pc, _run
    insts = _instances(seed=5, count=3)
    rng = np.random.default_rng(5)
    shuffled = []
    for s, g, sd in insts:
        p = rng.permutation(s.n)
        shuffled.append((O.State(s.x[p], s.v[p], s.C[p], s.F[p], s.m[p], s.vol[p], s.lam[p], s.mu[p],
                                 None if s.dFc is None else s.dFc[p]), g, sd[p]))
    pcs = [_pc(dm, s, "fp32") for s, g, _ in shuffled]
    grids = [dm.Grid(*g.dims, g.dx, g.min) for s, g, _ in shuffled]
    res = []
    for resort in (True, False):
        cg = dm.CompGraph.batch(pcs, grids, adjoint="exact")
        cg.set_resort(resort)
        n_total = len(cg.get_point_cloud(0))
        ranges = [cg.instance_range(i) for i in range(len(shuffled))]
        res.append(_run(cg, 4, [sd for _, _, sd in shuffled], ranges, n_total))
    (xa, ga), (xb, gb) = res
    assert rel_err(xa, xb) < 1e-6
    assert all(norm_err(ga[k], gb[k]) < 1e-4 for k in ga)
