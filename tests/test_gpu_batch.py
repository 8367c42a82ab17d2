"""Batched instances: independent simulations of
uneven particle count, grid size and material advanced in one launch per
kernel must give each instance the result it gets alone."""
import numpy as np
import pytest

import oracle as O
from helpers import norm_err, oracle_rollout, rel_err

pytestmark = pytest.mark.gpu


def _instances(seed=0, count=4):
    from diffmpm_bindings import workloads as W
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        G = int(rng.integers(8, 17))
        w = W.sphere32(seed=seed + i, G=G, rho=float(rng.uniform(40, 120)), radius=float(rng.uniform(0.15, 0.3)))
        n = w.n
        E = float(np.exp(rng.uniform(np.log(5e3), np.log(5e4))))
        lam, mu = W.lame(E, float(rng.uniform(0.2, 0.4)))
        s = O.State(w.x, w.v, 0.05 * rng.normal(size=(n, 3, 3)), np.eye(3) + 0.02 * rng.normal(size=(n, 3, 3)),
                    w.m, w.vol, np.full(n, lam), np.full(n, mu), 0.01 * rng.normal(size=(n, 3, 3)) if i % 2 else None)
        out.append((s, O.Grid(w.dims, w.dx, (0.0, 0.0, 0.0)), rng.normal(size=(n, 3)) / n))
    return out


def _pc(dm, s, prec):
    dt = np.float64 if prec == "fp64" else np.float32
    return dm.PointCloud.from_arrays(s.x.astype(dt), v=s.v.astype(dt), F=s.F.astype(dt), C_=s.C.astype(dt),
                                     dFc=None if s.dFc is None else s.dFc.astype(dt), m=s.m.astype(dt),
                                     vol=s.vol.astype(dt), lam=s.lam.astype(dt), mu=s.mu.astype(dt), precision=prec)


def _run(cg, T, seeds, ranges, n_total):
    cg.set_sim_params(dt=1e-3, drag=0.2, smoothing=0.1)
    cg.set_up_comp_graph(T + 1)
    cg.compute_forward_pass(0, 0)
    last = cg.get_point_cloud(T)
    gx = np.zeros((n_total, 3))
    for sd, r in zip(seeds, ranges):
        gx[r] = sd
    last.set("grad_x", gx)
    last.set("grad_v", np.zeros((n_total, 3)))
    last.set("grad_F", np.zeros((n_total, 3, 3)))
    last.set("grad_C", np.zeros((n_total, 3, 3)))
    cg.compute_backward_pass(0)
    xT = last.get("x", np.float64)
    g0 = {k: cg.get_point_cloud(0).get("grad_" + k, np.float64) for k in ("x", "v", "F", "dFc")}
    return xT, g0


@pytest.mark.parametrize("prec,checkpoint", [("fp32", 1), ("fp64", 1), ("fp32", 3)])
def test_batch_matches_single_instances(dm, prec, checkpoint):
    insts = _instances()
    T = 5
    pcs = [_pc(dm, s, prec) for s, g, _ in insts]
    grids = [dm.Grid(*g.dims, g.dx, g.min, precision=prec) for s, g, _ in insts]
    cg = dm.CompGraph.batch(pcs, grids, adjoint="exact", checkpoint_every=checkpoint)
    n_total = len(cg.get_point_cloud(0))
    ranges = [cg.instance_range(i) for i in range(len(insts))]
    assert all(o % 256 == 0 for o in cg.offsets)
    xT, g0 = _run(cg, T, [sd for _, _, sd in insts], ranges, n_total)
    tol_x = 1e-12 if prec == "fp64" else 1e-6
    tol_g = 1e-10 if prec == "fp64" else 1e-4
    for i, ((s, g, sd), r) in enumerate(zip(insts, ranges)):
        one = dm.CompGraph(pcs[i], grids[i], grids[i], adjoint="exact", checkpoint_every=checkpoint)
        xs, gs = _run(one, T, [sd], [slice(0, s.n)], s.n)
        assert rel_err(xT[r], xs) < tol_x, i
        for k in ("x", "v", "F", "dFc"):
            assert norm_err(g0[k][r], gs[k]) < tol_g, (i, k)


def test_batch_instance_matches_oracle(dm, orc):
    insts = _instances(seed=3, count=3)
    T = 4
    pcs = [_pc(dm, s, "fp64") for s, g, _ in insts]
    grids = [dm.Grid(*g.dims, g.dx, g.min, precision="fp64") for s, g, _ in insts]
    cg = dm.CompGraph.batch(pcs, grids, adjoint="exact")
    n_total = len(cg.get_point_cloud(0))
    ranges = [cg.instance_range(i) for i in range(len(insts))]
    xT, g0 = _run(cg, T, [sd for _, _, sd in insts], ranges, n_total)
    prm = O.Params(dt=1e-3, drag=0.2, smoothing=0.1, exact=True)
    for (s, g, sd), r in zip(insts, ranges):
        xw, gw = oracle_rollout(orc, g, prm, s, T, sd)
        assert rel_err(xT[r], xw) < 1e-10
        assert norm_err(g0["v"][r], gw.v) < 1e-9
        assert norm_err(g0["dFc"][r], gw.Ft) < 1e-9


def test_batch_rejects_mass_loss(dm):
    insts = _instances(count=2)
    pcs = [_pc(dm, s, "fp32") for s, g, _ in insts]
    grids = [dm.Grid(*g.dims, g.dx, g.min) for s, g, _ in insts]
    cg = dm.CompGraph.batch(pcs, grids)
    with pytest.raises(RuntimeError, match="single-instance"):
        cg.end_layer_mass_loss()


def test_batch_padding_rows_stay_zero(dm):
    """The rows between instances (each instance starts at a multiple of 256)
    are no particles: their gradients read back as zero, however the device
    memory behind them was used before."""
    insts = _instances(seed=4, count=3)
    pcs = [_pc(dm, s, "fp32") for s, g, _ in insts]
    grids = [dm.Grid(*g.dims, g.dx, g.min) for s, g, _ in insts]
    for det in (False, True):
        cg = dm.CompGraph.batch(pcs, grids, adjoint="exact", deterministic=det)
        n_total = len(cg.get_point_cloud(0))
        ranges = [cg.instance_range(i) for i in range(len(insts))]
        _, g0 = _run(cg, 4, [sd for _, _, sd in insts], ranges, n_total)
        pad = np.ones(n_total, bool)
        for r in ranges:
            pad[r] = False
        assert pad.any()
        for k, g in g0.items():
            assert not np.any(g[pad]), k


@pytest.mark.parametrize("checkpoint", [1, 2])
def test_batch_resort_in_rollout_matches_oracle(dm, orc, checkpoint):
    """Re-sort inside the rollout with instances: each instance's particles
    stay in its own slot range (padding last) and every instance still gets
    its own result (FP64, so the re-sort changes only summation order)."""
    insts = _instances(seed=5, count=3)
    T = 6
    pcs = [_pc(dm, s, "fp64") for s, g, _ in insts]
    grids = [dm.Grid(*g.dims, g.dx, g.min, precision="fp64") for s, g, _ in insts]
    cg = dm.CompGraph.batch(pcs, grids, adjoint="exact", checkpoint_every=checkpoint)
    cg.set_resort_every(2)
    n_total = len(cg.get_point_cloud(0))
    ranges = [cg.instance_range(i) for i in range(len(insts))]
    xT, g0 = _run(cg, T, [sd for _, _, sd in insts], ranges, n_total)
    assert cg.resort_every() == 2
    o2 = cg.particle_order(2)
    for r in ranges:  # each instance's slots hold that instance's particles
        assert np.array_equal(np.sort(o2[r]), np.arange(r.start, r.stop))
    prm = O.Params(dt=1e-3, drag=0.2, smoothing=0.1, exact=True)
    for (s, g, sd), r in zip(insts, ranges):
        xw, gw = oracle_rollout(orc, g, prm, s, T, sd)
        assert rel_err(xT[r], xw) < 1e-10
        assert norm_err(g0["v"][r], gw.v) < 1e-9
        assert norm_err(g0["dFc"][r], gw.Ft) < 1e-9
