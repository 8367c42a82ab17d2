"""Re-sort inside a rollout.  A forward pass re-sorts the particles by grid
cell at segment starts, so each segment runs in cell order as the particles
move; the backward pass carries the gradients back across each boundary.
The reference keeps one particle order throughout, so what a caller sees
must not change: the results agree with those without the re-sort to
summation-order noise, and with the oracle.  (The fixed-point scatters sum a
cell group's contributions in FP32 before rounding them to fixed point, and
cell groups depend on the order, so they are reproducible for one order, not
across orders: with them, two re-sorting runs give the same bits.)"""
import numpy as np
import pytest

import oracle as O
from helpers import get_grads, make_graph, norm_err, oracle_rollout, rel_err

pytestmark = pytest.mark.gpu


def _spinning(seed=0, G=24, omega=30.0):
    """A sphere spinning fast enough that its particles change cells within
    a few steps, plus some strain and a random control."""
    from diffmpm_bindings import workloads as W
    w = W.sphere32(seed=seed, G=G, rho=60.0)
    rng = np.random.default_rng(seed)
    n = w.n
    c = np.array([0.5, 0.5, 0.5])
    r = w.x - c
    v = w.v + omega * np.stack([-r[:, 1], r[:, 0], 0.5 * r[:, 2] * 0.0 + 0.3 * r[:, 0]], axis=1)
    s0 = O.State(w.x, v, 0.02 * rng.normal(size=(n, 3, 3)), np.eye(3) + 0.02 * rng.normal(size=(n, 3, 3)),
                 w.m, w.vol, w.lam, w.mu, 0.01 * rng.normal(size=(n, 3, 3)))
    return s0, O.Grid(w.dims, w.dx), rng


def _run(dm, s0, g, prm, T, seed_gx, every, **kw):
    cg, keep = make_graph(dm, s0, g, prm, layers=T + 1, adjoint="exact", resort_every=every, **kw)
    cg.enable_lame_grads(True)
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
    out["glam"] = cg.get_grad(0, "lam", np.float64)
    out["gmu"] = cg.get_grad(0, "mu", np.float64)
    return out, cg, keep


KEYS = ("xT", "gx", "gv", "gF", "gC", "gdFc", "glam", "gmu")


def _close(a, b):
    assert rel_err(a["xT"], b["xT"]) < 1e-6
    for k in KEYS[1:]:
        assert norm_err(a[k], b[k]) < 1e-4, k


@pytest.mark.parametrize("checkpoint_every,every", [(3, 3), (3, 6), (1, 4)])
def test_resort_in_rollout_fixed_point(dm, checkpoint_every, every):
    s0, g, rng = _spinning(1)
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.1, exact=True)
    T = 13
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    a, cg, _ = _run(dm, s0, g, prm, T, seed_gx, every, checkpoint_every=checkpoint_every, deterministic=True)
    a2, _, _ = _run(dm, s0, g, prm, T, seed_gx, every, checkpoint_every=checkpoint_every, deterministic=True)
    b, cb, _ = _run(dm, s0, g, prm, T, seed_gx, 0, checkpoint_every=checkpoint_every, deterministic=True)
    assert cg.resort_every() == every and cb.resort_every() == 0
    for k in KEYS:
        assert np.array_equal(a[k], a2[k]), k
    _close(a, b)
    # the re-sort happened: the boundary layers hold their own permutations
    o0 = cg.particle_order(0)
    for L in range(every, T, every):
        oL = cg.particle_order(L)
        assert np.array_equal(np.sort(oL), np.arange(s0.n))
        assert not np.array_equal(oL, o0), L
    # every stored layer reads back in the caller's order, as without re-sort
    for L in range(0, T + 1, checkpoint_every):
        pa, pb = cg.get_point_cloud(L), cb.get_point_cloud(L)
        for f in ("m", "vol", "lam", "mu"):
            assert np.array_equal(pa.get(f, np.float32), pb.get(f, np.float32)), (L, f)
        for f in ("x", "v", "F", "C"):
            assert rel_err(pa.get(f, np.float64), pb.get(f, np.float64)) < 1e-5, (L, f)


@pytest.mark.parametrize("checkpoint_every", [1, 3])
def test_resort_in_rollout_float_scatters(dm, orc, checkpoint_every):
    s0, g, rng = _spinning(2)
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.1, exact=True)
    T = 10
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    a, _, _ = _run(dm, s0, g, prm, T, seed_gx, 3, checkpoint_every=checkpoint_every)
    b, _, _ = _run(dm, s0, g, prm, T, seed_gx, 0, checkpoint_every=checkpoint_every)
    assert rel_err(a["xT"], b["xT"]) < 1e-6
    for k in KEYS[1:]:
        assert norm_err(a[k], b[k]) < 1e-4, k
    xw, gw = oracle_rollout(orc, g, prm, s0, T, seed_gx)
    assert rel_err(a["xT"], xw) < 1e-6
    assert norm_err(a["gdFc"], gw.Ft) < 2e-4


def test_resort_in_rollout_optimiser_steps(dm):
    """Adam on the controls of layer 0 and of a re-sorted layer across
    passes: the moments move with the particles, so the losses and the
    control agree with those without the re-sort, and two re-sorting runs
    give the same bits (fixed-point scatters)."""
    s0, g, rng = _spinning(3)
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.1, exact=True)
    T = 9
    tgt = rng.random(tuple(g.dims)) * 1e-4

    def losses(every, off_after=None):
        cg, keep = make_graph(dm, s0, g, prm, layers=T + 1, adjoint="exact", resort_every=every,
                              checkpoint_every=3, deterministic=True, target_mass=tgt)
        out = []
        for it in range(5):
            if it == off_after:
                cg.set_resort_every(0)  # the re-sorted layers go back to layer 0's order
            cg.compute_forward_pass(0, 0)
            out.append(cg.end_layer_mass_loss())
            for ctl in (0, 3):
                cg.compute_backward_pass(ctl)
                cg.adam_step(ctl, 0.01, cg.grad_norm(ctl), timestep=it + 1)
        out.append(cg.get_point_cloud(3).get("dFc", np.float32))
        return out

    a, a2, b, c = losses(3), losses(3), losses(0), losses(3, off_after=3)
    assert a[:-1] == a2[:-1]
    assert np.array_equal(a[-1], a2[-1])
    for r in (a, c):
        for la, lb in zip(r[:-1], b[:-1]):
            assert abs(la - lb) <= 1e-4 * abs(lb)
        assert norm_err(r[-1], b[-1]) < 1e-4


@pytest.mark.parametrize("checkpoint_every", [1, 3])
def test_resort_in_rollout_fp64_matches_oracle(dm, orc, checkpoint_every):
    """FP64: the re-sort changes only the order of additions, so the rollout
    and its gradients match the oracle to double-precision noise."""
    s0, g, rng = _spinning(4)
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.1, exact=True)
    T = 9
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    a, cg, _ = _run(dm, s0, g, prm, T, seed_gx, 3, checkpoint_every=checkpoint_every, precision="fp64")
    assert not np.array_equal(cg.particle_order(3), cg.particle_order(0))
    xw, gw = oracle_rollout(orc, g, prm, s0, T, seed_gx)
    assert rel_err(a["xT"], xw) < 1e-10
    assert norm_err(a["gv"], gw.v) < 1e-9
    assert norm_err(a["gdFc"], gw.Ft) < 1e-9
