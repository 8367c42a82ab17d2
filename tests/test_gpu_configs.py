"""Full-size parity on the two CPU-runnable workloads, against the FP64 oracle.

* 17,157-particle sphere (r = 0.25, 8 per cell, 33^3 nodes, dx = 1/32),
  Neo-Hookean E = 1e4, nu = 0.3, quadratic B-spline APIC, dt = 1e-3,
  20 steps, density 60 (the nominal density 1 is beyond the explicit CFL
  limit and diverges), full tape; loss = mean |x_T - target|^2 with the
  target a smooth sinusoidal displacement (amplitude 0.05) of x_0;
  gradients w.r.t. the initial velocity and the control F.
* 153,729-particle ellipsoid (semi-axes 0.35/0.25/0.2, 8 per cell, 65^3
  nodes), fixed-corotated E = 5e4, nu = 0.35, dt = 5e-4, 100 steps,
  checkpoint every 10 steps with recomputation, density for CFL 0.45.

Both run the exact adjoint.  Bars: FP64 engine 1e-9 relative; FP32 engine
x_T within 1e-5 and gradients within 1e-4 relative (the precision targets of the FP32 form).
"""
import functools

import numpy as np
import pytest

import oracle as O
from helpers import make_graph, norm_err, oracle_rollout, rel_err

pytestmark = pytest.mark.gpu


def _device(dm, s0, g, prm, T, seed_gx, prec, checkpoint, **kw):
    cg, keep = make_graph(dm, s0, g, prm, precision=prec, adjoint="exact", layers=T + 1,
                          checkpoint_every=checkpoint, **kw)
    cg.compute_forward_pass(0, 0)
    last = cg.get_point_cloud(T)
    xT = last.get("x", np.float64)
    last.set("grad_x", seed_gx)
    cg.compute_backward_pass(0)
    return xT, {"v": cg.get_grad(0, "v", np.float64), "dFc": cg.get_grad(0, "dFc", np.float64),
                "x": cg.get_grad(0, "x", np.float64)}


def _check(prec, xT, gd, xw, gw, what):
    ex = rel_err(xT, xw)
    errs = {k: norm_err(gd[k], w) for k, w in (("v", gw.v), ("dFc", gw.Ft if gw.Ft is not None else gw.F),
                                               ("x", gw.x))}
    print(f"{what} {prec}: x_T {ex:.2e}, " + ", ".join(f"dL/d{k} {e:.2e}" for k, e in errs.items()))
    assert ex < (1e-12 if prec == "fp64" else 1e-5)
    for k, e in errs.items():
        assert e < (1e-9 if prec == "fp64" else 1e-4), (k, e)


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_sphere17k_neohookean_quadratic_20_steps(dm, orc, prec):
    from diffmpm_bindings import workloads as W
    w = W.sphere32()
    assert w.n == 17157 and w.dims == (33, 33, 33)
    n, T = w.n, w.steps
    s0 = O.State(w.x, w.v, np.zeros((n, 3, 3)), w.F, w.m, w.vol, w.lam, w.mu, np.zeros((n, 3, 3)))
    g = O.Grid(w.dims, w.dx)
    prm = O.Params(dt=w.dt, drag=0.0, smoothing=0.0, exact=True, kernel=1, material=1)
    # loss = mean |x_T - target|^2: the seed is its gradient at the oracle's x_T
    s = s0
    for _ in range(T):
        s, _ = orc.forward_step(g, prm, s)
    seed_gx = 2.0 * (s.x - w.target) / n
    xw, gw = oracle_rollout(orc, g, prm, s0, T, seed_gx)
    xT, gd = _device(dm, s0, g, prm, T, seed_gx, prec, 1, kernel="quadratic", material="neohookean")
    _check(prec, xT, gd, xw, gw, "sphere17k")


@functools.lru_cache(maxsize=1)
def _ellipsoid_case():
    """Inputs and the oracle's rollout (about 20 s of FP64 CPU work), once."""
    from diffmpm_bindings import workloads as W
    w = W.ellipsoid64()
    n = w.n
    s0 = O.State(w.x, w.v, np.zeros((n, 3, 3)), w.F, w.m, w.vol, w.lam, w.mu)
    g = O.Grid(w.dims, w.dx)
    prm = O.Params(dt=w.dt, drag=0.0, smoothing=0.0, exact=True)
    seed_gx = np.random.default_rng(1).normal(size=(n, 3)) / n
    xw, gw = O.Oracle().rollout(g, prm, s0, w.steps, seed_gx)
    return w, s0, g, prm, seed_gx, xw, gw


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_ellipsoid154k_fcr_100_steps_checkpointed(dm, prec):
    w, s0, g, prm, seed_gx, xw, gw = _ellipsoid_case()
    assert w.n == 153729 and w.dims == (65, 65, 65)
    T = w.steps
    xT, gd = _device(dm, s0, g, prm, T, seed_gx, prec, w.checkpoint)
    # no smoothing: the control gradient dL/d(F + dFc) equals the oracle's dL/dF0
    _check(prec, xT, gd, xw, gw, "ellipsoid154k")
