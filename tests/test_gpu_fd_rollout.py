"""Gradients of a long checkpointed rollout against central finite
differences of the FP64 oracle (a down-scaled twin of the 2M-particle
rollout: a union of 8 seeded spheres, 40 steps, checkpoint every 20
steps with recomputation, exact adjoint).

The gradient with respect to the layer-0 control dFc, the initial velocity
v0 and the scalar Young's modulus E comes from the device autograd rollout
(``mpm_rollout``).  It is checked two ways:
* against the oracle's own FP64 exact adjoint of the same rollout, as whole
  gradients: FP64 engine 1e-10, FP32 engine 1e-4 relative;
* against central differences (L(p + eps d) - L(p - eps d)) / (2 eps) of the
  same loss from the oracle's FP64 forward, along 16 seeded random unit
  directions d in (dFc, v0, E / E0) jointly, eps = 1e-4.  Random unit
  directions in 72k dimensions see ~0.5% of the gradient, so the error is
  measured against |grad|: |dL.d - FD| <= tol |grad|, with tol 1e-6 for the
  oracle and the FP64 engine and 1e-4 for the FP32 engine (FP64-guarded
  stress), the gradient-error target.  At eps = 1e-4 a few directions
  straddle the ~1e-12 steps an iterative polar decomposition takes where its
  iteration count changes (the FD error there scales as 1/eps and is gone at
  eps = 1e-5); the median over directions is also checked relative to the
  directional derivative itself."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

T, EPS, NDIR = 40, 1e-4, 16


@pytest.fixture(scope="module")
def twin():
    from diffmpm_bindings import workloads as W
    w = W.spheres2m(seed=3, n=6000, G=32, steps=T, checkpoint=20)
    rng = np.random.default_rng(33)
    tgt = w.x + 0.02 * np.sin(2 * np.pi * w.x[:, [1, 2, 0]] + rng.random(3))
    dfc = 0.01 * rng.normal(size=(w.n, 3, 3))
    dirs = []
    for _ in range(NDIR):
        d_fc, d_v, d_e = rng.normal(size=(w.n, 3, 3)), rng.normal(size=(w.n, 3)), float(rng.normal())
        nrm = np.sqrt((d_fc ** 2).sum() + (d_v ** 2).sum() + d_e ** 2)
        dirs.append((d_fc / nrm, d_v / nrm, d_e / nrm * w.extra["E"]))
    return w, tgt, dfc, dirs


@pytest.fixture(scope="module")
def adjoint(orc, twin):
    """The oracle's exact adjoint of the rollout: dL/d dFc, dL/dv0, dL/dE."""
    w, tgt, dfc, _ = twin
    n = w.n
    nu = w.extra["nu"]
    lam, mu = orc.lame(w.extra["E"], nu)
    g = O.Grid(w.dims, w.dx)
    prm = O.Params(dt=w.dt, drag=w.drag, smoothing=w.smoothing, exact=True)
    states = [O.State(w.x, w.v, np.zeros((n, 3, 3)), w.F, w.m, w.vol, np.full(n, lam), np.full(n, mu), dfc)]
    steps = []
    for _ in range(T):
        s1, st = orc.forward_step(g, prm, states[-1])
        states.append(s1)
        steps.append(st)
    gg = O.Grads(2 * (states[-1].x - tgt) / (3 * n), np.zeros((n, 3)), np.zeros((n, 3, 3)), np.zeros((n, 3, 3)))
    glam, gmu = np.zeros(n), np.zeros(n)
    for t in range(T - 1, -1, -1):
        gg = orc.backward_step(g, prm, states[t], states[t + 1].C, steps[t], gg, want_ft=(t == 0), want_lame=True)
        glam += gg.lam
        gmu += gg.mu
    gE = glam.sum() * nu / ((1 + nu) * (1 - 2 * nu)) + gmu.sum() / (2 + 2 * nu)
    return gg.Ft, gg.v, gE


def _oracle_loss(orc, w, tgt, dfc, v0, E):
    lam, mu = orc.lame(E, w.extra["nu"])
    n = w.n
    s = O.State(w.x, v0, np.zeros((n, 3, 3)), w.F, w.m, w.vol, np.full(n, lam), np.full(n, mu), dfc)
    g = O.Grid(w.dims, w.dx)
    prm = O.Params(dt=w.dt, drag=w.drag, smoothing=w.smoothing, exact=True)
    for _ in range(T):
        s, _ = orc.forward_step(g, prm, s)
    return float(((s.x - tgt) ** 2).mean())


@pytest.fixture(scope="module")
def fd(orc, twin):
    w, tgt, dfc, dirs = twin
    E = w.extra["E"]
    out = []
    for d_fc, d_v, d_E in dirs:
        lp = _oracle_loss(orc, w, tgt, dfc + EPS * d_fc, w.v + EPS * d_v, E + EPS * d_E)
        lm = _oracle_loss(orc, w, tgt, dfc - EPS * d_fc, w.v - EPS * d_v, E - EPS * d_E)
        out.append((lp - lm) / (2 * EPS))
    return np.array(out)


def _gnorm(w, g_fc, g_v, g_E):
    return float(np.sqrt((g_fc ** 2).sum() + (g_v ** 2).sum() + (g_E * w.extra["E"]) ** 2))


def test_oracle_adjoint_matches_finite_differences(twin, fd, adjoint):
    w, _, _, dirs = twin
    g_fc, g_v, g_E = adjoint
    an = np.array([(g_fc * d_fc).sum() + (g_v * d_v).sum() + g_E * d_E for d_fc, d_v, d_E in dirs])
    assert np.abs(an - fd).max() <= 1e-6 * _gnorm(w, g_fc, g_v, g_E)
    assert np.median(np.abs(an - fd) / np.abs(fd)) <= 1e-7


@pytest.mark.parametrize("precision,tol,tol_adj", [("fp64", 1e-6, 1e-10), ("fp32", 1e-4, 1e-4)])
def test_rollout_gradient_matches_finite_differences(twin, fd, adjoint, precision, tol, tol_adj):
    torch = pytest.importorskip("torch")
    from diffmpm_bindings.rollout import Rollout, mpm_rollout
    w, tgt, dfc, dirs = twin
    dev = torch.device("cuda")
    dt = torch.float64 if precision == "fp64" else torch.float32
    sim = Rollout(w.n, w.dims, w.dx, steps=T, m=w.m[0], vol=w.vol[0], nu=w.extra["nu"], dt=w.dt,
                  precision=precision, checkpoint_every=20)
    x0 = torch.tensor(w.x, dtype=dt, device=dev)
    v0 = torch.tensor(w.v, dtype=dt, device=dev, requires_grad=True)
    F0 = torch.tensor(w.F, dtype=dt, device=dev)
    c0 = torch.tensor(dfc, dtype=dt, device=dev, requires_grad=True)
    E = torch.tensor(w.extra["E"], dtype=torch.float64, device=dev, requires_grad=True)
    xT, _ = mpm_rollout(x0, v0, F0, c0, E, sim)
    loss = ((xT.double() - torch.tensor(tgt, device=dev)) ** 2).mean()
    loss.backward()
    g_fc, g_v, g_E = c0.grad.double().cpu().numpy(), v0.grad.double().cpu().numpy(), float(E.grad)
    o_fc, o_v, o_E = adjoint
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
    assert rel(g_fc, o_fc) <= tol_adj and rel(g_v, o_v) <= tol_adj and abs(g_E - o_E) <= tol_adj * abs(o_E)
    an = np.array([(g_fc * d_fc).sum() + (g_v * d_v).sum() + g_E * d_E for d_fc, d_v, d_E in dirs])
    err = np.abs(an - fd) / _gnorm(w, o_fc, o_v, o_E)
    print(f"{precision}: |dL.d - FD| / |grad| max {err.max():.2e} over {NDIR} directions; "
          f"gradient vs oracle adjoint {rel(g_fc, o_fc):.2e} (dFc) {rel(g_v, o_v):.2e} (v0) "
          f"{abs(g_E - o_E) / abs(o_E):.2e} (E)")
    assert err.max() <= tol, err


def test_compgraph_gradient_accessors_match_oracle_adjoint(dm, twin, adjoint):
    """get_grad_v0 / get_grad_F / get_grad_E of a CompGraph backward pass
    (FP64, checkpoint every 20, Lame gradients on) against the oracle's FP64
    exact adjoint of the same rollout and loss."""
    w, tgt, dfc, _ = twin
    n = w.n
    E, nu = w.extra["E"], w.extra["nu"]
    lam, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 + 2 * nu)  # in double, as the oracle
    pc = dm.PointCloud.from_arrays(w.x, v=w.v, F=w.F, dFc=dfc, m=w.m, vol=w.vol, lam=np.full(n, lam),
                                   mu=np.full(n, mu), precision="fp64")
    grid = dm.Grid(*w.dims, w.dx, (0.0, 0.0, 0.0), precision="fp64")
    cg = dm.CompGraph(pc, grid, grid, adjoint="exact", checkpoint_every=20)
    cg.set_sim_params(dt=w.dt, drag=w.drag, smoothing=w.smoothing)
    cg.enable_lame_grads(True)
    cg.set_up_comp_graph(T + 1)
    cg.compute_forward_pass(0, 0)
    last = cg.get_point_cloud(T)
    last.set("grad_x", 2.0 * (last.get("x", np.float64) - tgt) / (3 * n))  # d mean((x_T - tgt)^2) / dx_T
    cg.compute_backward_pass(0)
    o_fc, o_v, o_E = adjoint
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
    assert rel(cg.get_grad_F(0, np.float64), o_fc) <= 1e-10
    assert rel(cg.get_grad_v0(np.float64), o_v) <= 1e-10
    assert abs(cg.get_grad_E(w.extra["E"]) - o_E) <= 1e-10 * abs(o_E)
