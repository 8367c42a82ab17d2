"""The oracle's exact adjoint is the derivative of its forward: central
finite differences along seeded random directions (FP64, eps = 1e-4 scaled),
the same check the GPU FP64 path is held to."""
import numpy as np
import pytest

import oracle as O
from helpers import oracle_loss, oracle_rollout


def _case(seed=0, smoothing=0.0, drag=0.0, f_ext=(0.0, 0.0, 0.0)):
    from diffmpm_bindings import workloads as W
    w = W.sphere32(seed=seed, G=8, rho=60.0)
    rng = np.random.default_rng(seed)
    n = w.n
    s0 = O.State(w.x, w.v, 0.1 * rng.normal(size=(n, 3, 3)), np.eye(3) + 0.02 * rng.normal(size=(n, 3, 3)),
                 w.m, w.vol, w.lam, w.mu, 0.01 * rng.normal(size=(n, 3, 3)))
    g = O.Grid(w.dims, w.dx)
    prm = O.Params(dt=1e-3, drag=drag, smoothing=smoothing, f_ext=f_ext, exact=True)
    seed_gx = rng.normal(size=(n, 3)) / n
    return s0, g, prm, seed_gx, rng


def _fd(orc, g, prm, s0, T, seed_gx, field, d, eps):
    import copy
    sp, sm = copy.deepcopy(s0), copy.deepcopy(s0)
    setattr(sp, field, getattr(s0, field) + eps * d)
    setattr(sm, field, getattr(s0, field) - eps * d)
    return (oracle_loss(orc, g, prm, sp, T, seed_gx) - oracle_loss(orc, g, prm, sm, T, seed_gx)) / (2 * eps)


@pytest.mark.parametrize("smoothing,drag,f_ext", [(0.0, 0.0, (0, 0, 0)), (0.3, 0.5, (0.0, -9.8, 0.0))])
def test_exact_adjoint_matches_fd(orc, smoothing, drag, f_ext):
    T = 3
    s0, g, prm, seed_gx, rng = _case(1, smoothing, drag, f_ext)
    _, gr = oracle_rollout(orc, g, prm, s0, T, seed_gx)
    grads = dict(v=gr.v, x=gr.x, C=gr.C, F=gr.F, dFc=gr.Ft)
    for field, eps in (("v", 1e-4), ("dFc", 1e-5), ("F", 1e-5), ("C", 1e-4), ("x", 1e-6)):
        for k in range(3):
            d = rng.normal(size=grads[field].shape)
            fd = _fd(orc, g, prm, s0, T, seed_gx, field, d, eps)
            an = float((grads[field] * d).sum())
            assert abs(an - fd) <= 1e-5 * max(abs(fd), 1e-12) + 1e-13, (field, an, fd)


def test_reference_adjoint_differs_from_fd(orc):
    """The reference's own adjoint (BackPropagation.cpp, incl. the repeated
    (I + dt C)^T dLdF at line 140) is not the derivative of its forward."""
    T = 3
    s0, g, prm, seed_gx, rng = _case(2)
    prm_ref = O.Params(dt=prm.dt, drag=prm.drag, smoothing=prm.smoothing, exact=False)
    _, gr = oracle_rollout(orc, g, prm_ref, s0, T, seed_gx)
    d = rng.normal(size=gr.F.shape)
    fd = _fd(orc, g, prm, s0, T, seed_gx, "dFc", d, 1e-5)
    an = float((gr.F * d).sum())
    assert abs(an - fd) > 1e-3 * abs(fd)


def test_exact_adjoint_matches_fd_under_compression(orc):
    """The compressive case (tests/helpers.compressive_case): the trust region
    rescales or zeroes C, F0 includes inverted, near-singular and strongly
    compressed matrices (J clamp, FP64-guard regime).  The exact adjoint is
    still the derivative of the forward pass."""
    from helpers import compressive_case, oracle_branch_counts
    s0, g, rng, _ = compressive_case(seed=1)
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.1, exact=True)
    T = 4
    counts = oracle_branch_counts(orc, g, prm, s0, T)
    assert all(min(c.values()) > 0 for c in counts), counts
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    _, gr = oracle_rollout(orc, g, prm, s0, T, seed_gx)
    grads = dict(v=gr.v, x=gr.x, F=gr.F, dFc=gr.Ft)
    # eps 1e-6 (1e-7 for x): smaller steps lose the difference to rounding in
    # this violent case, larger ones straddle the clamps' kinks
    for field, eps in (("v", 1e-6), ("dFc", 1e-6), ("F", 1e-6), ("x", 1e-7)):
        for _ in range(3):
            d = rng.normal(size=grads[field].shape)
            fd = _fd(orc, g, prm, s0, T, seed_gx, field, d, eps)
            an = float((grads[field] * d).sum())
            assert abs(an - fd) <= 1e-5 * abs(fd), (field, an, fd)
