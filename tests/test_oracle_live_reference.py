"""Random-input cross-check of the oracle against the reference compiled here
(skipped where the reference tree, and so oracle/_ref, is absent)."""
import numpy as np
import pytest

import oracle as O
from helpers import rel_err

pytestmark = pytest.mark.skipif(not O.Reference.available(64), reason="reference build (oracle/_ref) not present")


@pytest.fixture(scope="module")
def ref64():
    return O.Reference(64)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_step_pair_random(orc, ref64, seed):
    from diffmpm_bindings import workloads as W
    w = W.sphere32(seed=seed, G=12)
    rng = np.random.default_rng(seed)
    n = w.n
    s = O.State(w.x, w.v, 0.4 * rng.normal(size=(n, 3, 3)), np.eye(3) + 0.05 * rng.normal(size=(n, 3, 3)),
                w.m, w.vol, w.lam, w.mu, 0.02 * rng.normal(size=(n, 3, 3)))
    g = O.Grid(w.dims, w.dx)
    prm = O.Params(dt=1e-3, drag=0.5, smoothing=0.3, f_ext=(0.0, -9.8, 0.0))
    a, ga = orc.forward_step(g, prm, s)
    b, gb = ref64.forward_step(g, prm, s)
    for k in ("x", "v", "C", "F"):
        assert rel_err(getattr(a, k), getattr(b, k)) < 1e-9, k
    g1 = O.Grads(rng.normal(size=(n, 3)), rng.normal(size=(n, 3)), rng.normal(size=(n, 3, 3)),
                 rng.normal(size=(n, 3, 3)))
    oa = orc.backward_step(g, prm, s, a.C, ga, g1)
    ob = ref64.backward_step(g, prm, s, a.C, ga, g1)
    for k in ("x", "v", "F", "C"):
        assert rel_err(getattr(oa, k), getattr(ob, k)) < 1e-9, k


def test_inverted_and_degenerate_stress(orc, ref64):
    rng = np.random.default_rng(3)
    for i in range(300):
        F = rng.normal(size=(3, 3)) * rng.choice([0.05, 1.0, 3.0])
        dF = rng.normal(size=(3, 3))
        assert rel_err(orc.pk(F, 100.0, 50.0), ref64.pk(F, 100.0, 50.0)) < 1e-8
        assert rel_err(orc.pk_vjp(F, 100.0, 50.0, dF), ref64.hvp(F, 100.0, 50.0, dF)) < 1e-7


def test_optimizer_random_case(orc, ref64):
    """The oracle's OptimizeDefGradControlSequence against the reference's on
    another seeded case (drag, smoothing and gravity on)."""
    from diffmpm_bindings import workloads as W
    w = W.sphere32(seed=11, G=9)
    n = w.n
    rng = np.random.default_rng(11)
    s = O.State(w.x, w.v, np.zeros((n, 3, 3)), np.eye(3) + 0.02 * rng.normal(size=(n, 3, 3)), w.m, w.vol, w.lam,
                w.mu)
    g = O.Grid(w.dims, w.dx)
    tgt = np.zeros(g.n_nodes)
    orc.p2g_accumulate(g, w.x * 0.95 + 0.03, w.v, np.zeros((n, 3, 3)), w.m, tgt, np.zeros((g.n_nodes, 3)))
    prm = O.Params(dt=1e-3, drag=0.3, smoothing=0.2, f_ext=(0.0, -2.0, 0.0))
    kw = dict(num_steps=7, control_stride=3, max_gd_iters=3, max_ls_iters=3, initial_alpha=0.1, gd_tol=1e-4)
    hist, layers = orc.run_optimization(g, prm, s, tgt, **kw)
    loss, dfc, xT, _ = ref64.optimize(g, prm, s, tgt, **kw)
    assert abs(hist[-1] - loss) <= 1e-11 * loss
    for l, lay in enumerate(layers):
        assert np.abs(lay.dFc - dfc[l]).max() <= 1e-10 * max(1.0, np.abs(dfc[l]).max())
    assert rel_err(layers[-1].x, xT) < 1e-12
