"""GPU parity where the FP64 guard, the J clamp and the trust region switch in.

The FP32 engine forms the fixed-corotated stress in FP32 but switches to
FP64 near inversion: an SVD polar decomposition when J <= 0.05 (|F|/sqrt 3)^3
and FP64 det F / F^{-T} when J <= 0.25.  The reference clamps J at 1e-6
(Elasticity.cpp:52), regularises its rotation-derivative solve when
det A < 1e-6 (Elasticity.cpp:57-117) and rescales C under compression with
the J trust region (ForwardSimulation.cpp:135-152, kJmin = 0.6 at :13).

* The device constitutive functions (the ones P2G and its transpose inline,
  run on given matrices through mpm_constitutive) against the reference's
  own PK_FixedCorotatedElasticity / d2_FCE_psi_dF2_mult_by_dF outputs on 32
  matrices with det F from -12.5 to 1e-3 (tests/golden/reference_small.npz),
  with the branch each matrix took.
* A compressive rollout (tests/helpers.compressive_case) that enters every
  one of those branches, against the FP64 oracle, for both adjoints and both
  engine precisions, and the FP64 engine's exact adjoint against central
  differences.

FP32 bar: 1e-4 relative (the gradient precision target) on P, the stress
derivative and the rollout gradients; FP64 engine: 1e-9.
"""
import copy
import ctypes as C

import numpy as np
import pytest

import oracle as O
from helpers import compressive_case, get_grads, make_graph, norm_err, oracle_branch_counts, oracle_rollout, rel_err

pytestmark = pytest.mark.gpu

LAM, MU = 5769.23, 3846.15  # the Lame pair the golden constitutive cases use
BR_SVD, BR_INV64, BR_JCLAMP, BR_DR_REG = 1, 2, 4, 8


def _constitutive(dm, F, G, lam, mu, precision, adjoint, material=0):
    lib = dm._lib.lib
    F = np.ascontiguousarray(F, np.float64).reshape(-1, 3, 3)
    G = np.ascontiguousarray(G, np.float64).reshape(-1, 3, 3)
    n = len(F)
    lam = np.ascontiguousarray(np.broadcast_to(lam, (n,)), np.float64)
    mu = np.ascontiguousarray(np.broadcast_to(mu, (n,)), np.float64)
    P, dP = np.zeros((n, 3, 3)), np.zeros((n, 3, 3))
    br = np.zeros(n, np.int32)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    prec = {"fp32": 0, "fp64": 1}[precision]
    adj = {"reference": 0, "exact": 1}[adjoint]
    rc = lib.mpm_constitutive(n, prec, material, adj, dp(F), dp(G), dp(lam), dp(mu), dp(P), dp(dP),
                              br.ctypes.data_as(C.POINTER(C.c_int)))
    assert rc == 0, lib.mpm_last_error()
    return P, dP, br


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_device_stress_matches_reference_golden(dm, golden, prec):
    """P and the reference's stress derivative on the reference-made cases,
    each matrix on its own (inverted and near-singular F included)."""
    F, dF = golden["cons_F"], golden["cons_dF"]
    P, H, br = _constitutive(dm, F, dF, LAM, MU, prec, "reference")
    tol = 1e-4 if prec == "fp32" else 1e-9
    eP = [norm_err(P[i], golden["cons_P64"][i]) for i in range(len(F))]
    eH = [norm_err(H[i], golden["cons_H64"][i]) for i in range(len(F))]
    print(f"{prec}: max rel err P {max(eP):.2e}, dP/dF.dF {max(eH):.2e}")
    assert max(eP) < tol and max(eH) < tol, (max(eP), max(eH))
    det = np.linalg.det(F)
    # the guard and the clamp are the branches these matrices take
    assert ((br & BR_INV64) != 0).tolist() == (det <= 0.25).tolist()
    assert ((br & BR_JCLAMP) != 0).tolist() == (det <= 1e-6).tolist()
    assert (br & BR_SVD).astype(bool).sum() >= (det <= 0).sum() > 0
    print(f"{prec}: branches SVD {int((br & BR_SVD).astype(bool).sum())}, FP64 invariants "
          f"{int((br & BR_INV64).astype(bool).sum())}, J clamp {int((br & BR_JCLAMP).astype(bool).sum())} of {len(F)}")


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_device_exact_stress_derivative_matches_oracle(dm, orc, golden, prec):
    """The exact adjoint's stress VJP (the true derivative, also in the J-clamp
    branch, where it differs from the reference's) against the oracle's."""
    F, dF = golden["cons_F"], golden["cons_dF"]
    _, H, _ = _constitutive(dm, F, dF, LAM, MU, prec, "exact")
    tol = 1e-4 if prec == "fp32" else 1e-9
    e = [norm_err(H[i], orc.pk_vjp(F[i], LAM, MU, dF[i], exact=True)) for i in range(len(F))]
    print(f"{prec}: max rel err exact dP/dF^T G {max(e):.2e}")
    assert max(e) < tol


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_device_regularised_rotation_derivative(dm, orc, prec):
    """An inverted F whose two smallest signed singular values nearly cancel
    (0.6 and -(0.6 - 1e-7)) makes the rotation-derivative matrix
    A = tr(S) I - S nearly singular: the reference adds 1e-4 to its diagonal
    (Elasticity.cpp:57-117), and so must the device.  The solve is so
    ill-conditioned that the reference's own float build lands O(1) from
    its double build here, so the FP32 engine solves it in FP64 from the
    stored (FP32) F: it is held to the oracle at those FP32-rounded inputs.
    (At an exact tie the polar factor of an inverted F is not unique, so no
    two implementations need agree; such F are not used.)"""
    rng = np.random.default_rng(3)
    Fs = []
    for _ in range(6):
        Q1, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        Q2, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        Q1 *= np.sign(np.linalg.det(Q1))
        Q2 *= np.sign(np.linalg.det(Q2))
        Fs.append(Q1 @ np.diag([1.7, 0.6, -(0.6 - 1e-7)]) @ Q2.T)
    Fs = np.asarray(Fs)
    Gs = rng.normal(size=Fs.shape)
    _, H, br = _constitutive(dm, Fs, Gs, LAM, MU, prec, "reference")
    assert (br & BR_DR_REG).all(), br
    if prec == "fp32":
        r = lambda a: np.asarray(a, np.float32).astype(np.float64)  # noqa: E731
        want = [orc.pk_vjp(r(Fs[i]), float(np.float32(LAM)), float(np.float32(MU)), r(Gs[i])) for i in range(len(Fs))]
    else:
        want = [orc.pk_vjp(Fs[i], LAM, MU, Gs[i]) for i in range(len(Fs))]
    tol = 1e-4 if prec == "fp32" else 1e-8
    e = [norm_err(H[i], want[i]) for i in range(len(Fs))]
    print(f"{prec}: regularised solve, max rel err {max(e):.2e}")
    assert max(e) < tol


def _rollout(dm, s0, g, prm, T, seed_gx, precision, adjoint):
    cg, keep = make_graph(dm, s0, g, prm, precision=precision, adjoint=adjoint, layers=T + 1)
    cg.compute_forward_pass(0, 0)
    n = s0.n
    last = cg.get_point_cloud(T)
    last.set("grad_x", seed_gx)
    for k, shp in (("grad_v", (n, 3)), ("grad_F", (n, 3, 3)), ("grad_C", (n, 3, 3))):
        last.set(k, np.zeros(shp))
    cg.compute_backward_pass(0)
    xT = last.get("x", np.float64)
    g0 = get_grads(cg, 0)
    g0["dFc"] = cg.get_grad(0, "dFc", np.float64)
    return xT, g0, cg, keep


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("adjoint", ["reference", "exact"])
def test_compressive_rollout_matches_oracle(dm, orc, prec, adjoint):
    s0, g, rng, fam = compressive_case()
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.1, exact=adjoint == "exact")
    T = 4
    counts = oracle_branch_counts(orc, g, prm, s0, T)
    # every guarded branch is entered, at the first step and later ones
    for c in counts:
        assert min(c["inv64"], c["jclamp"], c["svd"], c["rescaled"], c["zeroed"]) > 0, c
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    xT, g0, cg, keep = _rollout(dm, s0, g, prm, T, seed_gx, prec, adjoint)
    xw, gw = oracle_rollout(orc, g, prm, s0, T, seed_gx)
    # the device takes those branches on its own layer-0 state (F + dFc)
    Ft = cg.get_point_cloud(0).get("F_total", np.float64)
    _, _, br = _constitutive(dm, Ft, np.zeros_like(Ft), s0.lam, s0.mu, prec, adjoint)
    assert (br & BR_SVD).astype(bool).sum() == counts[0]["svd"]
    assert (br & BR_INV64).astype(bool).sum() == counts[0]["inv64"]
    assert (br & BR_JCLAMP).astype(bool).sum() == counts[0]["jclamp"]
    ex = rel_err(xT, xw)
    errs = {k: norm_err(g0[k], w) for k, w in (("x", gw.x), ("v", gw.v), ("F", gw.F), ("C", gw.C),
                                               ("dFc", gw.Ft))}
    print(f"{prec} {adjoint}: x_T {ex:.2e}, " + ", ".join(f"g{k} {e:.2e}" for k, e in errs.items()) +
          f"; branches per step {counts}")
    assert ex < (1e-12 if prec == "fp64" else 1e-5)
    tol = 1e-9 if prec == "fp64" else 2e-5  # FP32 measured <= 1.1e-6 through every guard branch
    for k, e in errs.items():
        assert e < tol, (k, e)


def test_compressive_fp64_exact_adjoint_matches_finite_differences(dm):
    """The FP64 engine's exact adjoint through the trust-region rescale, the
    FP64 guard and the J clamp, against central differences of its own
    forward pass along seeded directions."""
    s0, g, rng, _ = compressive_case(seed=1)
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.1, exact=True)
    T = 4
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    _, g0, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, "fp64", "exact")

    def loss(s):
        cg, keep = make_graph(dm, s, g, prm, precision="fp64", adjoint="exact", layers=T + 1)
        cg.compute_forward_pass(0, 0)
        return float((cg.get_point_cloud(T).get("x", np.float64) * seed_gx).sum())

    # eps 1e-6 (1e-7 for x): smaller steps lose the difference to rounding in
    # this violent case, larger ones straddle the clamps' kinks
    for field, gkey, eps in (("v", "v", 1e-6), ("dFc", "dFc", 1e-6), ("F", "F", 1e-6), ("x", "x", 1e-7)):
        for _ in range(3):
            d = rng.normal(size=getattr(s0, field).shape)
            sp, sm = copy.deepcopy(s0), copy.deepcopy(s0)
            setattr(sp, field, getattr(s0, field) + eps * d)
            setattr(sm, field, getattr(s0, field) - eps * d)
            fd = (loss(sp) - loss(sm)) / (2 * eps)
            an = float((g0[gkey] * d).sum())
            print(f"{field}: adjoint {an:.9e} fd {fd:.9e} rel {abs(an - fd) / abs(fd):.1e}")
            assert abs(an - fd) <= 1e-5 * abs(fd), (field, an, fd)
