"""Shared helpers for the parity tests (test infrastructure)."""
from __future__ import annotations

import numpy as np


def rel_err(a, b):
    """max |a - b| / max |b| (0 when both vanish)."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / den) if den > 0 else float(np.abs(a).max())


def norm_err(a, b):
    """||a - b|| / ||b||."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a))


def golden_state(gd):
    import oracle as O
    return O.State(gd["x"], gd["v"], gd["C"], gd["F"], gd["m"], gd["vol"], gd["lam"], gd["mu"], gd["dFc"])


def golden_grid(gd):
    import oracle as O
    return O.Grid(tuple(int(d) for d in gd["dims"]), float(gd["dx"]), tuple(gd["gmin"]))


def golden_params(gd, exact=False):
    import oracle as O
    return O.Params(dt=float(gd["dt"]), drag=float(gd["drag"]), smoothing=float(gd["smoothing"]), exact=exact)


def make_graph(dm, s, grid, prm, precision="fp32", adjoint="reference", layers=2, checkpoint_every=1,
               kernel="cubic", material="fcr", target_mass=None, deterministic=False, resort=True,
               resort_every=None):
    """CompGraph on the GPU holding state s in layer 0 (oracle.State)."""
    dtype = np.float64 if precision == "fp64" else np.float32
    pc = dm.PointCloud.from_arrays(s.x.astype(dtype), v=s.v.astype(dtype), F=s.F.astype(dtype),
                                   dFc=None if s.dFc is None else s.dFc.astype(dtype), C_=s.C.astype(dtype),
                                   m=s.m.astype(dtype), vol=s.vol.astype(dtype), lam=s.lam.astype(dtype),
                                   mu=s.mu.astype(dtype), precision=precision)
    g = dm.Grid(*grid.dims, grid.dx, grid.min, precision=precision)
    tg = dm.Grid(*grid.dims, grid.dx, grid.min, precision=precision)
    if target_mass is not None:
        tg.set_node_masses(target_mass)
    cg = dm.CompGraph(pc, g, tg, adjoint=adjoint, kernel=kernel, material=material,
                      checkpoint_every=checkpoint_every, deterministic=deterministic)
    cg.set_sim_params(dt=prm.dt, drag=prm.drag, smoothing=prm.smoothing, f_ext=prm.f_ext,
                      bulk_viscosity=prm.bulk_visc, j_min=prm.j_min)
    cg.set_resort(resort)
    if resort_every is not None:
        cg.set_resort_every(resort_every)
    cg.set_up_comp_graph(layers)
    return cg, (pc, g, tg)


def layer_state(cg, i, dtype=np.float64):
    pc = cg.get_point_cloud(i)
    return {k: pc.get(k, dtype) for k in ("x", "v", "C", "F")}


def set_grads(cg, layer, g1):
    pc = cg.get_point_cloud(layer)
    pc.set("grad_x", g1.x)
    pc.set("grad_v", g1.v)
    pc.set("grad_F", g1.F)
    pc.set("grad_C", g1.C)


def get_grads(cg, layer, dtype=np.float64):
    pc = cg.get_point_cloud(layer)
    return {k: pc.get("grad_" + k, dtype) for k in ("x", "v", "F", "C")}


def oracle_rollout(orc, grid, prm, s0, T, seed_gx, want_ctl=True):
    """Forward T steps and the adjoint with the oracle; returns (x_T, layer-0
    grads incl. the control gradient)."""
    import oracle as O
    states, steps = [s0], []
    s = s0
    for _ in range(T):
        s1, st = orc.forward_step(grid, prm, s)
        states.append(s1)
        steps.append(st)
        s = s1
    n = s0.n
    g = O.Grads(np.asarray(seed_gx, np.float64).reshape(n, 3).copy(), np.zeros((n, 3)), np.zeros((n, 3, 3)),
                np.zeros((n, 3, 3)))
    for t in range(T - 1, -1, -1):
        g = orc.backward_step(grid, prm, states[t], states[t + 1].C, steps[t], g, want_ft=want_ctl and t == 0)
    return states[-1].x, g


def oracle_loss(orc, grid, prm, s0, T, seed_gx):
    s = s0
    for _ in range(T):
        s, _ = orc.forward_step(grid, prm, s)
    return float((np.asarray(seed_gx).reshape(-1, 3) * s.x).sum())


def golden_opt_case(go):
    """State, grid, target and optimiser arguments of reference_optimize.npz."""
    import oracle as O
    n = len(go["m"])
    s = O.State(go["x"], go["v"], np.zeros((n, 3, 3)), np.tile(np.eye(3), (n, 1, 1)), go["m"], go["vol"],
                go["lam"], go["mu"])
    g = O.Grid(tuple(int(d) for d in go["dims"]), float(go["dx"]))
    prm = O.Params(dt=float(go["dt"]), drag=float(go["drag"]), smoothing=float(go["smoothing"]))
    kw = {k: (float(go[k]) if k in ("initial_alpha", "gd_tol") else int(go[k]))
          for k in ("num_steps", "control_stride", "max_gd_iters", "max_ls_iters", "initial_alpha", "gd_tol")}
    return s, g, go["target"], prm, kw


def compressive_case(seed=0, G=16, k=150.0):
    """A rollout start in the regime where the guarded and clamped branches
    switch in.  Particles of a sphere (rho 60) move with v = -k (x - c), so
    the first G2P gives tr C ~ -3k (-450: det(I + dt C) ~ 0.61 at dt 1e-3,
    which trips the J trust region, ForwardSimulation.cpp:135-152).  F0
    comes in four families: near identity; uniformly compressed (J ~ 0.17:
    FP64 invariants, and J0 < kJmin makes the trust scale 0); near-singular
    anisotropic (F ~ diag(1.6, 1, 0.01): the FP64 SVD polar decomposition);
    inverted (F ~ diag(1, 1, -0.2): J clamped at 1e-6, Elasticity.cpp:52).
    Returns (state, grid, rng, family index per particle)."""
    import oracle as O
    from diffmpm_bindings import workloads as W
    w = W.sphere32(seed=seed, G=G, rho=60.0)
    rng = np.random.default_rng(seed)
    n = w.n
    v = -k * (w.x - np.array([0.5, 0.5, 0.5]))
    F = np.tile(np.eye(3), (n, 1, 1)) + 0.02 * rng.normal(size=(n, 3, 3))
    fam = rng.integers(0, 4, size=n)
    F[fam == 1] = 0.55 * np.eye(3) + 0.01 * rng.normal(size=((fam == 1).sum(), 3, 3))
    F[fam == 2] = np.diag([1.6, 1.0, 0.01]) + 0.005 * rng.normal(size=((fam == 2).sum(), 3, 3))
    F[fam == 3] = np.diag([1.0, 1.0, -0.2]) + 0.01 * rng.normal(size=((fam == 3).sum(), 3, 3))
    s0 = O.State(w.x, v, np.zeros((n, 3, 3)), F, w.m, w.vol, w.lam, w.mu, 0.01 * rng.normal(size=(n, 3, 3)))
    return s0, O.Grid(w.dims, w.dx), rng, fam


def oracle_branch_counts(orc, grid, prm, s0, T):
    """Per forward step of the oracle rollout: particles whose F + dFc takes
    the FP64 invariants (J <= 0.25), the J clamp (J <= 1e-6), the FP64 SVD
    guard (J <= 0.05 (|F|/sqrt 3)^3), and whose C was rescaled by the trust
    region (0 < s < 1) or zeroed by it (s <= 0)."""
    out = []
    s = s0
    for _ in range(T):
        Ft = s.F + (s.dFc if s.dFc is not None else 0.0)
        J = np.linalg.det(Ft)
        nrm = np.sqrt((Ft ** 2).sum(axis=(1, 2)))
        s1, st = orc.forward_step(grid, prm, s)
        tr = st["trust"]
        out.append(dict(inv64=int((J <= 0.25).sum()), jclamp=int((J <= 1e-6).sum()),
                        svd=int((J <= 0.05 * (nrm / np.sqrt(3)) ** 3).sum()),
                        rescaled=int(((tr > 0) & (tr < 1)).sum()), zeroed=int((tr <= 0).sum())))
        s = s1
    return out
