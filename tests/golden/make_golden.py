"""Generate golden vectors from the reference's own DiffMPMLib3D sources.

Runs where the reference tree is mounted: it builds oracle/_ref/libref{32,64}.so
(oracle/build_oracle.py) and records, for small seeded inputs, the outputs of
the reference's ForwardTimeStep, Back_Timestep, EndLayerMassLoss,
Descend_Adam, CalculatePointCloudVolumes, PK_FixedCorotatedElasticity and
d2_FCE_psi_dF2_mult_by_dF, plus a 5-step full-tape forward/backward through
CompGraph (reference_small.npz), and a run of the control-sequence
optimiser OptimizeDefGradControlSequence (reference_optimize.npz), the
mesh -> lattice sampler GeneratePointCloudFromWatertightTriangleMesh on two
procedural meshes (reference_mesh_sampling.npz), and run.py's E2E sequence of
OptimizeSingleTimestep calls with render gradients (reference_single.npz).  The
fixtures travel with the repository; the GPU tests compare against them
without the reference present.

Usage: REF_DIR=<reference checkout> python tests/golden/make_golden.py [--only small|optimize|mesh|single]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "shape-morphing-binder_gb300"))

import build_oracle  # noqa: E402
import oracle as O  # noqa: E402
from diffmpm_bindings import workloads as W  # noqa: E402

OUT = Path(__file__).resolve().parent


def small_state(seed=7, G=10, rng_scale=1.0):
    w = W.sphere32(seed=seed, G=G)
    rng = np.random.default_rng(seed + 100)
    n = w.n
    C0 = 0.5 * rng.normal(size=(n, 3, 3)) * rng_scale
    F0 = np.eye(3) + 0.04 * rng.normal(size=(n, 3, 3))
    dFc = 0.01 * rng.normal(size=(n, 3, 3))
    s = O.State(w.x, w.v, C0, F0, w.m, w.vol, w.lam, w.mu, dFc)
    return w, s, rng


def uv_ellipsoid(c=(0.5, 0.5, 0.5), axes=(0.3, 0.22, 0.18), nu=48, nv=24):
    """Closed triangle mesh of an ellipsoid (poles + rings), outward facing."""
    c, a = np.asarray(c), np.asarray(axes)
    V = [c + a * [0, 0, 1]]
    for i in range(1, nv):
        th = np.pi * i / nv
        for j in range(nu):
            ph = 2 * np.pi * j / nu
            V.append(c + a * [np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)])
    V.append(c + a * [0, 0, -1])
    F = []
    ring = lambda i, j: 1 + (i - 1) * nu + (j % nu)  # noqa: E731
    for j in range(nu):
        F.append([0, ring(1, j), ring(1, j + 1)])
    for i in range(1, nv - 1):
        for j in range(nu):
            F.append([ring(i, j), ring(i + 1, j), ring(i + 1, j + 1)])
            F.append([ring(i, j), ring(i + 1, j + 1), ring(i, j + 1)])
    last = len(V) - 1
    for j in range(nu):
        F.append([last, ring(nv - 1, j + 1), ring(nv - 1, j)])
    return np.asarray(V, np.float32), np.asarray(F, np.int32)


def torus(c=(0.5, 0.5, 0.5), R=0.25, r=0.1, nu=48, nv=24):
    """Closed triangle mesh of a torus around z (non-convex)."""
    c = np.asarray(c)
    V = []
    for i in range(nu):
        u = 2 * np.pi * i / nu
        for j in range(nv):
            v = 2 * np.pi * j / nv
            V.append(c + [(R + r * np.cos(v)) * np.cos(u), (R + r * np.cos(v)) * np.sin(u), r * np.sin(v)])
    idx = lambda i, j: (i % nu) * nv + (j % nv)  # noqa: E731
    F = []
    for i in range(nu):
        for j in range(nv):
            F.append([idx(i, j), idx(i + 1, j), idx(i + 1, j + 1)])
            F.append([idx(i, j), idx(i + 1, j + 1), idx(i, j + 1)])
    return np.asarray(V, np.float32), np.asarray(F, np.int32)


def make_mesh_sampling():
    """The reference's mesh -> lattice sampler on two procedural meshes."""
    r32 = O.Reference(32)
    rec = {}
    for name, (V, F), dx in (("ellipsoid", uv_ellipsoid(), 1.0 / 48), ("torus", torus(), 1.0 / 64)):
        pts = r32.sample_mesh(V, F, dx)
        rec[f"{name}_V"], rec[f"{name}_F"], rec[f"{name}_dx"], rec[f"{name}_points"] = V, F, dx, pts
        print(name, "triangles", len(F), "points kept", len(pts))
    np.savez_compressed(OUT / "reference_mesh_sampling.npz", **rec)
    print("wrote", OUT / "reference_mesh_sampling.npz")


OPT_CASE = dict(num_steps=6, control_stride=2, max_gd_iters=2, max_ls_iters=4, initial_alpha=0.05, gd_tol=1e-4)


def optimize_case():
    """Inputs of the optimiser fixture: 524 particles at rest-state F = I,
    C = 0; target masses from the particles shifted by (0.04, 0, 0.02)."""
    w = W.sphere32(seed=7, G=10)
    n = w.n
    s = O.State(w.x, w.v, np.zeros((n, 3, 3)), np.tile(np.eye(3), (n, 1, 1)), w.m, w.vol, w.lam, w.mu)
    g = O.Grid(w.dims, w.dx)
    tgt = np.zeros(g.n_nodes)
    O.Oracle().p2g_accumulate(g, w.x + np.array([0.04, 0.0, 0.02]), w.v, np.zeros((n, 3, 3)), w.m, tgt,
                              np.zeros((g.n_nodes, 3)))
    prm = O.Params(dt=1e-3, drag=0.5, smoothing=0.1)
    return w, s, g, tgt, prm


def make_optimize():
    r64, r32 = O.Reference(64), O.Reference(32)
    w, s, g, tgt, prm = optimize_case()
    rec = dict(dims=np.asarray(w.dims), dx=w.dx, dt=prm.dt, drag=prm.drag, smoothing=prm.smoothing, target=tgt,
               x=s.x, v=s.v, m=s.m, vol=s.vol, lam=s.lam, mu=s.mu, **{k: v for k, v in OPT_CASE.items()})
    for bits, ref in ((64, r64), (32, r32)):
        loss, dfc, xT, log = ref.optimize(g, prm, s, tgt, **OPT_CASE)
        rec[f"opt{bits}_loss"] = loss
        rec[f"opt{bits}_dFc"] = dfc
        rec[f"opt{bits}_xT"] = xT
        rec[f"opt{bits}_initial_loss"] = float(log.split("Initial loss = ")[1].split()[0])
    np.savez_compressed(OUT / "reference_optimize.npz", **rec)
    print("wrote", OUT / "reference_optimize.npz", "N =", s.n)


# run.py's E2E physics path: layers, then OptimizeSingleTimestep calls
# (t, max_gd_iters, initial_alpha, max_line_search_iters), with render
# gradients stored on the graph
SINGLE_CALLS = [(2, 2, 0.05, 4), (0, 2, 0.05, 4), (2, 1, 0.05, 4), (4, 2, 0.5, 3)]
SINGLE_LAYERS = 6


def single_case():
    """Inputs of the single-timestep fixture: the optimiser fixture's
    particles and target, dt 2e-3, drag 0.5, smoothing 0.1, seeded render
    gradients dL/dF (N,3,3) and dL/dx (N,3) (float32, as run.py passes them)."""
    w, s, g, tgt, _ = optimize_case()
    prm = O.Params(dt=2e-3, drag=0.5, smoothing=0.1)
    rng = np.random.default_rng(17)
    n = s.n
    rF = (1e-3 * rng.normal(size=(n, 3, 3))).astype(np.float32)
    rx = (1e-3 * rng.normal(size=(n, 3))).astype(np.float32)
    return w, s, g, tgt, prm, rF, rx


def make_single():
    """OptimizeSingleTimestep (CompGraph.cpp:369-465) as run.py's E2E path
    calls it, both builds, each in a fresh process: the reference's Adam step
    counter is a function-local static that starts at 0 and carries over
    between calls (CompGraph.cpp:396)."""
    import subprocess
    for bits in (64, 32):
        subprocess.check_call([sys.executable, __file__, "--single-bits", str(bits)])
    rec = dict(np.load(OUT / "reference_single_64.npz"))
    rec.update(np.load(OUT / "reference_single_32.npz"))
    (OUT / "reference_single_64.npz").unlink()
    (OUT / "reference_single_32.npz").unlink()
    np.savez_compressed(OUT / "reference_single.npz", **rec)
    print("wrote", OUT / "reference_single.npz")


def _make_single_bits(bits):
    ref = O.Reference(bits)
    w, s, g, tgt, prm, rF, rx = single_case()
    dfc, xT, loss, log = ref.optimize_single(g, prm, s, tgt, SINGLE_LAYERS, SINGLE_CALLS, rF, rx)
    accepted = [int(line.split("ls_iter=")[1].split(",")[0]) if "accepted" in line else -1
                for line in log.splitlines() if "Step accepted" in line or "Line search failed" in line]
    rec = {f"single{bits}_dFc": dfc, f"single{bits}_xT": xT, f"single{bits}_loss": loss,
           f"single{bits}_ls": np.asarray(accepted)}
    if bits == 64:
        rec.update(dims=np.asarray(w.dims), dx=w.dx, dt=prm.dt, drag=prm.drag, smoothing=prm.smoothing, target=tgt,
                   x=s.x, v=s.v, m=s.m, vol=s.vol, lam=s.lam, mu=s.mu, render_dLdF=rF, render_dLdx=rx,
                   calls=np.asarray(SINGLE_CALLS, np.float64), layers=SINGLE_LAYERS)
    np.savez(OUT / f"reference_single_{bits}.npz", **rec)
    print(bits, "losses", loss, "line-search outcomes", accepted)


def main(which=("small", "optimize", "mesh", "single")):
    build_oracle.build_oracle()
    outs = build_oracle.build_ref()
    if not outs:
        raise SystemExit("reference tree not found; golden vectors need the reference sources")
    if "optimize" in which:
        make_optimize()
    if "mesh" in which:
        make_mesh_sampling()
    if "single" in which:
        make_single()
    if "small" not in which:
        return
    r64, r32 = O.Reference(64), O.Reference(32)
    w, s, rng = small_state()
    g = O.Grid(w.dims, w.dx)
    prm = O.Params(dt=1e-3, drag=0.5, smoothing=0.1)
    n = s.n
    rec = dict(dims=np.asarray(w.dims), dx=w.dx, gmin=np.zeros(3), dt=prm.dt, drag=prm.drag, smoothing=prm.smoothing,
               x=s.x, v=s.v, C=s.C, F=s.F, dFc=s.dFc, m=s.m, vol=s.vol, lam=s.lam, mu=s.mu)
    # forward step
    for bits, ref in ((64, r64), (32, r32)):
        s1, gstep = ref.forward_step(g, prm, s)
        for k in ("x", "v", "C", "F"):
            rec[f"fwd{bits}_{k}"] = getattr(s1, k)
        rec[f"fwd{bits}_gm"] = gstep["m"]
        rec[f"fwd{bits}_gv"] = gstep["v"]
    # backward step (upstream grads seeded)
    s1, gstep = r64.forward_step(g, prm, s)
    g1 = O.Grads(rng.normal(size=(n, 3)), rng.normal(size=(n, 3)), 0.1 * rng.normal(size=(n, 3, 3)),
                 0.01 * rng.normal(size=(n, 3, 3)))
    rec.update(bwd_C1=s1.C, bwd_gm=gstep["m"], bwd_gv=gstep["v"], bwd_gx1=g1.x, bwd_gv1=g1.v, bwd_gF1=g1.F,
               bwd_gC1=g1.C)
    for bits, ref in ((64, r64), (32, r32)):
        gb = ref.backward_step(g, prm, s, s1.C, gstep, g1)
        for k in ("x", "v", "F", "C"):
            rec[f"bwd{bits}_g{k}"] = getattr(gb, k)
    # mass loss against a target made from shifted particles
    tgt = np.zeros(g.n_nodes)
    O.Oracle().p2g_accumulate(g, s1.x + 0.03, s1.v, s1.C, s.m, tgt, np.zeros((g.n_nodes, 3)))
    rec["loss_target"] = tgt
    for bits, ref in ((64, r64), (32, r32)):
        loss, d = ref.mass_loss(g, s1.x, s.m, tgt)
        rec[f"loss{bits}"] = loss
        rec[f"loss{bits}_gx"] = d["gx"]
        rec[f"loss{bits}_dLdm"] = d["dLdm"]
    # Adam, three steps
    gF = 0.1 * rng.normal(size=(n, 3, 3))
    rec["adam_gF"] = gF
    for bits, ref in ((64, r64), (32, r32)):
        dFc, mom, vec, vmax = s.dFc.copy(), np.zeros((n, 3, 3)), np.zeros((n, 3, 3)), np.zeros((n, 3, 3))
        for t in (1, 2, 3):
            ref.adam(gF * t, dFc, mom, vec, vmax, 0.05, timestep=t)
        rec[f"adam{bits}_dFc"] = dFc
        rec[f"adam{bits}_vmax"] = vmax
    # volumes into an empty grid
    for bits, ref in ((64, r64), (32, r32)):
        gm, gp = np.zeros(g.n_nodes), np.zeros((g.n_nodes, 3))
        rec[f"vol{bits}"] = ref.volumes(g, s.x, s.v, s.C, s.m, gm, gp)
        rec[f"vol{bits}_gm"] = gm
        rec[f"vol{bits}_gp"] = gp
    # constitutive, including inverted and near-singular F
    Fs = [np.eye(3) + 0.3 * rng.normal(size=(3, 3)) for _ in range(20)]
    Fs += [rng.normal(size=(3, 3)) for _ in range(10)]
    Fs += [np.diag([1.0, 1.0, -0.5]), np.diag([2.0, 0.5, 1e-3])]
    dFs = [rng.normal(size=(3, 3)) for _ in Fs]
    rec["cons_F"] = np.asarray(Fs)
    rec["cons_dF"] = np.asarray(dFs)
    rec["cons_P64"] = np.asarray([r64.pk(F, 5769.23, 3846.15) for F in Fs])
    rec["cons_H64"] = np.asarray([r64.hvp(F, 5769.23, 3846.15, d) for F, d in zip(Fs, dFs)])
    # 5-step full-tape rollout through CompGraph (stable density, smoothing on)
    prm_r = O.Params(dt=1e-3, drag=0.5, smoothing=0.1)
    s0 = O.State(s.x, s.v, np.zeros((n, 3, 3)), np.tile(np.eye(3), (n, 1, 1)), s.m, s.vol, s.lam, s.mu, s.dFc)
    seed = 2.0 * (s.x - (s.x + 0.02)) / n
    rec["roll_T"] = 5
    rec["roll_seed"] = seed
    for bits, ref in ((64, r64), (32, r32)):
        xT, gr, _ = ref.rollout(g, prm_r, s0, 5, seed)
        rec[f"roll{bits}_xT"] = xT
        for k in ("x", "v", "F", "C"):
            rec[f"roll{bits}_g{k}"] = getattr(gr, k)
    np.savez_compressed(OUT / "reference_small.npz", **rec)
    print("wrote", OUT / "reference_small.npz", "N =", n)


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=["small", "optimize", "mesh", "single"])
    ap.add_argument("--single-bits", type=int, choices=[32, 64], help=argparse.SUPPRESS)
    a = ap.parse_args()
    if a.single_bits:
        _make_single_bits(a.single_bits)
    else:
        main((a.only,) if a.only else ("small", "optimize", "mesh", "single"))
