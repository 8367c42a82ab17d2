#!/usr/bin/env python
"""bench.py -- fwd+bwd particle-steps/s of the differentiable MPM rollout.

Workload (default ``spheres2m``): 2,000,000 particles in a union of 8 seeded
spheres (radii 0.08-0.15) on 129^3 nodes, Fixed-Corotated material
(E=1e4, nu=0.3, density chosen for CFL 0.45 at dt=2.5e-4), cubic B-spline
APIC, 400 steps forward plus the exact adjoint, checkpoint every 20 steps
with recomputation.  One bench step is one such rollout (forward 400 steps,
loss gradient, backward 400 steps); value = particles * steps / time.

`value` is timed with inputs resident in HBM; `e2e` is the same rollout
driven through the drop-in bindings from pinned host buffers with the
host<->device copies inside the timed region.  L2 (129 MB) is flushed with a
256 MiB write between timed steps (outside the CUDA-event brackets).

`--impl reference` times the reference algorithm's CPU path: the FP64 CPU
restatement in oracle/ (the reference's own sources are not present on the
GPU host), on all host threads, over a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "shape-morphing-binder_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))
os.environ.setdefault("MPM_QUIET", "1")

METRIC = "fwd+bwd particle-steps/s on 1 GB300 vs plain FP64 GPU form at ≤1e-4 grad rel err"
UNIT = "particle-steps/s"


# ------------------------------------------------------------------ helpers

def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_workload(name: str, quick: bool = False, timesteps: int = 0, checkpoint: int = 0):
    from diffmpm_bindings import workloads as W
    if name == "spheres2m":
        w = W.spheres2m(n=200_000 if quick else 2_000_000, steps=40 if quick else 400, checkpoint=20)
        w.extra["grad_E"] = True  # gradients w.r.t. control F, v0 and the scalar E
    elif name == "ellipsoid64":
        w = W.ellipsoid64(steps=20 if quick else 100, checkpoint=10)
    elif name == "sphere32":
        # the 17k-particle sphere as specified: Neo-Hookean, quadratic B-spline APIC
        w = W.sphere32()
        w.checkpoint = 1
        w.extra.update(kernel="quadratic", material="neohookean")
    else:
        raise SystemExit(f"unknown workload {name}")
    if timesteps:
        w.steps = timesteps
    if checkpoint:
        w.checkpoint = checkpoint
    if w.target is None:
        rng = np.random.default_rng(11)
        w.target = w.x + 0.02 * np.sin(2 * np.pi * w.x[:, [1, 2, 0]] + rng.random(3))
    return w


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- our arm

# algorithmic bytes per particle and per active node for each kernel (FP32
# storage)
KERNEL_BYTES = {
    "p2g": (112, 16),
    # G2P of a step fused with the next step's P2G: G2P's bytes plus the
    # particle constants; the state it writes is not read back
    "g2p2g": (164, 32),
    "g2p": (148, 16),
    "g2p_adj": (184, 16),
    "p2g_adj": (380, 32),
    # the grid kernels also clear the next step's grid (16 B per node)
    "grid_update": (0, 48),
    "grid_adj": (0, 64),
}
# kernel ids (include/mpm.h) of the kernels with roofline bytes
K_IDS = {"p2g": 0, "grid_update": 1, "g2p": 2, "g2p_adj": 3, "grid_adj": 4, "p2g_adj": 5, "g2p2g": 10}
ALL_KERNELS = (1 << 13) - 1


def query_kernels(lib):
    import ctypes as C
    kern = {}
    for k in range(13):
        cnt, ms = C.c_longlong(), C.c_double()
        lib.mpm_profile_query(k, C.byref(cnt), C.byref(ms))
        if cnt.value:
            kern[lib.mpm_kernel_name(k).decode()] = (cnt.value, ms.value)
    return kern


def build_graph(dm, w, precision, checkpoint, adjoint="exact", deterministic=False):
    kernel, material = w.extra.get("kernel", "cubic"), w.extra.get("material", "fcr")
    dt = np.float64 if precision == "fp64" else np.float32
    Cm = w.extra.get("C")
    pc = dm.PointCloud.from_arrays(w.x.astype(dt), v=w.v.astype(dt), F=w.F.astype(dt), m=w.m.astype(dt),
                                   vol=w.vol.astype(dt), lam=w.lam.astype(dt), mu=w.mu.astype(dt),
                                   C_=None if Cm is None else Cm.astype(dt), precision=precision)
    grid = dm.Grid(*w.dims, w.dx, w.grid_min, precision=precision)
    cg = dm.CompGraph(pc, grid, grid, adjoint=adjoint, checkpoint_every=checkpoint, deterministic=deterministic,
                      kernel=kernel, material=material)
    cg.set_sim_params(dt=w.dt, drag=w.drag, smoothing=w.smoothing)
    return cg, (pc, grid)


def advance_workload(dm, w, steps):
    """The workload's state after `steps` forward steps (FP32), in the
    caller's particle order: the particles have drifted away from the cell
    order of the input, as they have late in a long rollout.  With the
    set-up re-sort (the default) the timed graph starts re-sorted, with
    --no-resort it keeps the drifted order: the pair measures what a re-sort
    at a stored layer would buy."""
    cg, keep = build_graph(dm, w, "fp32", w.checkpoint)
    cg.set_up_comp_graph(steps + 1)
    cg.compute_forward_pass(0, 0)
    last = cg.get_point_cloud(steps)
    w.x, w.v, w.F = last.get("x", np.float64), last.get("v", np.float64), last.get("F", np.float64)
    w.extra["C"] = last.get("C", np.float64)
    w.extra["advanced_steps"] = steps
    del cg, keep
    return w


def device_rollout(torch, cg, T, tgt, n):
    """Forward T steps, position-loss gradient on device, backward T steps."""
    cg.compute_forward_pass(0, 0)
    last = cg.get_point_cloud(T)
    xT = last.get_torch("x", device="cuda")
    # (in a batch the padding between instances has x = target = 0: zero gradient)
    g = (2.0 / n) * (xT - tgt)
    last.set("grad_x", g)
    cg.compute_backward_pass(0)


class BatchWorkload:
    """The batched workload: 64 instances of uneven size concatenated."""

    def __init__(self, quick=False, timesteps=0):
        from diffmpm_bindings import workloads as W
        self.parts = W.batched(count=8 if quick else 64, steps=10 if quick else 50)
        self.name = "batched64" if not quick else "batched8"
        self.steps = timesteps or self.parts[0].steps
        self.checkpoint = 10
        self.dt, self.drag, self.smoothing = self.parts[0].dt, 0.0, 0.0
        self.n = sum(p.n for p in self.parts)
        self.dims = (0, 0, 0)
        self.dx = None
        self.rho = float("nan")
        self.extra = {"E": "log-U[1e3,1e5]", "nu": "U[0.2,0.45]"}


def build_batch_graph(dm, bw, precision, deterministic=False):
    dt = np.float64 if precision == "fp64" else np.float32
    pcs, grids = [], []
    for w in bw.parts:
        pcs.append(dm.PointCloud.from_arrays(w.x.astype(dt), v=w.v.astype(dt), F=w.F.astype(dt), m=w.m.astype(dt),
                                             vol=w.vol.astype(dt), lam=w.lam.astype(dt), mu=w.mu.astype(dt),
                                             precision=precision))
        grids.append(dm.Grid(*w.dims, w.dx, w.grid_min, precision=precision))
    cg = dm.CompGraph.batch(pcs, grids, adjoint="exact", checkpoint_every=bw.checkpoint,
                            deterministic=deterministic)
    cg.set_sim_params(dt=bw.dt, drag=bw.drag, smoothing=bw.smoothing)
    n_pad = len(cg.get_point_cloud(0))
    tgt = np.zeros((n_pad, 3))
    rng = np.random.default_rng(11)
    for i, w in enumerate(bw.parts):
        tgt[cg.instance_range(i)] = w.x + 0.01 * rng.normal(size=w.x.shape)
    return cg, (pcs, grids), tgt, n_pad


def run_ours(args, rank, world, device):
    import torch
    import diffmpm_bindings as dm
    lib = dm._lib.lib
    lib.mpm_set_verbose(0)
    if args.workload == "batched":
        w = BatchWorkload(args.quick, args.timesteps)
        n, T = w.n, w.steps
        cg, keep, tgt_np, n_pad = build_batch_graph(dm, w, "fp32", deterministic=args.deterministic)
        w.target = tgt_np
        args.no_e2e, args.no_fp64, args.no_cpu = True, True, True
    else:
        w = make_workload(args.workload, args.quick, args.timesteps, args.checkpoint)
        if args.from_rollout:
            w = advance_workload(dm, w, args.from_rollout)
        if args.shuffle:
            p = np.random.default_rng(5).permutation(w.n)
            for k in ("x", "v", "F", "m", "vol", "lam", "mu", "target"):
                setattr(w, k, getattr(w, k)[p])
        n, T = w.n, w.steps
        cg, keep = build_graph(dm, w, "fp32", w.checkpoint, deterministic=args.deterministic)
        n_pad = n
    apply_resort(cg, args)
    if w.extra.get("grad_E"):
        cg.enable_lame_grads(True)
    cg.set_up_comp_graph(T + 1)
    stream = torch.cuda.current_stream(device)
    cg.set_stream(stream)
    tgt = torch.tensor(w.target, dtype=torch.float32, device=device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    if args.tiles:
        # fixed tile budgets (P2G, G2P transpose, P2G-transpose gather), e.g.
        # the ones the autotuner picked for a full run, for profiler captures
        tp, ta, tg = (int(v) for v in args.tiles.split(","))
        cg.set_tuning(tp, 1, ta, tg)
        tuning = cg.get_tuning()
    elif args.no_autotune:
        tuning = cg.get_tuning()
    else:
        # tune from the stored layer halfway through a computed rollout: its
        # particles have drifted from the set-up cell order as they do over
        # the timed rollouts (untimed set-up work)
        device_rollout(torch, cg, T, tgt, n)
        mid = (T // 2) // w.checkpoint * w.checkpoint
        tuning = cg.autotune(steps=4, layer=mid)

    # CUDA events around the launches of the selected kernels, on from the
    # warm-up on: the warm-up rollouts record the passes (with their event
    # nodes) that the timed rollouts then replay.  With --timed-profile top
    # the first warm-up rollout times every kernel and picks the largest
    # one with roofline bytes; only that one is timed from then on.
    lib.mpm_profile_select(ALL_KERNELS)
    lib.mpm_profile_enable(1)
    for i in range(args.warmup):
        if i == 0:
            lib.mpm_profile_reset()
        device_rollout(torch, cg, T, tgt, n)
        if i == 0 and args.timed_profile == "top":
            torch.cuda.synchronize(device)
            k0 = query_kernels(lib)
            pick = max((k for k in k0 if k in K_IDS), key=lambda k: k0[k][1])
            lib.mpm_profile_select(1 << K_IDS[pick])
    torch.cuda.synchronize(device)

    # ---- timed region (device-resident inputs)
    if args.profile_window:
        torch.cuda.profiler.start()  # an external profiler started with capture off begins here
    lib.mpm_profile_reset()
    launches0 = lib.mpm_launch_count()
    times = []
    barrier(world)
    torch.cuda.synchronize(device)
    with Clocks(device.index if device.index is not None else 0) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            device_rollout(torch, cg, T, tgt, n)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    torch.cuda.synchronize(device)
    barrier(world)
    launches = lib.mpm_launch_count() - launches0
    lib.mpm_profile_enable(0)
    if args.profile_window:
        torch.cuda.profiler.stop()
    kern = query_kernels(lib)
    kern_all, kern_src = kern, "the timed rollouts"
    if args.timed_profile == "top":
        # every kernel timed in one more rollout after the timed region
        lib.mpm_profile_select(ALL_KERNELS)
        lib.mpm_profile_reset()
        lib.mpm_profile_enable(1)
        device_rollout(torch, cg, T, tgt, n)
        torch.cuda.synchronize(device)
        lib.mpm_profile_enable(0)
        kern_all = {k: (c * args.steps, ms * args.steps) for k, (c, ms) in query_kernels(lib).items()}
        kern_src = "one untimed rollout after the timed region, scaled to the timed rollouts' count"
    t_total = max_over_ranks(torch, sum(times), world, device)
    value = job_value(world, n * T * args.steps, t_total)
    active = cg.active_nodes(0)

    # ---- roofline of the dominant kernel
    hbm, src = peaks()
    top = max((k for k in kern if k in KERNEL_BYTES), key=lambda k: kern[k][1])
    cnt, ms = kern[top]
    bp, bn = KERNEL_BYTES[top]
    if top == "p2g_adj" and w.extra.get("grad_E"):
        bp += 16  # read and write the running dL/dlam, dL/dmu
    algo = bp * n + bn * active
    achieved = algo / (ms / cnt / 1e3) / 1e9
    traffic = None
    tp = ROOT / "profiles" / "ncu_traffic.json"
    if tp.exists():
        d = json.loads(tp.read_text()).get(top)
        if d and d.get("bytes_per_particle"):
            traffic = d["bytes_per_particle"] * n
    total_ms = sum(v[1] for v in kern_all.values())
    roof = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
            "frac": round(achieved / hbm, 4), "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": traffic, "algorithmic_bytes_per_launch": algo, "launches": cnt,
            "avg_launch_ms": round(ms / cnt, 5),
            "kernel_share": {k: round(v[1] / total_ms, 4) for k, v in sorted(kern_all.items(), key=lambda x: -x[1][1])},
            "timed_kernels": sorted(kern), "kernel_share_source": kern_src}

    # ---- e2e through the public API with host buffers
    e2e = None if args.no_e2e else run_e2e(torch, dm, args, w, device, keep, tuning)

    # ---- plain FP64 form and accuracy (rank 0)
    fp64 = None
    if rank == 0 and not args.no_fp64:
        fp64 = run_fp64(torch, dm, w, device, args, value / world)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(w, args)

    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * t_total / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64-guarded stress)", "data": "synthetic (seeded)",
        "config": {"workload": w.name, "particles": n, "grid_nodes": list(w.dims), "dx": w.dx, "timesteps": T,
                   "instances": len(w.parts) if hasattr(w, "parts") else 1,
                   "checkpoint_every": w.checkpoint, "dt": w.dt, "density": round(w.rho, 3),
                   "material": "%s E=%s nu=%s" % ({"fcr": "fixed-corotated", "neohookean": "Neo-Hookean"}[
                       w.extra.get("material", "fcr")], w.extra["E"], w.extra["nu"]),
                   "kernel": "%s B-spline APIC" % w.extra.get("kernel", "cubic"), "adjoint": "exact",
                   "parallelism": f"replicas x{world}",
                   "l2": "flushed between timed steps (256 MiB write, outside the event brackets)",
                   "bench_step": "one rollout: forward T steps + loss gradient + backward T steps",
                   "tuning": tuning, "cuda_graphs": True, "deterministic": bool(args.deterministic),
                   "particle_order": ("shuffled" if args.shuffle else "cell-sorted input") +
                                     (f", advanced {args.from_rollout} steps (drifted)" if args.from_rollout else "") +
                                     ("" if args.no_resort else ", re-sorted by cell at set-up") +
                                     (f", and every {cg.resort_every()} layers inside the rollout"
                                      if cg.resort_every() else ""),
                   "gradients": "layer 0: x, v, F, C, control F" + (", lam, mu (dL/dE)" if w.extra.get("grad_E")
                                                                    else "")},
        "clocks": clk.summary(), "gpu_launches": int(launches), "e2e": e2e, "roofline": roof,
        "kernels_ms": {k: round(v[1], 3) for k, v in kern_all.items()}, "active_nodes": active,
        "native_libs": native_libs(),
    }
    if fp64:
        line["fp64_plain"] = fp64
    if cpu:
        line["cpu_baseline"] = cpu
    return line


def run_morph(args, device):
    """The control-optimisation episode end to end: a 500k-particle sphere morphed
    towards targets displaced by seeded real spherical harmonics (l <= 4),
    one episode per target.  Each episode is run_optimization
    (OptimizeDefGradControlSequence) over 200 steps per pass, control stride
    10 (20 control steps), lr 1e-2, 10 passes, FP64 Adam moments and the
    deterministic fixed-point scatters; the next episode starts from the last
    layer (promote_last_as_initial, as run.py does between episodes).
    Timed on the host clock around each synchronous run_optimization call
    (everything included: line-search forwards, loss read-backs).  --warmup
    runs short episodes (one pass), --steps the timed episodes."""
    import torch
    import diffmpm_bindings as dm
    from diffmpm_bindings import workloads as W
    lib = dm._lib.lib
    lib.mpm_set_verbose(0)
    n_part = 50_000 if args.quick else 500_000
    w0 = W.morph500k(n=n_part, episode=0)
    n = w0.n
    steps = args.timesteps or (40 if args.quick else 200)
    passes = 2 if args.quick else 10
    pc0 = dm.PointCloud.from_arrays(w0.x.astype(np.float32), v=w0.v.astype(np.float32), F=w0.F.astype(np.float32),
                                    m=w0.m.astype(np.float32), vol=w0.vol.astype(np.float32),
                                    lam=w0.lam.astype(np.float32), mu=w0.mu.astype(np.float32))
    grid = dm.Grid(*w0.dims, w0.dx, w0.grid_min)
    target = dm.Grid(*w0.dims, w0.dx, w0.grid_min)
    # exact adjoint: the reference-compatible one repeats (I + dt C)^T dL/dF
    # (BackPropagation.cpp:140), which doubles dL/dF every step -- 2^200 over a
    # 200-step pass, beyond the FP32 range
    cg = dm.CompGraph(pc0, grid, target, checkpoint_every=10, deterministic=not args.no_det, adjoint="exact")
    opt = dm.OptInput()
    opt.num_timesteps, opt.control_stride, opt.max_gd_iters, opt.max_ls_iters = steps + 1, 10, 1, 4
    opt.dt, opt.drag, opt.smoothing_factor = w0.dt, w0.drag, w0.smoothing
    opt.initial_alpha, opt.gd_tol = 1e-2, 1e-4

    def set_target(e):
        we = W.morph500k(n=n_part, episode=e)
        target.set_node_masses(np.zeros(target.num_nodes))
        tpc = dm.PointCloud.from_arrays(we.target.astype(np.float32), m=we.m.astype(np.float32))
        dm.p2g(tpc, target)

    for e in range(args.warmup):
        set_target(100 + e)
        cg.run_optimization(opt, passes=1)
    episodes = []
    f0, b0 = dm.step_count()
    total = 0.0
    with Clocks(device.index if device.index is not None else 0) as clk:
        for e in range(args.steps):
            set_target(e)
            torch.cuda.synchronize(device)
            t0 = time.perf_counter()
            cg.run_optimization(opt, passes=passes)
            torch.cuda.synchronize(device)
            dt_e = time.perf_counter() - t0
            total += dt_e
            h = cg.loss_history()
            episodes.append({"episode": e, "seconds": round(dt_e, 3), "initial_loss": float(h[0]),
                             "final_loss": float(h[-1]), "best_loss": float(np.nanmin(h)),
                             "losses_evaluated": int(len(h)), "nonfinite_trials": int((~np.isfinite(h)).sum())})
            cg.promote_last_as_initial()
    f1, b1 = dm.step_count()
    psteps = n * ((f1 - f0) + (b1 - b0))
    return {
        "metric": "control-optimisation episode (500k-particle sphere morph), particle-steps/s end to end", "value": round(psteps / total, 1),
        "unit": "particle-steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "seconds_per_episode": round(total / max(1, args.steps), 3), "seconds_total": round(total, 3),
        "higher_is_better": True, "dtype": "f32 (FP64-guarded stress, FP64 Adam moments)",
        "data": "synthetic (seeded)",
        "config": {"workload": "morph500k" if not args.quick else "morph50k", "particles": n,
                   "grid_nodes": list(w0.dims), "dx": w0.dx, "timesteps_per_pass": steps, "control_stride": 10,
                   "passes": passes, "episodes": args.steps, "lr": 1e-2, "max_line_search": 4,
                   "checkpoint_every": 10, "deterministic": not args.no_det, "adjoint": "exact",
                   "target": "sphere displaced by seeded real spherical harmonics, l <= 4"},
        "forward_steps": f1 - f0, "adjoint_steps": b1 - b0, "episodes": episodes, "clocks": clk.summary(),
    }


def run_render(args, device):
    """The Gaussian rasterizer (diff_gauss) on the particles of the
    500k-particle morph sphere: 500k Gaussians (covariance from F = I and half a
    grid spacing), 1024 x 1024, colors precomputed, normals from scale and
    rotation; one step = forward + backward of an image loss.  CUDA events on
    the current stream; the backward includes the host read of the number of
    rendered (tile, Gaussian) pairs that sizes the sort."""
    import torch
    import diff_gauss as dg
    from diffmpm_bindings import workloads as W
    w = W.morph500k(n=50_000 if args.quick else 500_000, episode=0)
    H = Wd = 256 if args.quick else 1024
    tanx, tany, view, proj, eye = W.camera(H, Wd, fovx_deg=45.0, eye=(0.5, 0.5, -0.9), target=(0.5, 0.5, 0.5))
    n = w.n
    g = torch.Generator(device="cpu").manual_seed(0)
    f32 = dict(dtype=torch.float32, device=device)
    means = torch.tensor(w.x, **f32).requires_grad_(True)
    scales = torch.full((n, 3), 0.5 * w.dx, **f32).requires_grad_(True)
    rots = torch.nn.functional.normalize(torch.randn(n, 4, generator=g), dim=1).to(**f32).requires_grad_(True)
    cols = torch.rand(n, 3, generator=g).to(**f32).requires_grad_(True)
    ops = (0.3 + 0.6 * torch.rand(n, 1, generator=g)).to(**f32).requires_grad_(True)
    st = dg.GaussianRasterizationSettings(H, Wd, tanx, tany, torch.ones(3, **f32), 1.0, view.to(**f32),
                                          proj.to(**f32), 0, eye.to(**f32), False, False)
    rast = dg.GaussianRasterizer(st)
    target = torch.rand((3, H, Wd), generator=g).to(**f32)

    def step():
        m2 = torch.zeros_like(means, requires_grad=True)
        color, depth, nrm, alpha, radii, _ = rast(means, m2, ops, colors_precomp=cols, scales=scales,
                                                  rotations=rots)
        loss = ((color - target) ** 2).mean() + 0.01 * alpha.mean()
        loss.backward()
        return radii

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(device)
    stream = torch.cuda.current_stream(device)
    times = []
    with Clocks(device.index if device.index is not None else 0) as clk:
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            radii = step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    ms = statistics.median(times)
    return {"metric": "Gaussian rasterizer forward+backward, Gaussians/s", "value": round(n / (ms / 1e3), 1),
            "unit": "Gaussians/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "render500k" if not args.quick else "render50k", "gaussians": n,
                       "image": [H, Wd], "visible": int((radii > 0).sum()), "sh": "precomputed colors",
                       "covariance": "scale 0.5 dx, random rotation", "outputs": "color, depth, normal, alpha"},
            "clocks": clk.summary()}


def apply_resort(cg, args):
    """Particle re-sorts: at set-up and inside the rollout (library defaults
    unless switched off or set)."""
    cg.set_resort(not args.no_resort)
    if args.no_resort:
        cg.set_resort_every(0)
    elif args.resort_every is not None:
        cg.set_resort_every(args.resort_every)


def run_e2e(torch, dm, args, w, device, keep, tuning=None):
    """Public API with pinned host buffers: x0, v0, F0 in; dL/dx_T seed in
    (computed on the host from x_T out, like run.py's gradient injection);
    dL/dv0 and dL/dF0 out."""
    n, T = w.n, w.steps
    pc0, grid = keep
    cg = dm.CompGraph(pc0, grid, grid, adjoint="exact", checkpoint_every=w.checkpoint,
                      deterministic=args.deterministic, kernel=w.extra.get("kernel", "cubic"),
                      material=w.extra.get("material", "fcr"))
    cg.set_sim_params(dt=w.dt, drag=w.drag, smoothing=w.smoothing)
    grad_E = bool(w.extra.get("grad_E"))
    if grad_E:
        cg.enable_lame_grads(True)
    apply_resort(cg, args)
    if tuning:  # the device arm's kernel configuration
        cg.set_tuning(tuning["tile_nodes"], tuning["scatter_mode"], tuning.get("adj_tile_nodes", -1),
                      tuning.get("gather_tile_nodes", -1), tuning.get("block_threads", -1))
    cg.set_up_comp_graph(T + 1)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).pin_memory()  # noqa: E731
    hx, hv, hF = pin(w.x), pin(w.v), pin(w.F)
    htgt = torch.from_numpy(np.ascontiguousarray(w.target, dtype=np.float32))
    out_x = torch.empty((n, 3), dtype=torch.float32).pin_memory()
    out_gv = torch.empty((n, 3), dtype=torch.float32).pin_memory()
    out_gF = torch.empty((n, 3, 3), dtype=torch.float32).pin_memory()
    out_gl = torch.empty((n,), dtype=torch.float32).pin_memory()
    out_gm = torch.empty((n,), dtype=torch.float32).pin_memory()
    seed = torch.empty((n, 3), dtype=torch.float32).pin_memory()
    h2d = (hx.numel() + hv.numel() + hF.numel() + seed.numel()) * 4
    d2h = (out_x.numel() + out_gv.numel() + out_gF.numel() + (2 * n if grad_E else 0)) * 4
    if grad_E:
        nu = float(w.extra["nu"])
        dlam, dmu = nu / ((1 + nu) * (1 - 2 * nu)), 1.0 / (2 * (1 + nu))  # d(lam, mu)/dE
    import ctypes as C
    lib = dm._lib.lib

    def get_into(pc, field, t):
        dm._lib.check(lib.mpm_pointcloud_get(pc._h, dm._lib.FIELDS[field], C.c_void_p(t.data_ptr()), 0, 0))

    def step():
        l0 = cg.get_point_cloud(0)
        l0.set("x", hx.numpy())
        l0.set("v", hv.numpy())
        l0.set("F", hF.numpy())
        cg.compute_forward_pass(0, 0)
        last = cg.get_point_cloud(T)
        get_into(last, "x", out_x)
        # host-side loss gradient, in place on the host threads (torch CPU ops)
        torch.sub(out_x, htgt, out=seed)
        seed.mul_(2.0 / n)
        last.set("grad_x", seed.numpy())
        cg.compute_backward_pass(0)
        get_into(l0, "grad_v", out_gv)
        get_into(l0, "grad_dFc", out_gF)
        if grad_E:
            get_into(l0, "grad_lam", out_gl)
            get_into(l0, "grad_mu", out_gm)
            return float(out_gl.sum(dtype=torch.float64)) * dlam + float(out_gm.sum(dtype=torch.float64)) * dmu
        return None

    for _ in range(max(1, min(args.warmup, 2))):
        step()
    torch.cuda.synchronize(device)
    ts = []
    k = max(1, min(args.steps, 3))
    for _ in range(k):
        t0 = time.perf_counter()
        step()
        ts.append(time.perf_counter() - t0)
    t = sum(ts)
    return {"value": round(n * T * k / t, 1), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "steps": k, "ms_per_step": round(1e3 * t / k, 3),
            "path": "diffmpm_bindings.CompGraph (C ABI) from pinned host buffers",
            "outputs": "x_T; dL/dv0, dL/d(control F)" + (", dL/dE" if grad_E else "")}


def run_fp64(torch, dm, w, device, args, fp32_value):
    """The plain all-FP64 GPU form (the metric's denominator) over the whole
    rollout, timed with CUDA events, and the FP32 path's error against it:
    x_T and the gradients w.r.t. the initial velocity, the control F and E.
    One FP64 rollout is timed as it runs (its ~10k launches cost well under 1%
    of its time, so no graph replay is needed); the FP32 rollout beside it is
    for the errors, and the speed-up uses the timed FP32 value."""
    T = min(w.steps, args.fp64_steps) if args.fp64_steps > 0 else w.steps
    n = w.n
    res = {}
    grads = {}
    for prec in ("fp64", "fp32"):
        cg, keep = build_graph(dm, w, prec, w.checkpoint)
        if w.extra.get("grad_E"):
            cg.enable_lame_grads(True)
        cg.set_up_comp_graph(T + 1)
        tdt = torch.float64 if prec == "fp64" else torch.float32
        tgt = torch.tensor(w.target, dtype=tdt, device=device)
        stream = torch.cuda.current_stream(device)
        cg.set_stream(stream)
        torch.cuda.synchronize(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        device_rollout(torch, cg, T, tgt, n)
        e1.record(stream)
        e1.synchronize()
        res[prec] = n * T / (e0.elapsed_time(e1) / 1e3)
        grads[prec] = {"x": cg.get_point_cloud(T).get("x", np.float64),
                       "gv": cg.get_grad(0, "v", np.float64), "gF": cg.get_grad(0, "dFc", np.float64)}
        if w.extra.get("grad_E"):
            nu = float(w.extra["nu"])
            grads[prec]["gE"] = np.array([cg.get_grad(0, "lam", np.float64).sum() * nu / ((1 + nu) * (1 - 2 * nu))
                                          + cg.get_grad(0, "mu", np.float64).sum() / (2 * (1 + nu))])
        del cg, keep
    rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))  # noqa: E731
    full = T == w.steps
    return {"value": round(res["fp64"], 1), "unit": UNIT, "timesteps": T, "whole_rollout": full,
            "fp32_value_timed": round(fp32_value, 1), "speedup_fp32_vs_fp64": round(fp32_value / res["fp64"], 2),
            "grad_v0_rel_err": rel(grads["fp32"]["gv"], grads["fp64"]["gv"]),
            "grad_dFc_rel_err": rel(grads["fp32"]["gF"], grads["fp64"]["gF"]),
            **({"grad_E_rel_err": rel(grads["fp32"]["gE"], grads["fp64"]["gE"])} if "gE" in grads["fp32"] else {}),
            "x_T_max_abs_err": float(np.abs(grads["fp32"]["x"] - grads["fp64"]["x"]).max()),
            "x_T_rel_err": rel(grads["fp32"]["x"], grads["fp64"]["x"])}


# ------------------------------------------------------------ CPU baseline

def cpu_sample(w, particles: int, T: int):
    import oracle as O
    sel = slice(0, min(particles, w.n))
    s = O.State(w.x[sel], w.v[sel], np.zeros((sel.stop, 3, 3)), w.F[sel], w.m[sel], w.vol[sel], w.lam[sel],
                w.mu[sel])
    g = O.Grid(w.dims, w.dx, w.grid_min)
    prm = O.Params(dt=w.dt, drag=w.drag, smoothing=w.smoothing, exact=False)
    seed = (2.0 / sel.stop) * (w.x[sel] - w.target[sel])
    return s, g, prm, seed


def cpu_model() -> str:
    """The host CPU's model name (/proc/cpuinfo, else lscpu), for the CPU legs."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def cpu_split(orc, O, g, prm, s, T, seed) -> dict:
    """The CPU sample again, step by step: forward and adjoint timed apart."""
    try:
        t1 = time.perf_counter()
        states, steps = [s], []
        for _ in range(T):
            s1, st = orc.forward_step(g, prm, states[-1])
            states.append(s1)
            steps.append(st)
        t2 = time.perf_counter()
        gg = O.Grads(seed, np.zeros((s.n, 3)), np.zeros((s.n, 3, 3)), np.zeros((s.n, 3, 3)))
        for t in range(T - 1, -1, -1):
            gg = orc.backward_step(g, prm, states[t], states[t + 1].C, steps[t], gg)
        t3 = time.perf_counter()
        return {"forward_s": round(t2 - t1, 3), "backward_s": round(t3 - t2, 3)}
    except Exception as e:  # a detail of the report; the measured value stands without it
        return {"split_error": str(e)[:120]}


def cpu_single_thread(orc, O, w, particles: int, T: int) -> dict:
    """The same algorithm on one host thread, over a smaller sample (an
    eighth of the particles): the reference's adjoint serialises its G2P
    transpose (BackPropagation.cpp:50-53), so its one-thread figure is the
    other number a reader needs."""
    threads = orc.threads()
    sub = max(1, particles // 8)
    s, g, prm, seed = cpu_sample(w, sub, T)
    try:
        orc.set_threads(1)
        t0 = time.perf_counter()
        orc.rollout(g, prm, s, T, seed)
        dt = time.perf_counter() - t0
    finally:
        orc.set_threads(threads)
    return {"value": round(s.n * T / dt, 1), "unit": UNIT, "cores": 1,
            "sample": f"{s.n} of {w.n} particles, {T} timestep(s) forward + reference adjoint"}


def cpu_baseline(w, args, split=True, single=True):
    import build_oracle
    build_oracle.build_oracle()
    import oracle as O
    orc = O.Oracle()
    particles = args.cpu_particles or w.n
    T = args.cpu_timesteps
    s, g, prm, seed = cpu_sample(w, particles, T)
    t0 = time.perf_counter()
    orc.rollout(g, prm, s, T, seed)
    dt = time.perf_counter() - t0
    extra = cpu_split(orc, O, g, prm, s, T, seed) if split else {}
    if single:
        extra["single_thread"] = cpu_single_thread(orc, O, w, particles, T)
    return {"value": round(s.n * T / dt, 1), "unit": UNIT, "cores": orc.threads(), "cpu": cpu_model(), "kind": "port",
            "sample": f"{s.n} of {w.n} particles of {w.name}, {T} timestep(s) forward + reference adjoint, "
                      f"full {w.dims[0]}^3 grid, FP64 CPU restatement (oracle/mpm_oracle.c, OpenMP)",
            **extra}


def native_libs() -> list[str]:
    """Shared libraries of this repository mapped into this process."""
    out = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if len(line.split()) >= 6 else ""
                if path.endswith(".so") and path.startswith(str(ROOT)):
                    out.add(str(Path(path).relative_to(ROOT)))
    except OSError:
        pass
    return sorted(out)


def run_reference(args, rank, world):
    if rank != 0:
        return None
    w = make_workload(args.workload, args.quick, args.timesteps)
    vals = []
    cb = None
    for i in range(args.warmup + args.steps):
        last = i == args.warmup + args.steps - 1
        cb = cpu_baseline(w, args, split=last, single=last)
        if i >= args.warmup:
            vals.append(cb["value"])
    v = float(np.mean(vals)) if vals else cb["value"]
    cb["value"] = round(v, 1)
    return {"metric": METRIC, "value": round(v, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": w.name, "particles": w.n, "timesteps": w.steps,
                       "note": "reference CPU path (restated in oracle/, OpenMP); each step is a bounded sample"},
            "cpu_baseline": cb, "e2e": {"value": round(v, 1), "unit": UNIT, "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0},
            "native_libs": native_libs()}


# ------------------------------------------------------------ distributed

def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def job_value(world, units_per_rank, t_max):
    """Whole-job throughput of independent replicas (weak scaling): every rank
    processes the same units; the job takes the slowest rank's time."""
    return world * units_per_rank / t_max


def max_over_ranks(torch, t, world, device):
    if world == 1:
        return t
    import torch.distributed as dist
    x = torch.tensor([t], dtype=torch.float64, device=device)
    dist.all_reduce(x, op=dist.ReduceOp.MAX)
    return float(x.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="spheres2m",
                    choices=["spheres2m", "ellipsoid64", "sphere32", "batched", "morph500k", "render500k"])
    ap.add_argument("--fp64-steps", type=int, default=0, help="0: the whole rollout")
    ap.add_argument("--cpu-particles", type=int, default=0, help="0: every particle")
    ap.add_argument("--cpu-timesteps", type=int, default=2)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--quick", action="store_true", help="reduced workload for smoke runs")
    ap.add_argument("--timesteps", type=int, default=0, help="override the workload's timestep count")
    ap.add_argument("--checkpoint", type=int, default=0,
                    help="override the workload's checkpoint interval (1: full tape, no recomputation)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--timed-profile", choices=("top", "all"), default="top",
                    help="kernels with CUDA events in the timed rollouts: the largest one (picked in the first "
                         "warm-up rollout; the full kernel table then comes from one more untimed rollout) or all")
    ap.add_argument("--profile-window", action="store_true",
                    help="start/stop an external profiler around the timed steps (ncu --profile-from-start off)")
    ap.add_argument("--tiles", default="", help="P2G,G2P-transpose,gather tile budgets instead of the autotuner")
    ap.add_argument("--deterministic", action="store_true",
                    help="fixed-point node sums (bitwise reproducible passes)")
    ap.add_argument("--no-det", action="store_true", help="morph500k: float atomics instead of fixed point")
    ap.add_argument("--shuffle", action="store_true", help="shuffle the particle order of the workload")
    ap.add_argument("--no-resort", action="store_true", help="keep the input particle order (no cell re-sort)")
    ap.add_argument("--resort-every", type=int, default=None,
                    help="re-sort inside the rollout every N layers (0 never; default: the library's choice)")
    ap.add_argument("--from-rollout", type=int, default=0,
                    help="start from the state after this many forward steps (drifted particle order)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
        line = run_reference(args, rank, world)
        if line:
            print(json.dumps(line), flush=True)
        return
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=device)
    import build_oracle  # noqa: F401  (oracle build for the CPU baseline happens lazily)
    if args.workload == "morph500k":
        if rank == 0:
            print(json.dumps(run_morph(args, device)), flush=True)
        return
    if args.workload == "render500k":
        if rank == 0:
            print(json.dumps(run_render(args, device)), flush=True)
        return
    line = run_ours(args, rank, world, device)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
