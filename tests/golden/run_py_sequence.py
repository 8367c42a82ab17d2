"""run.py's physics-only call sequence, written once against the module API.

``physics_episodes(dmb, cfg, workdir)`` makes the calls run.py makes when it
optimises physics only (no renderer), with the same arguments, on whatever
module ``dmb`` is:

* build_opt_input (run.py:318-349): OptInput and its fields from the
  config's ``simulation`` / ``optimization`` sections;
* initialize_point_clouds (run.py:355-359): load_point_cloud_from_obj for
  the input and the target mesh;
* initialize_grids (run.py:362-379): two Grids of
  int((max - min) / dx) + 1 nodes per axis;
* calculate_point_cloud_volumes on both (run.py:1278-1279), which also
  leaves each cloud's mass in its grid -- the target grid's masses are the
  loss target;
* initialize_comp_graph (run.py:382-387) and get_positions_from_pc of the
  target (run.py:1284);
* the episode loop (run.py:1340-1364): opt.current_episodes = ep,
  run_optimization(opt), promote_last_as_initial() between episodes.

After each episode it records, through the same API, what a caller can
read: the number of layers, every layer's control (get_def_grads_morph),
the last layer's positions (get_positions) and end_layer_mass_loss().

Run as a script (where the reference tree is present: REF_DIR), it builds
the reference's own pybind11 module from its sources (oracle/build_oracle.py,
float as shipped and widened to double), runs the sequence on each in a
fresh process, and writes tests/golden/reference_run_py.npz.  The meshes
are procedural (an ellipsoid and a displaced one), written as OBJ files to
a temporary directory; every configuration value, mesh vertex and lattice
point is exactly representable in float32, so both builds and both engine
precisions start from the same numbers.  tests/test_gpu_run_py.py makes the
identical call sequence through this repository's diffmpm_bindings.

Usage: REF_DIR=<reference checkout> python tests/golden/run_py_sequence.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent
ROOT = OUT.parents[1]

# run.py's config sections; values exact in float32 (dt = 2^-10, dx = 1/16)
CONFIG = {
    "simulation": {"grid_dx": 0.0625, "grid_min_point": [0.0, 0.0, 0.0], "grid_max_point": [1.0, 1.0, 1.0],
                   "points_per_cell_cuberoot": 2, "lam": 5769.0, "mu": 3846.0, "density": 64.0,
                   "dt": 0.0009765625, "drag": 0.5, "external_force": [0.0, -9.75, 0.0],
                   "smoothing_factor": 0.125},
    "optimization": {"num_animations": 2, "num_timesteps": 7, "control_stride": 2, "max_gd_iters": 2,
                     "max_ls_iters": 4, "initial_alpha": 0.0625, "gd_tol": 0.0001220703125},
}


def ellipsoid_mesh(centre, axes, nu=40, nv=20):
    """Closed outward-facing triangle mesh of an ellipsoid, float32 vertices."""
    c, a = np.asarray(centre, np.float64), np.asarray(axes, np.float64)
    V = [c + a * [0, 0, 1]]
    for i in range(1, nv):
        th = np.pi * i / nv
        for j in range(nu):
            ph = 2 * np.pi * j / nu
            V.append(c + a * [np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)])
    V.append(c + a * [0, 0, -1])
    ring = lambda i, j: 1 + (i - 1) * nu + (j % nu)  # noqa: E731
    F = [[0, ring(1, j), ring(1, j + 1)] for j in range(nu)]
    for i in range(1, nv - 1):
        for j in range(nu):
            F.append([ring(i, j), ring(i + 1, j), ring(i + 1, j + 1)])
            F.append([ring(i, j), ring(i + 1, j + 1), ring(i, j + 1)])
    last = len(V) - 1
    F += [[last, ring(nv - 1, j + 1), ring(nv - 1, j)] for j in range(nu)]
    return np.asarray(V, np.float32), np.asarray(F, np.int64)


def write_obj(path: Path, V, F):
    """Wavefront OBJ; each float32 vertex coordinate printed exactly."""
    with open(path, "w") as f:
        for v in V:
            f.write("v %r %r %r\n" % tuple(float(x) for x in v))
        for t in F:
            f.write("f %d %d %d\n" % tuple(int(i) + 1 for i in t))


def write_meshes(workdir: Path):
    """The input ellipsoid and the target (the same shape moved and
    stretched); the bounding-box corners are float32-exact so the sampling
    lattice (corner + i * dx / 2) is too."""
    workdir.mkdir(parents=True, exist_ok=True)
    src, tgt = workdir / "input.obj", workdir / "target.obj"
    write_obj(src, *ellipsoid_mesh((0.5, 0.5, 0.5), (0.1875, 0.15625, 0.125)))
    write_obj(tgt, *ellipsoid_mesh((0.53125, 0.5, 0.515625), (0.21875, 0.140625, 0.125)))
    return str(src), str(tgt)


def physics_episodes(dmb, cfg: dict, workdir: Path) -> dict:
    """run.py's physics-only sequence on module ``dmb``; returns per-episode
    records (see the module docstring)."""
    src, tgt = write_meshes(Path(workdir))
    sim, run = cfg["simulation"], cfg["optimization"]
    # build_opt_input (run.py:318-349)
    opt = dmb.OptInput()
    opt.mpm_input_mesh_path = src
    opt.mpm_target_mesh_path = tgt
    opt.grid_dx = float(sim["grid_dx"])
    opt.grid_min_point = sim["grid_min_point"]
    opt.grid_max_point = sim["grid_max_point"]
    opt.points_per_cell_cuberoot = int(sim.get("points_per_cell_cuberoot", 2))
    opt.lam = float(sim["lam"])
    opt.mu = float(sim["mu"])
    opt.p_density = float(sim["density"])
    opt.dt = float(sim["dt"])
    opt.drag = float(sim["drag"])
    opt.f_ext = sim["external_force"]
    opt.smoothing_factor = float(sim["smoothing_factor"])
    opt.num_animations = int(run["num_animations"])
    opt.num_timesteps = int(run["num_timesteps"])
    opt.control_stride = int(run["control_stride"])
    opt.max_gd_iters = int(run["max_gd_iters"])
    opt.max_ls_iters = int(run["max_ls_iters"])
    opt.initial_alpha = float(run["initial_alpha"])
    opt.gd_tol = float(run["gd_tol"])
    opt.current_episodes = 0
    # initialize_point_clouds (run.py:355-359)
    input_pc = dmb.load_point_cloud_from_obj(opt.mpm_input_mesh_path, opt)
    target_pc = dmb.load_point_cloud_from_obj(opt.mpm_target_mesh_path, opt)
    # initialize_grids (run.py:362-379)
    dims = [int((opt.grid_max_point[i] - opt.grid_min_point[i]) / opt.grid_dx) + 1 for i in range(3)]
    input_grid = dmb.Grid(dims[0], dims[1], dims[2], opt.grid_dx, opt.grid_min_point)
    target_grid = dmb.Grid(dims[0], dims[1], dims[2], opt.grid_dx, opt.grid_min_point)
    # run.py:1278-1279, 382-387, 1284
    dmb.calculate_point_cloud_volumes(input_pc, input_grid)
    dmb.calculate_point_cloud_volumes(target_pc, target_grid)
    cg = dmb.CompGraph(input_pc, input_grid, target_grid)
    tgt_x = np.asarray(dmb.get_positions_from_pc(target_pc), np.float64)
    rec = {"n_input": len(np.asarray(input_pc.get_positions())), "n_target": len(tgt_x),
           "input_x": np.asarray(input_pc.get_positions(), np.float64),
           "input_m": np.asarray(input_pc.get_masses(), np.float64)}
    # the episode loop (run.py:1340-1364), physics only
    for ep in range(int(opt.num_animations)):
        opt.current_episodes = ep
        cg.run_optimization(opt)
        L = cg.get_num_layers()
        rec[f"ep{ep}_layers"] = L
        rec[f"ep{ep}_dFc"] = np.stack([np.asarray(cg.get_point_cloud(i).get_def_grads_morph(), np.float64)
                                       for i in range(L)])
        rec[f"ep{ep}_xT"] = np.asarray(cg.get_point_cloud(L - 1).get_positions(), np.float64)
        rec[f"ep{ep}_loss"] = float(cg.end_layer_mass_loss())
        if ep < int(opt.num_animations) - 1:
            cg.promote_last_as_initial()
    return rec


def _run_reference(bits: int, out: Path):
    """One fresh process per build: import the reference module built from
    source (oracle/_ref/pymod{32,64}) and run the sequence."""
    import contextlib
    import io
    import os
    import tempfile
    sys.path.insert(0, str(ROOT / "oracle" / "_ref" / f"pymod{bits}"))
    import diffmpm_bindings as ref  # the reference's own module
    assert "_ref" in ref.__file__, ref.__file__
    with tempfile.TemporaryDirectory() as tmp:
        # the module prints progress to stdout (fd 1) from C++: keep it out
        fd = os.dup(1)
        with open(os.devnull, "w") as null, contextlib.redirect_stdout(io.StringIO()):
            os.dup2(null.fileno(), 1)
            try:
                rec = physics_episodes(ref, CONFIG, Path(tmp))
            finally:
                os.dup2(fd, 1)
                os.close(fd)
    np.savez(out, **{f"ref{bits}_{k}": v for k, v in rec.items()})
    print(bits, {k: v for k, v in rec.items() if k.endswith("loss") or k.startswith("n_")})


def main():
    import subprocess
    sys.path.insert(0, str(ROOT / "oracle"))
    import build_oracle
    for widen in (False, True):
        if build_oracle.build_ref_module(widen) is None:
            raise SystemExit("reference tree (REF_DIR) or pybind11 not found")
    rec = {}
    for bits in (32, 64):
        part = OUT / f"_run_py_{bits}.npz"
        subprocess.check_call([sys.executable, __file__, "--bits", str(bits), "--out", str(part)])
        rec.update(np.load(part))
        part.unlink()
    np.savez_compressed(OUT / "reference_run_py.npz", **rec)
    print("wrote", OUT / "reference_run_py.npz")


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--bits", type=int, choices=[32, 64])
    ap.add_argument("--out")
    a = ap.parse_args()
    if a.bits:
        _run_reference(a.bits, Path(a.out))
    else:
        main()
