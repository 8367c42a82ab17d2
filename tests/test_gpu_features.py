"""GPU tests of the engine features around the step: checkpointed rollouts,
finite-difference gradients of the FP64 form, shared-tile vs global-atomic
scatter, the optional kernel/material, CompGraph semantics (render
gradients, optimisation, promotion), edge cases and the autograd rollout."""
import copy

import numpy as np
import pytest

import oracle as O
from helpers import get_grads, layer_state, make_graph, norm_err, oracle_rollout, rel_err, set_grads

pytestmark = pytest.mark.gpu


def _case(seed=0, G=12, rho=60.0, smoothing=0.0, drag=0.0):
    from diffmpm_bindings import workloads as W
    w = W.sphere32(seed=seed, G=G, rho=rho)
    rng = np.random.default_rng(seed)
    n = w.n
    s0 = O.State(w.x, w.v, 0.05 * rng.normal(size=(n, 3, 3)), np.eye(3) + 0.02 * rng.normal(size=(n, 3, 3)),
                 w.m, w.vol, w.lam, w.mu, 0.01 * rng.normal(size=(n, 3, 3)))
    g = O.Grid(w.dims, w.dx)
    return s0, g, rng, smoothing, drag


def _rollout(dm, s0, g, prm, T, seed_gx, precision, adjoint="exact", checkpoint_every=1, **kw):
    cg, keep = make_graph(dm, s0, g, prm, precision=precision, adjoint=adjoint, layers=T + 1,
                          checkpoint_every=checkpoint_every, **kw)
    cg.compute_forward_pass(0, 0)
    n = s0.n
    last = cg.get_point_cloud(T)
    last.set("grad_x", seed_gx)
    last.set("grad_v", np.zeros((n, 3)))
    last.set("grad_F", np.zeros((n, 3, 3)))
    last.set("grad_C", np.zeros((n, 3, 3)))
    cg.compute_backward_pass(0)
    xT = last.get("x", np.float64)
    g0 = get_grads(cg, 0)
    g0["dFc"] = cg.get_grad(0, "dFc", np.float64)
    return xT, g0, cg, keep


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_multistep_exact_matches_oracle(dm, orc, prec):
    s0, g, rng, sm, dr = _case(1, smoothing=0.2, drag=0.3)
    prm = O.Params(dt=1e-3, drag=dr, smoothing=sm, exact=True)
    T = 8
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    xT, g0, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, prec)
    xw, gw = oracle_rollout(orc, g, prm, s0, T, seed_gx)
    tol = 1e-9 if prec == "fp64" else 1e-5  # FP32 measured <= 9.1e-7
    assert rel_err(xT, xw) < (1e-10 if prec == "fp64" else 1e-6)
    for k, want in (("x", gw.x), ("v", gw.v), ("F", gw.F), ("C", gw.C), ("dFc", gw.Ft)):
        e = norm_err(g0[k], want)
        print(f"{prec} T={T} exact g{k} {e:.3e}")
        assert e < tol, (k, e)


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_checkpointed_equals_full_tape(dm, prec):
    s0, g, rng, _, _ = _case(2)
    prm = O.Params(dt=1e-3, drag=0.0, smoothing=0.0, exact=True)
    T = 12
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    x1, g1, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, prec, checkpoint_every=1)
    x4, g4, cg4, _ = _rollout(dm, s0, g, prm, T, seed_gx, prec, checkpoint_every=5)
    assert rel_err(x4, x1) < (1e-12 if prec == "fp64" else 1e-6)
    for k in ("x", "v", "F", "C", "dFc"):
        assert norm_err(g4[k], g1[k]) < (1e-10 if prec == "fp64" else 1e-4), k
    with pytest.raises(Exception):
        cg4.get_point_cloud(3).get("x")  # non-stored layer of a checkpointed graph


def test_fp64_exact_gradient_matches_finite_differences(dm):
    """Central differences (eps = 1e-4 scaled) along seeded directions."""
    s0, g, rng, _, _ = _case(3, smoothing=0.1, drag=0.2)
    prm = O.Params(dt=1e-3, drag=0.2, smoothing=0.1, exact=True)
    T = 4
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    _, g0, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, "fp64")

    def loss(s):
        cg, keep = make_graph(dm, s, g, prm, precision="fp64", adjoint="exact", layers=T + 1)
        cg.compute_forward_pass(0, 0)
        return float((cg.get_point_cloud(T).get("x", np.float64) * seed_gx).sum())

    for field, gkey, eps in (("v", "v", 1e-4), ("dFc", "dFc", 1e-5), ("x", "x", 1e-6)):
        for _ in range(3):
            d = rng.normal(size=getattr(s0, field).shape)
            sp, sm_ = copy.deepcopy(s0), copy.deepcopy(s0)
            setattr(sp, field, getattr(s0, field) + eps * d)
            setattr(sm_, field, getattr(s0, field) - eps * d)
            fd = (loss(sp) - loss(sm_)) / (2 * eps)
            an = float((g0[gkey] * d).sum())
            assert abs(an - fd) <= 1e-5 * abs(fd) + 1e-12, (field, an, fd)


@pytest.mark.parametrize("mode,tile", [(0, 0), (0, 2048), (1, 0), (1, 64)])
def test_scatter_strategies_agree(dm, mode, tile):
    """Segmented vs per-particle scatter, with and without the shared node
    tile (tile 64 forces the global-atomic fallback for most blocks)."""
    s0, g, rng, _, _ = _case(4, G=16)
    prm = O.Params(dt=1e-3, drag=0.0, smoothing=0.0, exact=True)
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    lib = dm._lib.lib
    xb, gb, _, _ = _rollout(dm, s0, g, prm, 3, seed_gx, "fp32")  # defaults: segmented, no tile
    try:
        lib.mpm_set_scatter_mode(mode)
        lib.mpm_set_tile_nodes(tile)
        xa, ga, _, _ = _rollout(dm, s0, g, prm, 3, seed_gx, "fp32")
    finally:
        lib.mpm_set_scatter_mode(1)
        lib.mpm_set_tile_nodes(0)
    assert rel_err(xa, xb) < 1e-6
    for k in ("x", "v", "F"):
        assert norm_err(ga[k], gb[k]) < 1e-4, k


def test_unsorted_particles(dm, orc):
    """Shuffled particle order (segments of length one) gives the same step."""
    s0, g, rng, _, _ = _case(10, G=12)
    perm = rng.permutation(s0.n)
    sp = O.State(s0.x[perm], s0.v[perm], s0.C[perm], s0.F[perm], s0.m[perm], s0.vol[perm], s0.lam[perm],
                 s0.mu[perm], s0.dFc[perm])
    prm = O.Params(dt=1e-3, drag=0.0, smoothing=0.0)
    for resort in (False, True):  # shuffled slots, and re-sorted by cell behind the caller's order
        cg, keep = make_graph(dm, sp, g, prm, precision="fp32", layers=2, resort=resort)
        cg.compute_forward_pass(0, 0)
        want, _ = orc.forward_step(g, prm, sp)
        got = layer_state(cg, 1)
        assert rel_err(got["x"], want.x) < 1e-6 and rel_err(got["C"], want.C) < 1e-4


@pytest.mark.parametrize("kernel,material", [("quadratic", "fcr"), ("cubic", "neohookean"), ("quadratic", "neohookean")])
def test_optional_kernel_and_material(dm, orc, kernel, material):
    s0, g, rng, _, _ = _case(5)
    kid = {"cubic": 0, "quadratic": 1}[kernel]
    mid = {"fcr": 0, "neohookean": 1}[material]
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.0, exact=True, kernel=kid, material=mid)
    T = 4
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    xT, g0, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, "fp64", kernel=kernel, material=material)
    xw, gw = oracle_rollout(orc, g, prm, s0, T, seed_gx)
    assert rel_err(xT, xw) < 1e-10
    for k, want in (("x", gw.x), ("v", gw.v), ("dFc", gw.Ft)):
        assert norm_err(g0[k], want) < 1e-9, k


def test_particles_at_grid_boundary(dm, orc):
    """Stencils that leave the grid: out-of-range nodes are skipped (reference
    behaviour, ForwardSimulation.cpp:47-49); a ragged particle count."""
    rng = np.random.default_rng(6)
    n = 257
    x = rng.uniform(0.0, 1.0, size=(n, 3))
    x[:20] = rng.uniform(0.0, 0.03, size=(20, 3))
    x[20:40] = rng.uniform(0.97, 1.0, size=(20, 3))
    s0 = O.State(x, 0.3 * rng.normal(size=(n, 3)), 0.1 * rng.normal(size=(n, 3, 3)),
                 np.eye(3) + 0.02 * rng.normal(size=(n, 3, 3)), np.full(n, 1e-3), np.full(n, 1e-4),
                 np.full(n, 50.0), np.full(n, 30.0))
    g = O.Grid((9, 9, 9), 1.0 / 8)
    prm = O.Params(dt=1e-3, drag=0.0, smoothing=0.0, exact=False)
    for prec in ("fp64", "fp32"):
        cg, keep = make_graph(dm, s0, g, prm, precision=prec)
        cg.compute_forward_pass(0, 0)
        got = layer_state(cg, 1)
        want, step = orc.forward_step(g, prm, s0)
        assert rel_err(got["x"], want.x) < (1e-12 if prec == "fp64" else 1e-6)
        assert rel_err(got["v"], want.v) < (1e-10 if prec == "fp64" else 1e-4)
        g1 = O.Grads(rng.normal(size=(n, 3)), rng.normal(size=(n, 3)), rng.normal(size=(n, 3, 3)),
                     rng.normal(size=(n, 3, 3)))
        set_grads(cg, 1, g1)
        cg.compute_backward_pass(0)
        gb = orc.backward_step(g, prm, s0, want.C, step, g1)
        assert norm_err(get_grads(cg, 0)["x"], gb.x) < (1e-9 if prec == "fp64" else 2e-3)


def test_empty_point_cloud(dm):
    pc = dm.PointCloud.create(0)
    grid = dm.Grid(4, 4, 4, 0.25, (0, 0, 0))
    cg = dm.CompGraph(pc, grid, grid)
    cg.set_up_comp_graph(3)
    cg.compute_forward_pass(0, 0)
    cg.compute_backward_pass(0)
    assert cg.get_point_cloud(2).get_positions().shape == (0, 3)
    loss = cg.end_layer_mass_loss()
    assert np.isfinite(loss)


def test_compgraph_surface(dm, orc):
    """CompGraph semantics of bind.cpp: layers, IndexError, render gradients,
    optimisation steps, promotion."""
    s0, g, rng, _, _ = _case(7, G=12)
    prm = O.Params(dt=1e-3, drag=0.5, smoothing=0.1)
    tgt = np.zeros(g.n_nodes)
    orc.p2g_accumulate(g, s0.x + 0.02, s0.v, s0.C, s0.m, tgt, np.zeros((g.n_nodes, 3)))
    cg, keep = make_graph(dm, s0, g, prm, precision="fp32", layers=5, target_mass=tgt)
    assert cg.get_num_layers() == 5
    with pytest.raises(IndexError):
        cg.get_point_cloud(5)
    with pytest.raises(IndexError):
        cg.get_point_cloud_at_timestep(7)
    cg.compute_forward_pass(0, 0)
    l0 = cg.end_layer_mass_loss()
    n = s0.n
    assert not cg.has_render_gradients()
    dF, dx = 1e-3 * rng.normal(size=(n, 3, 3)).astype(np.float32), 1e-3 * rng.normal(size=(n, 3)).astype(np.float32)
    cg.set_render_gradients(dF, dx)
    info = cg.get_render_gradient_info()
    assert info["has_gradients"] and info["num_points"] == n
    assert abs(info["grad_F_norm"] - np.linalg.norm(dF)) < 1e-4 * np.linalg.norm(dF)
    cg.compute_backward_pass(0)
    # render gradients were added to the last layer's loss gradient
    last_gx = cg.get_grad(4, "x", np.float64)
    _, d = orc.mass_loss(g, O.Params(), cg.get_point_cloud(4).get("x", np.float64), s0.m, tgt)
    assert norm_err(last_gx, d["gx"] + dx) < 1e-4
    with pytest.raises(RuntimeError, match="dLdF must be"):
        cg.set_render_gradients(np.zeros((n, 3)), dx)
    with pytest.raises(RuntimeError, match="Shape mismatch"):
        cg.accumulate_render_grads(dF[:-1], dx[:-1])
    cg.clear_render_gradients()
    assert not cg.has_render_gradients()
    # one optimisation step at layer 0 must not increase the loss
    cg.optimize_single_timestep(0, max_gd_iters=1, initial_alpha=0.01, max_line_search_iters=6)
    cg.compute_forward_pass(0, 0)
    l1 = cg.end_layer_mass_loss()
    assert l1 <= l0 + 1e-7
    assert np.abs(cg.get_point_cloud(0).get_def_grads_morph()).max() > 0  # dFc moved
    F_tot = cg.get_point_cloud(0).get_def_grads_total()
    assert rel_err(F_tot, cg.get_point_cloud(0).get_def_grads() + cg.get_point_cloud(0).get_def_grads_morph()) < 1e-6
    # invalid index: message and return, no raise (CompGraph.cpp:377-380)
    cg.optimize_single_timestep(99)
    x_last = cg.get_point_cloud(4).get_positions()
    cg.promote_last_as_initial()
    assert cg.get_num_layers() == 1
    assert rel_err(cg.get_point_cloud(0).get_positions(), x_last) == 0.0


def test_run_optimization_reduces_loss(dm, orc):
    s0, g, rng, _, _ = _case(8, G=12)
    tgt = np.zeros(g.n_nodes)
    orc.p2g_accumulate(g, s0.x + np.array([0.03, 0.0, 0.0]), s0.v, s0.C, s0.m, tgt, np.zeros((g.n_nodes, 3)))
    prm = O.Params(dt=1e-3, drag=0.5, smoothing=0.1)
    cg, keep = make_graph(dm, s0, g, prm, precision="fp32", layers=1, target_mass=tgt)
    opt = dm.OptInput()
    opt.num_timesteps, opt.control_stride, opt.max_gd_iters, opt.max_ls_iters = 4, 2, 1, 4
    opt.dt, opt.drag, opt.smoothing_factor, opt.initial_alpha, opt.gd_tol = 1e-3, 0.5, 0.1, 0.01, 1e-4
    cg.set_up_comp_graph(4)
    cg.set_sim_params(dt=1e-3, drag=0.5, smoothing=0.1)
    cg.compute_forward_pass(0, 0)
    before = cg.end_layer_mass_loss()
    cg.run_optimization(opt)
    cg.compute_forward_pass(0, 0)
    after = cg.end_layer_mass_loss()
    assert after <= before + 1e-7


def test_autograd_rollout(dm):
    torch = pytest.importorskip("torch")
    from diffmpm_bindings.rollout import Rollout, mpm_rollout
    from diffmpm_bindings import workloads as W
    w = W.sphere32(seed=9, G=12, rho=60.0)
    dev = torch.device("cuda")
    sim = Rollout(w.n, w.dims, w.dx, steps=4, m=w.m[0], vol=w.vol[0], nu=0.3, dt=1e-3, precision="fp64",
                  checkpoint_every=2)
    x0 = torch.tensor(w.x, device=dev, requires_grad=True)
    v0 = torch.tensor(w.v, device=dev, requires_grad=True)
    F0 = torch.eye(3, dtype=torch.float64, device=dev).expand(w.n, 3, 3).contiguous().requires_grad_(True)
    dFc = torch.zeros((w.n, 3, 3), dtype=torch.float64, device=dev, requires_grad=True)
    E = torch.tensor(1e4, dtype=torch.float64, device=dev, requires_grad=True)
    tgt = x0.detach() + 0.01
    xT, FT = mpm_rollout(x0, v0, F0, dFc, E, sim)
    loss = ((xT - tgt) ** 2).mean() + 0.1 * ((FT - torch.eye(3, dtype=torch.float64, device=dev)) ** 2).mean()
    loss.backward()
    for t in (x0, v0, F0, dFc):
        assert t.grad is not None and torch.isfinite(t.grad).all()
    # dL/dE against central differences of the same rollout
    eps = 1.0

    def L(Ev):
        with torch.no_grad():
            a, b = mpm_rollout(x0.detach(), v0.detach(), F0.detach(), dFc.detach(), torch.tensor(Ev, dtype=torch.float64, device=dev), sim)
            return float((((a - tgt) ** 2).mean() + 0.1 * ((b - torch.eye(3, dtype=torch.float64, device=dev)) ** 2).mean()))
    fd = (L(1e4 + eps) - L(1e4 - eps)) / (2 * eps)
    assert abs(float(E.grad) - fd) <= 1e-4 * abs(fd) + 1e-14, (float(E.grad), fd)


@pytest.mark.parametrize("checkpoint_every", [1, 4])
def test_graph_replay_matches_eager(dm, checkpoint_every):
    """Forward/backward passes replayed from CUDA graphs equal eager passes;
    changing a control (dFc of layer 0) re-records."""
    s0, g, rng, _, _ = _case(11, G=12)
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.1, exact=True)
    T = 8
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n

    def run(cg):
        out = []
        for rep in range(5):  # eager, eager (allocations settle), record, replay, new control
            if rep == 4:
                cg.get_point_cloud(0).set("dFc", 0.02 * np.ones((s0.n, 3, 3)))
            cg.compute_forward_pass(0, 0)
            last = cg.get_point_cloud(T)
            last.set("grad_x", seed_gx)
            last.set("grad_v", np.zeros((s0.n, 3)))
            last.set("grad_F", np.zeros((s0.n, 3, 3)))
            last.set("grad_C", np.zeros((s0.n, 3, 3)))
            cg.compute_backward_pass(0)
            out.append((last.get("x", np.float64), cg.get_grad(0, "dFc", np.float64)))
        return out

    cg_a, ka = make_graph(dm, s0, g, prm, precision="fp64", adjoint="exact", layers=T + 1,
                          checkpoint_every=checkpoint_every)
    cg_b, kb = make_graph(dm, s0, g, prm, precision="fp64", adjoint="exact", layers=T + 1,
                          checkpoint_every=checkpoint_every)
    cg_b.use_graphs(False)
    ra, rb = run(cg_a), run(cg_b)
    for (xa, ga), (xb, gb) in zip(ra, rb):
        assert rel_err(xa, xb) < 1e-12 and norm_err(ga, gb) < 1e-10
    assert rel_err(ra[3][0], ra[2][0]) < 1e-12  # replay == recording run
    assert rel_err(ra[4][0], ra[3][0]) > 1e-9  # the dFc change took effect


def test_profiler_counts_graph_replays(dm):
    s0, g, rng, _, _ = _case(12, G=10)
    prm = O.Params(dt=1e-3, drag=0.0, smoothing=0.0)
    T = 3
    cg, keep = make_graph(dm, s0, g, prm, precision="fp32", layers=T + 1)
    lib = dm._lib.lib
    import ctypes as C
    for _ in range(3):
        cg.compute_forward_pass(0, 0)
    lib.mpm_profile_reset()
    lib.mpm_profile_enable(1)
    try:
        for _ in range(4):  # eager, record, replay, replay
            cg.compute_forward_pass(0, 0)
        cnt, ms, cnt2, ms2 = C.c_longlong(), C.c_double(), C.c_longlong(), C.c_double()
        lib.mpm_profile_query(0, C.byref(cnt), C.byref(ms))  # p2g
        lib.mpm_profile_query(10, C.byref(cnt2), C.byref(ms2))  # g2p2g: G2P fused with the next P2G
    finally:
        lib.mpm_profile_enable(0)
    # every step's P2G ran once per pass: the first on its own, the others
    # inside the fused G2P -> P2G kernel
    assert cnt.value == 4 and cnt2.value == 4 * (T - 1) and ms.value > 0 and ms2.value > 0
    # the launch counter counts kernels: P2G, then per step the grid update
    # and the fused kernel (plain G2P for the last step)
    n0 = lib.mpm_launch_count()
    cg.compute_forward_pass(0, 0)
    assert lib.mpm_launch_count() - n0 == 2 * T + 1


def test_autotune_picks_a_valid_configuration(dm, orc):
    s0, g, rng, _, _ = _case(13, G=12)
    prm = O.Params(dt=1e-3, drag=0.0, smoothing=0.0)
    cg, keep = make_graph(dm, s0, g, prm, precision="fp32", layers=3)
    res = cg.autotune(steps=2)
    assert res["tile_nodes"] in (0, 512, 1024, 2048) and res["scatter_mode"] in (0, 1) and res["ms_per_pass"] > 0
    assert res["adj_tile_nodes"] in (0, 512, 1024, 2048) and res["gather_tile_nodes"] in (1024, 2048, 2816)
    assert res["block_threads"] in (128, 256)
    assert cg.get_tuning() == {k: res[k] for k in ("tile_nodes", "scatter_mode", "adj_tile_nodes",
                                                   "gather_tile_nodes", "block_threads")}
    cg.compute_forward_pass(0, 0)
    want, _ = orc.forward_step(g, prm, s0)
    assert rel_err(cg.get_point_cloud(1).get("x", np.float64), want.x) < 1e-6


def test_autotune_from_a_stored_layer(dm):
    s0, g, rng, _, _ = _case(13, G=12)
    prm = O.Params(dt=1e-3, drag=0.0, smoothing=0.0)
    cg, keep = make_graph(dm, s0, g, prm, precision="fp32", layers=5, checkpoint_every=2)
    cg.compute_forward_pass(0, 0)
    res = cg.autotune(steps=2, layer=2)
    assert res["from_layer"] == 2 and res["tile_nodes"] in (0, 512, 1024, 2048) and res["ms_per_pass"] > 0
    with pytest.raises(IndexError):
        cg.autotune(steps=2, layer=9)
    with pytest.raises(RuntimeError, match="no state"):  # layer 3 is not stored (checkpoint every 2)
        cg.autotune(steps=2, layer=3)


def test_adjoint_tile_budgets_change_no_result(dm):
    """The adjoint kernels' own tile budgets (or tiles off): the P2G
    transpose's gather reads the same node values from the tile as from
    global memory, and the G2P transpose's fixed-point scatter sums the same
    integers, so the gradients are identical."""
    s0, g, rng, _, _ = _case(15, G=12)
    prm = O.Params(dt=1e-3, drag=0.1, smoothing=0.1, exact=True)
    T = 3
    seed = rng.normal(size=(s0.n, 3)) / s0.n
    outs = []
    for at, gt in ((-1, -1), (0, 0), (512, 64), (2048, 2816)):
        cg, keep = make_graph(dm, s0, g, prm, precision="fp32", adjoint="exact", layers=T + 1,
                              deterministic=True)
        cg.set_tuning(1024, 1, at, gt)
        tun = cg.get_tuning()
        assert (tun["adj_tile_nodes"], tun["gather_tile_nodes"]) == (1024 if at < 0 else at, 2048 if gt < 0 else gt)
        cg.compute_forward_pass(0, 0)
        last = cg.get_point_cloud(T)
        last.set("grad_x", seed)
        cg.compute_backward_pass(0)
        outs.append({k: cg.get_grad(0, k, np.float32) for k in ("x", "v", "F", "C", "dFc")})
    for o in outs[1:]:
        for k in o:
            assert np.array_equal(o[k], outs[0][k]), k
    assert dm._lib.lib.mpm_compgraph_set_adjoint_tiles(cg._h, 5000, -1) == dm._lib.MPM_ERR_ARG


def test_nonfinite_state_is_flagged_not_fatal(dm):
    """A NaN injected on the host flows through a pass without faulting and is
    reported by the state check; a clean state is not flagged."""
    s0, g, rng, _, _ = _case(14, G=10)
    prm = O.Params(dt=1e-3, drag=0.0, smoothing=0.0)
    T = 3
    cg, keep = make_graph(dm, s0, g, prm, precision="fp32", layers=T + 1)
    cg.compute_forward_pass(0, 0)
    assert not cg.has_nonfinite(T)
    v = s0.v.copy()
    v[7, 1] = np.nan
    cg.get_point_cloud(0).set("v", v)
    cg.compute_forward_pass(0, 0)
    assert cg.has_nonfinite(T) and cg.has_nonfinite(0)
    v[7, 1] = 0.0
    cg.get_point_cloud(0).set("v", v)
    cg.compute_forward_pass(0, 0)
    assert not cg.has_nonfinite(T)


@pytest.mark.parametrize("checkpoint_every", [1, 5])
def test_fused_forward_steps_agree_with_step_by_step(dm, orc, checkpoint_every):
    """Forward passes run each step's G2P fused with the next step's P2G
    (k_g2p2g): the same computation as the three kernels step by step, so
    the two agree to the order of the float atomics, and both match the
    oracle; full tape and checkpointed (where the scratch grids alternate)."""
    s0, g, rng, _, _ = _case(6, G=16, smoothing=0.1, drag=0.2)
    prm = O.Params(dt=1e-3, drag=0.2, smoothing=0.1, exact=True)
    T = 12
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    lib = dm._lib.lib
    xf, gf, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, "fp32", checkpoint_every=checkpoint_every)
    try:
        assert lib.mpm_set_fused_steps(0) == 0
        xs, gs, _, _ = _rollout(dm, s0, g, prm, T, seed_gx, "fp32", checkpoint_every=checkpoint_every)
    finally:
        lib.mpm_set_fused_steps(1)
    xw, gw = oracle_rollout(orc, g, prm, s0, T, seed_gx)
    assert rel_err(xf, xs) < 1e-6 and rel_err(xf, xw) < 1e-6
    for k, want in (("x", gw.x), ("v", gw.v), ("F", gw.F), ("C", gw.C), ("dFc", gw.Ft)):
        assert norm_err(gf[k], gs[k]) < 1e-5, k
        assert norm_err(gf[k], want) < 2e-4, k


@pytest.mark.parametrize("deterministic", [False, True])
def test_block_threads_128_matches_256(dm, orc, deterministic):
    """The step kernels at 128 threads (and particles) per block give the
    same results as at 256 (bit for bit with the fixed-point scatters) and
    match the oracle."""
    s0, g, rng, _, _ = _case(8, G=14, smoothing=0.1, drag=0.2)
    prm = O.Params(dt=1e-3, drag=0.2, smoothing=0.1, exact=True)
    T = 6
    seed_gx = rng.normal(size=(s0.n, 3)) / s0.n
    out = {}
    for threads in (256, 128):
        cg, keep = make_graph(dm, s0, g, prm, precision="fp32", adjoint="exact", layers=T + 1, checkpoint_every=3,
                              deterministic=deterministic)
        cg.set_tuning(block_threads=threads)
        assert cg.get_tuning()["block_threads"] == threads
        cg.compute_forward_pass(0, 0)
        last = cg.get_point_cloud(T)
        last.set("grad_x", seed_gx)
        cg.compute_backward_pass(0)
        out[threads] = (last.get("x", np.float64), get_grads(cg, 0), cg.get_grad(0, "dFc", np.float64))
    xw, gw = oracle_rollout(orc, g, prm, s0, T, seed_gx)
    (xa, ga, ca), (xb, gb, cb) = out[256], out[128]
    if deterministic:
        assert np.array_equal(xa, xb) and np.array_equal(ca, cb)
        for k in ga:
            assert np.array_equal(ga[k], gb[k]), k
    assert rel_err(xb, xw) < 1e-6 and norm_err(cb, gw.Ft) < 2e-4
    for k, want in (("x", gw.x), ("v", gw.v), ("F", gw.F), ("C", gw.C)):
        assert norm_err(gb[k], want) < 2e-4, k
