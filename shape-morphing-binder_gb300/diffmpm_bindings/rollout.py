"""torch.autograd.Function over a differentiable MPM rollout.

``Rollout`` owns a CompGraph (exact adjoint, optional checkpointing) and
moves CUDA tensors in and out through the C ABI without host copies.
``mpm_rollout(x0, v0, F0, dFc0, E, sim)`` returns (x_T, F_T) and
backpropagates to x0, v0, F0, the layer-0 control dFc0 and the scalar
Young's modulus E, so losses computed in torch (render losses, position
losses) reach the physics directly.  This replaces the reference's
CPU-tensor -> numpy -> set_render_gradients round trip
(bind.cpp:89-131,359-451; run.py:767-883) for device-resident callers.
"""
from __future__ import annotations

import numpy as np
import torch

from . import CompGraph, Grid, PointCloud


class Rollout:
    """A fixed-size simulation: N particles, a grid, T steps."""

    def __init__(self, n, dims, dx, grid_min=(0.0, 0.0, 0.0), *, steps, m, vol, nu, dt, drag=0.0, smoothing=0.0,
                 f_ext=(0.0, 0.0, 0.0), checkpoint_every=1, precision="fp32", kernel="cubic", material="fcr"):
        self.n, self.T = int(n), int(steps)
        self.nu = float(nu)
        self.precision = precision
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        npdt = np.float64 if precision == "fp64" else np.float32
        pc = PointCloud.create(self.n, precision)
        pc.set("m", np.broadcast_to(np.asarray(m, npdt), (self.n,)).copy())
        pc.set("vol", np.broadcast_to(np.asarray(vol, npdt), (self.n,)).copy())
        self.grid = Grid(*dims, dx, grid_min, precision=precision)
        self.cg = CompGraph(pc, self.grid, self.grid, adjoint="exact", kernel=kernel, material=material,
                            checkpoint_every=checkpoint_every)
        self.cg.set_sim_params(dt=dt, drag=drag, smoothing=smoothing, f_ext=f_ext)
        self.cg.set_up_comp_graph(self.T + 1)
        self.cg.enable_lame_grads(True)

    def _lame(self, E):
        nu = self.nu
        return E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 + 2 * nu)

    def load(self, x0, v0, F0, dFc0, E):
        l0 = self.cg.get_point_cloud(0)
        dev = x0.device
        for name, t in (("x", x0), ("v", v0), ("F", F0)):
            l0.set(name, t.detach().to(self.dtype).contiguous())
        if dFc0 is not None:
            l0.set("dFc", dFc0.detach().to(self.dtype).contiguous())
        lam, mu = self._lame(float(E))
        l0.set("lam", torch.full((self.n,), lam, dtype=self.dtype, device=dev))
        l0.set("mu", torch.full((self.n,), mu, dtype=self.dtype, device=dev))

    def forward(self, device):
        torch.cuda.current_stream(device).synchronize()
        self.cg.compute_forward_pass(0, 0)
        last = self.cg.get_point_cloud(self.T)
        return last.get_torch("x", device, self.dtype), last.get_torch("F", device, self.dtype)

    def backward(self, gx, gF, device):
        last = self.cg.get_point_cloud(self.T)
        z3 = torch.zeros((self.n, 3), dtype=self.dtype, device=device)
        z9 = torch.zeros((self.n, 3, 3), dtype=self.dtype, device=device)
        last.set("grad_x", (gx if gx is not None else z3).to(self.dtype).contiguous())
        last.set("grad_F", (gF if gF is not None else z9).to(self.dtype).contiguous())
        last.set("grad_v", z3)
        last.set("grad_C", z9)
        self.cg.compute_backward_pass(0)
        l0 = self.cg.get_point_cloud(0)
        out = {k: l0.get_torch("grad_" + k, device, self.dtype) for k in ("x", "v", "F", "dFc", "lam", "mu")}
        nu = self.nu
        dlam, dmu = nu / ((1 + nu) * (1 - 2 * nu)), 1.0 / (2 + 2 * nu)
        out["E"] = (out["lam"].sum() * dlam + out["mu"].sum() * dmu).reshape(())
        return out


class _RolloutFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, F0, dFc0, E, sim):
        sim.load(x0, v0, F0, dFc0, E)
        xT, FT = sim.forward(x0.device)
        ctx.sim = sim
        ctx.device = x0.device
        ctx.has_dfc = dFc0 is not None
        return xT, FT

    @staticmethod
    def backward(ctx, gxT, gFT):
        g = ctx.sim.backward(gxT, gFT, ctx.device)
        gE = g["E"].to(torch.float64)
        return g["x"], g["v"], g["F"], (g["dFc"] if ctx.has_dfc else None), gE, None


def mpm_rollout(x0, v0, F0, dFc0, E, sim: Rollout):
    """(x_T, F_T) = rollout(x0, v0, F0, dFc0, E); differentiable in all five.

    ``E`` is a 0-d tensor (float64 recommended).  The tensors must live on the
    CUDA device the simulation runs on.
    """
    if not torch.is_tensor(E):
        E = torch.tensor(float(E), dtype=torch.float64, device=x0.device)
    return _RolloutFn.apply(x0, v0, F0, dFc0, E, sim)
