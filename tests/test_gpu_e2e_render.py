"""End-to-end mode on the device (run.py:767-883 does this through CPU
tensors, numpy and set_render_gradients): the particles of a differentiable
MPM rollout are rendered as Gaussians (means = x_T, covariance
F_T Sigma0 F_T^T, the diff_gauss precomputed-covariance path), an image
loss is taken in torch, and its gradient flows back through the rasterizer's
adjoint into the rollout's adjoint to the initial velocity and the layer-0
control.  Checked against central finite differences of the same pipeline
with the FP64 rollout and the dense float64 renderer (tests/gs_reference.py)
along seeded directions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _pipeline(dm, w, T, H, W, cam, target):
    from diffmpm_bindings.rollout import Rollout
    sim = Rollout(w.n, w.dims, w.dx, steps=T, m=w.m[0], vol=w.vol[0], nu=w.extra["nu"], dt=w.dt,
                  precision="fp64", checkpoint_every=1)
    return sim


def _render_ours(xT, FT, cam, H, W, sigma0):
    import diff_gauss as dg
    tanx, tany, view, proj, eye = cam
    dev = xT.device
    cov = sigma0 ** 2 * FT @ FT.transpose(1, 2)
    c6 = torch.stack([cov[:, 0, 0], cov[:, 0, 1], cov[:, 0, 2], cov[:, 1, 1], cov[:, 1, 2], cov[:, 2, 2]], 1)
    n = xT.shape[0]
    st = dg.GaussianRasterizationSettings(H, W, tanx, tany, torch.tensor([1.0, 1.0, 1.0], device=dev), 1.0,
                                          view.to(dev, torch.float32), proj.to(dev, torch.float32), 0,
                                          eye.to(dev, torch.float32), False, False)
    e = torch.empty(0, device=dev)
    col = torch.tensor([0.8, 0.3, 0.2], device=dev).expand(n, 3).contiguous()
    op = torch.full((n, 1), 0.6, device=dev)
    nrm = torch.tensor([0.0, 0.0, -1.0], device=dev).expand(n, 3).contiguous()
    out = dg.rasterize_gaussians(xT.float(), torch.zeros_like(xT.float()), e, col, op, e, e, c6.float(), nrm, e, st)
    return out[0]


def _render_reference(xT, FT, cam, H, W, sigma0):
    import gs_reference as R
    tanx, tany, view, proj, eye = cam
    n = xT.shape[0]
    cov = sigma0 ** 2 * FT @ FT.transpose(1, 2)
    c6 = torch.stack([cov[:, 0, 0], cov[:, 0, 1], cov[:, 0, 2], cov[:, 1, 1], cov[:, 1, 2], cov[:, 2, 2]], 1)
    col = torch.tensor([0.8, 0.3, 0.2], dtype=torch.float64).expand(n, 3)
    op = torch.full((n, 1), 0.6, dtype=torch.float64)
    nrm = torch.tensor([0.0, 0.0, -1.0], dtype=torch.float64).expand(n, 3)
    return R.render(xT, op, H, W, tanx, tany, torch.ones(3, dtype=torch.float64), view, proj, eye, colors=col,
                    cov3D=c6, norm3D=nrm)[0]


def test_render_loss_gradient_reaches_the_rollout(dm, orc):
    import gs_reference as R
    import oracle as O
    from diffmpm_bindings import workloads as W
    from diffmpm_bindings.rollout import Rollout, mpm_rollout
    w = W.sphere32(seed=21, G=12, rho=60.0, radius=0.2)
    n, T, H, Wd = w.n, 5, 32, 32
    sigma0 = 0.5 * w.dx
    cam = R.camera(H, Wd, fovx_deg=40.0, eye=(0.5, 0.5, -1.2), target=(0.5, 0.5, 0.5))
    dev = torch.device("cuda")
    sim = Rollout(n, w.dims, w.dx, steps=T, m=w.m[0], vol=w.vol[0], nu=w.extra["nu"], dt=w.dt, precision="fp64")
    rng = np.random.default_rng(4)
    dfc0 = 0.02 * rng.normal(size=(n, 3, 3))
    target = torch.rand((3, H, Wd), generator=torch.Generator().manual_seed(1), dtype=torch.float64)
    x0 = torch.tensor(w.x, device=dev)
    v0 = torch.tensor(w.v, device=dev, requires_grad=True)
    F0 = torch.tensor(w.F, device=dev)
    c0 = torch.tensor(dfc0, device=dev, requires_grad=True)
    xT, FT = mpm_rollout(x0, v0, F0, c0, torch.tensor(w.extra["E"], dtype=torch.float64, device=dev), sim)
    img = _render_ours(xT, FT, cam, H, Wd, sigma0)
    loss = ((img.double() - target.to(dev)) ** 2).mean()
    loss.backward()
    gv, gc = v0.grad.cpu().numpy(), c0.grad.cpu().numpy()
    assert np.isfinite(gv).all() and np.abs(gv).max() > 0 and np.abs(gc).max() > 0

    def L(v, c):  # FP64 oracle rollout + dense float64 renderer
        lam, mu = orc.lame(w.extra["E"], w.extra["nu"])
        s = O.State(w.x, v, np.zeros((n, 3, 3)), w.F, w.m, w.vol, np.full(n, lam), np.full(n, mu), c)
        g = O.Grid(w.dims, w.dx)
        prm = O.Params(dt=w.dt, drag=0.0, smoothing=0.0, exact=True)
        for _ in range(T):
            s, _ = orc.forward_step(g, prm, s)
        im = _render_reference(torch.tensor(s.x), torch.tensor(s.F), cam, H, Wd, sigma0)
        return float(((im - target) ** 2).mean())

    gnorm = np.sqrt((gv ** 2).sum() + (gc ** 2).sum())
    eps = 1e-4
    for k in range(4):
        r = np.random.default_rng(50 + k)
        dv, dc = r.normal(size=gv.shape), r.normal(size=gc.shape)
        nrm = np.sqrt((dv ** 2).sum() + (dc ** 2).sum())
        dv, dc = dv / nrm, dc / nrm
        fd = (L(w.v + eps * dv, dfc0 + eps * dc) - L(w.v - eps * dv, dfc0 - eps * dc)) / (2 * eps)
        an = float((gv * dv).sum() + (gc * dc).sum())
        print(f"direction {k}: adjoint {an:.6e} FD {fd:.6e}")
        assert abs(an - fd) <= 2e-3 * gnorm, (an, fd, gnorm)
