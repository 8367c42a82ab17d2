"""Seeded synthetic particle sets for the benchmark workloads.

The reference ships no benchmark inputs; these generators stand in for them
with the workloads' shapes, sizes and value distributions:

* ``sphere32``    sphere r=0.25 in the unit cube, 8 particles per cell,
                  33^3 nodes (dx=1/32), E=1e4, nu=0.3, dt=1e-3, 20 steps.
* ``ellipsoid64`` ellipsoid semi-axes (0.35,0.25,0.2), 8 ppc, 65^3 nodes
                  (dx=1/64), E=5e4, nu=0.35, dt=5e-4, 100 steps, checkpoint 10.
* ``batched``     64 randomly scaled/rotated ellipsoids, N log-uniform in
                  [5k,200k], grids 32^3..96^3, E log-U[1e3,1e5], nu U[0.2,0.45].
* ``spheres2m``   union of 8 spheres r in [0.08,0.15], exactly N particles
                  (default 2M) on 129^3 nodes, 400 steps, checkpoint 20.
* ``morph500k``   500k-particle sphere and a target displaced by seeded
                  real spherical harmonics of degree <= 4.

Particle mass and volume follow GeometryLoading.cpp:122-140
(m = rho * pdx^3, vol = pdx^3 with pdx^3 = dx^3 / ppc).  Densities default to
values that keep the explicit step inside its CFL limit (c*dt/dx <= 0.5);
the nominal rho=1 diverges for sphere32 and ellipsoid64 (p-wave speed
sqrt((lam+2mu)/rho) ~ 116 for sphere32).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def lame(E: float, nu: float):
    """CalculateLameParameters (Elasticity.cpp:149-153)."""
    return E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), E / (2.0 + 2.0 * nu)


def stable_density(E, nu, dt, dx, cfl=0.45):
    lam, mu = lame(E, nu)
    c_max = cfl * dx / dt
    return (lam + 2.0 * mu) / (c_max * c_max)


@dataclass
class Workload:
    name: str
    x: np.ndarray            # (N,3) float64
    v: np.ndarray            # (N,3)
    F: np.ndarray            # (N,3,3)
    m: np.ndarray            # (N,)
    vol: np.ndarray          # (N,)
    lam: np.ndarray          # (N,)
    mu: np.ndarray           # (N,)
    dims: tuple
    dx: float
    grid_min: tuple
    dt: float
    steps: int
    checkpoint: int = 1
    drag: float = 0.0
    smoothing: float = 0.0
    f_ext: tuple = (0.0, 0.0, 0.0)
    rho: float = 1.0
    target: np.ndarray | None = None     # (N,3) target positions for the position loss
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])


def _uniform_in(rng, n, inside, lo, hi, batch=1 << 16):
    """Rejection-sample exactly n points uniformly inside ``inside``."""
    pts = []
    count = 0
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    while count < n:
        cand = lo + (hi - lo) * rng.random((batch, 3))
        cand = cand[inside(cand)]
        pts.append(cand)
        count += len(cand)
    return np.concatenate(pts)[:n]


def smooth_field(x, amp, rng):
    """Seeded smooth vector field amp * (sin 2pi(y+a), sin 2pi(z+b), sin 2pi(x+c))."""
    ph = rng.random(3)
    return amp * np.stack([np.sin(2 * np.pi * (x[:, 1] + ph[0])),
                           np.sin(2 * np.pi * (x[:, 2] + ph[1])),
                           np.sin(2 * np.pi * (x[:, 0] + ph[2]))], axis=1)


def _particles(x, E, nu, rho, dx, ppc):
    n = len(x)
    pvol = dx ** 3 / ppc
    lam, mu = lame(E, nu)
    F = np.broadcast_to(np.eye(3), (n, 3, 3)).copy()
    return F, np.full(n, rho * pvol), np.full(n, pvol), np.full(n, lam), np.full(n, mu)


def cell_sort(x, grid_min, dx):
    """Order particles by grid cell (z fastest), the layout the kernels favour."""
    cell = np.floor((x - np.asarray(grid_min)) / dx).astype(np.int64)
    key = (cell[:, 0] << 42) + (cell[:, 1] << 21) + cell[:, 2]
    return np.argsort(key, kind="stable")


def sphere32(seed=0, rho=None, G=32, ppc=8, radius=0.25, v_amp=0.5, sort=True) -> Workload:
    rng = np.random.default_rng(seed)
    dx = 1.0 / G
    E, nu, dt = 1e4, 0.3, 1e-3
    if rho is None:
        rho = 60.0
    n = int(round(ppc * (4.0 / 3.0) * math.pi * radius ** 3 / dx ** 3))
    c = np.array([0.5, 0.5, 0.5])
    x = _uniform_in(rng, n, lambda p: ((p - c) ** 2).sum(1) < radius ** 2, c - radius, c + radius)
    if sort:
        x = x[cell_sort(x, (0, 0, 0), dx)]
    F, m, vol, lam, mu = _particles(x, E, nu, rho, dx, ppc)
    v = smooth_field(x, v_amp, rng)
    tgt = x + 0.05 * np.stack([np.sin(2 * np.pi * x[:, 1]), np.sin(2 * np.pi * x[:, 2]),
                               np.sin(2 * np.pi * x[:, 0])], axis=1)
    return Workload("sphere32", x, v, F, m, vol, lam, mu, (G + 1,) * 3, dx, (0.0, 0.0, 0.0), dt, 20,
                    rho=rho, target=tgt, extra=dict(E=E, nu=nu, ppc=ppc))


def ellipsoid64(seed=1, rho=None, G=64, ppc=8, axes=(0.35, 0.25, 0.2), v_amp=0.5, sort=True,
                steps=100, checkpoint=10) -> Workload:
    rng = np.random.default_rng(seed)
    dx = 1.0 / G
    E, nu, dt = 5e4, 0.35, 5e-4
    if rho is None:
        rho = stable_density(E, nu, dt, dx)
    a = np.asarray(axes)
    n = int(round(ppc * (4.0 / 3.0) * math.pi * a.prod() / dx ** 3))
    c = np.array([0.5, 0.5, 0.5])
    x = _uniform_in(rng, n, lambda p: (((p - c) / a) ** 2).sum(1) < 1.0, c - a, c + a)
    if sort:
        x = x[cell_sort(x, (0, 0, 0), dx)]
    F, m, vol, lam, mu = _particles(x, E, nu, rho, dx, ppc)
    v = smooth_field(x, v_amp, rng)
    tgt = x + 0.05 * np.stack([np.sin(2 * np.pi * x[:, 1]), np.sin(2 * np.pi * x[:, 2]),
                               np.sin(2 * np.pi * x[:, 0])], axis=1)
    return Workload("ellipsoid64", x, v, F, m, vol, lam, mu, (G + 1,) * 3, dx, (0.0, 0.0, 0.0), dt, steps,
                    checkpoint=checkpoint, rho=rho, target=tgt, extra=dict(E=E, nu=nu, ppc=ppc))


def spheres2m(seed=3, n=2_000_000, G=128, rho=None, v_amp=0.5, sort=True, steps=400, checkpoint=20) -> Workload:
    """Union of 8 seeded spheres holding exactly n particles (ppc derived)."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / G
    E, nu = 1e4, 0.3
    dt = 2.5e-4
    if rho is None:
        rho = stable_density(E, nu, dt, dx)
    r = rng.uniform(0.08, 0.15, 8)
    cen = np.stack([rng.uniform(0.2 + rr, 0.8 - rr, 3) if rr < 0.3 else np.full(3, 0.5) for rr in r])
    inside = lambda p: (((p[:, None, :] - cen[None]) ** 2).sum(-1) < r[None] ** 2).any(1)
    lo, hi = (cen - r[:, None]).min(0), (cen + r[:, None]).max(0)
    x = _uniform_in(rng, n, inside, lo, hi)
    if sort:
        x = x[cell_sort(x, (0, 0, 0), dx)]
    # occupied volume estimate -> ppc so that mass/volume match the union's volume
    probe = lo + (hi - lo) * rng.random((400_000, 3))
    frac = inside(probe).mean()
    vol_union = frac * np.prod(hi - lo)
    ppc = n * dx ** 3 / vol_union
    F, m, vol, lam, mu = _particles(x, E, nu, rho, dx, ppc)
    v = smooth_field(x, v_amp, rng)
    return Workload("spheres2m", x, v, F, m, vol, lam, mu, (G + 1,) * 3, dx, (0.0, 0.0, 0.0), dt, steps,
                    checkpoint=checkpoint, rho=rho, extra=dict(E=E, nu=nu, ppc=ppc, radii=r, centres=cen))


def batched(seed=2, count=64, steps=50):
    """Independent instances of uneven size (list of Workloads)."""
    rng = np.random.default_rng(seed)
    out = []
    dt = 2e-4
    for i in range(count):
        n_i = int(round(math.exp(rng.uniform(math.log(5e3), math.log(2e5)))))
        G = int(rng.integers(32, 97))
        dx = 1.0 / G
        E = math.exp(rng.uniform(math.log(1e3), math.log(1e5)))
        nu = rng.uniform(0.2, 0.45)
        axes = rng.uniform(0.12, 0.3, 3)
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        rho = stable_density(E, nu, dt, dx)
        c = np.array([0.5, 0.5, 0.5])
        Rt = q.T
        inside = lambda p, Rt=Rt, axes=axes: ((((p - c) @ Rt.T) / axes) ** 2).sum(1) < 1.0
        rmax = axes.max()
        x = _uniform_in(rng, n_i, inside, c - rmax, c + rmax)
        x = x[cell_sort(x, (0, 0, 0), dx)]
        ppc = n_i * dx ** 3 / ((4.0 / 3.0) * math.pi * axes.prod())
        F, m, vol, lam, mu = _particles(x, E, nu, rho, dx, ppc)
        v = smooth_field(x, 0.3, rng)
        out.append(Workload(f"batched{i}", x, v, F, m, vol, lam, mu, (G + 1,) * 3, dx, (0.0, 0.0, 0.0), dt, steps,
                            rho=rho, extra=dict(E=E, nu=nu, ppc=ppc)))
    return out


def _real_sph_harm(l, m, theta, phi):
    """Real spherical harmonic (unnormalised) via associated Legendre recursion."""
    x = np.cos(theta)
    am = abs(m)
    # P_am^am
    pmm = np.ones_like(x)
    somx2 = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    fact = 1.0
    for _ in range(am):
        pmm = -pmm * fact * somx2
        fact += 2.0
    if l == am:
        plm = pmm
    else:
        pmmp1 = x * (2 * am + 1) * pmm
        if l == am + 1:
            plm = pmmp1
        else:
            for ll in range(am + 2, l + 1):
                pll = ((2 * ll - 1) * x * pmmp1 - (ll + am - 1) * pmm) / (ll - am)
                pmm, pmmp1 = pmmp1, pll
            plm = pmmp1
    if m > 0:
        return plm * np.cos(m * phi)
    if m < 0:
        return plm * np.sin(am * phi)
    return plm


def morph500k(seed=4, n=500_000, G=96, episode=0, amp=0.04, rho=None, sort=True) -> Workload:
    """500k-particle sphere -> sphere displaced by seeded real SH noise (l<=4)."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / G
    E, nu, dt = 1e4, 0.3, 5e-4
    if rho is None:
        rho = stable_density(E, nu, dt, dx)
    radius = 0.25
    c = np.array([0.5, 0.5, 0.5])
    x = _uniform_in(rng, n, lambda p: ((p - c) ** 2).sum(1) < radius ** 2, c - radius, c + radius)
    if sort:
        x = x[cell_sort(x, (0, 0, 0), dx)]
    ppc = n * dx ** 3 / ((4.0 / 3.0) * math.pi * radius ** 3)
    F, m, vol, lam, mu = _particles(x, E, nu, rho, dx, ppc)
    erng = np.random.default_rng(seed * 1000 + episode)
    d = x - c
    rr = np.linalg.norm(d, axis=1) + 1e-12
    theta = np.arccos(np.clip(d[:, 2] / rr, -1, 1))
    phi = np.arctan2(d[:, 1], d[:, 0])
    disp = np.zeros(n)
    for l in range(1, 5):
        for mm in range(-l, l + 1):
            disp += erng.normal() * _real_sph_harm(l, mm, theta, phi) / (1 + l * l)
    disp *= amp / (np.abs(disp).max() + 1e-12)
    tgt = x + (disp * rr / radius)[:, None] * d / rr[:, None]
    v = np.zeros_like(x)
    return Workload(f"morph500k_ep{episode}", x, v, F, m, vol, lam, mu, (G + 1,) * 3, dx, (0.0, 0.0, 0.0), dt,
                    200, rho=rho, target=tgt, extra=dict(E=E, nu=nu, ppc=ppc))


def camera(H, W, fovx_deg=50.0, eye=(0.0, 0.0, -3.0), target=(0.0, 0.0, 0.0), znear=0.01, zfar=100.0):
    """A look-at pinhole camera for the Gaussian rasterizer: (tanfovx, tanfovy,
    view, proj, position) with view and proj as flat 16-vectors in the
    rasterizer's convention (x' = m[0]x + m[4]y + m[8]z + m[12]), proj the
    full world-to-clip transform."""
    import torch
    tanx = math.tan(math.radians(fovx_deg) / 2)
    tany = tanx * H / W
    eye_t, tgt = torch.tensor(eye, dtype=torch.float64), torch.tensor(target, dtype=torch.float64)
    fwd = tgt - eye_t
    fwd = fwd / fwd.norm()
    up = torch.tensor([0.0, 1.0, 0.0], dtype=torch.float64)
    right = torch.cross(up, fwd, dim=0)
    right = right / right.norm()
    up2 = torch.cross(fwd, right, dim=0)
    Rw = torch.stack([right, up2, fwd])            # rows: camera axes in world
    tw = -Rw @ eye_t
    Wv = torch.eye(4, dtype=torch.float64)
    Wv[:3, :3], Wv[:3, 3] = Rw, tw                  # column-vector world->view
    Pr = torch.zeros(4, 4, dtype=torch.float64)
    Pr[0, 0], Pr[1, 1] = 1 / tanx, 1 / tany
    Pr[2, 2], Pr[2, 3] = zfar / (zfar - znear), -zfar * znear / (zfar - znear)
    Pr[3, 2] = 1.0
    view = Wv.T.contiguous().reshape(-1)            # flat layout m[4c+r] = Wv[r][c]
    proj = (Pr @ Wv).T.contiguous().reshape(-1)
    return tanx, tany, view, proj, eye_t
