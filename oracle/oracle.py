"""ctypes wrappers for the test oracle (TEST INFRASTRUCTURE ONLY).

``Oracle`` wraps ``liboracle.so`` (the FP64 restatement, ``mpm_oracle.c``);
``Reference`` wraps ``_ref/libref{32,64}.so`` (the reference's own sources,
built by ``build_oracle.py`` where the reference tree is present).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs
import this module; the product never does.

Conventions: positions/velocities (N,3) float64, matrices (N,3,3) float64
row-major, grid arrays flattened over (dx,dy,dz) with node (i,j,k) at
i*dy*dz + j*dz + k.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(_dp)


def _f64(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


class _OrcGrid(C.Structure):
    _fields_ = [("dims", C.c_int * 3), ("dx", C.c_double), ("min", C.c_double * 3)]


class _OrcParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("drag", C.c_double), ("smoothing", C.c_double),
                ("f_ext", C.c_double * 3), ("bulk_visc", C.c_double), ("j_min", C.c_double),
                ("exact", C.c_int), ("kernel", C.c_int), ("material", C.c_int)]


@dataclass
class Grid:
    dims: tuple
    dx: float
    min: tuple = (0.0, 0.0, 0.0)

    @property
    def n_nodes(self) -> int:
        return int(self.dims[0]) * int(self.dims[1]) * int(self.dims[2])

    def c(self) -> _OrcGrid:
        g = _OrcGrid()
        g.dims[:] = [int(d) for d in self.dims]
        g.dx = float(self.dx)
        g.min[:] = [float(m) for m in self.min]
        return g


@dataclass
class Params:
    dt: float = 1.0 / 120.0
    drag: float = 0.5
    smoothing: float = 0.1
    f_ext: tuple = (0.0, 0.0, 0.0)
    bulk_visc: float = 0.25
    j_min: float = 0.6
    exact: bool = False
    kernel: int = 0
    material: int = 0

    def c(self) -> _OrcParams:
        p = _OrcParams()
        p.dt, p.drag, p.smoothing = float(self.dt), float(self.drag), float(self.smoothing)
        p.f_ext[:] = [float(f) for f in self.f_ext]
        p.bulk_visc, p.j_min = float(self.bulk_visc), float(self.j_min)
        p.exact, p.kernel, p.material = int(bool(self.exact)), int(self.kernel), int(self.material)
        return p


@dataclass
class State:
    """One layer of particle state (double)."""
    x: np.ndarray
    v: np.ndarray
    C: np.ndarray
    F: np.ndarray
    m: np.ndarray
    vol: np.ndarray
    lam: np.ndarray
    mu: np.ndarray
    dFc: np.ndarray | None = None

    def __post_init__(self):
        n = len(self.m)
        self.x = _f64(self.x, (n, 3))
        self.v = _f64(self.v, (n, 3))
        self.C = _f64(self.C, (n, 3, 3))
        self.F = _f64(self.F, (n, 3, 3))
        self.m = _f64(self.m, (n,))
        self.vol = _f64(self.vol, (n,))
        self.lam = _f64(self.lam, (n,))
        self.mu = _f64(self.mu, (n,))
        self.dFc = _f64(self.dFc, (n, 3, 3)) if self.dFc is not None else None

    @property
    def n(self) -> int:
        return len(self.m)


@dataclass
class Grads:
    x: np.ndarray
    v: np.ndarray
    F: np.ndarray
    C: np.ndarray
    Ft: np.ndarray | None = None
    lam: np.ndarray | None = None
    mu: np.ndarray | None = None

    @staticmethod
    def zeros(n: int) -> "Grads":
        return Grads(np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3, 3)), np.zeros((n, 3, 3)))


def load_lib(path: Path) -> C.CDLL:
    return C.CDLL(str(path))


class Oracle:
    """FP64 CPU restatement of the reference path (mpm_oracle.c)."""

    def __init__(self, path: Path | None = None):
        path = path or HERE / "liboracle.so"
        if not path.exists():
            from build_oracle import build_oracle  # noqa: WPS433 (local recipe)
            build_oracle()
        self.lib = load_lib(path)
        L = self.lib
        L.orc_forward_step.restype = C.c_int
        L.orc_backward_step.restype = C.c_int
        L.orc_mass_loss.restype = C.c_double
        L.orc_grad_norm.restype = C.c_double
        L.orc_num_threads.restype = C.c_int
        L.orc_rollout.restype = C.c_int

    def threads(self) -> int:
        return self.lib.orc_num_threads()

    def set_threads(self, n: int) -> None:
        """OpenMP threads of the following calls (the process-wide setting)."""
        self.lib.orc_set_threads(C.c_int(int(n)))

    # -- constitutive
    def pk(self, F, lam, mu, material=0):
        F = _f64(F, (3, 3))
        P = np.zeros((3, 3))
        self.lib.orc_pk(C.c_int(material), _p(F), C.c_double(lam), C.c_double(mu), _p(P))
        return P

    def pk_vjp(self, F, lam, mu, G, material=0, exact=False):
        F, G = _f64(F, (3, 3)), _f64(G, (3, 3))
        out = np.zeros((3, 3))
        self.lib.orc_pk_vjp(C.c_int(material), C.c_int(int(exact)), _p(F), C.c_double(lam), C.c_double(mu),
                            _p(G), _p(out))
        return out

    def polar(self, F):
        F = _f64(F, (3, 3))
        R, S = np.zeros((3, 3)), np.zeros((3, 3))
        self.lib.orc_polar(_p(F), _p(R), _p(S))
        return R, S

    def lame(self, E, nu):
        lam, mu = C.c_double(), C.c_double()
        self.lib.orc_lame(C.c_double(E), C.c_double(nu), C.byref(lam), C.byref(mu))
        return lam.value, mu.value

    # -- steps
    def forward_step(self, grid: Grid, prm: Params, s: State):
        n, nn = s.n, grid.n_nodes
        out = State(np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3, 3)), np.zeros((n, 3, 3)),
                    s.m, s.vol, s.lam, s.mu)
        gm, gp, gv = np.zeros(nn), np.zeros((nn, 3)), np.zeros((nn, 3))
        trust = np.zeros(n)
        rc = self.lib.orc_forward_step(C.byref(grid.c()), C.byref(prm.c()), C.c_int(n),
                                       _p(s.x), _p(s.v), _p(s.C), _p(s.F), _p(s.dFc),
                                       _p(s.m), _p(s.vol), _p(s.lam), _p(s.mu),
                                       _p(out.x), _p(out.v), _p(out.C), _p(out.F),
                                       _p(gm), _p(gp), _p(gv), _p(trust))
        assert rc == 0
        return out, dict(m=gm, p=gp, v=gv, trust=trust)

    def backward_step(self, grid: Grid, prm: Params, s: State, C1, grid_step: dict, g1: Grads,
                      want_ft=False, want_lame=False):
        n = s.n
        g = Grads.zeros(n)
        gFt = np.zeros((n, 3, 3)) if want_ft else None
        glam = np.zeros(n) if want_lame else None
        gmu = np.zeros(n) if want_lame else None
        rc = self.lib.orc_backward_step(C.byref(grid.c()), C.byref(prm.c()), C.c_int(n),
                                        _p(s.x), _p(s.v), _p(s.C), _p(s.F), _p(s.dFc),
                                        _p(s.m), _p(s.vol), _p(s.lam), _p(s.mu),
                                        _p(_f64(C1, (n, 3, 3))), _p(_f64(grid_step.get("trust"))),
                                        _p(_f64(grid_step["m"])), _p(_f64(grid_step["v"])),
                                        _p(_f64(g1.x)), _p(_f64(g1.v)), _p(_f64(g1.F)), _p(_f64(g1.C)),
                                        _p(g.x), _p(g.v), _p(g.F), _p(g.C), _p(gFt), _p(glam), _p(gmu))
        assert rc == 0
        g.Ft, g.lam, g.mu = gFt, glam, gmu
        return g

    def mass_loss(self, grid: Grid, prm: Params, x, m, target_m):
        x, m, t = _f64(x), _f64(m), _f64(target_m)
        n, nn = len(m), grid.n_nodes
        gm, dLdm, gx = np.zeros(nn), np.zeros(nn), np.zeros((n, 3))
        loss = self.lib.orc_mass_loss(C.byref(grid.c()), C.byref(prm.c()), C.c_int(n), _p(x), _p(m), _p(t),
                                      _p(gm), _p(dLdm), _p(gx))
        return loss, dict(m=gm, dLdm=dLdm, gx=gx)

    def p2g_accumulate(self, grid: Grid, x, v, Cm, m, gm, gp, kernel=0):
        x, v, Cm, m = _f64(x), _f64(v), _f64(Cm), _f64(m)
        self.lib.orc_p2g_accumulate(C.byref(grid.c()), C.c_int(kernel), C.c_int(len(m)), _p(x), _p(v), _p(Cm),
                                    _p(m), _p(gm), _p(gp))

    def volumes(self, grid: Grid, x, v, Cm, m, gm, gp, kernel=0):
        x, v, Cm, m = _f64(x), _f64(v), _f64(Cm), _f64(m)
        vol = np.zeros(len(m))
        self.lib.orc_volumes(C.byref(grid.c()), C.c_int(kernel), C.c_int(len(m)), _p(x), _p(v), _p(Cm), _p(m),
                             _p(gm), _p(gp), _p(vol))
        return vol

    def grad_norm(self, dLdF):
        dLdF = _f64(dLdF)
        return self.lib.orc_grad_norm(C.c_int(dLdF.size // 9), _p(dLdF))

    def adam(self, dLdF, dFc, mom, vec, vmax, alpha, gnorm, beta1=0.9, beta2=0.999, eps=1e-3, timestep=1):
        """Updates dFc, mom, vec, vmax in place (float64 arrays)."""
        dLdF = _f64(dLdF)
        self.lib.orc_adam(C.c_int(dLdF.size // 9), _p(dLdF), _p(dFc), _p(mom), _p(vec), _p(vmax),
                          C.c_double(alpha), C.c_double(gnorm), C.c_double(beta1), C.c_double(beta2),
                          C.c_double(eps), C.c_int(timestep))

    def rollout(self, grid: Grid, prm: Params, s: State, T: int, seed_gx):
        n = s.n
        xT = np.zeros((n, 3))
        g = Grads.zeros(n)
        rc = self.lib.orc_rollout(C.byref(grid.c()), C.byref(prm.c()), C.c_int(n), C.c_int(T),
                                  _p(s.x), _p(s.v), _p(s.F), _p(s.dFc), _p(s.m), _p(s.vol), _p(s.lam), _p(s.mu),
                                  _p(_f64(seed_gx)), _p(xT), _p(g.x), _p(g.v), _p(g.F), _p(g.C))
        assert rc == 0
        return xT, g


    # -- CompGraph optimiser
    def run_optimization(self, grid: Grid, prm: Params, s0: State, target_m, num_steps: int, control_stride: int,
                         max_gd_iters: int, max_ls_iters: int, initial_alpha: float, gd_tol: float,
                         passes: int = 3):
        """OptimizeDefGradControlSequence (CompGraph.cpp:213-368) over the
        FP64 step, loss and Adam of this oracle.  Returns every loss it
        evaluates, in order (initial; per gradient step the loss before the
        step and each line-search trial; final), and the final layers.

        As in the reference: a forward pass from layer t rewrites layers
        t+1.. and zeroes their control (ForwardSimulation.cpp:155), so a
        rejected line-search trial leaves its states in the later layers;
        Adam moments live per layer and are restored with dFc on rejection
        (CompGraph.cpp:309-346); the control gradient is dL/dF of the
        control layer, or dL/d(F + dFc) for the exact adjoint."""
        L = int(num_steps)
        n = s0.n
        first = State(s0.x, s0.v, s0.C, s0.F, s0.m, s0.vol, s0.lam, s0.mu,
                      s0.dFc if s0.dFc is not None else np.zeros((n, 3, 3)))
        layers = [first] + [None] * (L - 1)
        steps = [None] * (L - 1)
        moments = {}
        hist = []

        def forward(start):  # ComputeForwardPass (CompGraph.cpp:131-141)
            for i in range(start, L - 1):
                nxt, st = self.forward_step(grid, prm, layers[i])
                nxt.dFc = np.zeros((n, 3, 3))
                layers[i + 1], steps[i] = nxt, st

        def eval_loss():  # EndLayerMassLoss (CompGraph.cpp:42-129)
            loss, aux = self.mass_loss(grid, prm, layers[-1].x, layers[-1].m, target_m)
            hist.append(loss)
            return loss, aux["gx"]

        def backward(ctl, gx):  # ComputeBackwardPass (CompGraph.cpp:143-211)
            g = Grads(np.array(gx, np.float64), np.zeros((n, 3)), np.zeros((n, 3, 3)), np.zeros((n, 3, 3)))
            for t in range(L - 2, ctl - 1, -1):
                g = self.backward_step(grid, prm, layers[t], layers[t + 1].C, steps[t], g, want_ft=(t == ctl))
            return g.Ft if prm.exact else g.F

        forward(0)
        _, gx = eval_loss()
        backward(0, gx)
        adam_t = 0
        for _ in range(passes):
            for ct in range(0, L - 1, max(1, control_stride)):
                alpha, init_norm = initial_alpha, 0.0
                for it in range(max_gd_iters):
                    forward(ct)
                    loss, gx = eval_loss()
                    if not np.isfinite(loss):
                        break
                    gc = backward(ct, gx)
                    gn = max(self.grad_norm(gc), 1e-12)
                    if it == 0:
                        init_norm = gn
                    if gn < gd_tol * init_norm:
                        break
                    lay = layers[ct]
                    mom = moments.setdefault(ct, [np.zeros((n, 3, 3)) for _ in range(3)])
                    bak = [lay.dFc.copy()] + [a.copy() for a in mom]
                    ok, a = False, alpha
                    for _ls in range(max_ls_iters):
                        self.adam(gc, lay.dFc, mom[0], mom[1], mom[2], a, gn, timestep=adam_t + 1)
                        forward(ct)
                        nl, _ = eval_loss()
                        if np.isfinite(nl) and nl < loss:
                            adam_t += 1
                            alpha = min(a * 1.1, initial_alpha)
                            ok = True
                            break
                        lay.dFc[...] = bak[0]
                        for dst, src in zip(mom, bak[1:]):
                            dst[...] = src
                        a *= 0.5
                    if not ok:
                        break
        eval_loss()
        return np.array(hist), layers


class OracleGraph:
    """CompGraph's layer tape, loss, backward with render gradients and
    OptimizeSingleTimestep (CompGraph.cpp:21-211, 369-465) over the FP64
    step, loss and Adam of ``Oracle``.  Test infrastructure: the checker for
    the engine's optimize_single_timestep.

    As in the reference: SetUpCompGraph copies layer 0 into every layer
    (CompGraph.cpp:30-40), so each layer has its own zero Adam moments; a
    forward pass from layer t rewrites layers t+1.. and zeroes their control
    (ForwardSimulation.cpp:155); EndLayerMassLoss sets the last layer's dL/dx
    and zeroes its other gradients; ComputeBackwardPass first adds the stored
    render gradients to the last layer (CompGraph.cpp:148-197); the control
    gradient is dL/dF of the control layer, or dL/d(F + dFc) for the exact
    adjoint.  OptimizeSingleTimestep's Adam step counter is a function-local
    static in the reference (CompGraph.cpp:396), shared by every graph of the
    process: here it is the class attribute ``adam_step``."""

    adam_step = 0

    def __init__(self, orc: "Oracle", grid: Grid, prm: Params, s0: State, target_m):
        self.orc, self.grid, self.prm = orc, grid, prm
        n = s0.n
        self.target = _f64(target_m)
        first = State(s0.x, s0.v, s0.C, s0.F, s0.m, s0.vol, s0.lam, s0.mu,
                      s0.dFc if s0.dFc is not None else np.zeros((n, 3, 3)))
        self.layers = [first]
        self.steps = []
        self.moments = {}
        self.render = None
        self.history = []

    @property
    def n(self) -> int:
        return self.layers[0].n

    def set_up(self, num_layers: int):
        import copy
        self.layers = [self.layers[0]] + [copy.deepcopy(self.layers[0]) for _ in range(num_layers - 1)]
        self.steps = [None] * (num_layers - 1)

    def set_render_gradients(self, dLdF, dLdx):
        n = self.n
        self.render = (_f64(dLdF, (n, 3, 3)), _f64(dLdx, (n, 3)))

    def forward(self, start: int):
        for i in range(start, len(self.layers) - 1):
            nxt, st = self.orc.forward_step(self.grid, self.prm, self.layers[i])
            nxt.dFc = np.zeros((self.n, 3, 3))
            self.layers[i + 1], self.steps[i] = nxt, st

    def loss(self):
        last = self.layers[-1]
        loss, aux = self.orc.mass_loss(self.grid, self.prm, last.x, last.m, self.target)
        self.last_gx = aux["gx"]
        self.history.append(loss)
        return loss

    def backward(self, ctl: int):
        n = self.n
        gx = np.array(self.last_gx, np.float64)
        gF = np.zeros((n, 3, 3))
        if self.render is not None:
            gF = gF + self.render[0]
            gx = gx + self.render[1]
        g = Grads(gx, np.zeros((n, 3)), gF, np.zeros((n, 3, 3)))
        for t in range(len(self.layers) - 2, ctl - 1, -1):
            g = self.orc.backward_step(self.grid, self.prm, self.layers[t], self.layers[t + 1].C, self.steps[t], g,
                                       want_ft=(t == ctl))
        return g.Ft if self.prm.exact else g.F

    def optimize_single_timestep(self, t: int, max_gd_iters: int = 1, episode: int = 0, initial_alpha: float = 1.0,
                                 max_ls_iters: int = 10):
        """OptimizeSingleTimestep (CompGraph.cpp:369-465); the losses it
        evaluates are appended to ``history``."""
        if t < 0 or t >= len(self.layers) - 1:
            return
        alpha = initial_alpha
        lay = self.layers[t]
        for _ in range(max_gd_iters):
            self.forward(t)
            loss = self.loss()
            if not np.isfinite(loss):
                break
            gc = self.backward(t)
            gn = max(self.orc.grad_norm(gc), 1e-12)
            mom = self.moments.setdefault(t, [np.zeros((self.n, 3, 3)) for _ in range(3)])
            bak = [lay.dFc.copy()] + [a.copy() for a in mom]
            ok, a = False, alpha
            for _ls in range(max_ls_iters):
                self.orc.adam(gc, lay.dFc, mom[0], mom[1], mom[2], a, gn, timestep=OracleGraph.adam_step + 1)
                self.forward(t)
                nl = self.loss()
                if np.isfinite(nl) and nl < loss:
                    OracleGraph.adam_step += 1
                    alpha = min(a * 1.1, initial_alpha)
                    ok = True
                    break
                lay.dFc[...] = bak[0]
                for dst, src in zip(mom, bak[1:]):
                    dst[...] = src
                a *= 0.5
            if not ok:
                break


class Reference:
    """The reference's own DiffMPMLib3D compiled from source (float or double)."""

    def __init__(self, bits: int = 64):
        path = HERE / "_ref" / f"libref{bits}.so"
        if not path.exists():
            raise FileNotFoundError(path)
        self.lib = load_lib(path)
        self.bits = bits
        self.lib.ref_mass_loss.restype = C.c_double
        self.lib.ref_adam.restype = C.c_double

    @staticmethod
    def available(bits: int = 64) -> bool:
        return (HERE / "_ref" / f"libref{bits}.so").exists()

    @staticmethod
    def _g(grid: Grid):
        dims = (C.c_int * 3)(*[int(d) for d in grid.dims])
        mn = np.asarray(grid.min, dtype=np.float64)
        return dims, C.c_double(grid.dx), mn

    def pk(self, F, lam, mu):
        P = np.zeros((3, 3))
        self.lib.ref_pk(_p(_f64(F, (3, 3))), C.c_double(lam), C.c_double(mu), _p(P))
        return P

    def hvp(self, F, lam, mu, dF):
        out = np.zeros((3, 3))
        self.lib.ref_hvp(_p(_f64(F, (3, 3))), C.c_double(lam), C.c_double(mu), _p(_f64(dF, (3, 3))), _p(out))
        return out

    def lame(self, E, nu):
        lam, mu = C.c_double(), C.c_double()
        self.lib.ref_lame(C.c_double(E), C.c_double(nu), C.byref(lam), C.byref(mu))
        return lam.value, mu.value

    def forward_step(self, grid: Grid, prm: Params, s: State):
        dims, dx, mn = self._g(grid)
        n, nn = s.n, grid.n_nodes
        out = State(np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3, 3)), np.zeros((n, 3, 3)),
                    s.m, s.vol, s.lam, s.mu)
        gm, gv = np.zeros(nn), np.zeros((nn, 3))
        fext = np.asarray(prm.f_ext, dtype=np.float64)
        self.lib.ref_forward_step(dims, dx, _p(mn), C.c_double(prm.dt), C.c_double(prm.drag),
                                  C.c_double(prm.smoothing), _p(fext), C.c_int(n),
                                  _p(s.x), _p(s.v), _p(s.C), _p(s.F), _p(s.dFc), _p(s.m), _p(s.vol),
                                  _p(s.lam), _p(s.mu), _p(out.x), _p(out.v), _p(out.C), _p(out.F), _p(gm), _p(gv))
        return out, dict(m=gm, v=gv)

    def backward_step(self, grid: Grid, prm: Params, s: State, C1, grid_step: dict, g1: Grads):
        dims, dx, mn = self._g(grid)
        n = s.n
        g = Grads.zeros(n)
        self.lib.ref_backward_step(dims, dx, _p(mn), C.c_double(prm.dt), C.c_double(prm.drag),
                                   C.c_double(prm.smoothing), C.c_int(n),
                                   _p(s.x), _p(s.v), _p(s.C), _p(s.F), _p(s.dFc), _p(s.m), _p(s.vol),
                                   _p(s.lam), _p(s.mu), _p(_f64(C1, (n, 3, 3))),
                                   _p(_f64(grid_step["m"])), _p(_f64(grid_step["v"])),
                                   _p(_f64(g1.x)), _p(_f64(g1.v)), _p(_f64(g1.F)), _p(_f64(g1.C)),
                                   _p(g.x), _p(g.v), _p(g.F), _p(g.C))
        return g

    def mass_loss(self, grid: Grid, x, m, target_m):
        dims, dx, mn = self._g(grid)
        x, m, t = _f64(x), _f64(m), _f64(target_m)
        n, nn = len(m), grid.n_nodes
        gm, dLdm, gx = np.zeros(nn), np.zeros(nn), np.zeros((n, 3))
        loss = self.lib.ref_mass_loss(dims, dx, _p(mn), C.c_int(n), _p(x), _p(m), _p(t), _p(gm), _p(dLdm), _p(gx))
        return loss, dict(m=gm, dLdm=dLdm, gx=gx)

    def adam(self, dLdF, dFc, mom, vec, vmax, alpha, beta1=0.9, beta2=0.999, eps=1e-3, timestep=1):
        dLdF = _f64(dLdF)
        return self.lib.ref_adam(C.c_int(dLdF.size // 9), _p(dLdF), _p(dFc), _p(mom), _p(vec), _p(vmax),
                                 C.c_double(alpha), C.c_double(beta1), C.c_double(beta2), C.c_double(eps),
                                 C.c_int(timestep))

    def volumes(self, grid: Grid, x, v, Cm, m, gm, gp):
        dims, dx, mn = self._g(grid)
        x, v, Cm, m = _f64(x), _f64(v), _f64(Cm), _f64(m)
        vol = np.zeros(len(m))
        self.lib.ref_volumes(dims, dx, _p(mn), C.c_int(len(m)), _p(x), _p(v), _p(Cm), _p(m), _p(gm), _p(gp),
                             _p(vol))
        return vol

    def rollout(self, grid: Grid, prm: Params, s: State, T: int, seed_gx):
        dims, dx, mn = self._g(grid)
        n = s.n
        xT = np.zeros((n, 3))
        g = Grads.zeros(n)
        tf, tb = C.c_double(), C.c_double()
        fext = np.asarray(prm.f_ext, dtype=np.float64)
        self.lib.ref_rollout(dims, dx, _p(mn), C.c_double(prm.dt), C.c_double(prm.drag), C.c_double(prm.smoothing),
                             _p(fext), C.c_int(n), C.c_int(T), _p(s.x), _p(s.v), _p(s.F), _p(s.dFc), _p(s.m),
                             _p(s.vol), _p(s.lam), _p(s.mu), _p(_f64(seed_gx)), _p(xT),
                             _p(g.x), _p(g.v), _p(g.F), _p(g.C), C.byref(tf), C.byref(tb))
        return xT, g, (tf.value, tb.value)

    def optimize(self, grid: Grid, prm: Params, s: State, target_m, num_steps: int, control_stride: int,
                 max_gd_iters: int, max_ls_iters: int, initial_alpha: float, gd_tol: float):
        """The reference's OptimizeDefGradControlSequence (3 passes, reference
        adjoint): final loss, every layer's dFc (L,N,3,3), last positions and
        the optimiser's printed lines."""
        dims, dx, mn = self._g(grid)
        n = s.n
        dfc = np.zeros((num_steps, n, 3, 3))
        xT = np.zeros((n, 3))
        log = C.create_string_buffer(1 << 16)
        fext = np.asarray(prm.f_ext, dtype=np.float64)
        self.lib.ref_optimize.restype = C.c_double
        loss = self.lib.ref_optimize(dims, dx, _p(mn), C.c_double(prm.dt), C.c_double(prm.drag),
                                     C.c_double(prm.smoothing), _p(fext), C.c_int(n), _p(s.x), _p(s.v), _p(s.F),
                                     _p(s.m), _p(s.vol), _p(s.lam), _p(s.mu), _p(_f64(target_m)),
                                     C.c_int(num_steps), C.c_int(control_stride), C.c_int(max_gd_iters),
                                     C.c_int(max_ls_iters), C.c_double(initial_alpha), C.c_double(gd_tol),
                                     _p(dfc), _p(xT), log, C.c_int(len(log)))
        return loss, dfc, xT, log.value.decode(errors="replace")

    def optimize_single(self, grid: Grid, prm: Params, s: State, target_m, num_layers: int, calls,
                        render_dLdF=None, render_dLdx=None):
        """run.py's E2E sequence (set_up_comp_graph, compute_forward_pass(0),
        optional set_render_gradients, then OptimizeSingleTimestep per call
        (t, max_gd, alpha, max_ls)) on the reference: per call, every layer's
        dFc (calls, L, N, 3, 3), the last positions (calls, N, 3) and
        EndLayerMassLoss, and the printed lines.  The reference's Adam step
        counter for this call is process-wide: call this once per process."""
        dims, dx, mn = self._g(grid)
        n, k = s.n, len(calls)
        t = (C.c_int * k)(*[int(c[0]) for c in calls])
        gd = (C.c_int * k)(*[int(c[1]) for c in calls])
        al = (C.c_double * k)(*[float(c[2]) for c in calls])
        ls = (C.c_int * k)(*[int(c[3]) for c in calls])
        dfc = np.zeros((k, num_layers, n, 3, 3))
        xT = np.zeros((k, n, 3))
        loss = np.zeros(k)
        log = C.create_string_buffer(1 << 16)
        fp = C.POINTER(C.c_float)
        rF = None if render_dLdF is None else np.ascontiguousarray(render_dLdF, np.float32).reshape(n, 9)
        rx = None if render_dLdx is None else np.ascontiguousarray(render_dLdx, np.float32).reshape(n, 3)
        rc = self.lib.ref_optimize_single(dims, dx, _p(mn), C.c_double(prm.dt), C.c_double(prm.drag),
                                          C.c_double(prm.smoothing), C.c_int(n), _p(s.x), _p(s.v), _p(s.F),
                                          _p(s.m), _p(s.vol), _p(s.lam), _p(s.mu), _p(_f64(target_m)),
                                          C.c_int(num_layers), None if rF is None else rF.ctypes.data_as(fp),
                                          None if rx is None else rx.ctypes.data_as(fp), C.c_int(k), t, gd, al, ls,
                                          _p(dfc), _p(xT), _p(loss), log, C.c_int(len(log)))
        assert rc == 0
        return dfc, xT, loss, log.value.decode(errors="replace")

    def sample_mesh(self, V, F, dx: float):
        """GeneratePointCloudFromWatertightTriangleMesh over the mesh's bounding
        box (the reference's lattice + libigl winding-number inside test)."""
        V = np.ascontiguousarray(V, np.float64).reshape(-1, 3)
        Fi = np.ascontiguousarray(F, np.int32).reshape(-1, 3)
        cap = 1
        for d in range(3):
            cap *= int(np.ceil((V[:, d].max() - V[:, d].min()) / dx)) + 2
        out = np.zeros((cap, 3))
        self.lib.ref_sample_mesh.restype = C.c_int
        k = self.lib.ref_sample_mesh(_p(V), C.c_int(len(V)), Fi.ctypes.data_as(_ip), C.c_int(len(Fi)),
                                     C.c_double(dx), _p(out), C.c_int(cap))
        return out[:min(k, cap)]
