"""diffmpm_bindings -- GB300-native drop-in for the reference's pybind11 module.

Same names, argument meanings and error behaviour as bind/bind.cpp:54-560
(``OptInput``, ``PointCloud``, ``Grid``, ``CompGraph`` and the module
functions), implemented over the C ABI of libmpm.so (include/mpm.h).  All
simulation work runs in hand-written sm_103a CUDA kernels; particle state
stays resident on the GPU and getters copy it out.

Additive API (not in the reference): ``PointCloud.from_arrays``,
``PointCloud.get(field)``, ``CompGraph.set_sim_params``, ``CompGraph.options``,
``CompGraph.get_grad(...)``, ``set_default_precision`` and the
``torch.autograd.Function`` in ``diffmpm_bindings.rollout``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import (MPM_ADJ_EXACT, MPM_ADJ_REFERENCE, MPM_DTYPE_F32, MPM_DTYPE_F64, MPM_FP32, MPM_FP64,
                   MPM_KERNEL_CUBIC, MPM_KERNEL_QUADRATIC, MPM_MAT_FCR, MPM_MAT_NEOHOOKEAN, MpmError,
                   MpmOptInput, MpmOptions, MpmParams, check, lib)

__all__ = ["OptInput", "PointCloud", "Grid", "CompGraph", "load_point_cloud_from_obj", "calculate_lame_parameters",
           "p2g", "calculate_point_cloud_volumes", "get_positions_from_pc", "set_default_precision", "MpmError"]

_default_precision = MPM_FP32


def set_default_precision(p) -> None:
    """'fp32' (FP32 with FP64 guard, the default) or 'fp64' (plain all-FP64)."""
    global _default_precision
    _default_precision = _prec(p)


def _prec(p):
    if p is None:
        return _default_precision
    if isinstance(p, str):
        return {"fp32": MPM_FP32, "float32": MPM_FP32, "fp64": MPM_FP64, "float64": MPM_FP64}[p.lower()]
    return int(p)


def _np_dtype(prec):
    return np.float64 if prec == MPM_FP64 else np.float32


def _vec3(v):
    a = np.asarray(v, dtype=np.float32).reshape(-1)
    if a.size != 3:
        raise TypeError("expected a 3-vector")
    return a


# ----------------------------------------------------------------- OptInput

class OptInput:
    """OptInput (bind.cpp:30-52, 58-80): 21 read/write fields."""

    _float_fields = ("grid_dx", "lam", "mu", "p_density", "dt", "drag", "initial_alpha", "gd_tol",
                     "smoothing_factor")
    _int_fields = ("points_per_cell_cuberoot", "num_animations", "num_timesteps", "control_stride",
                   "max_gd_iters", "max_ls_iters", "current_episodes")
    _vec_fields = ("grid_min_point", "grid_max_point", "f_ext")

    def __init__(self):
        object.__setattr__(self, "mpm_input_mesh_path", "")
        object.__setattr__(self, "mpm_target_mesh_path", "")
        for f in self._float_fields:
            object.__setattr__(self, f, 0.0)
        for f in self._int_fields:
            object.__setattr__(self, f, 0)
        for f in self._vec_fields:
            object.__setattr__(self, f, np.zeros(3, dtype=np.float32))

    def __setattr__(self, name, value):
        if name in self._float_fields:
            value = float(np.float32(value))
        elif name in self._int_fields:
            value = int(value)
        elif name in self._vec_fields:
            value = _vec3(value)
        elif name in ("mpm_input_mesh_path", "mpm_target_mesh_path"):
            value = str(value)
        else:
            raise AttributeError(f"'OptInput' object has no attribute '{name}'")
        object.__setattr__(self, name, value)


# --------------------------------------------------------------- PointCloud

class PointCloud:
    """PointCloud (PointCloud.h:10-66; bind.cpp:83-157), resident on the GPU."""

    def __init__(self, handle=None, owner=None):
        if handle is None:
            raise TypeError("PointCloud objects come from load_point_cloud_from_obj, PointCloud.from_arrays "
                            "or CompGraph.get_point_cloud")
        self._h = handle
        self._owner = owner

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.mpm_pointcloud_release(h)
            self._h = None

    # -- construction (additive)
    @classmethod
    def create(cls, n: int, precision=None) -> "PointCloud":
        h = C.c_void_p()
        check(lib.mpm_pointcloud_create(int(n), _prec(precision), C.byref(h)), "PointCloud")
        return cls(h)

    @classmethod
    def from_arrays(cls, x, v=None, F=None, dFc=None, C_=None, m=None, vol=None, lam=None, mu=None,
                    precision=None) -> "PointCloud":
        """Build a point cloud from (N,3)/(N,3,3)/(N,) arrays (host numpy or torch)."""
        x = np.asarray(x)
        n = int(x.shape[0])
        pc = cls.create(n, precision)
        pc.set("x", x)
        for name, val in (("v", v), ("F", F), ("dFc", dFc), ("C", C_), ("m", m), ("vol", vol), ("lam", lam),
                          ("mu", mu)):
            if val is not None:
                pc.set(name, val)
        return pc

    @property
    def size(self) -> int:
        n = C.c_int()
        check(lib.mpm_pointcloud_size(self._h, C.byref(n)))
        return n.value

    def __len__(self):
        return self.size

    @property
    def precision(self) -> int:
        p = C.c_int()
        check(lib.mpm_pointcloud_precision(self._h, C.byref(p)))
        return p.value

    def set(self, field: str, value) -> None:
        """Copy a field in from a host array or a CUDA torch tensor (additive)."""
        shape = (self.size,) + _lib.FIELD_SHAPE[field]
        try:
            import torch  # noqa: WPS433
            if isinstance(value, torch.Tensor):
                t = value.detach().contiguous()
                if tuple(t.shape) != shape:
                    raise RuntimeError(f"{field} must have shape {shape}, got {tuple(t.shape)}")
                if t.dtype not in (torch.float32, torch.float64):
                    t = t.float()
                dt = MPM_DTYPE_F64 if t.dtype == torch.float64 else MPM_DTYPE_F32
                if t.is_cuda:
                    check(lib.mpm_pointcloud_set(self._h, _lib.FIELDS[field], C.c_void_p(t.data_ptr()), dt, 1), field)
                    return
                value = t.numpy()
        except ImportError:
            pass
        a = np.asarray(value)
        if a.dtype not in (np.float32, np.float64):
            a = a.astype(np.float32)
        a = np.ascontiguousarray(a)
        if a.shape != shape:
            raise RuntimeError(f"{field} must have shape {shape}, got {a.shape}")
        dt = MPM_DTYPE_F64 if a.dtype == np.float64 else MPM_DTYPE_F32
        check(lib.mpm_pointcloud_set(self._h, _lib.FIELDS[field], a.ctypes.data_as(C.c_void_p), dt, 0), field)

    def get(self, field: str, dtype=np.float32) -> np.ndarray:
        """Copy a field out as a host array (additive)."""
        out = np.empty((self.size,) + _lib.FIELD_SHAPE[field], dtype=dtype)
        dt = MPM_DTYPE_F64 if out.dtype == np.float64 else MPM_DTYPE_F32
        check(lib.mpm_pointcloud_get(self._h, _lib.FIELDS[field], out.ctypes.data_as(C.c_void_p), dt, 0), field)
        return out

    def get_torch(self, field: str, device="cpu", dtype=None, requires_grad=False):
        """Copy a field into a torch tensor; on CUDA the copy stays on the device (additive)."""
        import torch
        dtype = dtype or torch.float32
        shape = (self.size,) + _lib.FIELD_SHAPE[field]
        t = torch.empty(shape, dtype=dtype, device=device)
        dt = MPM_DTYPE_F64 if dtype == torch.float64 else MPM_DTYPE_F32
        if t.is_cuda:
            torch.cuda.current_stream(t.device).synchronize()
            check(lib.mpm_pointcloud_get(self._h, _lib.FIELDS[field], C.c_void_p(t.data_ptr()), dt, 1), field)
        else:
            check(lib.mpm_pointcloud_get(self._h, _lib.FIELDS[field], C.c_void_p(t.data_ptr()), dt, 0), field)
        if requires_grad:
            t.requires_grad_(True)
        return t

    # -- reference getters (bind.cpp:84-157)
    def get_positions(self):
        """(N,3) float32 positions (PointCloud::GetPointPositions)."""
        return self.get("x")

    def get_masses(self):
        return self.get("m")

    def get_volumes(self):
        return self.get("vol")

    def get_def_grads(self):
        """(N,3,3) F only (PointCloud::GetPointDefGrads)."""
        return self.get("F")

    def get_def_grads_morph(self):
        """(N,3,3) control dFc."""
        return self.get("dFc")

    def get_def_grads_total(self):
        """(N,3,3) F + dFc."""
        return self.get("F_total")

    def get_point_determinants(self):
        """det(F + dFc) per particle (PointCloud::GetPointDeterminants)."""
        return np.linalg.det(self.get("F_total", np.float64)).astype(np.float32)

    def get_positions_torch(self, requires_grad=False):
        """CPU float32 leaf tensor (N,3) (bind.cpp:89-107)."""
        return self.get_torch("x", "cpu", requires_grad=requires_grad)

    def get_def_grads_total_torch(self, requires_grad=False):
        """CPU float32 leaf tensor (N,3,3) of F + dFc (bind.cpp:109-131)."""
        return self.get_torch("F_total", "cpu", requires_grad=requires_grad)


# --------------------------------------------------------------------- Grid

class Grid:
    """Grid(dim_x, dim_y, dim_z, dx, min_point) (Grid.cpp:7-26; bind.cpp:159-160)."""

    def __init__(self, dim_x, dim_y, dim_z, dx, min_point, precision=None):
        prec = _prec(precision)
        # dx and min_point are float in the reference (Grid.h:96-100): an FP32
        # grid keeps their float32 values, an FP64 grid the exact ones
        if prec == MPM_FP64:
            mn = np.asarray(min_point, dtype=np.float64).reshape(3).copy()
            dxv = float(dx)
        else:
            mn = np.asarray(_vec3(min_point), dtype=np.float64)
            dxv = float(np.float32(dx))
        h = C.c_void_p()
        check(lib.mpm_grid_create(int(dim_x), int(dim_y), int(dim_z), dxv, mn.ctypes.data_as(_lib._dp), prec,
                                  C.byref(h)), "Grid")
        self._h = h
        self.dims = (int(dim_x), int(dim_y), int(dim_z))
        self.dx = dxv
        self.min_point = mn.copy()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.mpm_grid_release(h)
            self._h = None

    @property
    def num_nodes(self) -> int:
        return self.dims[0] * self.dims[1] * self.dims[2]

    def get_node_masses(self, dtype=np.float32):
        out = np.empty(self.num_nodes, dtype=dtype)
        dt = MPM_DTYPE_F64 if out.dtype == np.float64 else MPM_DTYPE_F32
        check(lib.mpm_grid_get(self._h, 0, out.ctypes.data_as(C.c_void_p), dt, 0))
        return out

    def get_node_momenta(self, dtype=np.float32):
        out = np.empty((self.num_nodes, 3), dtype=dtype)
        dt = MPM_DTYPE_F64 if out.dtype == np.float64 else MPM_DTYPE_F32
        check(lib.mpm_grid_get(self._h, 1, out.ctypes.data_as(C.c_void_p), dt, 0))
        return out

    def set_node_masses(self, m):
        a = np.ascontiguousarray(np.asarray(m, dtype=np.float64).reshape(-1))
        if a.size != self.num_nodes:
            raise RuntimeError(f"expected {self.num_nodes} node masses, got {a.size}")
        check(lib.mpm_grid_set(self._h, 0, a.ctypes.data_as(C.c_void_p), MPM_DTYPE_F64, 0))

    def get_node_positions(self):
        i, j, k = np.meshgrid(*(np.arange(d, dtype=np.float32) for d in self.dims), indexing="ij")
        ijk = np.stack([i, j, k], -1).reshape(-1, 3)
        return (self.min_point.astype(np.float32) + ijk * np.float32(self.dx)).astype(np.float32)


# ---------------------------------------------------------------- CompGraph

class CompGraph:
    """CompGraph (CompGraph.h:20-99; bind.cpp:163-528) on the GPU.

    ``options`` (additive) selects precision ('fp32'/'fp64'), the adjoint
    ('reference' reproduces BackPropagation.cpp term for term, 'exact' is the
    true derivative), the kernel ('cubic'/'quadratic'), the material
    ('fcr'/'neohookean'), checkpointing (keep every k-th layer) and
    ``deterministic`` (FP32: node sums in 64-bit fixed point, bitwise
    reproducible).
    """

    def __init__(self, point_cloud: PointCloud, grid: Grid, target_grid: Grid, *, adjoint="reference",
                 kernel="cubic", material="fcr", checkpoint_every=1, deterministic=False):
        if point_cloud is None or grid is None:
            raise RuntimeError("PointCloud or Grid is null.")
        o = MpmOptions()
        lib.mpm_default_options(C.byref(o))
        o.precision = point_cloud.precision
        o.adjoint = {"reference": MPM_ADJ_REFERENCE, "exact": MPM_ADJ_EXACT}[adjoint] \
            if isinstance(adjoint, str) else int(adjoint)
        o.kernel = {"cubic": MPM_KERNEL_CUBIC, "quadratic": MPM_KERNEL_QUADRATIC}[kernel] \
            if isinstance(kernel, str) else int(kernel)
        o.material = {"fcr": MPM_MAT_FCR, "neohookean": MPM_MAT_NEOHOOKEAN}[material] \
            if isinstance(material, str) else int(material)
        o.checkpoint_every = int(checkpoint_every)
        o.deterministic = int(bool(deterministic))
        h = C.c_void_p()
        check(lib.mpm_compgraph_create(point_cloud._h, grid._h, target_grid._h if target_grid is not None else None,
                                       C.byref(o), C.byref(h)), "CompGraph")
        self._h = h
        self._target = target_grid  # aliased, like std::shared_ptr<const Grid>
        self._grid = grid
        self.precision = o.precision

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.mpm_compgraph_release(h)
            self._h = None

    @classmethod
    def batch(cls, point_clouds, grids, *, adjoint="reference", kernel="cubic", material="fcr",
              checkpoint_every=1, deterministic=False) -> "CompGraph":
        """Independent instances advanced together in one launch per kernel
        (additive).  ``instance_range(i)`` gives the
        slice of instance i in the concatenated layer arrays."""
        if len(point_clouds) != len(grids) or not point_clouds:
            raise RuntimeError("batch needs one grid per point cloud")
        o = MpmOptions()
        lib.mpm_default_options(C.byref(o))
        o.precision = point_clouds[0].precision
        o.adjoint = {"reference": MPM_ADJ_REFERENCE, "exact": MPM_ADJ_EXACT}[adjoint]
        o.kernel = {"cubic": MPM_KERNEL_CUBIC, "quadratic": MPM_KERNEL_QUADRATIC}[kernel]
        o.material = {"fcr": MPM_MAT_FCR, "neohookean": MPM_MAT_NEOHOOKEAN}[material]
        o.checkpoint_every = int(checkpoint_every)
        o.deterministic = int(bool(deterministic))
        k = len(point_clouds)
        pcs = (C.c_void_p * k)(*[p._h for p in point_clouds])
        gs = (C.c_void_p * k)(*[g._h for g in grids])
        h = C.c_void_p()
        check(lib.mpm_compgraph_create_batch(pcs, gs, k, C.byref(o), C.byref(h)), "CompGraph.batch")
        self = cls.__new__(cls)
        self._h = h
        self._target = None
        self._grid = list(grids)
        self.precision = o.precision
        cnt = C.c_int()
        po = (C.c_longlong * (k + 1))()
        check(lib.mpm_compgraph_batch_offsets(h, C.byref(cnt), po, None))
        self.sizes = [len(p) for p in point_clouds]
        self.offsets = [int(po[i]) for i in range(k)]
        return self

    def instance_range(self, i: int) -> slice:
        return slice(self.offsets[i], self.offsets[i] + self.sizes[i])

    # -- additive configuration
    @property
    def options(self) -> dict:
        o = MpmOptions()
        check(lib.mpm_compgraph_get_options(self._h, C.byref(o)))
        return dict(precision=o.precision, adjoint=o.adjoint, kernel=o.kernel, material=o.material,
                    checkpoint_every=o.checkpoint_every, deterministic=bool(o.deterministic))

    def resort(self):
        """Order the particles by grid cell (additive; the order callers see
        does not change)."""
        check(lib.mpm_compgraph_resort(self._h))

    def set_resort(self, on=True):
        """Re-sort at set_up_comp_graph (default on)."""
        check(lib.mpm_compgraph_set_resort(self._h, int(bool(on))))

    def set_resort_every(self, layers=-1):
        """Re-sort inside a rollout every `layers` layers (segment starts);
        -1 automatic, 0 never (additive)."""
        check(lib.mpm_compgraph_set_resort_every(self._h, int(layers)))

    def resort_every(self) -> int:
        """The in-rollout re-sort interval in effect (0: never)."""
        v = C.c_int()
        check(lib.mpm_compgraph_get_resort_every(self._h, C.byref(v)))
        return v.value

    def particle_order(self, layer: int) -> np.ndarray:
        """Slot p of the layer's device planes holds the caller's particle
        out[p] (diagnostics)."""
        out = np.empty(len(self.get_point_cloud(layer)), np.int32)
        check(lib.mpm_compgraph_particle_order(self._h, int(layer), out.ctypes.data_as(C.POINTER(C.c_int))))
        return out

    def set_deterministic(self, on=True):
        """Fixed-point node sums (FP32 graphs): bitwise reproducible passes."""
        check(lib.mpm_compgraph_set_deterministic(self._h, int(bool(on))))

    def get_sim_params(self) -> dict:
        p = MpmParams()
        check(lib.mpm_compgraph_get_params(self._h, C.byref(p)))
        return dict(dt=p.dt, drag=p.drag, smoothing=p.smoothing, f_ext=tuple(p.f_ext), bulk_viscosity=p.bulk_viscosity,
                    j_min=p.j_min)

    def set_sim_params(self, dt=None, drag=None, smoothing=None, f_ext=None, bulk_viscosity=None, j_min=None):
        """Set the simulation parameters CompGraph keeps private (CompGraph.h:78-83)."""
        p = MpmParams()
        check(lib.mpm_compgraph_get_params(self._h, C.byref(p)))
        if dt is not None:
            p.dt = float(dt)
        if drag is not None:
            p.drag = float(drag)
        if smoothing is not None:
            p.smoothing = float(smoothing)
        if f_ext is not None:
            p.f_ext[:] = [float(v) for v in np.asarray(f_ext).reshape(3)]
        if bulk_viscosity is not None:
            p.bulk_viscosity = float(bulk_viscosity)
        if j_min is not None:
            p.j_min = float(j_min)
        check(lib.mpm_compgraph_set_params(self._h, C.byref(p)))

    def set_stream(self, stream) -> None:
        """Run on a torch.cuda.Stream / raw cudaStream_t (None: the graph's own)."""
        ptr = getattr(stream, "cuda_stream", stream)
        check(lib.mpm_compgraph_set_stream(self._h, C.c_void_p(ptr) if ptr else None))

    def autotune(self, steps: int = 4, layer: int = 0) -> dict:
        """Pick the fastest scatter strategy, node-tile budgets and block size
        for this graph by timing short forward+backward passes from the state of
        `layer` (additive; a stored layer deep in a computed rollout reflects
        the particle drift of long rollouts)."""
        t, m, ms = C.c_int(), C.c_int(), C.c_double()
        check(lib.mpm_compgraph_autotune_from(self._h, int(layer), int(steps), C.byref(t), C.byref(m), C.byref(ms)),
              "autotune")
        out = self.get_tuning()
        out.update(ms_per_pass=ms.value, steps=int(steps), from_layer=int(layer))
        return out

    def set_tuning(self, tile_nodes=-1, scatter_mode=-1, adj_tile_nodes=-1, gather_tile_nodes=-1,
                   block_threads=-1):
        """P2G's tile budget and the scatter strategy, the tile budgets of
        the G2P transpose's scatter and the P2G transpose's gather, and the
        threads (= particles) per block of the step kernels (-1: library
        defaults; the adjoint budgets follow P2G's; 256 threads)."""
        check(lib.mpm_compgraph_set_tuning(self._h, int(tile_nodes), int(scatter_mode)))
        check(lib.mpm_compgraph_set_adjoint_tiles(self._h, int(adj_tile_nodes), int(gather_tile_nodes)))
        check(lib.mpm_compgraph_set_block_threads(self._h, int(block_threads)))

    def get_tuning(self) -> dict:
        t, m, at, gt, th = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(lib.mpm_compgraph_get_tuning(self._h, C.byref(t), C.byref(m)))
        check(lib.mpm_compgraph_get_adjoint_tiles(self._h, C.byref(at), C.byref(gt)))
        check(lib.mpm_compgraph_get_block_threads(self._h, C.byref(th)))
        return {"tile_nodes": t.value, "scatter_mode": m.value, "adj_tile_nodes": at.value,
                "gather_tile_nodes": gt.value, "block_threads": th.value}

    def use_graphs(self, on=True):
        """Replay forward/backward passes as CUDA graphs (default on)."""
        check(lib.mpm_compgraph_use_graphs(self._h, int(bool(on))))

    def enable_lame_grads(self, on=True):
        check(lib.mpm_compgraph_enable_lame_grads(self._h, int(bool(on))))

    def synchronize(self):
        check(lib.mpm_compgraph_synchronize(self._h))

    # -- reference surface
    def run_optimization(self, opt: OptInput, *, passes: int | None = None):
        """OptimizeDefGradControlSequence (CompGraph.cpp:213-368).  ``passes``
        (additive) replaces the reference's fixed 3 passes over the control
        steps."""
        o = MpmOptInput()
        o.passes = int(passes or 0)
        o.num_timesteps, o.control_stride = opt.num_timesteps, opt.control_stride
        o.max_gd_iters, o.max_ls_iters, o.current_episodes = opt.max_gd_iters, opt.max_ls_iters, opt.current_episodes
        o.dt, o.drag, o.smoothing_factor = opt.dt, opt.drag, opt.smoothing_factor
        o.initial_alpha, o.gd_tol = opt.initial_alpha, opt.gd_tol
        o.f_ext[:] = [float(v) for v in opt.f_ext]
        check(lib.mpm_compgraph_run_optimization(self._h, C.byref(o)), "run_optimization")

    def loss_history(self) -> np.ndarray:
        """Every loss the last run_optimization or optimize_single_timestep
        evaluated, in order (additive)."""
        n = C.c_int()
        check(lib.mpm_compgraph_loss_history(self._h, None, 0, C.byref(n)))
        out = np.zeros(n.value)
        check(lib.mpm_compgraph_loss_history(self._h, out.ctypes.data_as(_lib._dp), n.value, C.byref(n)))
        return out

    def get_num_layers(self) -> int:
        n = C.c_int()
        check(lib.mpm_compgraph_num_layers(self._h, C.byref(n)))
        return n.value

    def get_point_cloud(self, layer_idx: int) -> PointCloud:
        if layer_idx < 0:
            raise TypeError("layer_idx must be non-negative")
        if layer_idx >= self.get_num_layers():
            raise IndexError("Layer index out of range.")
        h = C.c_void_p()
        check(lib.mpm_compgraph_layer(self._h, int(layer_idx), C.byref(h)))
        return PointCloud(h, owner=self)

    def get_point_cloud_at_timestep(self, timestep_idx: int) -> PointCloud:
        n = self.get_num_layers()
        if timestep_idx < 0 or timestep_idx >= n:
            raise IndexError(f"Timestep index {timestep_idx} out of range [0, {n})")
        h = C.c_void_p()
        check(lib.mpm_compgraph_layer(self._h, int(timestep_idx), C.byref(h)))
        return PointCloud(h, owner=self)

    def end_layer_mass_loss(self) -> float:
        out = C.c_double()
        check(lib.mpm_compgraph_mass_loss(self._h, C.byref(out)), "end_layer_mass_loss")
        # the reference returns a float; the FP64 engine returns its double
        return out.value if self.precision == MPM_FP64 else float(np.float32(out.value))

    @staticmethod
    def _render_arrays(dLdF_render, dLdx_render, verb):
        gF = np.asarray(dLdF_render, dtype=np.float32)
        gX = np.asarray(dLdx_render, dtype=np.float32)
        if gF.ndim != 3 or gF.shape[1] != 3 or gF.shape[2] != 3:
            sh = tuple(gF.shape) + (0,) * (3 - gF.ndim)
            raise RuntimeError(f"dLdF must be (N,3,3), got {verb}({sh[0]},{sh[1]},{sh[2]})")
        if gX.ndim != 2 or gX.shape[1] != 3:
            sh = tuple(gX.shape) + (0,) * (2 - gX.ndim)
            raise RuntimeError(f"dLdx must be (N,3), got {verb}({sh[0]},{sh[1]})")
        return np.ascontiguousarray(gF), np.ascontiguousarray(gX)

    def accumulate_render_grads(self, dLdF_render, dLdx_render):
        gF, gX = self._render_arrays(dLdF_render, dLdx_render, "")
        n = self.get_point_cloud(self.get_num_layers() - 1).size
        if gF.shape[0] != n or gX.shape[0] != n:
            raise RuntimeError(f"Shape mismatch: point cloud has {n} points, but got dLdF with {gF.shape[0]} "
                               f"and dLdx with {gX.shape[0]}")
        check(lib.mpm_compgraph_accumulate_render_grads(self._h, gF.ctypes.data_as(_lib._fp),
                                                        gX.ctypes.data_as(_lib._fp), n))

    def promote_last_as_initial(self, carry_grid=False):
        check(lib.mpm_compgraph_promote_last_as_initial(self._h, int(bool(carry_grid))))

    def optimize_single_timestep(self, timestep_idx, max_gd_iters=1, current_episode=0, initial_alpha=1.0,
                                 max_line_search_iters=10):
        check(lib.mpm_compgraph_optimize_single_timestep(self._h, int(timestep_idx), int(max_gd_iters),
                                                         int(current_episode), float(np.float32(initial_alpha)),
                                                         int(max_line_search_iters)), "optimize_single_timestep")

    def set_up_comp_graph(self, num_layers):
        check(lib.mpm_compgraph_set_up(self._h, int(num_layers)), "set_up_comp_graph")

    def compute_forward_pass(self, start_layer, current_episode=0):
        check(lib.mpm_compgraph_forward(self._h, int(start_layer), int(current_episode)), "compute_forward_pass")

    def compute_backward_pass(self, control_layer):
        check(lib.mpm_compgraph_backward(self._h, int(control_layer)), "compute_backward_pass")

    def set_render_gradients(self, dLdF_render, dLdx_render):
        if self.get_num_layers() < 1:
            raise RuntimeError("CompGraph has no layers!")
        gF, gX = self._render_arrays(dLdF_render, dLdx_render, "shape ")
        if gX.shape[0] != gF.shape[0]:
            raise RuntimeError(f"Shape mismatch: dLdF has {gF.shape[0]} points, but dLdx has {gX.shape[0]}")
        check(lib.mpm_compgraph_set_render_gradients(self._h, gF.ctypes.data_as(_lib._fp),
                                                     gX.ctypes.data_as(_lib._fp), int(gF.shape[0])))

    def clear_render_gradients(self):
        check(lib.mpm_compgraph_clear_render_gradients(self._h))

    def has_render_gradients(self) -> bool:
        return bool(self.get_render_gradient_info()["has_gradients"])

    def get_render_gradient_info(self) -> dict:
        has, n = C.c_int(), C.c_int()
        nf, nx = C.c_double(), C.c_double()
        check(lib.mpm_compgraph_render_gradient_info(self._h, C.byref(has), C.byref(n), C.byref(nf), C.byref(nx)))
        return {"has_gradients": bool(has.value), "num_points": int(n.value),
                "grad_F_norm": float(np.float32(nf.value)), "grad_x_norm": float(np.float32(nx.value))}

    # -- additive gradient access
    def get_grad(self, layer: int, field: str = "F", dtype=np.float32) -> np.ndarray:
        """dL/d{x,v,F,C,dFc,lam,mu} of a layer after compute_backward_pass."""
        return self.get_point_cloud(layer).get("grad_" + field, dtype)

    def get_grad_v0(self, dtype=np.float32) -> np.ndarray:
        """dL/dv of layer 0, (N, 3)."""
        return self.get_grad(0, "v", dtype)

    def get_grad_F(self, layer: int = 0, dtype=np.float32) -> np.ndarray:
        """dL/d(control F) of a layer, (N, 3, 3): the gradient the control
        optimisation descends (ForwardSimulation.cpp uses F + dFc)."""
        return self.get_grad(layer, "dFc", dtype)

    def get_grad_E(self, young_modulus: float, layer: int = 0) -> float:
        """dL/dE for a material whose Lame parameters all scale with one
        Young's modulus E at fixed Poisson ratio (lam, mu proportional to E):
        (sum dL/dlam * lam + sum dL/dmu * mu) / E.  Needs
        enable_lame_grads(True) before the backward pass; the sums run from
        `layer` (the control layer of that pass) to the end."""
        pc = self.get_point_cloud(layer)
        glam, gmu = pc.get("grad_lam", np.float64), pc.get("grad_mu", np.float64)
        lam, mu = pc.get("lam", np.float64), pc.get("mu", np.float64)
        return float((glam @ lam + gmu @ mu) / float(young_modulus))

    def grad_norm(self, layer: int) -> float:
        out = C.c_double()
        check(lib.mpm_compgraph_grad_norm(self._h, int(layer), C.byref(out)))
        return out.value

    def adam_step(self, layer, alpha, grad_norm, beta1=0.9, beta2=0.999, eps=1e-3, timestep=1):
        check(lib.mpm_compgraph_adam_step(self._h, int(layer), float(alpha), float(grad_norm), float(beta1),
                                          float(beta2), float(eps), int(timestep)))

    def has_nonfinite(self, layer: int, grads: bool = False) -> bool:
        """NaN/Inf anywhere in the layer's state (and gradient) planes (additive)."""
        f = C.c_int()
        check(lib.mpm_compgraph_nonfinite(self._h, int(layer), int(bool(grads)), C.byref(f)))
        return bool(f.value)

    def active_nodes(self, layer: int = 0) -> int:
        out = C.c_ulonglong()
        check(lib.mpm_compgraph_active_nodes(self._h, int(layer), C.byref(out)))
        return int(out.value)


# ------------------------------------------------------------------ utilities

def calculate_lame_parameters(young_mod, poisson):
    """(lam, mu) computed in float32 like Elasticity.cpp:149-153."""
    E, nu = np.float32(young_mod), np.float32(poisson)
    one = np.float32(1.0)
    lam = E * nu / ((one + nu) * (one - np.float32(2.0) * nu))
    mu = E / (np.float32(2.0) + np.float32(2.0) * nu)
    return float(lam), float(mu)


def p2g(pc: PointCloud, grid: Grid):
    """P2G(pc, grid, dt=0, drag=0) into the un-reset grid (bind.cpp:546-549)."""
    if pc is None or grid is None:
        raise RuntimeError("PointCloud or Grid is null.")
    check(lib.mpm_p2g(pc._h, grid._h))


def calculate_point_cloud_volumes(pc: PointCloud, grid: Grid):
    """CalculatePointCloudVolumes (ForwardSimulation.cpp:234-271; bind.cpp:551-554)."""
    if pc is None or grid is None:
        raise RuntimeError("PointCloud or Grid is null.")
    check(lib.mpm_calculate_point_cloud_volumes(pc._h, grid._h))


def get_positions_from_pc(pc: PointCloud):
    if pc is None:
        raise RuntimeError("PointCloud is null.")
    return pc.get_positions()


def load_point_cloud_from_obj(obj_path: str, opt: OptInput, precision=None) -> PointCloud:
    """Mesh -> lattice points inside it (GeometryLoading.cpp:85-143; bind.cpp:531-538)."""
    from .geometry import lattice_inside_mesh, read_obj
    try:
        V, Fc = read_obj(obj_path)
    except Exception as e:  # noqa: BLE001
        raise RuntimeError(f"Failed to load PointCloud from: {obj_path}") from e
    point_dx = np.float32(opt.grid_dx) / np.float32(opt.points_per_cell_cuberoot)
    pts = lattice_inside_mesh(V, Fc, float(point_dx))
    n = len(pts)
    m = np.float32(point_dx) ** 3 * np.float32(opt.p_density)
    vol = m / np.float32(opt.p_density)
    return PointCloud.from_arrays(pts.astype(np.float32), m=np.full(n, m, np.float32),
                                  vol=np.full(n, vol, np.float32), lam=np.full(n, opt.lam, np.float32),
                                  mu=np.full(n, opt.mu, np.float32), precision=precision)


def single_timestep_adam_step(set_to=None) -> int:
    """OptimizeSingleTimestep's process-wide Adam step counter (a
    function-local static in the reference, CompGraph.cpp:396): returns it
    and, with ``set_to``, replaces it afterwards (additive)."""
    cur = C.c_int()
    new = None if set_to is None else C.byref(C.c_int(int(set_to)))
    check(lib.mpm_single_timestep_adam_step(C.byref(cur), new), "single_timestep_adam_step")
    return cur.value


def step_count():
    """(forward, adjoint) particle-layer steps executed since load (additive)."""
    f, b = C.c_longlong(), C.c_longlong()
    lib.mpm_step_count(C.byref(f), C.byref(b))
    return f.value, b.value
