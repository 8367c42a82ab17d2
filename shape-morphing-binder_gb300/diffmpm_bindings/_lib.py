"""ctypes binding of libmpm.so (the C ABI in include/mpm.h).

The library is built in-tree by ``shape-morphing-binder_gb300/build.py``.
It is opened on first use (the first call through ``lib``), so importing the
package -- e.g. for its numpy-only workload generators -- maps no native
code.  Opening fails loudly when the library is missing: there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

# the in-tree build; MPM_LIB_PATH names another build of the same library
LIB_PATH = Path(os.environ.get("MPM_LIB_PATH") or Path(__file__).resolve().parent / "libmpm.so")

MPM_OK, MPM_ERR_ARG, MPM_ERR_SHAPE, MPM_ERR_OOM, MPM_ERR_NONFINITE, MPM_ERR_TIMEOUT, MPM_ERR_CUDA, \
    MPM_ERR_STATE, MPM_ERR_RANGE = range(9)
MPM_FP32, MPM_FP64 = 0, 1
MPM_DTYPE_F32, MPM_DTYPE_F64 = 0, 1
MPM_ADJ_REFERENCE, MPM_ADJ_EXACT = 0, 1
MPM_KERNEL_CUBIC, MPM_KERNEL_QUADRATIC = 0, 1
MPM_MAT_FCR, MPM_MAT_NEOHOOKEAN = 0, 1

FIELDS = dict(x=0, v=1, F=2, C=3, dFc=4, F_total=5, m=6, vol=7, lam=8, mu=9,
              grad_x=10, grad_v=11, grad_F=12, grad_C=13, grad_dFc=14, grad_lam=15, grad_mu=16)
FIELD_SHAPE = dict(x=(3,), v=(3,), F=(3, 3), C=(3, 3), dFc=(3, 3), F_total=(3, 3), m=(), vol=(), lam=(), mu=(),
                   grad_x=(3,), grad_v=(3,), grad_F=(3, 3), grad_C=(3, 3), grad_dFc=(3, 3), grad_lam=(), grad_mu=())
GRID_FIELDS = dict(mass=0, momentum=1, velocity=2)


class MpmParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("drag", C.c_double), ("smoothing", C.c_double), ("f_ext", C.c_double * 3),
                ("bulk_viscosity", C.c_double), ("j_min", C.c_double)]


class MpmOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("adjoint", C.c_int), ("kernel", C.c_int), ("material", C.c_int),
                ("checkpoint_every", C.c_int), ("deterministic", C.c_int)]


class MpmOptInput(C.Structure):
    _fields_ = [("num_timesteps", C.c_int), ("control_stride", C.c_int), ("max_gd_iters", C.c_int),
                ("max_ls_iters", C.c_int), ("current_episodes", C.c_int), ("dt", C.c_double),
                ("drag", C.c_double), ("smoothing_factor", C.c_double), ("initial_alpha", C.c_double),
                ("gd_tol", C.c_double), ("f_ext", C.c_double * 3), ("passes", C.c_int)]


_vp = C.c_void_p
_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)

# name -> (argtypes) ; all return int unless listed in _RESTYPE
_SIGS = {
    "mpm_version": [],
    "mpm_last_error": [],
    "mpm_default_params": [C.POINTER(MpmParams)],
    "mpm_default_options": [C.POINTER(MpmOptions)],
    "mpm_set_verbose": [C.c_int],
    "mpm_set_tile_nodes": [C.c_int],
    "mpm_set_scatter_mode": [C.c_int],
    "mpm_set_fused_steps": [C.c_int],
    "mpm_lame": [C.c_double, C.c_double, _dp, _dp],
    "mpm_pointcloud_create": [C.c_int, C.c_int, C.POINTER(_vp)],
    "mpm_pointcloud_set": [_vp, C.c_int, _vp, C.c_int, C.c_int],
    "mpm_pointcloud_get": [_vp, C.c_int, _vp, C.c_int, C.c_int],
    "mpm_pointcloud_size": [_vp, _ip],
    "mpm_pointcloud_precision": [_vp, _ip],
    "mpm_pointcloud_release": [_vp],
    "mpm_grid_create": [C.c_int, C.c_int, C.c_int, C.c_double, _dp, C.c_int, C.POINTER(_vp)],
    "mpm_grid_info": [_vp, _ip, _dp, _dp],
    "mpm_grid_get": [_vp, C.c_int, _vp, C.c_int, C.c_int],
    "mpm_grid_set": [_vp, C.c_int, _vp, C.c_int, C.c_int],
    "mpm_grid_release": [_vp],
    "mpm_p2g": [_vp, _vp],
    "mpm_calculate_point_cloud_volumes": [_vp, _vp],
    "mpm_compgraph_create": [_vp, _vp, _vp, C.POINTER(MpmOptions), C.POINTER(_vp)],
    "mpm_compgraph_release": [_vp],
    "mpm_compgraph_create_batch": [C.POINTER(_vp), C.POINTER(_vp), C.c_int, C.POINTER(MpmOptions), C.POINTER(_vp)],
    "mpm_compgraph_batch_offsets": [_vp, _ip, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)],
    "mpm_compgraph_set_params": [_vp, C.POINTER(MpmParams)],
    "mpm_compgraph_get_params": [_vp, C.POINTER(MpmParams)],
    "mpm_compgraph_get_options": [_vp, C.POINTER(MpmOptions)],
    "mpm_compgraph_set_stream": [_vp, _vp],
    "mpm_compgraph_set_up": [_vp, C.c_int],
    "mpm_compgraph_num_layers": [_vp, _ip],
    "mpm_compgraph_forward": [_vp, C.c_int, C.c_int],
    "mpm_compgraph_backward": [_vp, C.c_int],
    "mpm_compgraph_mass_loss": [_vp, _dp],
    "mpm_compgraph_accumulate_render_grads": [_vp, _fp, _fp, C.c_int],
    "mpm_compgraph_set_render_gradients": [_vp, _fp, _fp, C.c_int],
    "mpm_compgraph_clear_render_gradients": [_vp],
    "mpm_compgraph_render_gradient_info": [_vp, _ip, _ip, _dp, _dp],
    "mpm_compgraph_layer": [_vp, C.c_int, C.POINTER(_vp)],
    "mpm_compgraph_promote_last_as_initial": [_vp, C.c_int],
    "mpm_compgraph_grad_norm": [_vp, C.c_int, _dp],
    "mpm_compgraph_adam_step": [_vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int],
    "mpm_compgraph_optimize_single_timestep": [_vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int],
    "mpm_compgraph_run_optimization": [_vp, C.POINTER(MpmOptInput)],
    "mpm_compgraph_active_nodes": [_vp, C.c_int, C.POINTER(C.c_ulonglong)],
    "mpm_compgraph_enable_lame_grads": [_vp, C.c_int],
    "mpm_compgraph_use_graphs": [_vp, C.c_int],
    "mpm_compgraph_set_tuning": [_vp, C.c_int, C.c_int],
    "mpm_compgraph_set_deterministic": [_vp, C.c_int],
    "mpm_compgraph_resort": [_vp],
    "mpm_compgraph_nonfinite": [_vp, C.c_int, C.c_int, _ip],
    "mpm_winding_numbers": [C.c_int, _vp, C.c_int, _vp, _vp, C.c_int, _vp],
    # Gaussian-splatting rasterizer (include/gsplat.h; structs passed by pointer)
    "gs_scratch_bytes": [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)],
    "gs_preprocess": [_vp, _vp, _vp, C.c_size_t, _ip, _vp],
    "gs_render": [_vp, _vp, C.c_int, _vp, _vp, C.c_size_t, _vp, _vp],
    "gs_backward": [_vp, _vp, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "mpm_compgraph_set_resort": [_vp, C.c_int],
    "mpm_compgraph_set_resort_every": [_vp, C.c_int],
    "mpm_compgraph_get_resort_every": [_vp, _ip],
    "mpm_compgraph_particle_order": [_vp, C.c_int, _ip],
    "mpm_compgraph_loss_history": [_vp, _dp, C.c_int, _ip],
    "mpm_step_count": [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)],
    "mpm_compgraph_get_tuning": [_vp, _ip, _ip],
    "mpm_compgraph_autotune": [_vp, C.c_int, _ip, _ip, _dp],
    "mpm_compgraph_autotune_from": [_vp, C.c_int, C.c_int, _ip, _ip, _dp],
    "mpm_compgraph_set_adjoint_tiles": [_vp, C.c_int, C.c_int],
    "mpm_compgraph_get_adjoint_tiles": [_vp, _ip, _ip],
    "mpm_compgraph_set_block_threads": [_vp, C.c_int],
    "mpm_compgraph_get_block_threads": [_vp, _ip],
    "mpm_compgraph_synchronize": [_vp],
    "mpm_profile_enable": [C.c_int],
    "mpm_profile_select": [C.c_ulonglong],
    "mpm_profile_reset": [],
    "mpm_profile_query": [C.c_int, C.POINTER(C.c_longlong), _dp],
    "mpm_kernel_name": [C.c_int],
    "mpm_launch_count": [],
    "mpm_mass_loss_noalloc": [C.c_int, _vp, _vp, _vp, _ip, C.c_double, _dp, C.c_int, _vp, _dp, _vp],
    "mpm_constitutive": [C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _ip],
    "mpm_single_timestep_adam_step": [_ip, _ip],
}
_RESTYPE = {"mpm_last_error": C.c_char_p, "mpm_kernel_name": C.c_char_p, "mpm_launch_count": C.c_longlong, "mpm_default_params": None, "mpm_default_options": None,
            "mpm_set_verbose": None, "mpm_step_count": None}


class MpmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class MpmIndexError(IndexError):
    pass


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"libmpm.so not found at {LIB_PATH}; build it with "
            "`python shape-morphing-binder_gb300/build.py` (no CPU fallback exists)")
    lib = C.CDLL(str(LIB_PATH))
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPE.get(name, C.c_int)
    if os.environ.get("MPM_QUIET"):
        lib.mpm_set_verbose(0)
    return lib


class _LazyLib:
    """libmpm.so, opened by the first attribute lookup (a C entry point).

    Each entry point is cached on this object after its first lookup, so
    later calls cost one attribute access, as with a plain ctypes.CDLL."""

    def __init__(self):
        self._cdll = None

    def loaded(self) -> bool:
        return self._cdll is not None

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        if self._cdll is None:
            self._cdll = _load()
        fn = getattr(self._cdll, name)
        setattr(self, name, fn)
        return fn


lib = _LazyLib()


def check(rc: int, what: str = ""):
    if rc == MPM_OK:
        return
    msg = lib.mpm_last_error().decode("utf-8", "replace")
    if rc == MPM_ERR_RANGE:
        raise MpmIndexError(msg)
    raise MpmError(rc, f"{what}: {msg}" if what else msg)


def exported_symbols() -> list[str]:
    return sorted(_SIGS)

