"""ctypes binding of libgfs (include/gfs.h).

The binding mirrors pyfluid's pybindings (src/pyfluid/pybindings.py:1-36) with
one change: every call's status is checked, including calls that return a
value (pybindings.execute_lib_func skips check_success for those,
pybindings.py:26-36), and a failure raises GFSError with the library's message.

There is no fallback: if libgfs.so is missing the first call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgfs.so")

GFS_OK = 0
GFS_ERR_INVALID = 1
GFS_ERR_CUDA = 2
GFS_ERR_NOMEM = 3
GFS_ERR_TIMEOUT = 4
GFS_ERR_STATE = 5
PRECISION_PLAIN = 0
PRECISION_MIXED = 1
SWEEP_AUTO = 0
SWEEP_BLOCK = 1
SWEEP_CLUSTER_4X2 = 2
SWEEP_CLUSTER_2X2 = 3
SWEEP_WARP = 4
STAGE_UPDATE_FLUID_CELLS = 1
STAGE_BODY_FORCES = 6
STAGE_PRESSURE = 7
STAGE_APPLY_PRESSURE = 8
STAGE_EXTRAPOLATE = 9
STAGE_ALL = 12

_ERR_NAMES = {1: "invalid argument", 2: "CUDA error", 3: "out of device memory",
              4: "wavefront wait timed out", 5: "call out of order"}


class GFSError(RuntimeError):
    def __init__(self, code: int, func: str, message: str):
        self.code = code
        super().__init__(f"{func} - {_ERR_NAMES.get(code, 'error')} ({code}): {message}")


class SimParams(ctypes.Structure):
    _fields_ = [("density", ctypes.c_double), ("ratio_pic", ctypes.c_double), ("cfl", ctypes.c_double),
                ("gravity", ctypes.c_float * 3), ("max_particles_per_cell", ctypes.c_int),
                ("precision", ctypes.c_int), ("tol", ctypes.c_double), ("max_cg_iterations", ctypes.c_int)]


class StepStats(ctypes.Structure):
    _fields_ = [("num_particles", ctypes.c_int64), ("num_fluid_cells", ctypes.c_int64),
                ("cg_iterations", ctypes.c_int), ("refinements", ctypes.c_int), ("sweeps", ctypes.c_int),
                ("cg_max_residual", ctypes.c_double), ("pressure_ms", ctypes.c_double),
                ("step_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class FluidSourceC(ctypes.Structure):
    _fields_ = [("shape", ctypes.c_int), ("outflow", ctypes.c_int), ("active", ctypes.c_int),
                ("position", ctypes.c_float * 3), ("radius", ctypes.c_double), ("size", ctypes.c_double * 3),
                ("velocity", ctypes.c_float * 3)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double

# name -> argtypes (every function returns int status)
_SIGNATURES = {
    "gfs_ctx_create": [_I, ctypes.POINTER(_P)],
    "gfs_ctx_destroy": [_P],
    "gfs_ctx_synchronize": [_P],
    "gfs_ctx_stream": [_P, ctypes.POINTER(_P)],
    "gfs_ctx_device_name": [_P, ctypes.c_char_p, _I],
    "gfs_ctx_launch_count": [_P, ctypes.POINTER(_I64)],
    "gfs_ctx_profile_enable": [_P, _I],
    "gfs_ctx_profile_reset": [_P],
    "gfs_ctx_profile_read": [_P, _I, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(_D), ctypes.POINTER(_I64)],
    "gfs_ctx_set_sweep_kernel": [_P, _I],
    "gfs_ctx_last_sweep_kernel": [_P, ctypes.POINTER(_I)],
    "gfs_ctx_set_wait_limit": [_P, _I64],
    "gfs_ctx_inject_wait_timeout": [_P, _I],
    "gfs_scalar_field_add_point_values": [_P, _P, _P, _I64, _D, _P, _D, _I, _I, _I, _P, _P, _I, _D],
    "gfs_velocity_scalar_field": [_P, _I, _I, _I, _I, _D, _P, _P, _I64, _P, _P],
    "gfs_tricubic_interpolate": [_P, _I, _I, _I, _D, _P, _P, _P, _P, _I64, _P],
    "gfs_advect_particles": [_P, _I, _I, _I, _I, _D, _P, _P, _P, _D, _P, _I64, _P],
    "gfs_tricubic_interpolate_noalloc": [_I, _I, _I, _D, _P, _P, _P, _P, _I64, _P, _P],
    "gfs_pressure_solve": [_P, _I, _I, _I, _D, _D, _D, _P, _P, _P, _P, _I, _D, _I, _P,
                           ctypes.POINTER(_I64), ctypes.POINTER(_I), ctypes.POINTER(_D)],
    "gfs_sim_default_params": [ctypes.POINTER(SimParams)],
    "gfs_sim_create": [_P, _I, _I, _I, _D, _I64, ctypes.POINTER(_P)],
    "gfs_sim_destroy": [_P],
    "gfs_sim_set_params": [_P, ctypes.POINTER(SimParams)],
    "gfs_sim_get_params": [_P, ctypes.POINTER(SimParams)],
    "gfs_sim_set_material": [_P, _P],
    "gfs_sim_get_material": [_P, _P],
    "gfs_sim_set_particles": [_P, _P, _P, _P, _I64],
    "gfs_sim_add_solid_cells": [_P, _P, _I],
    "gfs_sim_remove_solid_cells": [_P, _P, _I],
    "gfs_sim_initialize": [_P, _P, _I, _P, _I, ctypes.POINTER(_I64)],
    "gfs_seed_fluid_particles": [_I, _I, _I, _D, _P, _P, _I, _P, _I, _D, ctypes.c_uint64, _P, _I64,
                                 ctypes.POINTER(_I64)],
    "gfs_sim_num_particles": [_P, ctypes.POINTER(_I64)],
    "gfs_sim_get_particles": [_P, _P, _P, _P, ctypes.POINTER(_I64)],
    "gfs_sim_get_velocity_field": [_P, _P, _P, _P],
    "gfs_sim_get_pressure_grid": [_P, _P],
    "gfs_sim_step": [_P, _D, ctypes.POINTER(StepStats)],
    "gfs_sim_step_host": [_P, _D, _P, _P, _P, ctypes.POINTER(_I64), ctypes.POINTER(StepStats)],
    "gfs_sim_step_stages": [_P, _D, _I, ctypes.POINTER(StepStats)],
    "gfs_sim_get_saved_velocity_field": [_P, _P, _P, _P],
    "gfs_sim_add_marker_particle_points": [_P, _D, _P, _D, _I, _I, _I, _P, _I, _D],
    "gfs_sim_pressure_check": [_P, _D, _D, ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.POINTER(_I)],
    "gfs_sim_set_fluid_sources": [_P, ctypes.POINTER(FluidSourceC), _I],
    "gfs_sim_set_marker_particle_jitter": [_P, _D, ctypes.c_uint64],
    "gfs_sim_update_fluid_sources": [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)],
    "gfs_sim_add_fluid_cells": [_P, _P, _I, _P],
    "gfs_sim_remove_fluid_cells": [_P, _P, _I],
    "gfs_savestate_read_header": [ctypes.c_char_p, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                                  ctypes.POINTER(_D), ctypes.POINTER(_I), ctypes.POINTER(_I64),
                                  ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I)],
    "gfs_sim_save_state": [_P, ctypes.c_char_p, _I],
    "gfs_sim_load_state": [_P, ctypes.c_char_p, ctypes.POINTER(_I)],
    "gfs_diff_create": [_P, _I, _I64, _D, ctypes.POINTER(_P)],
    "gfs_diff_destroy": [_P],
    "gfs_diff_forward": [_P, _P, _P, _P, _P, _P, _P, _P],
    "gfs_diff_backward": [_P, _P, _P, _P, _P, _P, _P, _P],
    "gfs_diff_info": [_P, ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.POINTER(_I64)],
}

# entry points declared in include/gfs.h (checked by the CPU test suite)
EXPORTS = sorted(list(_SIGNATURES) + ["gfs_last_error", "gfs_version"])

_lib = None
_lock = threading.Lock()


def _errcheck(result, func, args):
    if result != GFS_OK:
        msg = _lib.gfs_last_error().decode("utf-8", "replace")
        raise GFSError(int(result), func.__name__, msg)
    return result


def load(path: str | None = None):
    """Load libgfs.so (raises GFSError-free OSError / RuntimeError if absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(f"libgfs.so is not built ({p}); run gridfluidsim3d_gb300.build.build()")
        L = ctypes.CDLL(p)
        L.gfs_last_error.argtypes = []
        L.gfs_last_error.restype = ctypes.c_char_p
        L.gfs_version.argtypes = []
        L.gfs_version.restype = ctypes.c_char_p
        for name, argt in _SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = argt
            f.restype = ctypes.c_int
            f.errcheck = _errcheck
        _lib = L
        return _lib


def lib():
    return _lib if _lib is not None else load()


def loaded_path() -> str | None:
    return LIB_PATH if _lib is not None else None
