"""ctypes binding of the C ABI in include/wpf.h (libwpf_gb300.so).

The library is the only implementation of the time step: there is no CPU or
PyTorch fallback, so loading fails loudly when it is missing or when no CUDA
device is usable.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

WPF_OK = 0
WPF_ERR_ARG = 1
WPF_ERR_CUDA = 2
WPF_ERR_NOT_CONVERGED = 3
WPF_ERR_NONFINITE = 4
WPF_ERR_TIMEOUT = 5
WPF_ERR_NOMEM = 6
WPF_ERR_SINGULAR = 7
WPF_ERR_TOO_LARGE = 8
NOALLOC_MAX_PLANES = 4096

SOLVER_FP64 = 0
SOLVER_MIXED = 1
SOLVER_NO_GRAPHS = 1   # wpf_solver_opts.flags bits
SOLVER_EXTRAPOLATE = 2
SOLVER_NO_TMA = 4
SOLVER_STEP_GRAPH = 8
SOLVER_NET_ALWAYS = 16
SOLVER_FP64_UPDATE = 32
SOLVER_NET_COARSE = 64
SOLVER_FIXED_START = 128


class WpfError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {strerror(status)} (status {status})")


class Params(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("ix_ref", C.c_int32), ("iy_ref", C.c_int32), ("iz_ref", C.c_int32),
                ("dx", C.c_double), ("epsilon", C.c_double), ("lambda_", C.c_double),
                ("porosity", C.c_double), ("viscosity", C.c_double), ("diffusion", C.c_double),
                ("ral", C.c_double), ("rat", C.c_double), ("permeab_hole", C.c_double),
                ("alpha", C.c_double), ("tfac", C.c_double)]


class Well(C.Structure):
    _fields_ = [("ix", C.c_int32), ("iy", C.c_int32), ("iz", C.c_int32), ("pad", C.c_int32),
                ("pressure", C.c_double), ("injection", C.c_double), ("phase", C.c_double),
                ("concent", C.c_double)]


class SolverOpts(C.Structure):
    _fields_ = [("mode", C.c_int32), ("max_outer", C.c_int32), ("max_inner", C.c_int32),
                ("smooth_sweeps", C.c_int32), ("rtol", C.c_double), ("inner_rtol", C.c_double),
                ("sweep_min_cells", C.c_int64), ("w_from_level", C.c_int32), ("flags", C.c_int32),
                ("sweep_zchunk", C.c_int32), ("row_blocks_per_sm", C.c_int32)]


class StepStats(C.Structure):
    _fields_ = [("outer_iterations", C.c_int32), ("inner_iterations", C.c_int32),
                ("converged", C.c_int32), ("overshoot_cells", C.c_int32), ("relres", C.c_double),
                ("taumin", C.c_double), ("dtime", C.c_double), ("max_courant", C.c_double),
                ("solve_ms", C.c_double), ("update_ms", C.c_double),
                ("kernel_launches", C.c_int32), ("warm_start", C.c_int32),
                ("relres0", C.c_double), ("active_cells", C.c_int32), ("device_resident", C.c_int32),
                ("interface_cells", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Diag(C.Structure):
    _fields_ = [("pv", C.c_double), ("vcal", C.c_double), ("rwhmax", C.c_double),
                ("phase_max", C.c_double), ("phase_min", C.c_double),
                ("concent_max", C.c_double), ("concent_min", C.c_double),
                ("pressure_ref", C.c_double), ("inlet_flux", C.c_double),
                ("phase_max_outlet", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


H = C.c_void_p
DP = C.POINTER(C.c_double)

# name -> (restype, argtypes); every function declared in include/wpf.h
SIGNATURES = {
    "wpf_create": (C.c_int, [C.POINTER(Params), C.POINTER(H)]),
    "wpf_destroy": (C.c_int, [H]),
    "wpf_strerror": (C.c_char_p, [C.c_int]),
    "wpf_device_bytes": (C.c_int, [H, C.POINTER(C.c_int64)]),
    "wpf_set_wells": (C.c_int, [H, C.POINTER(Well), C.c_int32]),
    "wpf_upload": (C.c_int, [H, DP, DP, DP, DP]),
    "wpf_download": (C.c_int, [H, DP, DP, DP, DP, DP, DP, DP]),
    "wpf_set_solver": (C.c_int, [H, C.POINTER(SolverOpts)]),
    "wpf_get_solver": (C.c_int, [H, C.POINTER(SolverOpts)]),
    "wpf_calc_permeability": (C.c_int, [H]),
    "wpf_solve_pressure": (C.c_int, [H, C.POINTER(StepStats)]),
    "wpf_calc_velocity": (C.c_int, [H]),
    "wpf_calc_phase_deriv": (C.c_int, [H, DP, C.POINTER(C.c_int32)]),
    "wpf_calc_concent_deriv": (C.c_int, [H]),
    "wpf_evolve_phase": (C.c_int, [H, C.c_double]),
    "wpf_evolve_concent": (C.c_int, [H, C.c_double]),
    "wpf_step": (C.c_int, [H, C.c_int32, DP, C.POINTER(StepStats)]),
    "wpf_run": (C.c_int, [H, C.c_int32, C.c_int32, DP, C.POINTER(StepStats)]),
    "wpf_reduce": (C.c_int, [H, C.POINTER(Diag)]),
    "wpf_reduce_noalloc": (C.c_int, [C.POINTER(Params), C.c_void_p, C.c_void_p,
                                     C.POINTER(Diag), C.c_void_p]),
    "wpf_get_taumin": (C.c_int, [H, DP]),
    "wpf_set_taumin": (C.c_int, [H, C.c_double]),
    "wpf_get_stream": (C.c_int, [H, C.POINTER(C.c_void_p)]),
    "wpf_launch_count": (C.c_int, [H, C.POINTER(C.c_int64)]),
    "wpf_set_kernel_timing": (C.c_int, [H, C.c_uint32]),
    "wpf_kernel_times": (C.c_int, [H, DP, C.POINTER(C.c_int64), C.c_int32]),
    "wpf_host_alloc": (C.c_int, [C.c_int64, C.POINTER(C.c_void_p)]),
    "wpf_host_free": (C.c_int, [C.c_void_p]),
    "wpf_snapshot": (C.c_int, [H, C.c_void_p]),
    "wpf_snapshot_wait": (C.c_int, [H]),
    "wpf_ensemble_run": (C.c_int, [C.POINTER(H), C.c_int32, C.c_int32, C.c_int32, C.c_int32, DP,
                                   C.POINTER(StepStats), C.POINTER(C.c_int32)]),
    "wpf_check_conversions": (C.c_int, [DP, C.c_int64, C.POINTER(C.c_int64)]),
    "wpf_check_reciprocal": (C.c_int, [DP, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "wpf_measure_fp64_rate": (C.c_int, [DP]),
    # include/wpf_net.h: the learned warm start
    "wpf_net_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "wpf_net_destroy": (C.c_int, [C.c_void_p]),
    "wpf_net_init": (C.c_int, [C.c_void_p, C.c_uint64]),
    "wpf_net_param_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "wpf_net_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "wpf_net_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "wpf_net_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "wpf_net_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                     C.POINTER(C.c_float), C.c_void_p]),
    "wpf_net_get_grads": (C.c_int, [C.c_void_p, C.c_void_p]),
    "wpf_net_get_activation": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64]),
    "wpf_conv3d": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                             C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "wpf_conv3d_wgrad": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "wpf_set_warm_start_net": (C.c_int, [H, C.c_void_p]),
    "wpf_ws_features": (C.c_int, [H, C.c_double, C.c_void_p]),
    "wpf_ws_target": (C.c_int, [H, C.c_void_p]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load libwpf_gb300.so (building it in-tree first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if not os.path.exists(path) or not _build.up_to_date():
        if not build_if_missing:
            raise RuntimeError(f"libwpf_gb300 is not built ({path})")
        _build.build()
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def strerror(status: int) -> str:
    try:
        return load(build_if_missing=False).wpf_strerror(status).decode()
    except Exception:  # library not loadable: fall back to the status number
        return f"status {status}"


def check(status: int, what: str, ok=(WPF_OK,)):
    if status not in ok:
        raise WpfError(status, what)
    return status
