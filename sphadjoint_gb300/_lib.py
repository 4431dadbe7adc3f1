"""ctypes binding of libsphgb300.so (the C ABI declared in include/sphadjoint_gb300.h).

The library is built in-tree by ``sphadjoint_gb300.build``. There is no CPU
fallback: if the shared library is missing or cannot be loaded, importing the
binding raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import buildlib as _build

_lib = None

SPH_F64, SPH_F32 = 0, 1
FLAG_NL_OVERFLOW, FLAG_DISPLACEMENT, FLAG_NONFINITE = 1, 2, 4

KERNELS = ["assign", "scan", "bucket", "rank", "nl_build", "density", "accel_integrate",
           "tape", "gather", "accel_drag", "pass1", "pass2", "theta_node", "misc"]
KERNEL_ID = {k: i for i, k in enumerate(KERNELS)}


class sph_params(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("h", "m", "rho0", "c", "mu", "gx", "gy", "dt", "Lx", "Ly", "kw")] + \
               [("ngx", C.c_int32), ("ngy", C.c_int32), ("eos", C.c_int32),
                ("gamma", C.c_int32), ("visc", C.c_int32), ("pad", C.c_int32),
                ("alpha", C.c_double)]


class SPHError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"sphadjoint_gb300 error {code}: {msg}")
        self.code = code


class CapacityError(SPHError, ValueError):
    """simulate! with a tape that is too short (ArgumentError in the reference)."""


class ArgumentError(SPHError, ValueError):
    pass


class sph_request(C.Structure):
    _fields_ = [("p", sph_params), ("N", C.c_int64), ("X0", C.c_void_p), ("V0", C.c_void_p),
                ("theta", C.c_void_p), ("nsteps", C.c_int64), ("snapshots", C.c_int32),
                ("objective", C.c_int32), ("obj_args", C.c_double * 3), ("skin", C.c_double),
                ("interval", C.c_int32), ("maxnb", C.c_int32), ("gX", C.c_void_p),
                ("gV", C.c_void_p), ("gtheta", C.c_void_p)]


_P = C.c_void_p
_PP = C.POINTER(C.c_void_p)
_I32 = C.c_int32
_I64 = C.c_int64
_U32P = C.POINTER(C.c_uint32)
_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)
_DP = C.POINTER(C.c_double)
_SP = C.POINTER(sph_params)

_SIGS = {
    "sph_last_error": (C.c_char_p, []),
    "sph_version": (_I32, []),
    "sph_set_stream": (_I32, [_P]),
    "sph_synchronize": (_I32, []),
    "sph_field_create": (_I32, [_I32, _I32, _I32, _P, _PP]),
    "sph_field_upload": (_I32, [_P, _P]),
    "sph_field_upload_device": (_I32, [_P, _P]),
    "sph_field_destroy": (_I32, [_P]),
    "sph_state_create": (_I32, [_SP, _I64, _P, _P, _I32, C.c_double, _I32, _I32, _PP]),
    "sph_state_destroy": (_I32, [_P]),
    "sph_state_set": (_I32, [_P, _P, _P]),
    "sph_state_get": (_I32, [_P, _P, _P]),
    "sph_state_fields": (_I32, [_P, _P, _P, _P, _P, _P]),
    "sph_state_keep_accel": (_I32, [_P, _I32]),
    "sph_state_take_flags": (_I32, [_P, _U32P]),
    "sph_state_grid": (_I32, [_P, _I32P, _I32P, _DP, _I64P]),
    "sph_build_cells": (_I32, [_P]),
    "sph_build_neighbors": (_I32, [_P]),
    "sph_get_celllist": (_I32, [_P, _P, _P, _P]),
    "sph_get_neighbors": (_I32, [_P, _P, _P]),
    "sph_step": (_I32, [_P, _P, _SP]),
    "sph_simulate": (_I32, [_P, _P, _SP, _I64, _P, _U32P]),
    "sph_tape_create": (_I32, [_I64, _I64, _I32, _PP]),
    "sph_tape_create_checkpointed": (_I32, [_I64, _I64, _I32, _I32, _PP]),
    "sph_tape_plan": (_I32, [_SP, _I64, _I64, _I32, C.c_double, _I64, _I32P, _I64P]),
    "sph_tape_create_auto": (_I32, [_SP, _I64, _I64, _I32, C.c_double, _I64, _PP]),
    "sph_tape_snapshots": (_I32, [_P, _I32P]),
    "sph_tape_destroy": (_I32, [_P]),
    "sph_tape_reset": (_I32, [_P]),
    "sph_tape_length": (_I32, [_P, _I64P]),
    "sph_tape_get": (_I32, [_P, _I64, _P, _P]),
    "sph_tape_recomputed_steps": (_I32, [_P, _I64P]),
    "sph_workspace_create": (_I32, [_I64, _SP, _I32, _PP]),
    "sph_workspace_destroy": (_I32, [_P]),
    "sph_backward": (_I32, [_P, _P, _P, _SP, _P, _P, _P, C.c_double, _I32, _I32, _U32P]),
    "sph_workspace_get": (_I32, [_P, _P, _P, _P]),
    "sph_state_assign": (_I32, [_P, _P]),
    "sph_autotune": (_I32, [_P, _P, _I32, _I32P]),
    "sph_set_block_sizes": (_I32, [_P, _I32P]),
    "sph_get_block_sizes": (_I32, [_P, _I32P]),
    "sph_set_group_lanes": (_I32, [_I32]),
    "sph_set_density_form": (_I32, [_I32]),
    "sph_set_launch_overlap": (_I32, [_I32]),
    "sph_set_step_graphs": (_I32, [_I32]),
    "sph_get_step_graphs": (_I32, [_I32P]),
    "sph_step_graph_counts": (_I32, [_I64P, _I64P]),
    "sph_get_density_form": (_I32, [_I32P]),
    "sph_capture_begin": (_I32, []),
    "sph_capture_end": (_I32, [_PP]),
    "sph_graph_launch": (_I32, [_P]),
    "sph_graph_nodes": (_I32, [_P, _I64P]),
    "sph_graph_destroy": (_I32, [_P]),
    "sph_workspace_objective_value": (_I32, [_P, _DP]),
    "sph_workspace_take_flags": (_I32, [_P, _U32P]),
    "sph_get_group_lanes": (_I32, [_I32P]),
    "sph_objective": (_I32, [_P, _P, _I32, _DP, _SP, _DP]),
    "sph_backward_seeded": (_I32, [_P, _P, _P, _SP, _P, C.c_double, _I32, _I32, _U32P]),
    "sph_batch_create": (_I32, [_I32, _SP, _I64P, _P, _P, _I32, C.c_double, _I32, _I32, _PP]),
    "sph_batch_field_create": (_I32, [_I32, _I32P, _I32P, _I32, _P, _PP]),
    "sph_batch_workspace_create": (_I32, [_I32, _SP, _I64P, _I32, _PP]),
    "sph_batch_size": (_I32, [_P, _I32P]),
    "sph_batch_take_flags": (_I32, [_P, _U32P]),
    "sph_batch_objective": (_I32, [_P, _P, _I32, _DP, _DP]),
    "sph_server_create": (_I32, [_I32, _I64, _I32, _PP]),
    "sph_server_create_packed": (_I32, [_I32, _I64, _I32, _PP]),
    "sph_server_destroy": (_I32, [_P]),
    "sph_server_submit": (_I32, [_P, C.POINTER(sph_request), _I64P]),
    "sph_server_wait": (_I32, [_P, _I64, _DP, _DP, _U32P]),
    "sph_server_poll": (_I32, [_P, _I64, _I32P]),
    "sph_server_stats": (_I32, [_P, _DP, _DP, _DP, _I64P, _I64P, _I32P]),
    "sph_server_reset_stats": (_I32, [_P]),
    "sph_request_bytes": (_I64, [C.POINTER(sph_request), _I32]),
    "sph_launch_count": (_I64, []),
    "sph_profile_enable": (_I32, [_I32, _I32]),
    "sph_profile_read": (_I32, [_I32, _DP, _I64P]),
    "sph_profile_reset": (_I32, []),
    "sph_plan_cost": (_I64, [_I64, _I64]),
    "sph_plan_split": (_I64, [_I64, _I64]),
    "sph_design_create": (_I32, [_I32, _I32, _I32, C.c_double, C.c_double, C.c_double, _PP]),
    "sph_design_destroy": (_I32, [_P]),
    "sph_design_set": (_I32, [_P, _P]),
    "sph_design_get": (_I32, [_P, _P, _P, _P]),
    "sph_design_to_theta": (_I32, [_P, _P]),
    "sph_design_gradient": (_I32, [_P, _P, _DP]),
    "sph_design_candidate": (_I32, [_P, C.c_double, _P]),
    "sph_design_accept": (_I32, [_P]),
    "sph_design_apply": (_I32, [_P, _I32, _P, _P]),
    "sph_build_cells_noalloc": (_I32, [_P, _I64, _I32, C.c_double, _I32, _I32, _I32P, _I32P,
                                       _I32P, _P]),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) the CUDA library; raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing and (not os.path.exists(path) or _build._stale()):
        _build.build()
    if not os.path.exists(path):
        raise ImportError(f"libsphgb300.so not found at {path}; run sphadjoint_gb300.build")
    L = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(code: int) -> None:
    if code != 0:
        msg = _lib.sph_last_error().decode(errors="replace")
        if code == 2:
            raise CapacityError(code, msg)
        if code == 1:
            raise ArgumentError(code, msg)
        raise SPHError(code, msg)
