"""ctypes binding of libsns_gpu.so (include/sns_gpu.h).

The structures mirror the C layouts exactly (which mirror the reference's
include/param.h, parallel.h, fluid.h, temperature.h). Loading the library
needs no GPU; every compute entry point needs one. There is no fallback: if
the library is missing, importing this module raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_bool, c_char_p, c_double, c_int, c_longlong, c_size_t, c_void_p

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_lib", "libsns_gpu.so")

SNS_OK = 0
SNS_ERR_ARG = 1
SNS_ERR_UNSUPPORTED = 2
SNS_ERR_CUDA = 3
SNS_ERR_OOM = 4
SNS_ERR_STATE = 5
SNS_ERR_NONFINITE = 6

SNS_FORM_EXACT = 0
SNS_FORM_PARALLEL = 1

_PD = POINTER(c_double)


class RkCoef(ctypes.Structure):
    _fields_ = [("alpha", c_double), ("beta", c_double), ("gamma", c_double)]


class Schedule(ctypes.Structure):
    _fields_ = [("rate", c_double), ("after", c_double), ("next", c_double)]


class Param(ctypes.Structure):
    """param_t (include/param.h:28-54 of the reference)."""

    _fields_ = [
        ("load_flow_field", c_bool), ("dirname_restart", c_char_p),
        ("with_temperature", c_bool), ("with_thermal_forcing", c_bool),
        ("itot", c_int), ("jtot", c_int), ("lx", c_double), ("ly", c_double),
        ("stretch", c_double), ("xf", _PD), ("xc", _PD), ("dxf", _PD), ("dxc", _PD),
        ("yf", _PD), ("yc", _PD), ("dy", c_double), ("Ra", c_double), ("Pr", c_double),
        ("rkcoefs", RkCoef * 3), ("time", c_double), ("dt", c_double),
        ("step", c_int), ("implicitx", c_int), ("implicity", c_int),
        ("expimp_wtimes", (c_double * 2) * 2), ("timemax", c_double), ("wtimemax", c_double),
        ("log", Schedule), ("save", Schedule), ("stat", Schedule),
    ]


class Parallel(ctypes.Structure):
    """parallel_t (include/parallel.h:10-13)."""

    _fields_ = [("mpisize", c_int), ("mpirank", c_int), ("ymrank", c_int), ("yprank", c_int)]


class Fluid(ctypes.Structure):
    """fluid_t (include/fluid.h:8-13)."""

    _fields_ = [("ux", _PD), ("uy", _PD), ("p", _PD), ("psi", _PD),
                ("srcuxa", _PD), ("srcuxb", _PD), ("srcuxg", _PD),
                ("srcuya", _PD), ("srcuyb", _PD), ("srcuyg", _PD)]


class Temperature(ctypes.Structure):
    """temperature_t (include/temperature.h:8-12)."""

    _fields_ = [("temp", _PD), ("tempforcex", _PD), ("srctempa", _PD), ("srctempb", _PD), ("srctempg", _PD)]


class CaseDesc(ctypes.Structure):
    """sns_case_desc (include/sns_batch.h)."""

    _fields_ = [("itot", c_int), ("jtot", c_int), ("ly", c_double), ("stretch", c_double), ("Ra", c_double),
                ("Pr", c_double), ("with_temperature", c_int), ("with_thermal_forcing", c_int),
                ("steps", c_longlong), ("seed", ctypes.c_ulonglong), ("fixed_dt", c_double),
                ("compensated", c_int)]


class Tuning(ctypes.Structure):
    """sns_batch_tuning (include/sns_batch.h)."""

    _fields_ = [("tile_x", c_int), ("tile_rows", c_int), ("modes_per_block", c_int), ("fcols_shift", c_int)]


class Statistics(ctypes.Structure):
    _fields_ = [("num", c_int), ("ux1", _PD), ("ux2", _PD), ("uy1", _PD), ("uy2", _PD), ("temp1", _PD),
                ("temp2", _PD)]


PP, PL, PF, PT = POINTER(Param), POINTER(Parallel), POINTER(Fluid), POINTER(Temperature)
PS = POINTER(Statistics)
PCD = POINTER(CaseDesc)

# name -> (restype, argtypes)
PROTOTYPES = {
    "fluid_init": (PF, [PP, PL]),
    "fluid_finalise": (c_int, [PF]),
    "fluid_update_boundaries_ux": (c_int, [PP, PL, _PD]),
    "fluid_update_boundaries_uy": (c_int, [PP, PL, _PD]),
    "fluid_update_boundaries_p": (c_int, [PP, PL, _PD]),
    "fluid_update_velocity": (c_int, [PP, PL, c_int, PF, PT]),
    "fluid_compute_potential": (c_int, [PP, PL, c_int, PF]),
    "fluid_correct_velocity": (c_int, [PP, PL, c_int, PF]),
    "fluid_update_pressure": (c_int, [PP, PL, c_int, PF]),
    "temperature_init": (PT, [PP, PL]),
    "temperature_finalise": (c_int, [PT]),
    "temperature_compute_force": (c_int, [PP, PL, PT]),
    "temperature_update_temp": (c_int, [PP, PL, c_int, PF, PT]),
    "temperature_update_boundaries_temp": (c_int, [PP, PL, _PD]),
    "param_decide_dt": (c_int, [PP, PL, PF]),
    "sns_param_create": (PP, [c_int, c_int, c_double, c_double, c_double, c_double, c_int, c_int]),
    "sns_param_destroy": (c_int, [PP]),
    "sns_parallel_create": (PL, []),
    "sns_parallel_destroy": (c_int, [PL]),
    "sns_sync_to_host": (c_int, [PP, PF, PT]),
    "sns_sync_to_device": (c_int, [PP, PF, PT]),
    "sns_sync_state_to_host": (c_int, [PP, PF, PT]),
    "sns_sync_state_to_device": (c_int, [PP, PF, PT]),
    "sns_synchronize": (c_int, [PF]),
    "sns_stream": (c_void_p, [PF]),
    "sns_integrate": (c_int, [PP, PL, PF, PT]),
    "sns_run": (c_int, [PP, PL, PF, PT, c_int]),
    "sns_last_error": (c_char_p, []),
    "sns_kernel_launches": (c_longlong, []),
    "sns_allocations": (c_longlong, []),
    "sns_abi_layout": (c_int, [POINTER(c_size_t), c_int]),
    "sns_diagnostics": (c_int, [PP, PF, PT, _PD]),
    "sns_diagnostics_static": (c_int, [PP, PF, PT, _PD]),
    "param_estimate_cost": (c_int, [PP, PL]),
    "sns_set_fused": (c_int, [PF, c_int]),
    "sns_set_form": (c_int, [PF, c_int]),
    "sns_get_form": (c_int, [PF]),
    "sns_set_wait_limit": (c_int, [PF, ctypes.c_uint, c_int]),
    "sns_cost_model": (c_int, [c_int, c_int, c_int, c_double, c_int, _PD]),
    "sns_measure_cost": (c_int, [PP, PL, c_int, _PD]),
    "statistics_init": (PS, [PP, PL]),
    "statistics_finalise": (c_int, [PS]),
    "statistics_collect": (c_int, [PP, PL, PF, PT, PS]),
    "statistics_output": (c_int, [PP, PL, PS]),
    "sns_statistics_output_to": (c_int, [PP, PS, c_char_p]),
    "sns_checkpoint": (c_int, [PP, PF, PT, ctypes.c_char_p]),
    "sns_checkpoint_wait": (c_int, [PF]),
    "sns_restart": (c_int, [PP, PF, PT, ctypes.c_char_p]),
    "sns_npy_write": (c_int, [c_char_p, c_char_p, c_int, POINTER(c_size_t), c_void_p, c_size_t]),
    "sns_npy_read": (c_int, [c_char_p, c_char_p, c_int, POINTER(c_size_t), c_void_p, c_size_t]),
    "sns_profile": (c_int, [PF, c_int]),
    "sns_profile_read": (c_int, [PF, POINTER(c_double), POINTER(c_longlong), c_int]),
    "sns_profile_kind_name": (c_char_p, [c_int]),
    "sns_fp64_issue_rate": (c_int, [_PD]),
    # include/sns_batch.h
    "sns_batch_create": (c_void_p, [c_size_t, c_int]),
    "sns_batch_destroy": (c_int, [c_void_p]),
    "sns_batch_case_bytes": (c_size_t, [PCD]),
    "sns_batch_free_bytes": (c_size_t, [c_void_p]),
    "sns_batch_add": (c_int, [c_void_p, PCD, _PD, POINTER(c_int)]),
    "sns_batch_remove": (c_int, [c_void_p, c_int]),
    "sns_batch_step": (c_int, [c_void_p, c_int]),
    "sns_batch_synchronize": (c_int, [c_void_p]),
    "sns_batch_set_wait_limit": (c_int, [c_void_p, ctypes.c_uint, c_int]),
    "sns_batch_set_persistent": (c_int, [c_void_p, c_int]),
    "sns_batch_stream": (c_void_p, [c_void_p]),
    "sns_batch_state": (c_int, [c_void_p, c_int, _PD, _PD, _PD, _PD, _PD]),
    "sns_batch_case_status": (c_int, [c_void_p, c_int, _PD, _PD, POINTER(c_longlong), POINTER(c_int)]),
    "sns_batch_cases": (c_int, [c_void_p, POINTER(c_int), c_int]),
    "sns_batch_active_cells": (c_longlong, [c_void_p]),
    "sns_batch_initial_temperature": (c_int, [PCD, _PD]),
    "sns_batch_diagnostics": (c_int, [c_void_p, c_int, _PD]),
    "sns_batch_get_tuning": (c_int, [c_void_p, POINTER(Tuning)]),
    "sns_batch_checkpoint": (c_int, [c_void_p, c_int, c_char_p]),
    "sns_batch_add_restart": (c_int, [c_void_p, PCD, c_char_p, POINTER(c_int)]),
    "sns_batch_set_tuning": (c_int, [c_void_p, POINTER(Tuning)]),
    "sns_batch_autotune": (c_int, [c_void_p, c_int, POINTER(Tuning), _PD]),
    "sns_serve": (c_int, [PCD, _PD, c_int, c_size_t, c_int, c_int, _PD, _PD, _PD, c_void_p, c_void_p]),
}

# void (*sns_done_fn)(int request, sns_batch *batch, int slot, void *user)
DONE_FN = ctypes.CFUNCTYPE(None, c_int, c_void_p, c_int, c_void_p)

_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with simplenavierstokessolver_gb300/build.py "
                               "(or __graft_entry__.build()); there is no CPU fallback")
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def last_error() -> str:
    return (lib().sns_last_error() or b"").decode(errors="replace")


class SnsError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what} failed with status {code}: {last_error()}")
        self.code = code


def check(code: int, what: str) -> None:
    if code != SNS_OK:
        raise SnsError(code, what)


def fp64_issue_rate() -> dict:
    """FP64 additions and multiplications per second of the current device
    (sns_fp64_issue_rate), in Gop/s"""
    out = (c_double * 2)()
    check(lib().sns_fp64_issue_rate(out), "sns_fp64_issue_rate")
    return {"dadd_gops": out[0], "dmul_gops": out[1]}
