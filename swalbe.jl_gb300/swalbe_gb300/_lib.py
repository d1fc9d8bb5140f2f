"""ctypes binding of libswalbe_gb300.so (include/swalbe_gb300.h).

The product path has no CPU fallback: if the library has not been built, or
no CUDA device is present when a state is created, the call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

from .build import LIB_PATH

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                      "include", "swalbe_gb300.h")

SWB_OK = 0
SWB_ERR_ARG = -1
SWB_ERR_OOM = -2
SWB_ERR_CUDA = -3
SWB_ERR_NAN = -4
SWB_ERR_UNSUPPORTED = -5
SWB_ERR_CANCELLED = -6
SWB_ERR_NOT_FOUND = -7
SWB_ERR_BUSY = -8

SWB_F64, SWB_F32, SWB_F16, SWB_PLAIN64 = 0, 1, 2, 3

FIELD = {"height": 0, "velx": 1, "vely": 2, "pressure": 3, "fout": 4, "feq": 5, "Fx": 6, "Fy": 7,
         "slipx": 8, "slipy": 9, "h∇px": 10, "h∇py": 11, "vsq": 12}

FIELD_HEIGHT, FIELD_VELX, FIELD_VELY, FIELD_PRESSURE, FIELD_FOUT = 0, 1, 2, 3, 4

MEAS_MASS, MEAS_WETTED, MEAS_MAXMIN, MEAS_AREA, MEAS_ALL = 1, 2, 4, 8, 15
RECORD_CAPACITY = 65536  # SWB_RECORD_CAPACITY: per-step records the device ring holds
STEP_AUTO, STEP_PER_ITERATION, STEP_MULTI = 0, 1, 2


class Params(C.Structure):
    _fields_ = [("Lx", C.c_int32), ("Ly", C.c_int32), ("Tmax", C.c_int32), ("tdump", C.c_int32),
                ("tau", C.c_double), ("cs", C.c_double), ("mu", C.c_double),
                ("delta", C.c_double), ("kbt", C.c_double), ("gamma", C.c_double),
                ("n", C.c_int32), ("m", C.c_int32), ("hmin", C.c_double),
                ("hcrit", C.c_double), ("theta", C.c_double), ("g", C.c_double)]


class Measure(C.Structure):
    _fields_ = [("t", C.c_int64), ("mass", C.c_double), ("wetted", C.c_int64),
                ("hmax", C.c_double), ("hmin", C.c_double), ("area", C.c_double),
                ("energy", C.c_double)]


class RequestInfo(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int32), ("steps_done", C.c_int64),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("admitted", C.c_int64), ("completed", C.c_int64),
                ("rejected", C.c_int64), ("queued", C.c_int64), ("running", C.c_int64),
                ("lattice_updates", C.c_double), ("busy_seconds", C.c_double),
                ("hbm_in_use", C.c_size_t), ("hbm_budget", C.c_size_t), ("ticks", C.c_int64),
                ("device_seconds", C.c_double)]


class SwbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; "
                "g.build()'` (there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        p, i, d, i64 = C.c_void_p, C.c_int, C.c_double, C.c_int64
        PP = C.POINTER(Params)
        sig = {
            "swb_abi_version": (i, []),
            "swb_last_error": (C.c_char_p, [p]),
            "swb_status_string": (C.c_char_p, [i]),
            "swb_state_bytes": (i, [PP, i, C.POINTER(C.c_size_t)]),
            "swb_create": (i, [PP, i, C.POINTER(p)]),
            "swb_destroy": (i, [p]),
            "swb_get_params": (i, [p, PP, C.POINTER(i)]),
            "swb_set_field": (i, [p, i, p]),
            "swb_get_field": (i, [p, i, p]),
            "swb_set_field_device": (i, [p, i, p]),
            "swb_set_stream": (i, [p, p]),
            "swb_get_stream": (i, [p, C.POINTER(p)]),
            "swb_launch_count": (i, [C.POINTER(C.c_uint64)]),
            "swb_set_theta": (i, [p, d]),
            "swb_set_theta_field": (i, [p, p]),
            "swb_set_theta_wave": (i, [p, d, d, d]),
            "swb_set_inclination": (i, [p, d, d, i, i64, i64, i64]),
            "swb_set_measures": (i, [p, i, d]),
            "swb_set_mass_correction": (i, [p, i]),
            "swb_set_geometry": (i, [p, i, i]),
            "swb_get_geometry": (i, [p, C.POINTER(i), C.POINTER(i)]),
            "swb_set_step_mode": (i, [p, i]),
            "swb_get_step_mode": (i, [p, C.POINTER(i)]),
            "swb_step": (i, [p, i64]),
            "swb_sync": (i, [p]),
            "swb_steps_done": (i, [p, C.POINTER(i64)]),
            "swb_get_measures": (i, [p, C.POINTER(Measure), i64, C.POINTER(i64)]),
            "swb_measures_dropped": (i, [p, C.POINTER(i64)]),
            "swb_measure_now": (i, [p, d, C.POINTER(Measure)]),
            "swb_measure_field_noalloc": (i, [p, i, i, d, p, d, p, C.POINTER(Measure)]),
            "swb_op_filmpressure": (i, [p]),
            "swb_op_hgradp": (i, [p]),
            "swb_op_slippage": (i, [p]),
            "swb_op_force_sum": (i, [p]),
            "swb_op_inclination": (i, [p, d, d, i64, i64, i64]),
            "swb_op_equilibrium": (i, [p]),
            "swb_op_bgk_stream": (i, [p]),
            "swb_op_moments": (i, [p]),
            "swb_batch_create": (i, [PP, i, i, C.POINTER(p)]),
            "swb_batch_destroy": (i, [p]),
            "swb_batch_set_height": (i, [p, i, p]),
            "swb_batch_get_height": (i, [p, i, p]),
            "swb_batch_set_theta_wave": (i, [p, i, d, d, d]),
            "swb_batch_step": (i, [p, i64]),
            "swb_batch_sync": (i, [p]),
            "swb_batch_tile": (i, [p, C.POINTER(i), C.POINTER(i), C.POINTER(i)]),
            "swb_batch_geometry": (i, [p, C.POINTER(i), C.POINTER(i), C.POINTER(i)]),
            "swb_server_create": (i, [C.c_size_t, i, i, C.POINTER(p)]),
            "swb_server_destroy": (i, [p]),
            "swb_server_submit": (i, [p, PP, p, d, d, d, i64, C.POINTER(i64)]),
            "swb_server_set_queue_limit": (i, [p, i64]),
            "swb_server_set_policy": (i, [p, i, i64]),
            "swb_server_set_geometry": (i, [p, i, i]),
            "swb_count_droplets": (i, [p, i, i, d, C.POINTER(i64)]),
            "swb_set_thermal_seed": (i, [p, C.c_uint64]),
            "swb_thermal_field": (i, [p, i64, p, p]),
            "swb_op_thermal": (i, [p, i64]),
            "swb_batch_set_geometry": (i, [p, i, i]),
            "swb_set_substrate_motion": (i, [p, i64, i, i]),
            "swb_set_snapshots": (i, [p, i64, i64]),
            "swb_get_snapshots": (i, [p, p, i64, C.POINTER(i64), p]),
            "swb1d_create": (i, [C.POINTER(Params), i, i, i, C.POINTER(p)]),
            "swb1d_destroy": (i, [p]),
            "swb1d_set_field": (i, [p, i, i, p]),
            "swb1d_get_field": (i, [p, i, i, p]),
            "swb1d_step": (i, [p, i64]),
            "swb1d_sync": (i, [p]),
            "swb1d_get_measures": (i, [p, i, p, i64, C.POINTER(i64)]),
            "swb_server_poll": (i, [p, i64, p, C.POINTER(RequestInfo)]),
            "swb_server_cancel": (i, [p, i64]),
            "swb_server_stats_get": (i, [p, C.POINTER(ServerStats)]),
            "swb_server_clock": (d, [p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, handle=None) -> int:
    if status < 0:
        msg = lib().swb_last_error(handle)
        raise SwbError(status, (msg or b"").decode() or lib().swb_status_string(status).decode())
    return status


def header_functions(path: str = HEADER):
    """Names of the functions include/swalbe_gb300.h declares."""
    txt = open(path).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(swb_\w+)\s*\(", txt,
                                 re.M)))
