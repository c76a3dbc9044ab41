"""ctypes binding of libgpu4snn.so (include/gpu4snn.h).

The library is the only compute path: there is no CPU fallback.  If the shared object is
missing the import of this module succeeds but every call raises, naming the build step.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libgpu4snn.so")

# status codes
OK = 0
ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_TIMEOUT = -1, -2, -3, -4
ERR_OVERFLOW, ERR_IO, ERR_BUDGET, ERR_CANCELLED, ERR_STATE = -5, -6, -7, -8, -9
ERR_NAMES = {
    ERR_INVALID: "G4S_ERR_INVALID", ERR_CUDA: "G4S_ERR_CUDA", ERR_NOMEM: "G4S_ERR_NOMEM",
    ERR_TIMEOUT: "G4S_ERR_TIMEOUT", ERR_OVERFLOW: "G4S_ERR_OVERFLOW", ERR_IO: "G4S_ERR_IO",
    ERR_BUDGET: "G4S_ERR_BUDGET", ERR_CANCELLED: "G4S_ERR_CANCELLED", ERR_STATE: "G4S_ERR_STATE",
}

# propagation schemes (the reference's `dynamic`, gpu4snn.cu:1083)
ALG_AP, ALG_N, ALG_S, ALG_AB, ALG_SKL, ALG_AUTO = 0, 1, 2, 3, 4, 5
ALG_NAMES = {"AP": ALG_AP, "N": ALG_N, "S": ALG_S, "AB": ALG_AB, "SKL": ALG_SKL, "AUTO": ALG_AUTO}

CONN_PHILOX, CONN_GLIBC = 0, 1

FAULT_BARRIER_STALL, FAULT_ALLOC = 1, 2


class G4SError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


class NetDesc(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("nsyn", C.c_int32),
        ("exc_permille", C.c_int32),
        ("self_loops", C.c_int32),
        ("conn_law", C.c_int32),
        ("seed", C.c_uint64),
        ("drive_scale", C.c_float),
        ("record_raster", C.c_int32),
        ("raster_budget_bytes", C.c_int64),
    ]


class NetInfo(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("nsyn", C.c_int32),
        ("stride", C.c_int32),
        ("steps_done", C.c_int64),
        ("total_spikes", C.c_int64),
        ("raster_size", C.c_int64),
        ("last_run_ms", C.c_double),
        ("last_run_wall_ms", C.c_double),
        ("last_run_spikes", C.c_int64),
        ("last_algorithm", C.c_int32),
        ("persistent_blocks", C.c_int32),
        ("device_bytes", C.c_int64),
        ("last_run_kernel_ms", C.c_double),
        ("last_run_launches", C.c_int64),
    ]


class Request(C.Structure):
    _fields_ = [("n", C.c_int64), ("nsyn", C.c_int32), ("steps", C.c_int32), ("seed", C.c_uint64),
                ("drive_scale", C.c_float), ("record_raster", C.c_int32)]


class RequestResult(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int32), ("steps_done", C.c_int32), ("total_spikes", C.c_int64),
                ("latency_ms", C.c_double), ("queue_ms", C.c_double), ("rate_hz", C.c_double),
                ("isi_cv", C.c_double), ("create_ms", C.c_double), ("device_ms", C.c_double),
                ("sm_ms", C.c_double), ("rounds", C.c_int32), ("team", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [("rounds", C.c_int64), ("launches", C.c_int64), ("completed", C.c_int64), ("queued", C.c_int64),
                ("resident", C.c_int64), ("events", C.c_int64), ("busy_ms", C.c_double), ("wall_ms", C.c_double),
                ("bytes_in_use", C.c_int64), ("peak_bytes", C.c_int64)]


# (name, restype, argtypes) of every exported entry point
_P = C.c_void_p
SIGNATURES = [
    ("g4s_abi_version", C.c_int, []),
    ("g4s_last_error", C.c_char_p, []),
    ("g4s_set_device", C.c_int, [C.c_int32]),
    ("g4s_net_create", C.c_int, [C.POINTER(NetDesc), C.POINTER(_P)]),
    ("g4s_net_create_from_tables", C.c_int, [C.POINTER(NetDesc), _P, _P, C.c_int32, C.POINTER(_P)]),
    ("g4s_net_load_tables", C.c_int, [_P, _P, _P, C.c_int32]),
    ("g4s_net_reset", C.c_int, [_P]),
    ("g4s_net_run", C.c_int, [_P, C.c_int32, C.c_int32]),
    ("g4s_net_get_info", C.c_int, [_P, C.POINTER(NetInfo)]),
    ("g4s_net_raster", C.c_int, [_P, _P, _P, C.c_int64, C.POINTER(C.c_int64)]),
    ("g4s_net_counts", C.c_int, [_P, _P, C.c_int64, C.POINTER(C.c_int64)]),
    ("g4s_net_step_times", C.c_int, [_P, _P, _P, C.c_int64, C.POINTER(C.c_int64)]),
    ("g4s_net_state", C.c_int, [_P] * 9),
    ("g4s_net_currents", C.c_int, [_P, _P]),
    ("g4s_net_tables", C.c_int, [_P, C.c_int64, C.c_int64, _P, _P]),
    ("g4s_net_stats", C.c_int, [_P, _P, _P, _P]),
    ("g4s_net_set_barrier_timeout", C.c_int, [_P, C.c_uint64]),
    ("g4s_net_set_geometry", C.c_int, [_P, C.c_int32, C.c_int32]),
    ("g4s_net_set_block_threads", C.c_int, [_P, C.c_int32]),
    ("g4s_net_get_block_threads", C.c_int, [_P, C.POINTER(C.c_int32)]),
    ("g4s_net_get_geometry", C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]),
    ("g4s_net_get_delivery", C.c_int, [_P, C.POINTER(C.c_int32)]),
    ("g4s_nets_run", C.c_int, [_P, _P, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    ("g4s_net_autotune", C.c_int, [_P, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                   C.POINTER(C.c_double)]),
    ("g4s_net_destroy", C.c_int, [_P]),
    ("g4s_inject_fault", C.c_int, [_P, C.c_int32]),
    ("g4s_net_write_results", C.c_int, [_P, C.c_char_p, _P, C.c_double, C.c_double]),
    ("g4s_run_protocol", C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64,
                                   C.c_int32, C.c_char_p]),
    ("g4s_conn_glibc", C.c_int, [C.c_uint32, C.c_int32, C.c_int32, C.c_int32, _P, _P]),
    ("g4s_net_fp64_check", C.c_int, [_P, C.c_int32, _P, _P, _P, C.POINTER(C.c_int32), _P, _P]),
    ("g4s_run_noalloc", C.c_int, [_P, C.c_int64, C.c_int32, C.c_int32, C.c_int32, _P, _P, _P, C.c_int64, _P, _P]),
    ("g4s_server_start", C.c_int, [C.c_int64, C.c_int32, C.POINTER(_P)]),
    ("g4s_server_submit", C.c_int, [_P, C.POINTER(Request), C.POINTER(C.c_int64)]),
    ("g4s_server_poll", C.c_int, [_P, _P, C.c_int32, C.POINTER(C.c_int32)]),
    ("g4s_server_result", C.c_int, [_P, C.c_int64, _P, _P, C.c_int64, C.POINTER(C.c_int64), _P, _P, _P]),
    ("g4s_server_release", C.c_int, [_P, C.c_int64]),
    ("g4s_server_get_stats", C.c_int, [_P, C.POINTER(ServerStats)]),
    ("g4s_server_stop", C.c_int, [_P, C.c_int32]),
    ("g4s_net_stream_raster", C.c_int, [_P, C.c_char_p]),
    ("g4s_net_write_raster_file", C.c_int, [_P, C.c_char_p]),
    ("g4s_net_save_tables", C.c_int, [_P, C.c_char_p]),
    ("g4s_net_create_from_file", C.c_int, [C.POINTER(NetDesc), C.c_char_p, C.POINTER(_P)]),
    ("g4s_pinned_alloc", C.c_int, [C.c_uint64, C.POINTER(_P)]),
    ("g4s_pinned_free", C.c_int, [_P]),
]


def pinned_empty(shape, dtype) -> tuple[np.ndarray, C.c_void_p]:
    """A numpy array over page-locked host memory; free it with pinned_free(handle)."""
    dt = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dt.itemsize
    p = C.c_void_p()
    check(load().g4s_pinned_alloc(nbytes, C.byref(p)))
    buf = (C.c_byte * nbytes).from_address(p.value)
    return np.frombuffer(buf, dtype=dt).reshape(shape), p


def pinned_free(p: C.c_void_p):
    check(load().g4s_pinned_free(p))

_lib = None


def load(path: str = LIB_PATH):
    """Load libgpu4snn.so; raises if it has not been built (no fallback exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with `python -m gpu4snn_gb300.build` "
                               "(the CUDA library is the only implementation)")
        L = C.CDLL(path)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int):
    if rc != OK:
        msg = load().g4s_last_error()
        raise G4SError(rc, msg.decode() if msg else "")
    return rc


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)
