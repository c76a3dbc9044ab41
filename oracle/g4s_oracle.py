"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests, the smoke check and bench.py's CPU-baseline leg import this module; it is the
checker, never the product.  The C library restates the reference's algorithm
(gpu4snn.cu:286-320, 356-414, 862-899); see g4s_oracle.h for the line-by-line map.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libg4s_oracle.so")
REF_TABLES = os.path.join(HERE, "_ref", "gpu4snn_tables")

FP32, FP64 = 0, 1


class Desc(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("nsyn", C.c_int32),
        ("stride", C.c_int32),
        ("exc_permille", C.c_int32),
        ("self_loops", C.c_int32),
        ("seed", C.c_uint64),
        ("drive_scale", C.c_float),
        ("pad_", C.c_int32),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle and the reference-kernel harness with make (gcc, -ffp-contract=off)."""
    harness = os.path.join(HERE, "_build", "g4s_refgpu")
    if force or not os.path.exists(LIB_PATH) or not os.path.exists(harness):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        p = C.c_void_p
        L.g4o_philox4x64_10.argtypes = [p, p, p]
        L.g4o_philox4x32_10.argtypes = [p, p, p]
        L.g4o_logf.argtypes = [C.c_float]
        L.g4o_logf.restype = C.c_float
        L.g4o_normal.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        L.g4o_normal.restype = C.c_float
        L.g4o_param_r.argtypes = [C.c_uint64, C.c_uint64]
        L.g4o_param_r.restype = C.c_float
        L.g4o_conn_draw.argtypes = [C.c_uint64, C.c_int64, C.c_int, C.c_int64, C.c_int64]
        L.g4o_conn_draw.restype = C.c_int64
        L.g4o_conn_philox.argtypes = [C.POINTER(Desc), C.c_int64, C.c_int64, p, p]
        L.g4o_conn_glibc.argtypes = [C.c_uint, C.c_int32, C.c_int32, p, p]
        L.g4o_sort_rows.argtypes = [p, p, C.c_int64, C.c_int32]
        L.g4o_wfix.argtypes = [C.c_float]
        L.g4o_wfix.restype = C.c_int64
        L.g4o_sim_create.argtypes = [C.POINTER(Desc), p, p, C.c_int]
        L.g4o_sim_create.restype = p
        L.g4o_sim_destroy.argtypes = [p]
        L.g4o_sim_run.argtypes = [p, C.c_int32, C.c_int32]
        L.g4o_sim_step_index.argtypes = [p]
        L.g4o_sim_step_index.restype = C.c_int64
        L.g4o_sim_raster_size.argtypes = [p]
        L.g4o_sim_raster_size.restype = C.c_int64
        L.g4o_sim_raster.argtypes = [p, p, p, C.c_int64]
        L.g4o_sim_raster.restype = C.c_int64
        L.g4o_sim_counts.argtypes = [p, p, C.c_int64]
        L.g4o_sim_counts.restype = C.c_int64
        L.g4o_sim_state.argtypes = [p] + [p] * 8
        L.g4o_sim_state64.argtypes = [p, p, p]
        L.g4o_sim_acc.argtypes = [p, p]
        L.g4o_sim_stats.argtypes = [p, p, p, p]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def philox4x64_10(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, dtype=np.uint64)
    k = np.asarray(key, dtype=np.uint64)
    out = np.zeros(4, dtype=np.uint64)
    lib().g4o_philox4x64_10(_ptr(c), _ptr(k), _ptr(out))
    return out


def philox4x32_10(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().g4o_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return out


def logf(x: float) -> float:
    return lib().g4o_logf(x)


def normal(seed: int, neuron: int, step: int) -> float:
    return lib().g4o_normal(seed, neuron, step)


def wfix(w: float) -> int:
    return lib().g4o_wfix(w)


def row_stride(nsyn: int) -> int:
    return (nsyn + 3) // 4 * 4


def make_desc(n, nsyn, seed, drive_scale=1.0, self_loops=0, exc_permille=800, stride=None) -> Desc:
    return Desc(n=n, nsyn=nsyn, stride=row_stride(nsyn) if stride is None else stride,
                exc_permille=exc_permille, self_loops=self_loops, seed=seed,
                drive_scale=drive_scale, pad_=0)


def conn_philox(desc: Desc, row0: int = 0, nrows: int | None = None):
    nrows = desc.n - row0 if nrows is None else nrows
    idx = np.empty((nrows, desc.stride), dtype=np.int32)
    w = np.empty((nrows, desc.stride), dtype=np.float32)
    if lib().g4o_conn_philox(C.byref(desc), row0, nrows, _ptr(idx), _ptr(w)) != 0:
        raise ValueError("invalid connectivity request")
    return idx, w


def sort_rows(idx: np.ndarray, w: np.ndarray):
    """Sort every row in place into the library's order (target as unsigned, then weight bits)."""
    assert idx.flags.c_contiguous and w.flags.c_contiguous and idx.shape == w.shape
    assert idx.dtype == np.int32 and w.dtype == np.float32
    if lib().g4o_sort_rows(_ptr(idx), _ptr(w), idx.shape[0], idx.shape[1]) != 0:
        raise MemoryError("row sort failed")


def conn_glibc(seed: int, n: int, nsyn: int):
    idx = np.empty((n, nsyn), dtype=np.int32)
    w = np.empty((n, nsyn), dtype=np.float32)
    if lib().g4o_conn_glibc(seed, n, nsyn, _ptr(idx), _ptr(w)) != 0:
        raise ValueError("invalid connectivity request")
    return idx, w


def ref_tables(seed: int, n: int, nsyn: int, workdir: str):
    """Run the reference's own host generator (oracle/_ref, built by `make ref`)."""
    os.makedirs(workdir, exist_ok=True)
    env = dict(os.environ, G4S_REF_SEED=str(seed), G4S_REF_OUT=workdir)
    subprocess.run([REF_TABLES, str(n), str(nsyn), "1"], env=env, check=True,
                   stdout=subprocess.DEVNULL)
    w = np.fromfile(os.path.join(workdir, "conn_w.bin"), dtype=np.float32).reshape(n, nsyn)
    idx = np.fromfile(os.path.join(workdir, "conn_idx.bin"), dtype=np.int32).reshape(n, nsyn)
    return idx, w


@dataclass
class Stats:
    rate_hz: float
    isi_cv: float
    total_spikes: int


class Sim:
    """One oracle network; the tables must outlive the object (they are not copied)."""

    def __init__(self, desc: Desc, idx: np.ndarray, w: np.ndarray, mode: int = FP32):
        self.desc = desc
        self._idx = np.ascontiguousarray(idx, dtype=np.int32)
        self._w = np.ascontiguousarray(w, dtype=np.float32)
        assert self._idx.shape == (desc.n, desc.stride) and self._w.shape == self._idx.shape
        self._h = lib().g4o_sim_create(C.byref(desc), _ptr(self._idx), _ptr(self._w), mode)
        if not self._h:
            raise MemoryError("oracle simulation could not be created")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().g4o_sim_destroy(h)
            self._h = None

    def run(self, steps: int, threads: int = 1):
        if lib().g4o_sim_run(self._h, steps, threads) != 0:
            raise RuntimeError("oracle run failed")

    @property
    def step(self) -> int:
        return lib().g4o_sim_step_index(self._h)

    def raster(self):
        n = lib().g4o_sim_raster_size(self._h)
        t = np.empty(n, dtype=np.int32)
        i = np.empty(n, dtype=np.int32)
        lib().g4o_sim_raster(self._h, _ptr(t), _ptr(i), n)
        return t, i

    def counts(self) -> np.ndarray:
        c = np.empty(self.step, dtype=np.int32)
        lib().g4o_sim_counts(self._h, _ptr(c), c.size)
        return c

    def state(self) -> dict:
        n = self.desc.n
        out = {k: np.empty(n, dtype=np.float32) for k in ("v", "u", "I", "a", "b", "c", "d")}
        out["nospks"] = np.empty(n, dtype=np.int32)
        lib().g4o_sim_state(self._h, *(_ptr(out[k]) for k in ("v", "u", "I", "a", "b", "c", "d", "nospks")))
        return out

    def state64(self):
        n = self.desc.n
        v = np.empty(n, dtype=np.float64)
        u = np.empty(n, dtype=np.float64)
        lib().g4o_sim_state64(self._h, _ptr(v), _ptr(u))
        return v, u

    def acc(self) -> np.ndarray:
        a = np.empty(self.desc.n, dtype=np.int64)
        lib().g4o_sim_acc(self._h, _ptr(a))
        return a

    def stats(self) -> Stats:
        r = C.c_double()
        cv = C.c_double()
        tot = C.c_int64()
        lib().g4o_sim_stats(self._h, C.byref(r), C.byref(cv), C.byref(tot))
        return Stats(r.value, cv.value, tot.value)
