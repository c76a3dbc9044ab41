"""Network handle: the Python face of one simulated Izhikevich network.

Mirrors the reference's objects: the neuron record (gpu4snn.cu:50-62), the connectivity
tables (d_conn_idx / d_conn_w, gpu4snn.cu:762-773), the step loop with its five schemes
(gpu4snn.cu:1215-1300) and the per-run outputs (gpu4snn.cu:1109-1140, 1256-1327).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import CONN_GLIBC, CONN_PHILOX, check, load, ptr


def row_stride(nsyn: int) -> int:
    return (nsyn + 3) // 4 * 4


@dataclass
class Stats:
    rate_hz: float
    isi_cv: float
    total_spikes: int


class Network:
    """One network on the current CUDA device.

    n, nsyn       neurons and distinct targets per neuron (the reference's N, Nsyn)
    seed          seeds the tables, the neuron parameters and the thalamic drive
    drive_scale   gains (5, 2) x scale; the reference's modes 0/1/2 are 0.5/1.0/1.5
    self_loops    allow a neuron to target itself (the reference's generator does)
    conn_law      CONN_PHILOX (GPU generator) or CONN_GLIBC (the reference's rand() law)
    tables        optional (idx, w) host arrays [n][stride] to upload instead
    tables_file   optional tables checkpoint (save_tables) to build from instead
    """

    def __init__(self, n: int, nsyn: int, seed: int = 1, drive_scale: float = 1.0, self_loops: bool = False,
                 conn_law: int = CONN_PHILOX, exc_permille: int = 800, record_raster: bool = True,
                 raster_budget_bytes: int = 0, tables: tuple[np.ndarray, np.ndarray] | None = None,
                 tables_file: str | None = None):
        L = load()
        self.desc = _lib.NetDesc(n=n, nsyn=nsyn, exc_permille=exc_permille, self_loops=int(self_loops),
                                 conn_law=conn_law, seed=seed, drive_scale=drive_scale,
                                 record_raster=int(record_raster), raster_budget_bytes=raster_budget_bytes)
        h = C.c_void_p()
        if tables_file is not None:
            check(L.g4s_net_create_from_file(C.byref(self.desc), tables_file.encode(), C.byref(h)))
        elif tables is None:
            check(L.g4s_net_create(C.byref(self.desc), C.byref(h)))
        else:
            idx = np.ascontiguousarray(tables[0], dtype=np.int32)
            w = np.ascontiguousarray(tables[1], dtype=np.float32)
            check(L.g4s_net_create_from_tables(C.byref(self.desc), ptr(idx), ptr(w), idx.shape[1], C.byref(h)))
        self._h = h
        self.n, self.nsyn, self.stride = n, nsyn, row_stride(nsyn)

    # -- lifetime ---------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            check(load().g4s_net_destroy(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- stepping ---------------------------------------------------------------------
    def reset(self):
        check(load().g4s_net_reset(self._h))

    def run(self, steps: int, algorithm: int = _lib.ALG_AUTO):
        check(load().g4s_net_run(self._h, steps, algorithm))

    def set_barrier_timeout(self, ns: int):
        check(load().g4s_net_set_barrier_timeout(self._h, ns))

    def inject_fault(self, kind: int):
        check(load().g4s_inject_fault(self._h, kind))

    def set_geometry(self, owner_blocks: int = 0, delivery: int = -1):
        """SKL owner CTAs (0 = automatic) and delivery mapping of a multi-CTA team (-1
        automatic, 0 segment runs, 1 eight lanes a spike)."""
        check(load().g4s_net_set_geometry(self._h, owner_blocks, delivery))

    def set_block_threads(self, threads: int):
        """Threads per CTA of the SKL team kernel: 1024, 768 or 0 (automatic, the default);
        results do not depend on it."""
        check(load().g4s_net_set_block_threads(self._h, threads))

    def block_threads(self) -> int:
        t = C.c_int32()
        check(load().g4s_net_get_block_threads(self._h, C.byref(t)))
        return t.value

    def autotune(self, probe_steps: int = 100) -> tuple[int, int, float]:
        """Time the candidate schemes on this network (state restored afterwards) and keep
        the fastest for ALG_AUTO.  Returns (scheme, team size, us per step)."""
        a, t, us = C.c_int32(), C.c_int32(), C.c_double()
        check(load().g4s_net_autotune(self._h, probe_steps, C.byref(a), C.byref(t), C.byref(us)))
        return a.value, t.value, us.value

    def geometry(self) -> tuple[int, int]:
        """(owner CTAs, neurons per CTA) of the SKL kernel; (0, 0) on the fallback kernel."""
        p, rc = C.c_int32(), C.c_int64()
        check(load().g4s_net_get_geometry(self._h, C.byref(p), C.byref(rc)))
        return p.value, rc.value

    def delivery(self) -> int:
        """Delivery mapping in use: 0 segment runs, 1 eight lanes a spike, -1 without a
        multi-CTA team."""
        d = C.c_int32()
        check(load().g4s_net_get_delivery(self._h, C.byref(d)))
        return d.value

    def load_tables(self, idx: np.ndarray, w: np.ndarray):
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        w = np.ascontiguousarray(w, dtype=np.float32)
        check(load().g4s_net_load_tables(self._h, ptr(idx), ptr(w), idx.shape[1]))

    # -- results ----------------------------------------------------------------------
    def info(self) -> _lib.NetInfo:
        inf = _lib.NetInfo()
        check(load().g4s_net_get_info(self._h, C.byref(inf)))
        return inf

    def raster(self) -> tuple[np.ndarray, np.ndarray]:
        size = C.c_int64()
        check(load().g4s_net_raster(self._h, None, None, 0, C.byref(size)))
        t = np.empty(size.value, dtype=np.int32)
        i = np.empty(size.value, dtype=np.int32)
        check(load().g4s_net_raster(self._h, ptr(t), ptr(i), size.value, C.byref(size)))
        return t, i

    def counts(self) -> np.ndarray:
        size = C.c_int64()
        check(load().g4s_net_counts(self._h, None, 0, C.byref(size)))
        c = np.empty(size.value, dtype=np.int32)
        check(load().g4s_net_counts(self._h, ptr(c), size.value, C.byref(size)))
        return c

    def step_times(self) -> tuple[np.ndarray, np.ndarray]:
        size = C.c_int64()
        check(load().g4s_net_step_times(self._h, None, None, 0, C.byref(size)))
        u = np.empty(size.value, dtype=np.float32)
        s = np.empty(size.value, dtype=np.float32)
        check(load().g4s_net_step_times(self._h, ptr(u), ptr(s), size.value, C.byref(size)))
        return u, s

    def state(self) -> dict:
        out = {k: np.empty(self.n, dtype=np.float32) for k in ("v", "u", "I", "a", "b", "c", "d")}
        out["nospks"] = np.empty(self.n, dtype=np.int32)
        check(load().g4s_net_state(self._h, *(ptr(out[k]) for k in ("v", "u", "I", "a", "b", "c", "d", "nospks"))))
        return out

    def currents(self) -> np.ndarray:
        a = np.empty(self.n, dtype=np.int64)
        check(load().g4s_net_currents(self._h, ptr(a)))
        return a

    def tables(self, row0: int = 0, nrows: int | None = None) -> tuple[np.ndarray, np.ndarray]:
        nrows = self.n - row0 if nrows is None else nrows
        idx = np.empty((nrows, self.stride), dtype=np.int32)
        w = np.empty((nrows, self.stride), dtype=np.float32)
        check(load().g4s_net_tables(self._h, row0, nrows, ptr(idx), ptr(w)))
        return idx, w

    def stats(self) -> Stats:
        r, cv, tot = C.c_double(), C.c_double(), C.c_int64()
        check(load().g4s_net_stats(self._h, C.byref(r), C.byref(cv), C.byref(tot)))
        return Stats(r.value, cv.value, tot.value)

    def fp64_check(self, steps: int) -> dict:
        """On-device FP64 check (g4s_net_fp64_check): from step 0, `steps` steps of this
        network in lockstep with an FP64 twin on the GPU.  Returns per-step max, p99 and
        median |v32 - v64| (mV), the first step whose spike sets differ (-1: none) and the
        twin's final v, u."""
        mx, p99, p50 = (np.zeros(steps) for _ in range(3))
        v64, u64 = np.empty(self.n), np.empty(self.n)
        first = C.c_int32()
        check(load().g4s_net_fp64_check(self._h, steps, ptr(mx), ptr(p99), ptr(p50), C.byref(first), ptr(v64),
                                        ptr(u64)))
        return {"max": mx, "p99": p99, "median": p50, "first_divergent": first.value, "v64": v64, "u64": u64}

    def write_results(self, directory: str, elapsed_ms: float, elapsed_with_data_ms: float):
        check(load().g4s_net_write_results(self._h, directory.encode(), None, elapsed_ms, elapsed_with_data_ms))

    def stream_raster(self, path: str | None):
        """Stream the raster of the following runs to a binary file (None ends the stream);
        read it with gpu4snn_gb300.formats.read_raster."""
        check(load().g4s_net_stream_raster(self._h, None if path is None else path.encode()))

    def write_raster_file(self, path: str):
        check(load().g4s_net_write_raster_file(self._h, path.encode()))

    def save_tables(self, path: str):
        """Checkpoint the (sorted) tables; Network(..., tables_file=path) rebuilds from it."""
        check(load().g4s_net_save_tables(self._h, path.encode()))


def run_batch(nets: list[Network], steps) -> tuple[float, int]:
    """Advance several networks together in shared persistent launches of the SKL team
    kernel; network i runs steps[i] further steps.  Returns (device ms, launches)."""
    if isinstance(steps, int):
        steps = [steps] * len(nets)
    handles = (C.c_void_p * len(nets))(*[n._h.value for n in nets])
    st = np.ascontiguousarray(steps, dtype=np.int32)
    ms, nl = C.c_double(), C.c_int64()
    check(load().g4s_nets_run(C.cast(handles, C.c_void_p), ptr(st), len(nets), C.byref(ms), C.byref(nl)))
    return ms.value, nl.value


def conn_glibc(seed: int, n: int, nsyn: int, stride: int | None = None) -> tuple[np.ndarray, np.ndarray]:
    """The reference's host tables (glibc rand after srand(seed), gpu4snn.cu:873-898)."""
    stride = row_stride(nsyn) if stride is None else stride
    idx = np.empty((n, stride), dtype=np.int32)
    w = np.empty((n, stride), dtype=np.float32)
    check(load().g4s_conn_glibc(seed, n, nsyn, stride, ptr(idx), ptr(w)))
    return idx, w


def run_protocol(n: int, nsyn: int, iterations: int, algorithm: int = -1, mode: int = -1, seed: int = 1,
                 conn_law: int = CONN_PHILOX, results_root: str = "."):
    """The reference's experiment sweep (gpu4snn.cu:1082-1329)."""
    check(load().g4s_run_protocol(n, nsyn, iterations, algorithm, mode, seed, conn_law, results_root.encode()))


__all__ = ["Network", "Stats", "conn_glibc", "run_batch", "run_protocol", "row_stride", "CONN_GLIBC", "CONN_PHILOX"]
