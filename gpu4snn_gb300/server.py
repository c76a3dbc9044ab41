"""Python face of the simulation server (g4s_server_*): continuous batching of simulation
requests on one GPU under a device-memory budget."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check, load, ptr


@dataclass
class Result:
    id: int
    status: int
    steps_done: int
    total_spikes: int
    latency_ms: float
    queue_ms: float
    rate_hz: float
    isi_cv: float
    create_ms: float = 0.0  # network creation at admission
    device_ms: float = 0.0  # device time of its steps in the rounds
    sm_ms: float = 0.0      # the same times the CTAs of its team
    rounds: int = 0
    team: int = 0


class Server:
    """Requests are admitted while they fit `hbm_budget_bytes` and advanced together, one
    persistent launch per round: `quantum` steps in a request's first round, then as many as
    the median resident request runs in `quantum` steps (rounds of even duration); arrivals
    join at the next round."""

    def __init__(self, hbm_budget_bytes: int, quantum: int = 250):
        h = C.c_void_p()
        check(load().g4s_server_start(hbm_budget_bytes, quantum, C.byref(h)))
        self._h = h
        self.sizes: dict[int, int] = {}

    def submit(self, n: int, nsyn: int, steps: int, seed: int, drive_scale: float = 1.0,
               record_raster: bool = False) -> int:
        req = _lib.Request(n=n, nsyn=nsyn, steps=steps, seed=seed, drive_scale=drive_scale,
                           record_raster=int(record_raster))
        rid = C.c_int64()
        check(load().g4s_server_submit(self._h, C.byref(req), C.byref(rid)))
        self.sizes[rid.value] = n
        return rid.value

    def poll(self, cap: int = 4096) -> list[Result]:
        buf = (_lib.RequestResult * cap)()
        k = C.c_int32()
        check(load().g4s_server_poll(self._h, C.cast(buf, C.c_void_p), cap, C.byref(k)))
        return [Result(r.id, r.status, r.steps_done, r.total_spikes, r.latency_ms, r.queue_ms, r.rate_hz, r.isi_cv,
                       r.create_ms, r.device_ms, r.sm_ms, r.rounds, r.team) for r in buf[:k.value]]

    def result(self, rid: int) -> dict:
        n = self.sizes[rid]
        size = C.c_int64()
        check(load().g4s_server_result(self._h, rid, None, None, 0, C.byref(size), None, None, None))
        t = np.empty(size.value, dtype=np.int32)
        i = np.empty(size.value, dtype=np.int32)
        v = np.empty(n, dtype=np.float32)
        u = np.empty(n, dtype=np.float32)
        nos = np.empty(n, dtype=np.int32)
        check(load().g4s_server_result(self._h, rid, ptr(t), ptr(i), size.value, C.byref(size), ptr(v), ptr(u),
                                       ptr(nos)))
        return {"t": t, "id": i, "v": v, "u": u, "nospks": nos}

    def release(self, rid: int):
        check(load().g4s_server_release(self._h, rid))

    def stats(self) -> _lib.ServerStats:
        st = _lib.ServerStats()
        check(load().g4s_server_get_stats(self._h, C.byref(st)))
        return st

    def stop(self, drain: bool = True):
        if getattr(self, "_h", None) and self._h.value:
            check(load().g4s_server_stop(self._h, int(drain)))
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.stop(drain=True)
