"""Host logic of the reference-kernel harness and of the bench's served breakdown (CPU).

raster_stats computes, from a (step, neuron) raster such as the reference's kernels
produce, the statistics the oracle and the library compute on the fly (mean rate over all
neurons, mean per-neuron ISI CV over neurons with at least two intervals): on an oracle
run both must agree to rounding.  The served breakdown's bound is the largest of the mix's
SM time spread over every SM, the total creation time and the longest request."""
import importlib.util
import os
from types import SimpleNamespace

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_raster_stats_match_the_oracle(oracle):
    from oracle import refgpu as R
    n, nsyn, steps = 1500, 200, 600
    d = oracle.make_desc(n, nsyn, 4, drive_scale=1.5)
    idx, w = oracle.conn_philox(d)
    sim = oracle.Sim(d, idx, w)
    sim.run(steps, threads=4)
    t, i = sim.raster()
    st = sim.stats()
    rate, cv = R.raster_stats(t, i, n, steps)
    assert rate == pytest.approx(st.rate_hz, rel=1e-12)
    assert cv == pytest.approx(st.isi_cv, rel=1e-9)
    # order of the raster does not matter
    perm = np.random.default_rng(0).permutation(len(t))
    assert R.raster_stats(t[perm], i[perm], n, steps) == pytest.approx((rate, cv), rel=1e-9)


def test_raster_stats_edge_cases(oracle):
    from oracle import refgpu as R
    e = np.zeros(0, dtype=np.int32)
    assert R.raster_stats(e, e, 10, 100) == (0.0, 0.0)
    # one neuron, intervals 10, 10, 20: mean 40/3, population sd sqrt(200/9)
    t = np.array([0, 10, 20, 40], dtype=np.int32)
    i = np.zeros(4, dtype=np.int32)
    rate, cv = R.raster_stats(t, i, 2, 100)
    assert rate == pytest.approx(4 * 1000.0 / 200)
    assert cv == pytest.approx(np.sqrt(200.0 / 9.0) / (40.0 / 3.0))


def test_refgpu_unavailable_names_the_missing_part(tmp_path):
    from oracle import refgpu as R
    why = R.unavailable(str(tmp_path / "absent.cubin"))
    assert why is not None and "absent.cubin" in why


def test_served_breakdown_bound():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    N = np.array([1000, 50_000, 200_000])
    T = np.array([500, 5000, 20_000])
    res = [SimpleNamespace(device_ms=10.0, sm_ms=10.0, team=1, create_ms=2.0, queue_ms=1.0, latency_ms=20.0),
           SimpleNamespace(device_ms=100.0, sm_ms=700.0, team=7, create_ms=5.0, queue_ms=3.0, latency_ms=150.0),
           SimpleNamespace(device_ms=400.0, sm_ms=10_000.0, team=25, create_ms=9.0, queue_ms=4.0, latency_ms=500.0)]
    b = bench.served_breakdown(N, T, res, np.array([15.0, 120.0, 450.0]), np.array([9.0, 90.0, 380.0]), 600.0,
                               sms=10)
    assert b["sm_ms"] == 10_710.0 and b["create_ms"] == 16.0 and b["longest_request_ms"] == 409.0
    assert b["bound_ms"] == 1071.0 and b["best_speedup_in_this_geometry"] == pytest.approx(600.0 / 1071.0)
    assert sum(x["requests"] for x in b["bins"]) == 3
