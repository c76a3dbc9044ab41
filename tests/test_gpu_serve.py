"""GPU tests of the serving layer (continuous batching) and of the autotuner."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _wait_all(srv, count, timeout=180.0):
    results, deadline = {}, time.time() + timeout
    while len(results) < count and time.time() < deadline:
        for r in srv.poll():
            results[r.id] = r
        time.sleep(0.002)
    return results


def test_server_results_same_alone_and_in_mix(g4s):
    """Requests of uneven size, fan-out, length, seed and drive, some arriving while
    others run, give exactly the rasters and final states of the same networks run alone."""
    from gpu4snn_gb300.server import Server
    specs = [(3000, 200, 150, 101, 1.0), (12000, 500, 90, 102, 1.3), (800, 300, 200, 103, 0.7),
             (40000, 100, 60, 104, 1.0), (5000, 1000, 120, 105, 2.0), (20000, 50, 80, 106, 0.9)]
    with Server(hbm_budget_bytes=8 << 30, quantum=37) as srv:
        ids = []
        for k, (n, s, st, seed, d) in enumerate(specs):
            ids.append(srv.submit(n, s, st, seed, d, record_raster=True))
            if k == 2:
                time.sleep(0.05)
        results = _wait_all(srv, len(specs))
        assert len(results) == len(specs)
        stats = srv.stats()
        assert stats.rounds > 1 and stats.peak_bytes <= 8 << 30
        for rid, (n, s, st, seed, d) in zip(ids, specs):
            r = results[rid]
            assert r.status == 0 and r.steps_done == st
            got = srv.result(rid)
            with g4s.Network(n, s, seed=seed, drive_scale=d) as alone:
                alone.run(st, g4s.ALG_SKL)
                t, i = alone.raster()
                assert np.array_equal(got["t"], t) and np.array_equal(got["id"], i), n
                s_ = alone.state()
                assert np.array_equal(got["v"].view(np.uint32), s_["v"].view(np.uint32))
                assert np.array_equal(got["u"].view(np.uint32), s_["u"].view(np.uint32))
                assert np.array_equal(got["nospks"], s_["nospks"])
                assert r.total_spikes == len(t)
            srv.release(rid)


def test_served_requests_against_the_oracle(g4s, oracle):
    """Spot checks of served requests: each served raster equals the FP32 oracle's bit for
    bit, and for sampled requests the firing rate and ISI CV are within 1% of the FP64
    oracle's (the same random draws in double precision; 0.47% and 0.13% here: the runs are
    chaotic, so the precisions' trajectories separate, but their statistics agree)."""
    from gpu4snn_gb300.server import Server
    specs = [(2500, 1000, 2000, 1, 1.0, True), (4000, 400, 2000, 9, 1.3, True), (3000, 600, 2000, 21, 0.8, False)]
    with Server(hbm_budget_bytes=4 << 30, quantum=250) as srv:
        ids = [srv.submit(n, s, st, seed, d, record_raster=True) for n, s, st, seed, d, _ in specs]
        results = _wait_all(srv, len(specs))
        assert len(results) == len(specs)
        for rid, (n, s, st, seed, d, fp64) in zip(ids, specs):
            r = results[rid]
            assert r.status == 0 and r.steps_done == st
            got = srv.result(rid)
            desc = oracle.make_desc(n, s, seed, drive_scale=d)
            idx, w = oracle.conn_philox(desc)
            s32 = oracle.Sim(desc, idx, w, oracle.FP32)
            s32.run(st, threads=8)
            t, i = s32.raster()
            assert np.array_equal(got["t"], t) and np.array_equal(got["id"], i), n
            if fp64:
                s64 = oracle.Sim(desc, idx, w, oracle.FP64)
                s64.run(st)
                ref = s64.stats()
                assert abs(r.rate_hz - ref.rate_hz) / ref.rate_hz < 0.01
                assert abs(r.isi_cv - ref.isi_cv) / ref.isi_cv < 0.01
            srv.release(rid)


def test_server_budget_and_rejections(g4s):
    from gpu4snn_gb300 import _lib
    from gpu4snn_gb300.server import Server
    # a budget that holds one of these requests at a time: they queue and all complete
    with Server(hbm_budget_bytes=200 << 20, quantum=50) as srv:
        ids = [srv.submit(20000, 400, 120, 200 + k, 1.0) for k in range(4)]
        with pytest.raises(_lib.G4SError) as e:
            srv.submit(400000, 2000, 10, 1, 1.0)
        assert e.value.code == _lib.ERR_BUDGET
        with pytest.raises(_lib.G4SError) as e:
            srv.submit(100, 200, 10, 1, 1.0)
        assert e.value.code == _lib.ERR_INVALID
        results = _wait_all(srv, len(ids))
        assert sorted(results) == sorted(ids) and all(r.status == 0 for r in results.values())
        assert srv.stats().peak_bytes <= 200 << 20


def test_server_stop_without_drain(g4s):
    """Stopping with requests queued, resident and finishing: the resident ones finish,
    the retire thread frees every finished network, the queued ones are dropped, and the
    call returns; a second server then runs normally."""
    from gpu4snn_gb300.server import Server
    srv = Server(hbm_budget_bytes=300 << 20, quantum=40)
    for k in range(8):
        srv.submit(15000 + 1000 * k, 300, 60 + 20 * k, 300 + k, 1.0)
    time.sleep(0.05)
    done_before = len(srv.poll())
    t0 = time.time()
    srv.stop(drain=False)
    assert time.time() - t0 < 120.0 and done_before <= 8
    with Server(hbm_budget_bytes=300 << 20, quantum=40) as srv2:
        rid = srv2.submit(8000, 200, 50, 7, 1.0)
        res = _wait_all(srv2, 1)
        assert res[rid].status == 0 and res[rid].steps_done == 50


def test_autotune_does_not_perturb(g4s, oracle):
    n, nsyn, seed = 20000, 300, 7
    d = oracle.make_desc(n, nsyn, seed)
    idx, w = oracle.conn_philox(d)
    sim = oracle.Sim(d, idx, w)
    sim.run(100, threads=8)
    with g4s.Network(n, nsyn, seed=seed) as net:
        net.run(50, g4s.ALG_SKL)
        alg, team, us = net.autotune(30)
        assert alg in (0, 3, 4) and us > 0
        net.run(50, g4s.ALG_AUTO)
        assert net.info().steps_done == 100
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
        assert np.array_equal(net.state()["v"].view(np.uint32), sim.state()["v"].view(np.uint32))
