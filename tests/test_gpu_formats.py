"""The GPU-side writers of the binary files: a streamed raster equals the raster of the same
run kept in memory, and a network rebuilt from a tables checkpoint runs identically."""
from __future__ import annotations

import numpy as np
import pytest

from gpu4snn_gb300 import formats as F

pytestmark = pytest.mark.gpu


def test_streamed_raster_equals_host_raster(g4s, tmp_path):
    n, nsyn, seed = 2000, 200, 13
    p = str(tmp_path / "stream.g4s")
    # a small raster buffer forces many device chunks per run (one file chunk each)
    with g4s.Network(n, nsyn, seed=seed, raster_budget_bytes=64 << 10) as a, \
            g4s.Network(n, nsyn, seed=seed, raster_budget_bytes=64 << 10) as b:
        a.stream_raster(p)
        a.run(100, g4s.ALG_SKL)
        a.run(50, g4s.ALG_SKL)
        a.stream_raster(None)
        b.run(100, g4s.ALG_SKL)
        b.run(50, g4s.ALG_SKL)
        t, i = b.raster()
        r = F.read_raster(p)
        assert r.complete and r.n == n and r.t0 == 0 and len(r.counts) == 150
        assert np.array_equal(r.counts, b.counts())
        assert np.array_equal(r.times(), t) and np.array_equal(r.ids, i)
        assert len(a.raster()[0]) == 0  # streamed, not kept in host memory
        q = str(tmp_path / "whole.g4s")
        b.write_raster_file(q)
        w = F.read_raster(q)
        assert np.array_equal(w.counts, b.counts()) and np.array_equal(w.ids, i)
        with pytest.raises(g4s.G4SError):  # a's host raster does not hold the streamed steps
            a.write_raster_file(q)


def test_stream_needs_a_recorded_raster(g4s, tmp_path):
    with g4s.Network(500, 50, seed=1, record_raster=False) as net:
        with pytest.raises(g4s.G4SError):
            net.stream_raster(str(tmp_path / "x.g4s"))


def test_tables_checkpoint_rebuilds_the_same_network(g4s, tmp_path):
    n, nsyn, seed = 3000, 300, 21
    p = str(tmp_path / "tables.g4s")
    with g4s.Network(n, nsyn, seed=seed) as a:
        a.save_tables(p)
        a.run(200)
        ta, ia = a.raster()
        idx, w = a.tables()
    t = F.read_tables(p)
    assert t.n == n and t.nsyn == nsyn and t.seed == seed and t.flags == 1
    assert np.array_equal(t.idx, idx) and np.array_equal(t.w.view(np.uint32), w.view(np.uint32))
    with g4s.Network(n, nsyn, seed=seed, tables_file=p) as b:
        b.run(200)
        tb, ib = b.raster()
    assert np.array_equal(ta, tb) and np.array_equal(ia, ib)
    with pytest.raises(g4s.G4SError):
        g4s.Network(n + 1, nsyn, seed=seed, tables_file=p)


def test_protocol_results_feed_the_sweep_summary(g4s, tmp_path):
    from gpu4snn_gb300 import summary as S
    g4s.run_protocol(500, 50, 100, algorithm=-1, mode=1, seed=3, results_root=str(tmp_path))
    runs = S.collect(str(tmp_path))
    assert sorted(r.alg for r in runs) == [0, 1, 2, 3, 4] and all(r.n == 500 and r.mode == 1 for r in runs)
    assert len({r.spikes for r in runs}) == 1  # every scheme simulates the same network identically
    rows = S.speedup_table(runs, n=500, nsyn=50, modes=(1,))
    assert len(rows) == 6 and all(r[7] > 0 for r in rows)
