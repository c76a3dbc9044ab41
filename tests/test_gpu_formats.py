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


def _g(x) -> str:
    """A float field as the reference's ofstream writes it: default precision 6, no fixed
    or scientific flag, i.e. printf's %g of the float's double value (gpu4snn.cu:727-729)."""
    return "%g" % float(np.float32(x))


def _records(st, init: bool) -> bytes:
    """neuroninfo.csv / neuroninfoafter.csv bytes for a state dict (writeNeuronInfo's field
    order a b c d v u I id nospks, gpu4snn.cu:727-729; header gpu4snn.cu:1124, 1326)."""
    n = len(st["a"])
    out = ["a b c d v u I id nospks\n"]
    for i in range(n):
        b = st["b"][i]
        v, u, I, k = ((-65.0, np.float32(b) * np.float32(-65.0), 0.0, 0) if init
                      else (st["v"][i], st["u"][i], st["I"][i], int(st["nospks"][i])))
        out.append(f"{_g(st['a'][i])} {_g(b)} {_g(st['c'][i])} {_g(st['d'][i])} {_g(v)} {_g(u)} {_g(I)} {i} {k}\n")
    return "".join(out).encode()


@pytest.mark.parametrize("law", ["philox", "glibc"])
def test_protocol_result_files_byte_for_byte(g4s, oracle, tmp_path, law):
    """g4s_run_protocol's five files per (mode, scheme) against the reference's formats:
    neuroninfo.csv, spiketimes.csv and neuroninfoafter.csv byte for byte against the same
    run of the oracle (their content is the exact state and raster); computetime.csv and
    sim_overview.csv by grammar (their times are measured), with their integer columns
    against the oracle: headers (gpu4snn.cu:1124, 1134, 1140, 1312), single spaces, the
    %g floats, one row per neuron / spike / step, and no newline after sim_overview.csv's
    one row (gpu4snn.cu:1313).  Both connectivity laws: the GPU generator's, and the
    reference's own glibc rand() law (self loops allowed, gpu4snn.cu:873-898)."""
    import re
    n, nsyn, steps, seed = 500, 100, 200, 5
    glibc = law == "glibc"
    g4s.run_protocol(n, nsyn, steps, algorithm=-1, mode=-1, seed=seed, results_root=str(tmp_path),
                     conn_law=g4s.CONN_GLIBC if glibc else g4s.CONN_PHILOX)
    num = r"-?(?:\d+(?:\.\d*)?|\.\d+)(?:e[+-]\d+)?|inf|nan"
    for m, scale in enumerate((0.5, 1.0, 1.5)):
        d = oracle.make_desc(n, nsyn, seed, drive_scale=scale, self_loops=1 if glibc else 0)
        idx, w = oracle.conn_glibc(seed, n, nsyn) if glibc else oracle.conn_philox(d)
        sim = oracle.Sim(d, idx, w)
        init = sim.state()
        sim.run(steps)
        t, i = sim.raster()
        counts = sim.counts()
        spikes_txt = ("SpkTime NeuronID\n" + "".join(f"{a} {b}\n" for a, b in zip(t, i))).encode()
        for alg in range(5):
            p = tmp_path / "Results" / f"N{n}Nsyn{nsyn}Regime{m}Alg{alg}"
            assert sorted(x.name for x in p.iterdir()) == ["computetime.csv", "neuroninfo.csv", "neuroninfoafter.csv",
                                                          "sim_overview.csv", "spiketimes.csv"]
            assert (p / "neuroninfo.csv").read_bytes() == _records(init, True)
            assert (p / "spiketimes.csv").read_bytes() == spikes_txt
            assert (p / "neuroninfoafter.csv").read_bytes() == _records(sim.state(), False)
            ct = (p / "computetime.csv").read_bytes().decode()
            lines = ct.split("\n")
            assert lines[0] == "TimeStep SpksPerStep TimeKernelUpdate TimeSpent" and lines[-1] == ""
            assert len(lines) == steps + 2
            for k, row in enumerate(lines[1:-1]):
                f = row.split(" ")
                assert len(f) == 4 and f[0] == str(k) and f[1] == str(counts[k])
                assert all(re.fullmatch(num, x) and _g(float(x)) == x for x in f[2:]), row
            ov = (p / "sim_overview.csv").read_bytes().decode()
            head, row = ov.split("\n")
            assert head == "N elapsed(ms) elapsedwithdata(ms) totalspkcount" and not row.endswith("\n")
            f = row.split(" ")
            assert len(f) == 4 and f[0] == str(n) and f[3] == str(len(t))
            assert all(re.fullmatch(num, x) and ("%g" % float(x)) == x for x in f[1:3]), row
