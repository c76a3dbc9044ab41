"""Edge cases of the CUDA path against the oracle: the smallest network, a fully connected
one, a silent one, long rows, and handles driven from concurrent host threads."""
from __future__ import annotations

import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALGS = [0, 1, 2, 3, 4]


def _same_floats(x, y):
    """Bit-identical, except that any NaN matches any NaN (the GPU's and the host CPU's
    invalid operations produce NaNs with different payloads)."""
    nx, ny = np.isnan(x), np.isnan(y)
    return np.array_equal(nx, ny) and np.array_equal(x[~nx].view(np.uint32), y[~ny].view(np.uint32))


def _check(net, sim):
    assert np.array_equal(net.counts(), sim.counts())
    assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
    s, o = net.state(), sim.state()
    for k in ("v", "u", "a", "b", "c", "d"):
        assert _same_floats(s[k], o[k]), k
    assert np.array_equal(s["nospks"], o["nospks"])
    assert np.array_equal(net.currents(), sim.acc())


@pytest.mark.parametrize("alg", ALGS)
def test_two_neurons(g4s, oracle, alg):
    d = oracle.make_desc(2, 1, 5, drive_scale=1.5)
    idx, w = oracle.conn_philox(d)
    assert sorted(idx[:, 0].tolist()) == [0, 1] and idx[0, 0] == 1  # each targets the other
    sim = oracle.Sim(d, idx, w)
    sim.run(300)
    # weights of (1000 / Nsyn) x U drive the membrane to overflow: u becomes NaN (both sides)
    with g4s.Network(2, 1, seed=5, drive_scale=1.5) as net:
        net.run(300, alg)
        _check(net, sim)


@pytest.mark.parametrize("p", [1, 4, 16])
def test_fully_connected(g4s, oracle, p):
    n, nsyn, seed = 300, 299, 6
    d = oracle.make_desc(n, nsyn, seed)
    idx, w = oracle.conn_philox(d)
    rows = np.sort(np.where(idx >= 0, idx, n), axis=1)[:, :nsyn]
    assert all(np.array_equal(r, np.delete(np.arange(n), i)) for i, r in enumerate(rows))
    sim = oracle.Sim(d, idx, w)
    sim.run(200)
    with g4s.Network(n, nsyn, seed=seed) as net:
        net.set_geometry(p, 0)
        net.run(200, 4)
        _check(net, sim)


def test_silent_network(g4s, oracle):
    """No drive: no neuron ever fires, every step's exchange and delivery are empty."""
    n, nsyn, seed = 20_000, 100, 7
    d = oracle.make_desc(n, nsyn, seed, drive_scale=0.0)
    sim = oracle.Sim(d, *oracle.conn_philox(d))
    sim.run(100)
    assert sim.counts().sum() == 0
    with g4s.Network(n, nsyn, seed=seed, drive_scale=0.0) as net:
        assert net.geometry()[0] > 1
        net.run(100, 4)
        assert net.counts().sum() == 0 and net.info().total_spikes == 0
        _check(net, sim)


def test_long_rows(g4s, oracle):
    """8192 synapses per neuron (half the longest row the device sort takes)."""
    n, nsyn, seed = 9000, 8192, 8
    d = oracle.make_desc(n, nsyn, seed)
    sim = oracle.Sim(d, *oracle.conn_philox(d))
    sim.run(60, threads=16)
    for p in (0, 2):
        with g4s.Network(n, nsyn, seed=seed) as net:
            net.set_geometry(p, 0)
            net.run(60, 4)
            _check(net, sim)


def test_concurrent_handles_from_two_threads(g4s):
    """Distinct handles on distinct host threads give the results of sequential runs."""
    specs = [(30_000, 500, 11, 1.0), (12_000, 800, 12, 1.5)]
    ref = []
    for n, s, seed, drive in specs:
        with g4s.Network(n, s, seed=seed, drive_scale=drive) as net:
            net.run(400, 4)
            ref.append(net.raster())
    out, errs = [None, None], []

    def work(k):
        try:
            n, s, seed, drive = specs[k]
            with g4s.Network(n, s, seed=seed, drive_scale=drive) as net:
                net.run(400, 4)
                out[k] = net.raster()
        except Exception as e:  # surfaced below
            errs.append(e)

    ts = [threading.Thread(target=work, args=(k,)) for k in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errs
    for a, b in zip(out, ref):
        assert np.array_equal(np.stack(a), np.stack(b))
