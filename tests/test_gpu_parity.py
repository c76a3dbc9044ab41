"""GPU parity: the CUDA path against the CPU oracle, bit-exact (integer tables, Q32.32
currents, binary32 neuron state) on the same seeds."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALGS = [0, 1, 2, 3, 4]


def oracle_tables(O, n, nsyn, seed, self_loops=0):
    d = O.make_desc(n, nsyn, seed, self_loops=self_loops)
    return d, O.conn_philox(d)


def sorted_rows(idx, w):
    """The library keeps each row sorted by target (unused slots, negative, last); the
    oracle's rows are in draw order.  Same pairs, same order after this."""
    order = np.argsort(idx.view(np.uint32), axis=1, kind="stable")
    return np.take_along_axis(idx, order, 1), np.take_along_axis(w, order, 1)


def same_tables(gi, gw, oi, ow):
    si, sw = sorted_rows(oi, ow)
    return np.array_equal(gi, si) and np.array_equal(gw.view(np.uint32), sw.view(np.uint32))


@pytest.mark.parametrize("n,nsyn,seed,self_loops", [(2500, 1000, 1, 0), (1000, 999, 5, 0), (300, 37, 9, 0),
                                                    (257, 257, 11, 1), (5000, 3, 2, 0)])
def test_tables_bit_exact(g4s, oracle, n, nsyn, seed, self_loops):
    _, (idx, w) = oracle_tables(oracle, n, nsyn, seed, self_loops)
    with g4s.Network(n, nsyn, seed=seed, self_loops=bool(self_loops)) as net:
        gi, gw = net.tables()
    assert same_tables(gi, gw, idx, w)


@pytest.mark.parametrize("n,nsyn,seed", [(100_000, 1000, 2), (300_000, 1000, 6)])
def test_tables_large_sampled_rows(g4s, oracle, n, nsyn, seed):
    """Sampled rows of large tables: 100k x 1000 keeps each row's targets in a bitmap of the
    n targets, 300k x 1000 in a hash set (the smaller of the two)."""
    d = oracle.make_desc(n, nsyn, seed)
    with g4s.Network(n, nsyn, seed=seed, record_raster=False) as net:
        for row0 in (0, 1, n // 2 - 1, (n * 4) // 5 - 1, (n * 4) // 5, n - 3):
            gi, gw = net.tables(row0, 3)
            oi, ow = oracle.conn_philox(d, row0, 3)
            assert same_tables(gi, gw, oi, ow)


def test_tables_long_sampled_rows(g4s, oracle):
    """Rows of 10,000 synapses (the row sort's widest form: 16 keys per thread, 1024 threads)."""
    n, nsyn, seed = 12_000, 10_000, 4
    d = oracle.make_desc(n, nsyn, seed)
    with g4s.Network(n, nsyn, seed=seed, record_raster=False) as net:
        for row0 in (0, 5_999, n - 3):
            gi, gw = net.tables(row0, 3)
            oi, ow = oracle.conn_philox(d, row0, 3)
            assert same_tables(gi, gw, oi, ow)


def compare_state(net, sim):
    s, o = net.state(), sim.state()
    for k in ("v", "u", "a", "b", "c", "d"):
        assert np.array_equal(s[k].view(np.uint32), o[k].view(np.uint32)), k
    assert np.array_equal(s["nospks"], o["nospks"])
    assert np.array_equal(net.currents(), sim.acc())


@pytest.mark.parametrize("alg", ALGS)
def test_step_parity_200(g4s, oracle, alg):
    n, nsyn, seed = 2500, 1000, 1
    d, (idx, w) = oracle_tables(oracle, n, nsyn, seed)
    sim = oracle.Sim(d, idx, w)
    sim.run(200, threads=8)
    with g4s.Network(n, nsyn, seed=seed) as net:
        net.run(200, alg)
        t, i = net.raster()
        ot, oi = sim.raster()
        assert np.array_equal(t, ot) and np.array_equal(i, oi)
        assert np.array_equal(net.counts(), sim.counts())
        compare_state(net, sim)
        s = net.state()
        assert np.array_equal(s["I"].view(np.uint32), sim.state()["I"].view(np.uint32))


def test_full_config_skl_2000(g4s, oracle):
    n, nsyn, seed = 2500, 1000, 1
    d, (idx, w) = oracle_tables(oracle, n, nsyn, seed)
    sim = oracle.Sim(d, idx, w)
    sim.run(2000, threads=8)
    with g4s.Network(n, nsyn, seed=seed) as net:
        net.run(1000, 4)
        net.run(1000, 5)
        t, i = net.raster()
        ot, oi = sim.raster()
        assert np.array_equal(t, ot) and np.array_equal(i, oi)
        compare_state(net, sim)
        st, os_ = net.stats(), sim.stats()
        assert st.total_spikes == os_.total_spikes
        assert abs(st.rate_hz - os_.rate_hz) < 1e-9
        assert abs(st.isi_cv - os_.isi_cv) < 1e-9


@pytest.mark.parametrize("drive", [0.5, 1.5, 2.0])
def test_drive_modes(g4s, oracle, drive):
    n, nsyn, seed = 3000, 500, 4
    d = oracle.make_desc(n, nsyn, seed, drive_scale=drive)
    idx, w = oracle.conn_philox(d)
    sim = oracle.Sim(d, idx, w)
    sim.run(150, threads=8)
    with g4s.Network(n, nsyn, seed=seed, drive_scale=drive) as net:
        net.run(150, 4)
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
        compare_state(net, sim)


def test_chunked_run_matches(g4s, oracle):
    """A tiny raster budget forces many chunks; results must not change."""
    n, nsyn, seed = 2000, 200, 3
    d, (idx, w) = oracle_tables(oracle, n, nsyn, seed)
    sim = oracle.Sim(d, idx, w)
    sim.run(300, threads=8)
    for alg in (2, 4):
        with g4s.Network(n, nsyn, seed=seed, raster_budget_bytes=4 * n * 7) as net:
            net.run(300, alg)
            assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
            compare_state(net, sim)


def test_large_raster_matches_oracle(g4s, oracle):
    """N=100,000 x 1000 for 4000 steps (about 2.8 million spikes): the host files chunks of
    more than 2^20 ids on several threads and copies the raster out on several threads;
    the raster, counts and state equal the oracle's."""
    n, nsyn, seed, steps = 100_000, 1000, 2, 4000
    d, (idx, w) = oracle_tables(oracle, n, nsyn, seed)
    sim = oracle.Sim(d, idx, w)
    sim.run(steps, threads=16)
    with g4s.Network(n, nsyn, seed=seed) as net:
        net.run(steps, 4)
        t, i = net.raster()
        assert len(t) > (1 << 21)
        ot, oi = sim.raster()
        assert np.array_equal(t, ot) and np.array_equal(i, oi)
        assert np.array_equal(net.counts(), sim.counts())
        compare_state(net, sim)


@pytest.mark.parametrize("alg", [0, 1, 2, 3])
def test_host_driven_chunk_graphs(g4s, oracle, alg):
    """The host-driven schemes run their 512-step chunks as CUDA graphs, replayed for every
    chunk (the chunk's first step read from device memory): two runs of 1200 steps (captured
    chunks, replays, a last chunk launched step by step) equal the oracle's 2400 steps."""
    n, nsyn, seed = 1000, 100, 9
    d, (idx, w) = oracle_tables(oracle, n, nsyn, seed)
    sim = oracle.Sim(d, idx, w)
    sim.run(2400, threads=8)
    with g4s.Network(n, nsyn, seed=seed) as net:
        net.run(1200, alg)
        net.run(1200, alg)
        assert net.info().steps_done == 2400
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
        compare_state(net, sim)


def test_glibc_tables_on_gpu(g4s, oracle):
    n, nsyn, seed = 2500, 1000, 3
    idx, w = oracle.conn_glibc(seed, n, nsyn)
    d = oracle.make_desc(n, nsyn, seed, self_loops=1)
    sim = oracle.Sim(d, idx, w)
    sim.run(100, threads=8)
    with g4s.Network(n, nsyn, seed=seed, self_loops=True, conn_law=g4s.CONN_GLIBC) as net:
        gi, gw = net.tables()
        assert same_tables(gi, gw, idx, w)
        net.run(100, 3)
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
        compare_state(net, sim)


def test_barrier_timeout_is_reported(g4s, oracle):
    """An injected stall makes the first grid barrier wait for a block that does not exist;
    the wait runs out after the 50 ms limit, the host gets G4S_ERR_TIMEOUT and the context
    and the handle stay usable."""
    from gpu4snn_gb300 import _lib
    n, nsyn, seed = 2000, 100, 1
    with g4s.Network(n, nsyn, seed=seed) as net:
        net.set_barrier_timeout(50_000_000)
        net.inject_fault(_lib.FAULT_BARRIER_STALL)
        with pytest.raises(g4s.G4SError) as e:
            net.run(10, 4)
        assert e.value.code == _lib.ERR_TIMEOUT
        net.set_barrier_timeout(2_000_000_000)
        net.reset()
        net.run(40, 4)
        d = oracle.make_desc(n, nsyn, seed)
        idx, w = oracle.conn_philox(d)
        sim = oracle.Sim(d, idx, w)
        sim.run(40)
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))


@pytest.mark.parametrize("p,n,mode", [(1, 2500, 0), (2, 2500, 0), (3, 3001, 1), (7, 5003, 0), (152, 4099, 1),
                                      (0, 20011, 0), (0, 20011, 1), (40, 9000, 1)])
def test_owner_geometries(g4s, oracle, p, n, mode):
    """The owner-computes SKL kernel under forced geometries (one CTA, odd counts, more
    CTAs than 2048-neuron slices, slices that do not divide N) and both delivery mappings
    of a multi-CTA team, against the oracle."""
    nsyn, seed = 300, 21
    d, (idx, w) = oracle_tables(oracle, n, nsyn, seed)
    sim = oracle.Sim(d, idx, w)
    sim.run(120, threads=8)
    with g4s.Network(n, nsyn, seed=seed) as net:
        net.set_geometry(p, mode)
        gp, rc = net.geometry()
        assert (p == 0 or gp == p) and rc > 0
        net.run(70, 4)
        net.run(50, 4)
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
        compare_state(net, sim)


@pytest.mark.parametrize("n,nsyn,p,want", [(20_000, 4000, 0, 1), (20_000, 1000, 0, 0), (30_000, 600, 16, 1),
                                           (30_000, 600, 32, 0)])
def test_automatic_delivery_mapping(g4s, oracle, n, nsyn, p, want):
    """Untouched, a multi-CTA team delivers by eight-lane groups when a rank's segment of a
    row averages 24 synapses or more (Nsyn / team), else by segment runs; either way the
    raster, state and pending currents equal the oracle's."""
    seed = 29
    d, (idx, w) = oracle_tables(oracle, n, nsyn, seed)
    sim = oracle.Sim(d, idx, w)
    sim.run(60, threads=8)
    with g4s.Network(n, nsyn, seed=seed) as net:
        if p:
            net.set_geometry(p)
        gp, _ = net.geometry()
        assert gp > 1 and (p == 0 or gp == p)
        assert net.delivery() == want and (nsyn >= 24 * gp) == (want == 1)
        net.run(60, 4)
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
        compare_state(net, sim)


@pytest.mark.parametrize("n,drive,p,mode", [(100_000, 1.0, 0, 0), (50_000, 1.5, 8, 0), (50_000, 1.5, 8, 1),
                                            (300_000, 1.5, 0, 0), (3000, 1.0, 1, 0)])
def test_block_threads_768_same_results(g4s, n, drive, p, mode):
    """The 768-thread team kernel gives the 1024-thread kernel's results bit for bit in every
    delivery path: the flat mapping (N=100,000), segment runs and eight-lane groups on
    6,250-neuron slices, the dense list of large steps (N=300,000 at drive 1.5), one CTA."""
    nsyn, out = 1000, []
    for threads in (1024, 768):
        with g4s.Network(n, nsyn, seed=17, drive_scale=drive) as net:
            net.set_geometry(p, mode)
            net.set_block_threads(threads)
            assert net.block_threads() == threads
            net.run(150, 4)
            out.append((np.stack(net.raster()), net.state()["v"].view(np.uint32).copy(), net.currents()))
    (ra, va, ca), (rb, vb, cb) = out
    assert ra.shape[1] > 1000
    assert np.array_equal(ra, rb) and np.array_equal(va, vb) and np.array_equal(ca, cb)


def test_block_threads_automatic_choice(g4s):
    """Untuned, the team kernel's CTA size follows the expected synapses per CTA and step
    (N=100,000 at ~8 Hz: ~5,000, under 32,768, so 768 threads); a size that is set stays,
    0 restores the automatic choice, other sizes are refused."""
    from gpu4snn_gb300 import _lib
    with g4s.Network(100_000, 1000, seed=2, record_raster=False) as net:
        assert net.block_threads() == 768
        net.set_block_threads(1024)
        assert net.block_threads() == 1024
        net.run(20, 4)
        assert net.block_threads() == 1024
        net.set_block_threads(0)
        assert net.block_threads() == 768
        with pytest.raises(g4s.G4SError) as e:
            net.set_block_threads(512)
        assert e.value.code == _lib.ERR_INVALID


def test_upload_with_a_target_out_of_range(g4s, oracle):
    """A target >= n anywhere in a large upload (validated in parallel, block by block) is
    refused with its position, and the network keeps its tables: it still runs as before."""
    from gpu4snn_gb300 import _lib
    n, nsyn, seed = 20_000, 300, 12
    d, (idx, w) = oracle_tables(oracle, n, nsyn, seed)
    sim = oracle.Sim(d, idx, w)
    sim.run(60, threads=8)
    with g4s.Network(n, nsyn, seed=seed) as net:
        for pos in (n * nsyn - 1, 3_000_001, 5):
            bad = idx.copy()
            bad.flat[pos] = n
            bad.flat[n * nsyn - 2] = n + 7  # (a later offender: the first is reported)
            with pytest.raises(g4s.G4SError) as e:
                net.load_tables(bad, w)
            assert e.value.code == _lib.ERR_INVALID
            assert f"table entry {min(pos, n * nsyn - 2)} " in str(e.value)
        net.run(60, 4)
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))


def test_uploaded_tables_with_holes(g4s, oracle):
    """Caller tables may leave slots unused (negative target) anywhere in a row."""
    n, nsyn, seed = 3000, 200, 8
    d, (idx, w) = oracle_tables(oracle, n, nsyn, seed)
    rng = np.random.default_rng(0)
    holes = rng.random(idx.shape) < 0.1
    idx = idx.copy()
    idx[holes] = -1
    sim = oracle.Sim(d, idx, w)
    sim.run(100, threads=8)
    for alg in (2, 4):
        with g4s.Network(n, nsyn, seed=seed, tables=(idx, w)) as net:
            gi, gw = net.tables()
            valid = gi >= 0
            assert valid.sum() == (idx >= 0).sum()
            net.run(100, alg)
            assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
            compare_state(net, sim)


def test_sorted_and_shuffled_uploads_agree(g4s):
    """Rows uploaded in the device's sorted order skip the row sort; the same rows shuffled
    are sorted first.  Both give the same device tables and the same run."""
    n, nsyn, seed = 20_000, 500, 14
    with g4s.Network(n, nsyn, seed=seed) as ref:
        idx, w = ref.tables()
        ref.run(200, 4)
        t_ref, i_ref = ref.raster()
    rng = np.random.default_rng(3)
    perm = np.argsort(rng.random(idx.shape), axis=1)
    shuffled = (np.take_along_axis(idx, perm, axis=1), np.take_along_axis(w, perm, axis=1))
    assert not np.array_equal(shuffled[0], idx)
    for tabs in ((idx, w), shuffled):
        with g4s.Network(n, nsyn, seed=seed, tables=tabs) as net:
            gi, gw = net.tables()
            assert np.array_equal(gi, idx) and np.array_equal(gw.view(np.uint32), w.view(np.uint32))
            net.run(200, 4)
            t, i = net.raster()
            assert np.array_equal(t, t_ref) and np.array_equal(i, i_ref)


@pytest.mark.parametrize("p", [0, 8])
def test_weights_of_every_magnitude(g4s, oracle, p):
    """Weights spread over 2^-34 .. 2^4 (tiny ones round in Q32.32, ties included), both
    signs: the team kernel's currents and raster equal the oracle's."""
    n, nsyn, seed = 2000, 64, 12
    d, (idx, w) = oracle_tables(oracle, n, nsyn, seed)
    rng = np.random.default_rng(1)
    mag = np.ldexp(rng.uniform(1.0, 2.0, w.shape), rng.integers(-34, 4, w.shape)).astype(np.float32)
    ties = rng.random(w.shape) < 0.2  # w 2^32 = j + 1/2 exactly
    mag[ties] = np.ldexp(2.0 * rng.integers(0, 64, int(ties.sum())) + 1.0, -33).astype(np.float32)
    w = np.where(rng.random(w.shape) < 0.5, -mag, mag).astype(np.float32)
    w[idx < 0] = 0.0
    sim = oracle.Sim(d, idx, w)
    sim.run(60, threads=8)
    with g4s.Network(n, nsyn, seed=seed, tables=(idx, w)) as net:
        net.set_geometry(p, 0)
        net.run(60, 4)
        assert net.geometry()[0] >= 1  # the team kernel ran (tables within its exactness bound)
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
        compare_state(net, sim)


def test_group_delivery_dense_list(g4s, oracle):
    """The eight-lane group delivery on steps whose ids overflow the shared-memory window and
    are read, tagged, from the dense global list: 8 CTAs of 16,384 neurons (a 1,728-id
    window), segments of ~37 synapses (Nsyn 300 / 8, so the automatic choice is the groups),
    a strong drive; against the oracle."""
    n, nsyn, seed, drive, steps, p = 131_072, 300, 33, 2.0, 40, 8
    d = oracle.make_desc(n, nsyn, seed, drive_scale=drive)
    idx, w = oracle.conn_philox(d)
    sim = oracle.Sim(d, idx, w)
    sim.run(steps, threads=16)
    with g4s.Network(n, nsyn, seed=seed, drive_scale=drive) as net:
        net.set_geometry(p)
        assert net.geometry() == (p, n // p) and net.delivery() == 1
        net.run(steps, 4)
        assert sim.counts().max() > 1728  # the dense-list path runs
        assert np.array_equal(net.counts(), sim.counts())
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
        compare_state(net, sim)


def test_large_steps_dense_list(g4s, oracle):
    """Steps with more than 4096 spikes (the ids go through the dense global list instead of
    the shared-memory window) and ranks with more than 31 spikes (ids beyond the record
    lines): N=200,000 under a strong drive, against the oracle."""
    n, nsyn, seed, drive, steps = 200_000, 1000, 4, 2.0, 60
    d, (idx, w) = oracle_tables(oracle, n, nsyn, seed)
    d = oracle.make_desc(n, nsyn, seed, drive_scale=drive)
    sim = oracle.Sim(d, idx, w)
    sim.run(steps, threads=16)
    assert sim.counts().max() > 4096  # the dense-list path runs
    with g4s.Network(n, nsyn, seed=seed, drive_scale=drive) as net:
        assert net.geometry()[0] > 1
        net.run(steps, 4)
        assert np.array_equal(net.counts(), sim.counts())
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
        compare_state(net, sim)


def test_owner_large_network(g4s, oracle):
    """N=100,000, Nsyn=1000 (the scaled configuration) on the full GPU: many clusters."""
    n, nsyn, seed = 100_000, 1000, 2
    d, (idx, w) = oracle_tables(oracle, n, nsyn, seed)
    sim = oracle.Sim(d, idx, w)
    sim.run(200, threads=16)
    with g4s.Network(n, nsyn, seed=seed) as net:
        p, rc = net.geometry()
        assert p > 1
        net.run(200, 4)
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster()))
        compare_state(net, sim)


@pytest.mark.parametrize("p,delivery", [(8, 0), (8, 1), (0, 0)])
def test_team_without_interleaved_rows(g4s, p, delivery):
    """The team kernel's segment reads come from the interleaved (target, weight) rows; a
    network that finds no room for them (an allocation failure injected on the host) runs
    on the separate target and weight arrays with identical results.  8 CTAs: 6,250-neuron
    slices, segment runs (0) or eight lanes a spike (1); the default geometry adds the flat
    mapping."""
    from gpu4snn_gb300 import _lib
    n, nsyn, seed, steps = 50_000, 1000, 41, 300
    with g4s.Network(n, nsyn, seed=seed, drive_scale=1.5) as a, \
            g4s.Network(n, nsyn, seed=seed, drive_scale=1.5) as b:
        a.set_geometry(p, delivery)
        b.set_geometry(p, delivery)
        a.run(steps, 4)
        b.inject_fault(_lib.FAULT_ALLOC)  # b's first team run finds no room for the pairs
        b.run(steps, 4)
        assert a.info().device_bytes - b.info().device_bytes == n * nsyn * 8
        assert a.counts().sum() > steps * 100
        assert np.array_equal(np.stack(a.raster()), np.stack(b.raster()))
        sa, sb = a.state(), b.state()
        for k in ("v", "u"):
            assert np.array_equal(sa[k].view(np.uint32), sb[k].view(np.uint32)), k
        assert np.array_equal(a.currents(), b.currents())


def test_batch_matches_individual_runs(g4s, oracle):
    """Networks of uneven size, fan-out, seed and drive advanced together by the team
    kernel give exactly the results of each run alone (and of the oracle)."""
    specs = [(1500, 100, 31, 0.8, 120), (4000, 800, 32, 1.2, 90), (20011, 300, 33, 1.0, 60),
             (700, 699, 34, 2.0, 150), (3001, 37, 35, 0.5, 110)]
    nets = [g4s.Network(n, s, seed=sd, drive_scale=dr, raster_budget_bytes=4 * n * 64) for n, s, sd, dr, _ in specs]
    g4s.run_batch(nets, [st for *_, st in specs])
    for net, (n, nsyn, seed, drive, steps) in zip(nets, specs):
        d = oracle.make_desc(n, nsyn, seed, drive_scale=drive)
        idx, w = oracle.conn_philox(d)
        sim = oracle.Sim(d, idx, w)
        sim.run(steps, threads=8)
        assert net.info().steps_done == steps
        assert np.array_equal(np.stack(net.raster()), np.stack(sim.raster())), (n, nsyn)
        compare_state(net, sim)
        with g4s.Network(n, nsyn, seed=seed, drive_scale=drive) as alone:
            alone.run(steps, 4)
            assert np.array_equal(np.stack(alone.raster()), np.stack(net.raster()))
        net.close()
