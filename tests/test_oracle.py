"""CPU tests of the oracle: pinned against numpy's Philox and the reference's own tables,
plus the statistical and structural properties the reference's algorithm implies."""
import hashlib
import json
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _plus(ctr, k):
    """counter + k as a 256-bit little-endian number of four 64-bit words"""
    v = sum(int(c) << (64 * i) for i, c in enumerate(ctr)) + k
    v %= 1 << 256
    return [(v >> (64 * i)) & (2**64 - 1) for i in range(4)]


def test_philox_known_answers(oracle):
    for case in _load("philox_kat.json"):
        key = [int(k) for k in case["key"]]
        ctr = [int(c) for c in case["counter"]]
        for k, block in enumerate(case["blocks"]):
            got = oracle.philox4x64_10(_plus(ctr, k + 1), key)
            assert [int(x) for x in got] == [int(b) for b in block]


def test_philox_matches_numpy_live(oracle):
    rng = np.random.default_rng(5)
    for _ in range(50):
        key = [int(x) for x in rng.integers(0, 2**63, 2)]
        ctr = [int(x) for x in rng.integers(0, 2**63, 4)]
        ref = np.random.Philox(counter=np.array(ctr, dtype=np.uint64), key=np.array(key, dtype=np.uint64)).random_raw(4)
        assert [int(x) for x in oracle.philox4x64_10(_plus(ctr, 1), key)] == [int(x) for x in ref]


def test_philox4x32_known_answers(oracle):
    """Block k of the cuRAND host Philox4x32-10 generator with seed s is the function at
    counter (0, 0, k, 0) and key (s low word, s high word)."""
    for case in _load("philox4x32_kat.json"):
        s = int(case["seed"])
        key = [s & 0xFFFFFFFF, s >> 32]
        for k, block in enumerate(case["blocks"]):
            assert [int(x) for x in oracle.philox4x32_10([0, 0, k, 0], key)] == block


def test_log_accuracy(oracle):
    xs = np.concatenate([np.random.default_rng(0).random(20000), np.geomspace(1e-30, 1.0, 2000, endpoint=False)])
    xs = xs[xs > 0].astype(np.float32)
    for x in xs:
        ref = math.log(float(x))
        got = oracle.logf(float(x))
        assert abs(got - ref) <= 2.5e-7 * max(1.0, abs(ref)), (x, got, ref)


def test_normal_distribution(oracle):
    z = np.array([oracle.normal(3, i, t) for i in range(400) for t in range(100)])
    assert abs(z.mean()) < 0.02
    assert abs(z.std() - 1.0) < 0.02
    assert abs(((z - z.mean()) ** 4).mean() / z.var() ** 2 - 3.0) < 0.15
    # Kolmogorov-Smirnov distance against the normal CDF
    zs = np.sort(z)
    cdf = 0.5 * (1 + np.vectorize(math.erf)(zs / math.sqrt(2)))
    ks = np.max(np.abs(cdf - np.arange(1, len(zs) + 1) / len(zs)))
    assert ks < 1.63 / math.sqrt(len(zs))  # 1% level


@pytest.mark.parametrize("n,nsyn,seed,self_loops", [(2500, 1000, 1, 0), (500, 499, 2, 0), (64, 64, 3, 1),
                                                    (1000, 37, 4, 0)])
def test_philox_tables_structure(oracle, n, nsyn, seed, self_loops):
    d = oracle.make_desc(n, nsyn, seed, self_loops=self_loops)
    idx, w = oracle.conn_philox(d)
    stride = d.stride
    assert idx.shape == (n, stride)
    body = idx[:, :nsyn]
    assert body.min() >= 0 and body.max() < n
    assert (idx[:, nsyn:] == -1).all() and (w[:, nsyn:] == 0).all()
    s = np.sort(body, axis=1)
    assert (np.diff(s, axis=1) > 0).all(), "targets of a row must be distinct"
    if not self_loops:
        assert not (body == np.arange(n)[:, None]).any()
    nexc = n * 4 // 5
    scale = np.float32(1000.0) / np.float32(nsyn)
    assert (w[:nexc, :nsyn] >= 0).all() and (w[:nexc, :nsyn] < scale * 0.5).all()
    assert (w[nexc:, :nsyn] <= 0).all() and (w[nexc:, :nsyn] > -scale).all()


def test_philox_tables_uniform_targets(oracle):
    n, nsyn = 2000, 500
    idx, _ = oracle.conn_philox(oracle.make_desc(n, nsyn, 8))
    indeg = np.bincount(idx.ravel(), minlength=n)
    # in-degree ~ Binomial(n-1, nsyn/(n-1)): mean nsyn, var ~ nsyn (1 - nsyn/(n-1))
    assert abs(indeg.mean() - nsyn) < 1e-9
    assert 0.8 < indeg.var() / (nsyn * (1 - nsyn / (n - 1))) < 1.2


def test_tables_rows_are_independent(oracle):
    d = oracle.make_desc(3000, 100, 6)
    idx, w = oracle.conn_philox(d)
    i2, w2 = oracle.conn_philox(d, 1234, 10)
    assert np.array_equal(idx[1234:1244], i2) and np.array_equal(w[1234:1244], w2)


@pytest.mark.parametrize("fn", ["ref_tables_N20_S5_seed7.npz", "ref_tables_N200_S50_seed3.npz",
                                "ref_tables_N101_S101_seed11.npz"])
def test_glibc_tables_match_reference(oracle, fn):
    """The oracle's restatement of gpu4snn.cu:873-898 reproduces the reference's own tables."""
    g = np.load(os.path.join(GOLDEN, fn))
    n, nsyn = g["idx"].shape
    seed = int(fn.split("seed")[1].split(".")[0])
    idx, w = oracle.conn_glibc(seed, n, nsyn)
    assert np.array_equal(idx, g["idx"])
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))


def test_glibc_tables_match_reference_digest(oracle):
    for rec in _load("ref_tables_digest.json"):
        idx, w = oracle.conn_glibc(rec["seed"], rec["n"], rec["nsyn"])
        assert _digest(idx, w) == rec["sha256"]
        assert idx[0, :16].tolist() == rec["row0_idx"]


def test_oracle_regression_record(oracle):
    rec = _load("oracle_small.json")
    d = oracle.make_desc(rec["n"], rec["nsyn"], rec["seed"])
    idx, w = oracle.conn_philox(d)
    assert _digest(idx, w) == rec["tables_sha256"]
    sim = oracle.Sim(d, idx, w)
    sim.run(rec["steps"])
    t, i = sim.raster()
    assert len(t) == rec["spikes"] and _digest(t, i) == rec["raster_sha256"]
    assert _digest(sim.state()["v"]) == rec["v_sha256"]


def test_openmp_equals_serial(oracle):
    d = oracle.make_desc(3000, 300, 12, drive_scale=1.5)
    idx, w = oracle.conn_philox(d)
    a, b = oracle.Sim(d, idx, w), oracle.Sim(d, idx, w)
    a.run(150, threads=1)
    b.run(150, threads=4)
    assert np.array_equal(np.stack(a.raster()), np.stack(b.raster()))
    assert np.array_equal(a.acc(), b.acc())
    assert np.array_equal(a.state()["u"].view(np.uint32), b.state()["u"].view(np.uint32))


def test_fixed_point_is_order_independent(oracle):
    """Q32.32 sums of the weights of a row do not depend on the summation order."""
    d = oracle.make_desc(500, 200, 2)
    _, w = oracle.conn_philox(d)
    q = np.array([oracle.wfix(float(x)) for x in w[7, :200]], dtype=np.int64)
    perm = np.random.default_rng(1).permutation(200)
    assert int(q.sum()) == int(q[perm].sum())
    assert all(q[j] == np.int64(np.rint(np.float64(w[7, j]) * 2**32)) for j in range(200))


@pytest.mark.parametrize("drive,min_identical", [(0.5, 200), (1.0, 60), (1.5, 95)])
def test_fp32_against_fp64(oracle, drive, min_identical):
    """FP32 mirror vs the FP64 oracle, N=2500, Nsyn=1000, seed 1, in lockstep.  The rasters
    are identical for the first `min_identical` steps (all 200 in the quiet regime; the
    balanced and irregular regimes are chaotic and separate at steps 67 and 100); until
    then the median |v32 - v64| stays below 1e-4 mV at every step.  Neurons on the upswing
    to threshold amplify the rounding difference, so the tail (p99.9) is larger."""
    d = oracle.make_desc(2500, 1000, 1, drive_scale=drive)
    idx, w = oracle.conn_philox(d)
    s32, s64 = oracle.Sim(d, idx, w, oracle.FP32), oracle.Sim(d, idx, w, oracle.FP64)
    for step in range(min_identical):
        s32.run(1)
        s64.run(1)
        v64, _ = s64.state64()
        dv = np.abs(s32.state()["v"].astype(np.float64) - v64)
        assert np.median(dv) < 1e-4, (step, np.median(dv))
    assert np.array_equal(np.stack(s32.raster()), np.stack(s64.raster()))


def test_rate_and_isi_agree_fp32_fp64_full_run(oracle):
    """Long runs are chaotic, so FP32 and FP64 trajectories separate; firing rate and ISI CV
    of the 2000-step N=2500 run must agree within 1%."""
    d = oracle.make_desc(2500, 1000, 1)
    idx, w = oracle.conn_philox(d)
    s32, s64 = oracle.Sim(d, idx, w, oracle.FP32), oracle.Sim(d, idx, w, oracle.FP64)
    s32.run(2000, threads=4)
    s64.run(2000)
    a, b = s32.stats(), s64.stats()
    assert abs(a.rate_hz - b.rate_hz) / b.rate_hz < 0.01
    assert abs(a.isi_cv - b.isi_cv) / b.isi_cv < 0.01


def test_sort_rows_matches_numpy_order(oracle):
    """The oracle's parallel radix row sort puts every row in the library's order: target as
    unsigned (so padding, -1, last), equal targets by weight bits; generated rows (distinct
    targets, padded stride) and rows with repeated targets and negative weights alike."""
    rng = np.random.default_rng(3)
    d = oracle.make_desc(700, 37, 9)  # stride 40: three padding slots a row
    idx, w = oracle.conn_philox(d)
    rep_i = rng.integers(0, 50, size=(300, 64)).astype(np.int32)
    rep_i[:, -5:] = -1
    rep_w = rng.standard_normal((300, 64)).astype(np.float32)
    for ti, tw in ((idx, w), (rep_i, rep_w)):
        key = (ti.view(np.uint32).astype(np.uint64) << np.uint64(32)) | tw.view(np.uint32).astype(np.uint64)
        order = np.argsort(key, axis=1, kind="stable")
        want_i, want_w = np.take_along_axis(ti, order, 1), np.take_along_axis(tw, order, 1)
        gi, gw = ti.copy(), tw.copy()
        oracle.sort_rows(gi, gw)
        assert np.array_equal(gi, want_i) and np.array_equal(gw.view(np.uint32), want_w.view(np.uint32))
