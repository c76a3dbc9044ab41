"""The oracle's step pinned to the reference's own CUDA kernels run on this GPU.

The reference seeds cuRAND and glibc from time(NULL) (gpu4snn.cu:841, 873) and ships no
tests or golden outputs, so its update and drive can only be pinned statistically.  These
tests run its kernels (gpu4snn.cu compiled unmodified into a cubin by `make -C oracle
refcubin`, driven by oracle/refgpu/g4s_refgpu.c with fixed cuRAND seeds) on the
reference's own tables (its glibc law, reproduced bit for bit by the oracle), and compare
firing rate and mean ISI CV with the oracle's FP32 mirror over ten seeds per drive mode
(gains 2.5/1, 5/2, 7.5/3: the reference's modes 0, 1, 2, gpu4snn.cu:362-374).

Criterion: for each mode and statistic, the two means agree within 3.5 standard errors of
their difference (seed-to-seed spread of each side over its seeds), and every oracle seed
lies within four standard deviations of the reference's seed mean.  Both are tests that
the oracle and the reference draw from the same distribution: their seeds are unrelated
(Philox against cuRAND XORWOW streams), so no tighter comparison exists.
"""
import os
import subprocess

import numpy as np
import pytest

N, NSYN, STEPS, SEEDS = 2500, 1000, 2000, 10
MODES = ((0, 0.5), (1, 1.0), (2, 1.5))


@pytest.fixture(scope="module")
def refgpu(oracle):
    from oracle import refgpu as R
    why = R.unavailable()
    if why:
        pytest.skip(why)
    return R


@pytest.fixture(scope="module")
def glibc_tables(oracle):
    return oracle.conn_glibc(1, N, NSYN)


@pytest.mark.gpu
@pytest.mark.parametrize("mode,scale", MODES)
def test_oracle_rate_and_isi_within_reference_spread(oracle, refgpu, glibc_tables, mode, scale):
    idx, w = glibc_tables
    ref = refgpu.run(idx, w, steps=STEPS, schemes=(2,), modes=(mode,), seeds=tuple(range(1, SEEDS + 1)), raster=True)
    assert len(ref) == SEEDS and all(len(r["t"]) == r["spikes"] for r in ref)
    rr = np.array([refgpu.raster_stats(r["t"], r["id"], N, STEPS) for r in ref])
    oo = []
    for s in range(1, SEEDS + 1):
        sim = oracle.Sim(oracle.make_desc(N, NSYN, s, drive_scale=scale, self_loops=1), idx, w)
        sim.run(STEPS, os.cpu_count() or 1)
        st = sim.stats()
        oo.append((st.rate_hz, st.isi_cv))
    oo = np.array(oo)
    for k, name in enumerate(("rate", "ISI CV")):
        mr, sr = rr[:, k].mean(), rr[:, k].std(ddof=1)
        mo, so = oo[:, k].mean(), oo[:, k].std(ddof=1)
        se = np.sqrt(sr ** 2 / SEEDS + so ** 2 / SEEDS)
        print(f"mode {mode} {name}: reference {mr:.4f} +- {sr:.4f}, oracle {mo:.4f} +- {so:.4f}")
        assert abs(mo - mr) <= 3.5 * se, (mode, name, mr, sr, mo, so)
        assert np.all(np.abs(oo[:, k] - mr) <= 4 * sr), (mode, name, oo[:, k], mr, sr)


@pytest.mark.gpu
def test_reference_schemes_agree_with_each_other(oracle, refgpu, glibc_tables):
    """The harness runs each of the reference's five schemes on the same seed: the same
    parameters and drive, so the totals differ only by float-atomic order (and the AP
    scheme's own race, gpu4snn.cu:409), far inside the seed-to-seed spread."""
    idx, w = glibc_tables
    res = refgpu.run(idx, w, steps=STEPS, schemes=(0, 1, 2, 3, 4), modes=(1,), seeds=(3,))
    tot = np.array([r["spikes"] for r in res], dtype=float)
    assert len(tot) == 5
    assert res[4]["skl_total"] == res[4]["spikes"]
    # balanced mode: ~7.3 Hz, i.e. ~36,500 spikes; the seed-to-seed sd is ~0.06 Hz (~300)
    assert tot.max() - tot.min() < 0.02 * tot.mean(), tot
    assert 6.5 < tot.mean() * 1000.0 / (N * STEPS) < 8.0


@pytest.mark.gpu
def test_reference_refuses_int_overflow(oracle):
    """N x Nsyn >= 2^31 overflows the reference's int synapse indices (gpu4snn.cu:460, 569,
    692, 767): the harness refuses it before it opens a file or touches the GPU."""
    from oracle import refgpu
    r = subprocess.run([refgpu.HARNESS, "--cubin", refgpu.CUBIN_O3, "--n", "250000", "--nsyn", "10000",
                        "--idx", "/dev/null", "--w", "/dev/null", "--steps", "1"], capture_output=True, text=True)
    assert r.returncode == 0 and "cannot run" in r.stdout
