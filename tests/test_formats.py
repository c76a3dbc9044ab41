"""Binary raster and table files (gpu4snn_gb300.formats; the GPU writers are in
test_gpu_formats.py), and the reference's text raster format."""
from __future__ import annotations

import os
import struct

import numpy as np
import pytest

from gpu4snn_gb300 import formats as F


def _raster(seed=3, steps=57, n=400):
    rng = np.random.default_rng(seed)
    counts = rng.integers(0, 9, steps).astype(np.int32)
    ids = np.concatenate([np.sort(rng.choice(n, c, replace=False)) for c in counts]).astype(np.int32)
    return counts, ids


@pytest.mark.parametrize("chunk", [0, 1, 10, 1000])
def test_raster_round_trip(tmp_path, chunk):
    counts, ids = _raster()
    p = str(tmp_path / "r.g4s")
    F.write_raster(p, 400, counts, ids, t0=5, chunk=chunk)
    r = F.read_raster(p)
    assert r.n == 400 and r.t0 == 5 and r.complete
    assert np.array_equal(r.counts, counts) and np.array_equal(r.ids, ids)
    t = r.times()
    assert len(t) == len(ids) and t[0] >= 5 and np.all(np.diff(t) >= 0)


def test_raster_empty_and_unclosed(tmp_path):
    p = str(tmp_path / "e.g4s")
    F.write_raster(p, 10, np.zeros(0, np.int32), np.zeros(0, np.int32))
    r = F.read_raster(p)
    assert len(r.counts) == 0 and len(r.ids) == 0 and r.complete
    # a stream that was not closed: header totals still zero, chunks readable
    counts, ids = _raster(steps=8)
    F.write_raster(p, 400, counts, ids, chunk=3)
    with open(p, "r+b") as f:
        f.seek(24)
        f.write(struct.pack("<qq", 0, 0))
    r = F.read_raster(p)
    assert not r.complete and np.array_equal(r.counts, counts) and np.array_equal(r.ids, ids)


def test_raster_rejects_bad_files(tmp_path):
    p = str(tmp_path / "b.g4s")
    with open(p, "wb") as f:
        f.write(b"NOTARAST" + bytes(32))
    with pytest.raises(ValueError):
        F.read_raster(p)
    counts, ids = _raster(steps=6)
    F.write_raster(p, 400, counts, ids)
    size = os.path.getsize(p)
    with open(p, "r+b") as f:
        f.truncate(size - 4)
    with pytest.raises(ValueError):
        F.read_raster(p)
    with pytest.raises(ValueError):
        F.write_raster(p, 400, counts, ids[:-1])


def test_raster_to_text_is_the_reference_format(tmp_path):
    counts = np.array([2, 0, 1], np.int32)
    ids = np.array([3, 7, 1], np.int32)
    p, q = str(tmp_path / "r.g4s"), str(tmp_path / "spiketimes.csv")
    F.write_raster(p, 10, counts, ids)
    F.raster_to_text(F.read_raster(p), q)
    assert open(q).read() == "SpkTime NeuronID\n0 3\n0 7\n2 1\n"


def test_tables_round_trip(tmp_path, oracle):
    d = oracle.make_desc(300, 37, 9)
    idx, w = oracle.conn_philox(d)
    p = str(tmp_path / "t.g4s")
    F.write_tables(p, idx, w, nsyn=37, seed=9)
    t = F.read_tables(p)
    assert (t.n, t.nsyn, t.stride, t.seed, t.exc_permille, t.flags) == (300, 37, idx.shape[1], 9, 800, 1)
    assert np.array_equal(t.idx, idx) and np.array_equal(t.w.view(np.uint32), w.view(np.uint32))
    with open(p, "r+b") as f:
        f.truncate(os.path.getsize(p) - 8)
    with pytest.raises(ValueError):
        F.read_tables(p)
