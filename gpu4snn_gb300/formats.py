"""Readers and writers of the library's binary files (numpy only, no GPU needed).

Raster file "G4SRAS01" (written by g4s_net_stream_raster / g4s_net_write_raster_file):
    char[8] magic; int64 n; int64 first step; int64 steps; int64 spikes;
    then chunks to the end of the file: int32 cs; int32 counts[cs]; int32 ids[sum counts]
    (ids ascending within each step).
Tables file "G4STAB01" (written by g4s_net_save_tables):
    char[8] magic; int64 n; int32 nsyn; int32 stride; uint64 seed; int32 conn_law;
    int32 self_loops; int32 exc_permille; int32 flags; int32 reserved[2];
    int32 idx[n][stride]; float w[n][stride].
The reference's text raster (spiketimes.csv, gpu4snn.cu:1256-1261: header "SpkTime
NeuronID", one "t i" row per spike) is converted by `raster_to_text`.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass

import numpy as np

RASTER_MAGIC = b"G4SRAS01"
TABLES_MAGIC = b"G4STAB01"
_RASTER_HDR = struct.Struct("<8sqqqq")
_TABLES_HDR = struct.Struct("<8sqiiQiiiiii")


@dataclass
class Raster:
    n: int            # neurons of the network
    t0: int           # step of counts[0]
    counts: np.ndarray  # int32 [steps] spikes per step
    ids: np.ndarray     # int32 [spikes] neuron ids, step after step, ascending within a step
    complete: bool    # the header's totals were written (the stream was closed)

    def times(self) -> np.ndarray:
        """Step of every spike (int32), aligned with `ids`."""
        return np.repeat(np.arange(self.t0, self.t0 + len(self.counts), dtype=np.int32), self.counts)


def read_raster(path: str) -> Raster:
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < _RASTER_HDR.size:
        raise ValueError(f"{path}: not a raster file")
    magic, n, t0, steps, spikes = _RASTER_HDR.unpack_from(data, 0)
    if magic != RASTER_MAGIC:
        raise ValueError(f"{path}: not a raster file")
    counts, ids, off = [], [], _RASTER_HDR.size
    while off + 4 <= len(data):
        (cs,) = struct.unpack_from("<i", data, off)
        off += 4
        if cs < 0 or off + 4 * cs > len(data):
            raise ValueError(f"{path}: truncated chunk")
        c = np.frombuffer(data, dtype="<i4", count=cs, offset=off)
        off += 4 * cs
        k = int(c.sum())
        if off + 4 * k > len(data):
            raise ValueError(f"{path}: truncated chunk")
        counts.append(c)
        ids.append(np.frombuffer(data, dtype="<i4", count=k, offset=off))
        off += 4 * k
    counts = np.concatenate(counts).astype(np.int32) if counts else np.zeros(0, np.int32)
    ids = np.concatenate(ids).astype(np.int32) if ids else np.zeros(0, np.int32)
    complete = steps == len(counts) and spikes == len(ids)
    if (steps or spikes) and not complete:
        raise ValueError(f"{path}: header totals ({steps} steps, {spikes} spikes) disagree with the chunks")
    return Raster(int(n), int(t0), counts, ids, complete)


def write_raster(path: str, n: int, counts, ids, t0: int = 0, chunk: int = 0) -> None:
    """Write a raster file (one chunk, or chunks of `chunk` steps)."""
    counts = np.ascontiguousarray(counts, dtype="<i4")
    ids = np.ascontiguousarray(ids, dtype="<i4")
    if int(counts.sum()) != len(ids):
        raise ValueError("counts do not add up to the ids")
    with open(path, "wb") as f:
        f.write(_RASTER_HDR.pack(RASTER_MAGIC, n, t0, len(counts), len(ids)))
        step = chunk or max(1, len(counts))
        pos = 0
        for s0 in range(0, len(counts), step):
            c = counts[s0:s0 + step]
            k = int(c.sum())
            f.write(struct.pack("<i", len(c)))
            f.write(c.tobytes())
            f.write(ids[pos:pos + k].tobytes())
            pos += k


def raster_to_text(r: Raster, path: str) -> None:
    """The reference's spiketimes.csv: header "SpkTime NeuronID", one "t i" row per spike."""
    t = r.times()
    with open(path, "w") as f:
        f.write("SpkTime NeuronID\n")
        for a, b in zip(t.tolist(), r.ids.tolist()):
            f.write(f"{a} {b}\n")


@dataclass
class Tables:
    n: int
    nsyn: int
    stride: int
    seed: int
    conn_law: int
    self_loops: int
    exc_permille: int
    flags: int
    idx: np.ndarray  # int32 [n][stride]
    w: np.ndarray    # float32 [n][stride]


def read_tables(path: str) -> Tables:
    with open(path, "rb") as f:
        hdr = f.read(_TABLES_HDR.size)
        if len(hdr) < _TABLES_HDR.size:
            raise ValueError(f"{path}: not a tables file")
        magic, n, nsyn, stride, seed, law, loops, exc, flags, _, _ = _TABLES_HDR.unpack(hdr)
        if magic != TABLES_MAGIC or n < 1 or nsyn < 1 or stride < nsyn or stride % 4:
            raise ValueError(f"{path}: not a tables file")
        cnt = n * stride
        idx = np.fromfile(f, dtype="<i4", count=cnt)
        w = np.fromfile(f, dtype="<f4", count=cnt)
    if idx.size != cnt or w.size != cnt:
        raise ValueError(f"{path}: truncated tables file")
    return Tables(n, nsyn, stride, seed, law, loops, exc, flags, idx.reshape(n, stride), w.reshape(n, stride))


def write_tables(path: str, idx: np.ndarray, w: np.ndarray, nsyn: int, seed: int = 0, conn_law: int = 0,
                 self_loops: int = 0, exc_permille: int = 800, sorted_rows: bool = True) -> None:
    idx = np.ascontiguousarray(idx, dtype="<i4")
    w = np.ascontiguousarray(w, dtype="<f4")
    n, stride = idx.shape
    if w.shape != idx.shape or stride % 4 or stride < nsyn:
        raise ValueError("tables must be [n][stride] with stride a multiple of 4 and >= nsyn")
    with open(path, "wb") as f:
        f.write(_TABLES_HDR.pack(TABLES_MAGIC, n, nsyn, stride, seed, conn_law, self_loops, exc_permille,
                                 1 if sorted_rows else 0, 0, 0))
        f.write(idx.tobytes())
        f.write(w.tobytes())


__all__ = ["Raster", "Tables", "read_raster", "write_raster", "raster_to_text", "read_tables", "write_tables"]
