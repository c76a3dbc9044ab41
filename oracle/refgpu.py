"""The reference's own CUDA kernels on this GPU (baseline and test infrastructure only).

`make -C oracle refcubin` compiles the reference's gpu4snn.cu, unmodified, into linked
cubins (`_ref/gpu4snn_O3.cubin`, and `_ref/gpu4snn_G.cubin` with the shipped `-G -O0`
flags of the reference's makefile:16).  `_build/g4s_refgpu` (refgpu/g4s_refgpu.c, this
project's host code) loads a cubin with the driver API and runs randgeneratorinit,
initNeuron and one of the five schemes the way the reference's main does
(gpu4snn.cu:780-1300), with a fixed cuRAND seed.  Only tests and bench.py's reference legs
use this module; the product never does.
"""
from __future__ import annotations

import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN_O3 = os.path.join(HERE, "_ref", "gpu4snn_O3.cubin")
CUBIN_G = os.path.join(HERE, "_ref", "gpu4snn_G.cubin")
HARNESS = os.path.join(HERE, "_build", "g4s_refgpu")

SCHEMES = {0: "AP", 1: "N", 2: "S", 3: "AB", 4: "SKL"}


def unavailable(cubin: str = CUBIN_O3) -> str | None:
    """None when the harness and the cubin are present, else why not."""
    if not os.path.exists(cubin):
        return (f"{os.path.basename(cubin)} absent: it is built from the reference's source "
                "(make -C oracle refcubin with G4S_REFERENCE_DIR set) where that source exists")
    if not os.path.exists(HARNESS):
        return "oracle/_build/g4s_refgpu absent (make -C oracle)"
    return None


def run(idx: np.ndarray, w: np.ndarray, *, steps: int, schemes=(0, 1, 2, 3, 4), modes=(1,), seeds=(1,),
        cubin: str = CUBIN_O3, raster: bool = False, reps: int = 1, timeout: float = 1800.0) -> list[dict]:
    """Run the reference's kernels on tables idx/w ([N][Nsyn], dense rows) for every
    (scheme, mode, seed); one dict per run (see g4s_refgpu.c).  With raster=True the
    host-driven schemes copy their spike flags back every step, and each dict carries the
    run's raster as "t", "id" (int32, ordered by step then neuron)."""
    why = unavailable(cubin)
    if why:
        raise RuntimeError(why)
    n, nsyn = idx.shape
    with tempfile.TemporaryDirectory(prefix="g4s_refgpu_") as tmp:
        fi, fw = os.path.join(tmp, "idx.bin"), os.path.join(tmp, "w.bin")
        np.ascontiguousarray(idx, dtype=np.int32).tofile(fi)
        np.ascontiguousarray(w, dtype=np.float32).tofile(fw)
        cmd = [HARNESS, "--cubin", cubin, "--n", str(n), "--nsyn", str(nsyn), "--idx", fi, "--w", fw,
               "--steps", str(steps), "--reps", str(reps),
               "--schemes", ",".join(map(str, schemes)), "--modes", ",".join(map(str, modes)),
               "--seeds", ",".join(map(str, seeds))]
        prefix = os.path.join(tmp, "raster")
        if raster:
            cmd += ["--raster", prefix]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"g4s_refgpu failed ({r.returncode}): {r.stderr.strip()[-2000:]}")
        out = [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]
        for d in out:
            if "error" in d:
                continue
            path = f"{prefix}_s{d['scheme']}_m{d['mode']}_r{d['seed']}.bin"
            if raster and os.path.exists(path):
                pairs = np.fromfile(path, dtype=np.int32).reshape(-1, 2)
                d["t"], d["id"] = pairs[:, 0].copy(), pairs[:, 1].copy()
        return out


def raster_stats(t: np.ndarray, ids: np.ndarray, n: int, steps: int) -> tuple[float, float]:
    """Mean rate (Hz, 1 ms steps) and mean per-neuron ISI CV over neurons with at least two
    intervals: the definitions of the oracle's and the library's FP64 statistics."""
    rate = len(t) * 1000.0 / (n * steps)
    order = np.lexsort((t, ids))
    t, ids = t[order].astype(np.int64), ids[order]
    same = ids[1:] == ids[:-1]
    isi = (t[1:] - t[:-1])[same]
    owner = ids[1:][same]
    cnt = np.bincount(owner, minlength=n)
    s1 = np.bincount(owner, weights=isi, minlength=n)
    s2 = np.bincount(owner, weights=isi.astype(np.float64) ** 2, minlength=n)
    ok = cnt >= 2
    if not ok.any():
        return rate, 0.0
    m = cnt[ok].astype(np.float64)
    mean = s1[ok] / m
    var = (m * s2[ok] - s1[ok] ** 2) / (m * m)
    return rate, float(np.mean(np.sqrt(np.maximum(var, 0.0)) / mean))


def _fmt(x, nd=3):
    return f"{x:.{nd}f}"


def summary(seeds: int = 10) -> str:
    """Markdown summary of the reference's kernels on this GPU beside this library on the
    same tables: us per step and synaptic events/s per scheme (N=2,500 on the reference's
    own glibc tables, N=100,000 on the Philox tables of the bench's network, rows in draw
    order), at -O3 and at the shipped -G -O0, and the firing rate / ISI CV of the
    reference's kernels and of the oracle over `seeds` seeds per drive mode."""
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    from oracle import g4s_oracle as O
    import gpu4snn_gb300 as g

    lines = ["| network | scheme | build | steps | spikes | us/step | events/s |", "|---|---|---|---|---|---|---|"]
    cases = []
    idx, w = O.conn_glibc(1, 2500, 1000)
    cases.append(("N=2,500 x 1000 (glibc tables, seed 1)", idx, w, 2000, 1, True))
    d = O.make_desc(100_000, 1000, 2)
    idx5, w5 = O.conn_philox(d)
    cases.append(("N=100,000 x 1000 (Philox tables, seed 2)", idx5, w5, 1000, 2, False))
    for label, ti, tw, steps, seed, glibc in cases:
        n, nsyn = ti.shape
        for cubin, build, st in ((CUBIN_O3, "-O3", steps), (CUBIN_G, "-G -O0", steps if n <= 2500 else 200)):
            for r in run(ti, tw, steps=st, schemes=(0, 1, 2, 3, 4), modes=(1,), seeds=(7,), cubin=cubin, reps=2):
                if r["rep"] != 1:
                    continue
                us = r["ms"] * 1e3 / st
                ev = r["spikes"] * nsyn / (r["ms"] * 1e-3)
                lines.append(f"| {label} | {SCHEMES[r['scheme']]} (reference, grid {r['grid']} x {r['block']}) | {build} "
                             f"| {st} | {r['spikes']} | {_fmt(us, 2)} | {ev:.3e} |")
        with g.Network(n, nsyn, seed=seed, self_loops=glibc, tables=(ti, tw) if glibc else None,
                       record_raster=False) as net:
            for alg in (0, 1, 2, 3, 4):
                net.run(steps, alg)
                net.run(steps, alg)
                inf = net.info()
                us = inf.last_run_ms * 1e3 / steps
                ev = inf.last_run_spikes * nsyn / (inf.last_run_ms * 1e-3)
                lines.append(f"| {label} | {SCHEMES[alg]} (this library) | -O3 | {steps} | {inf.last_run_spikes} "
                             f"| {_fmt(us, 2)} | {ev:.3e} |")
    lines += ["", f"Firing rate and ISI CV, N=2,500 x 1000 on the glibc tables of seed 1, 2000 steps, {seeds} seeds "
                  "per mode (the reference: scheme S at -O3, cuRAND seeds 1..k; the oracle: FP32 mirror, seeds 1..k):",
              "", "| mode (gains) | reference rate Hz | oracle rate Hz | reference ISI CV | oracle ISI CV |",
              "|---|---|---|---|---|"]
    for mode, scale in ((0, 0.5), (1, 1.0), (2, 1.5)):
        ref = run(idx, w, steps=2000, schemes=(2,), modes=(mode,), seeds=tuple(range(1, seeds + 1)), raster=True)
        rr = np.array([raster_stats(r["t"], r["id"], 2500, 2000) for r in ref])
        oo = []
        for s in range(1, seeds + 1):
            sim = O.Sim(O.make_desc(2500, 1000, s, drive_scale=scale, self_loops=1), idx, w)
            sim.run(2000, os.cpu_count() or 1)
            st = sim.stats()
            oo.append((st.rate_hz, st.isi_cv))
        oo = np.array(oo)
        cell = lambda a: f"{a.mean():.4f} +- {a.std(ddof=1):.4f}"
        lines.append(f"| {mode} ({5 * scale:g}, {2 * scale:g}) | {cell(rr[:, 0])} | {cell(oo[:, 0])} "
                     f"| {cell(rr[:, 1])} | {cell(oo[:, 1])} |")
    return "\n".join(lines)


def summary_large(steps: int = 100, ap_steps: int = 10) -> str:
    """The same comparison at N=10^6 x 1000 (the bench's `n1m` network, balanced mode): the
    reference's five kernels at -O3 (AP for fewer steps: each spike launches a child grid of
    ceil(N / block) CTAs) and this library's SKL team on the same connectivity."""
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    from oracle import g4s_oracle as O
    import gpu4snn_gb300 as g

    n, nsyn, seed = 1_000_000, 1000, 3
    idx, w = O.conn_philox(O.make_desc(n, nsyn, seed))
    label = "N=1,000,000 x 1000 (Philox tables, seed 3)"
    lines = ["| network | scheme | build | steps | spikes | us/step | events/s |", "|---|---|---|---|---|---|---|"]
    for schemes, st in (((1, 2, 3, 4), steps), ((0,), ap_steps)):
        for r in run(idx, w, steps=st, schemes=schemes, modes=(1,), seeds=(7,), reps=2):
            if r["rep"] != 1:
                continue
            lines.append(f"| {label} | {SCHEMES[r['scheme']]} (reference, grid {r['grid']} x {r['block']}, "
                         f"pending-launch limit {r['pending_launch_limit']}) | -O3 | {st} | {r['spikes']} "
                         f"| {_fmt(r['ms'] * 1e3 / st, 2)} | {r['spikes'] * nsyn / (r['ms'] * 1e-3):.3e} |")
    del idx, w
    with g.Network(n, nsyn, seed=seed, record_raster=False) as net:
        net.run(1000, 4)
        net.run(1000, 4)
        inf = net.info()
        lines.append(f"| {label} | SKL (this library) | -O3 | 1000 | {inf.last_run_spikes} "
                     f"| {_fmt(inf.last_run_ms, 2)} | {inf.last_run_spikes * nsyn / (inf.last_run_ms * 1e-3):.3e} |")
    return "\n".join(lines)


if __name__ == "__main__":
    import sys
    print(summary_large() if sys.argv[1:] == ["large"] else summary())
