"""Summary of an experiment sweep: the speed-up table of the reference's notebook
(`GPU4SNN - Demo Notebook.ipynb`, the cells that load `sim_overview.csv` per GPU, iteration
count, drive mode and scheme and compare the new schemes SKL and AB with the old AP, N and
S), with the standard library and numpy instead of pandas.

    python -m gpu4snn_gb300.summary <root> [--N 2500] [--Nsyn 1000] [--metric elapsedwithdata]
                                            [--modes 1 2] [--csv table.csv]

<root> holds the driver's layout `<gpu>/<iterations>/Results/N{N}Nsyn{S}Regime{mode}Alg{alg}/`
(gpu4snn.py:45-47) or directly `Results/...` (the library's g4s_run_protocol).
"""
from __future__ import annotations

import argparse
import csv
import os
import re
import sys
from dataclasses import dataclass

import numpy as np

ALG_NAMES = {0: "AP", 1: "N", 2: "S", 3: "AB", 4: "SKL"}
_DIR = re.compile(r"^N(\d+)Nsyn(\d+)Regime(\d+)Alg(\d+)$")


@dataclass
class Run:
    gpu: str
    iterations: int
    n: int
    nsyn: int
    mode: int
    alg: int
    elapsed_ms: float
    elapsedwithdata_ms: float
    spikes: int


def read_overview(path: str) -> tuple[int, float, float, int]:
    """sim_overview.csv (gpu4snn.cu:1311-1313): header `N elapsed(ms) elapsedwithdata(ms)
    totalspkcount` and one row, without a trailing newline."""
    with open(path) as f:
        lines = [l for l in f.read().splitlines() if l.strip()]
    if len(lines) < 2 or lines[0].split() != ["N", "elapsed(ms)", "elapsedwithdata(ms)", "totalspkcount"]:
        raise ValueError(f"{path}: not a sim_overview.csv")
    n, e, ewd, spk = lines[1].split()
    return int(n), float(e), float(ewd), int(spk)


def collect(root: str) -> list[Run]:
    """Every run under `root` (driver layout or a bare Results directory)."""
    runs = []
    for dirpath, dirnames, filenames in os.walk(root):
        m = _DIR.match(os.path.basename(dirpath))
        if not m or "sim_overview.csv" not in filenames:
            continue
        res = os.path.dirname(dirpath)  # .../Results
        parent = os.path.dirname(res)
        it, gpu = os.path.basename(parent), os.path.basename(os.path.dirname(parent))
        iterations = int(it) if it.isdigit() else 0
        if not it.isdigit():
            gpu = ""
        n, e, ewd, spk = read_overview(os.path.join(dirpath, "sim_overview.csv"))
        runs.append(Run(gpu, iterations, int(m.group(1)), int(m.group(2)), int(m.group(3)), int(m.group(4)), e, ewd,
                        spk))
    return sorted(runs, key=lambda r: (r.gpu, r.iterations, r.n, r.nsyn, r.mode, r.alg))


COLUMNS = ["GPU", "Iterations", "Mode", "Old Alg.", "New Alg.", "t_old", "t_new", "speed_up", "is_speed_up",
           "spikes_old", "spikes_new"]


def speedup_table(runs: list[Run], n: int = 2500, nsyn: int = 1000, metric: str = "elapsedwithdata",
                  modes=(1, 2), new=(4, 3), old=(0, 1, 2)) -> list[list]:
    """Rows of the notebook's table: for every GPU, drive mode, new scheme, old scheme and
    iteration count, t_old, t_new, speed_up = t_old / t_new and whether it exceeds 1."""
    key = "elapsedwithdata_ms" if metric == "elapsedwithdata" else "elapsed_ms"
    by = {(r.gpu, r.iterations, r.mode, r.alg): r for r in runs if r.n == n and r.nsyn == nsyn}
    gpus = sorted({g for g, _, _, _ in by})
    its = sorted({i for _, i, _, _ in by})
    rows = []
    for gpu in gpus:
        for mode in modes:
            for a_new in new:
                for a_old in old:
                    for it in its:
                        ro, rn = by.get((gpu, it, mode, a_old)), by.get((gpu, it, mode, a_new))
                        if ro is None or rn is None:
                            continue
                        t_old, t_new = getattr(ro, key), getattr(rn, key)
                        sp = t_old / t_new if t_new > 0 else float("inf")
                        rows.append([gpu, it, mode, ALG_NAMES[a_old], ALG_NAMES[a_new], t_old, t_new, sp,
                                     "Y" if sp > 1.0 else "N", ro.spikes, rn.spikes])
    return rows


def mean_speedups(rows: list[list]) -> dict[tuple[str, str], float]:
    """Geometric mean of speed_up per (new, old) scheme pair."""
    acc: dict[tuple[str, str], list[float]] = {}
    for r in rows:
        acc.setdefault((r[4], r[3]), []).append(r[7])
    return {k: float(np.exp(np.mean(np.log(v)))) for k, v in acc.items()}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("root")
    ap.add_argument("--N", type=int, default=2500)
    ap.add_argument("--Nsyn", type=int, default=1000)
    ap.add_argument("--metric", choices=["elapsed", "elapsedwithdata"], default="elapsedwithdata")
    ap.add_argument("--modes", type=int, nargs="+", default=[1, 2])
    ap.add_argument("--csv", default="")
    a = ap.parse_args(argv)
    rows = speedup_table(collect(a.root), a.N, a.Nsyn, a.metric, tuple(a.modes))
    if a.csv:
        with open(a.csv, "w", newline="") as f:
            w = csv.writer(f)
            w.writerow(COLUMNS)
            w.writerows(rows)
    print(" ".join(f"{c:>11s}" for c in COLUMNS))
    for r in rows:
        print(" ".join(f"{x:>11.3f}" if isinstance(x, float) else f"{str(x):>11s}" for x in r))
    for (new, old), g in sorted(mean_speedups(rows).items()):
        print(f"{new} over {old}: geometric-mean speed-up {g:.2f}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
