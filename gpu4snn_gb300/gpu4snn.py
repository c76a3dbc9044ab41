"""Drop-in driver for the reference's gpu4snn.py.

    python -m gpu4snn_gb300.gpu4snn <gpu_name> <iterations> [options]

As the reference (gpu4snn.py:19-47): N=2500 and Nsyn=1000 unless given, every drive
regime (0 quiet, 1 balanced, 2 irregular) and every scheme (0 AP, 1 N, 2 S, 3 AB, 4 SKL),
results in ./<gpu_name>/<iterations>/Results/N{N}Nsyn{Nsyn}Regime{m}Alg{a}/ with the
reference's five files.  Instead of `make` and a subprocess it calls libgpu4snn.so through
ctypes; pandas and matplotlib are not needed.
"""
from __future__ import annotations

import argparse
import os
import shutil
import sys

from ._lib import ALG_NAMES, CONN_GLIBC, CONN_PHILOX
from .network import run_protocol


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("gpu_name")
    ap.add_argument("iterations", type=int)
    ap.add_argument("--N", type=int, default=2500)
    ap.add_argument("--Nsyn", type=int, default=1000)
    ap.add_argument("--algorithm", default="all", help="all, AP, N, S, AB, SKL, auto or 0..5")
    ap.add_argument("--mode", default="all", help="all or 0, 1, 2")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--conn", choices=["philox", "glibc"], default="philox",
                    help="glibc: the reference's own table law (srand(seed), rand())")
    a = ap.parse_args(argv)
    alg = -1 if a.algorithm.lower() == "all" else (
        int(a.algorithm) if a.algorithm.isdigit() else ALG_NAMES[a.algorithm.upper()])
    mode = -1 if a.mode == "all" else int(a.mode)
    run_protocol(a.N, a.Nsyn, a.iterations, alg, mode, a.seed,
                 CONN_GLIBC if a.conn == "glibc" else CONN_PHILOX, ".")
    dest = os.path.join(".", a.gpu_name, str(a.iterations))
    os.makedirs(dest, exist_ok=True)
    target = os.path.join(dest, "Results")
    if os.path.isdir(target):
        for entry in os.listdir("Results"):
            src, dst = os.path.join("Results", entry), os.path.join(target, entry)
            if os.path.isdir(dst):
                shutil.rmtree(dst)
            shutil.move(src, dst)
        os.rmdir("Results")
    else:
        shutil.move("Results", target)
    return 0


if __name__ == "__main__":
    sys.exit(main())
