"""Multi-process paths of bench.py on the CPU (gloo, world size 2).

The simulation step does not shard: `bench.py --gpus N` runs N independent replicas whose
only communication is the host-side reduction of the timing (max over ranks) and of the
events (sum), and the reference arm prints from rank 0 alone.  Both are exercised here with
two ranks over gloo on 127.0.0.1, no GPU.
"""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_ranks(argv: list[str], world: int = 2, timeout: int = 240) -> list[subprocess.CompletedProcess]:
    port = _free_port()
    procs = []
    for rank in range(world):
        env = dict(os.environ, WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen(argv, cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                      text=True))
    out = []
    for p in procs:
        o, e = p.communicate(timeout=timeout)
        out.append(subprocess.CompletedProcess(p.args, p.returncode, o, e))
    return out


def test_reductions_over_two_ranks():
    snippet = (
        "import json, sys; sys.path.insert(0, '.'); import bench\n"
        "ws, rank, local, pg = bench.dist_setup()\n"
        "mx = bench.reduce_max(pg, 1.5 + rank)\n"
        "sm = bench.reduce_sum(pg, 10.0 * (rank + 1))\n"
        "print(json.dumps({'ws': ws, 'rank': rank, 'max': mx, 'sum': sm}))\n"
    )
    res = _run_ranks([sys.executable, "-c", snippet])
    for r in res:
        assert r.returncode == 0, r.stderr
    got = sorted((json.loads(r.stdout.strip().splitlines()[-1]) for r in res), key=lambda d: d["rank"])
    assert [d["rank"] for d in got] == [0, 1]
    for d in got:
        assert d["ws"] == 2
        assert d["max"] == 2.5  # the slowest rank's time
        assert d["sum"] == 30.0  # all ranks' events


def test_reference_arm_prints_from_rank_zero_only():
    res = _run_ranks([sys.executable, "bench.py", "--impl", "reference", "--workload", "n2500", "--steps", "1",
                      "--warmup", "3"])
    for r in res:
        assert r.returncode == 0, r.stderr
    lines0 = [l for l in res[0].stdout.splitlines() if l.strip()]
    assert len(lines0) == 1
    line = json.loads(lines0[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    assert res[1].stdout.strip() == ""


def test_reference_arm_at_another_drive():
    """`--drive` replaces the workload's drive scale: the line's config says so, and the quiet
    regime (0.5) fires far less than the balanced one on the same network."""
    rates = {}
    for drive in ("0.5", "1.0"):
        r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "n2500", "--drive", drive,
                            "--steps", "1", "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=240)
        assert r.returncode == 0, r.stderr
        line = json.loads([l for l in r.stdout.splitlines() if l.strip()][-1])
        assert line["config"]["drive_scale"] == float(drive)
        rates[drive] = line["value"]
    assert rates["0.5"] < 0.1 * rates["1.0"]
