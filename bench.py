"""Benchmark of the GPU4SNN simulation step on GB300 (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Workload (default "n100k"): one randomly connected Izhikevich network, N=100,000 neurons,
Nsyn=1000 distinct targets each (1e8 synapses, int32 target + fp32 weight = 0.8 GB), the
balanced drive (gains 5 and 2), seed 2.  One bench step is one 10,000-step simulation
(10 s of model time).  The tables (0.8 GB) are larger than L2 (129 MB) and are streamed
from HBM every step, so no L2 flush is needed between bench steps.

Metric: synaptic events/s = sum over steps of spikes x Nsyn, divided by the device time of
the runs (CUDA events on the library's launching stream).  `roofline` reports the
persistent step kernel against the measured HBM copy bandwidth; `e2e` is the same metric
through the C ABI with host tables uploaded from pinned memory, a reset, the run and the
raster read back, every step.  `cpu_baseline` is the oracle's OpenMP port on the host cores.

`reference_gpu`: the reference's own CUDA kernels (gpu4snn.cu compiled unmodified for
sm_103a into a cubin, driven by this project's harness oracle/refgpu/g4s_refgpu.c) on the
same network's connectivity and drive mode, each of its five schemes timed with CUDA
events, and the headline's speed-up over its best scheme.  `large`: the N=10^6 x 1000 and
N=250,000 x 10,000 networks, each timed like the headline (its own roofline, clocks and
DRAM traffic).  `e2e` runs as many steps as the timed leg.

--impl reference times the reference's algorithm on the CPU (the oracle's OpenMP port of
gpu4snn.cu's step, all host threads) on the same network: the reference has no CPU
implementation of the step (its kernels' GPU timings are the `reference_gpu` block).

Multi-GPU: the path does not shard; `--gpus N` under torchrun runs N independent replicas
(seed + rank), value = all ranks' events / the slowest rank's time ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (N, Nsyn, sim steps per bench step, drive scale, seed)
    "n100k": (100_000, 1000, 10_000, 1.0, 2),
    "n1m": (1_000_000, 1000, 1000, 1.0, 3),
    "n250k_s10k": (250_000, 10_000, 500, 1.0, 4),
    "n2500": (2500, 1000, 2000, 1.0, 1),
    "n25k": (25_000, 1000, 500, 1.0, 5),  # small profiling case: 0.2 GB of tables, still > L2
    "n300k": (300_000, 1000, 50, 1.0, 6),  # profiling case for large-N delivery: 2.4 GB of tables
    "n100k_200": (100_000, 1000, 200, 1.0, 2),  # profiling case: the N=100,000 network, 200-step launches
    "n30k_s4k": (30_000, 4000, 100, 1.0, 7),  # profiling case for long segments (~26 synapses a rank, the
                                              # eight-lane group delivery): 1.9 GB of tables with their copy
    "n25k_s10k": (25_000, 10_000, 50, 1.0, 8),  # profiling case with the segment length of N=250,000 x
                                                # 10,000 (~66 synapses a rank): 4 GB of tables with their copy
}
# algorithmic bytes: delivery = spikes x Nsyn x (4 B target + 4 B weight) and the spike
# statistics (32 B read + 32 B written per spike); the neuron state (v,u read + write 16 B
# and the parameter r 4 B per neuron and step, a,b,c,d being recomputed from r; the currents
# stay in shared memory) only when it is not kept on chip: the team kernel holds slices of
# up to RESIDENT_SLICE neurons in shared memory for a whole launch
UPDATE_BYTES_PER_NEURON = 20
STAT_BYTES_PER_SPIKE = 64
RESIDENT_SLICE = 2048


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.path = tempfile.mktemp(prefix="g4s_clocks_", suffix=".csv")
        self.proc = None

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        # the timed region starts once the sampler has written its first sample, so that its
        # start-up (loading the management library) stays out of it (once, on a fresh host, a
        # lone timed launch that began with the sampler's start-up measured 30 times its
        # usual time)
        t0 = time.perf_counter()
        while self.proc and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return None
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return ws, rank, local, pg


def reduce_max(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def cpu_port_rate(n, nsyn, seed, drive, threads, min_seconds, max_steps, warm_steps):
    """Events/s of the oracle's OpenMP port on a bounded sample of the workload."""
    from oracle import g4s_oracle as O
    d = O.make_desc(n, nsyn, seed, drive_scale=drive)
    idx, w = O.conn_philox(d)
    sim = O.Sim(d, idx, w)
    sim.run(warm_steps, threads=threads)
    spikes0, steps, t0 = len(sim.raster()[0]), 0, time.perf_counter()
    while steps < max_steps and time.perf_counter() - t0 < min_seconds:
        sim.run(25, threads=threads)
        steps += 25
    dt = time.perf_counter() - t0
    ev = (len(sim.raster()[0]) - spikes0) * nsyn
    return ev / dt, steps, dt


def run_reference(a, cfg, ws, rank, pg):
    if rank != 0:
        return 0
    n, nsyn, T, drive, seed = cfg
    threads = os.cpu_count() or 1
    from oracle import g4s_oracle as O
    O.build()
    d = O.make_desc(n, nsyn, seed, drive_scale=drive)
    idx, w = O.conn_philox(d)
    sim = O.Sim(d, idx, w)
    per = max(1, min(T, 100))
    for _ in range(a.warmup):
        sim.run(per, threads=threads)
    s0 = len(sim.raster()[0])
    t0 = time.perf_counter()
    for _ in range(a.steps):
        sim.run(per, threads=threads)
    dt = time.perf_counter() - t0
    ev = (len(sim.raster()[0]) - s0) * nsyn
    v = ev / dt
    sample = (f"{a.steps} x {per} simulation steps (after {a.warmup} x {per} warm-up) of the N={n}, Nsyn={nsyn} "
              f"network, oracle OpenMP port, {threads} threads")
    line = {"impl": "reference", "metric": "synaptic events/s", "value": v, "unit": "events/s", "n_gpus": ws,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": dt * 1e3 / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic (seeded Philox network)",
            "config": workload_config(a.workload, cfg),
            "cpu_baseline": {"value": v, "unit": "events/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def workload_config(name, cfg):
    n, nsyn, T, drive, seed = cfg
    return {"workload": name, "N": n, "Nsyn": nsyn, "sim_steps_per_bench_step": T, "drive_scale": drive,
            "seed": seed, "synapses": n * nsyn, "table_bytes": n * ((nsyn + 3) // 4 * 4) * 8,
            "l2": "tables larger than L2 (129 MB), streamed from HBM every step; no flush",
            "parallelism": "replicas"}


ALG_LABEL = {0: "AP", 1: "N", 2: "S", 3: "AB", 4: "SKL", 5: "AUTO"}


def schemes_leg(g, net, nsyn, steps):
    """Each of the five schemes on the same network for `steps` steps, after a warm-up run
    of the same length (which also captures the host-driven schemes' chunk graphs; the
    simulation continues from one run to the next; the dynamics are stationary)."""
    out = {}
    for alg in (0, 1, 2, 3, 4):
        net.run(steps, alg)
        net.run(steps, alg)
        inf = net.info()
        out[ALG_LABEL[alg]] = {"events_per_s": inf.last_run_spikes * nsyn / (inf.last_run_ms * 1e-3),
                               "us_per_step": inf.last_run_ms * 1e3 / steps, "steps": steps}
    return out


def ensemble(count, seed=5):
    """The batched ensemble: N log-uniform in [1e3, 5e4], Nsyn uniform in [100, 2000]
    (at most N-1), drive scale U(0.5, 2), steps uniform in [1000, 5000], own seeds."""
    import numpy as np
    rng = np.random.default_rng(seed)
    N = np.exp(rng.uniform(np.log(1000), np.log(50000), count)).astype(int)
    S = np.minimum(rng.integers(100, 2001, count), N - 1)
    D = rng.uniform(0.5, 2.0, count)
    T = rng.integers(1000, 5001, count)
    seeds = rng.integers(1, 2**62, count)
    return N, S, D, T, seeds


def batched_leg(g, count):
    """All networks in shared persistent launches vs one network per launch, in turn."""
    N, S, D, T, seeds = ensemble(count)
    nets = [g.Network(int(n), int(s), seed=int(sd), drive_scale=float(d), record_raster=False)
            for n, s, sd, d in zip(N, S, seeds, D)]
    g.run_batch(nets, T.tolist())  # warm-up
    for x in nets:
        x.reset()
    t0 = time.perf_counter()
    ms, launches = g.run_batch(nets, T.tolist())
    wall = time.perf_counter() - t0
    ev = sum(x.info().last_run_spikes * int(s) for x, s in zip(nets, S))
    counts_b = [x.info().last_run_spikes for x in nets]
    for x in nets:
        x.reset()
    p_ms, p_ev = 0.0, 0
    for x, t, s in zip(nets, T, S):
        x.run(int(t), g.ALG_AUTO)
        inf = x.info()
        p_ms += inf.last_run_ms
        p_ev += inf.last_run_spikes * int(s)
    same = counts_b == [x.info().last_run_spikes for x in nets]
    for x in nets:
        x.close()
    return {"networks": count, "synapses": int((N * S).sum()), "launches": int(launches),
            "device_ms": ms, "wall_ms": wall * 1e3, "sims_per_s": count / (ms * 1e-3), "events_per_s": ev / (ms * 1e-3),
            "plain_device_ms": p_ms, "plain_sims_per_s": count / (p_ms * 1e-3),
            "plain_events_per_s": p_ev / (p_ms * 1e-3), "speedup_vs_plain": p_ms / ms,
            "identical_spike_counts": same,
            "workload": "N log-U[1e3,5e4], Nsyn U[100,2000] (<= N-1), drive U(0.5,2), steps U[1000,5000], seed 5"}


def served_leg(g, count, lams):
    """Poisson arrivals of simulation requests to the continuous-batching server (150 GB
    budget), against serving the same requests one network per launch, in turn."""
    import numpy as np
    from gpu4snn_gb300.server import Server
    rng = np.random.default_rng(6)
    N = np.exp(rng.uniform(np.log(1e3), np.log(2e5), count)).astype(int)
    S = np.minimum(rng.integers(100, 2001, count), N - 1)
    T = np.exp(rng.uniform(np.log(500), np.log(2e4), count)).astype(int)
    D = rng.uniform(0.5, 2.0, count)
    seeds = rng.integers(1, 2**62, count)
    out = {"requests": count, "workload": "N log-U[1e3,2e5], Nsyn U[100,2000] (<= N-1), steps log-U[500,2e4], "
                                          "drive U(0.5,2), seed 6; budget 150 GB, quantum 250 steps"}
    for lam in lams:
        gaps = rng.exponential(1.0 / lam, count)
        with Server(hbm_budget_bytes=150 << 30, quantum=250) as srv:
            t0 = time.perf_counter()
            for k in range(count):
                while time.perf_counter() - t0 < gaps[:k + 1].sum():
                    time.sleep(0.0002)
                srv.submit(int(N[k]), int(S[k]), int(T[k]), int(seeds[k]), float(D[k]))
            res = {}
            while len(res) < count:
                for r in srv.poll():
                    res[r.id] = r
                time.sleep(0.001)
            wall = time.perf_counter() - t0
            st = srv.stats()
        lat = np.array([r.latency_ms for r in res.values()])
        out[f"lambda_{lam:g}"] = {"req_per_s": count / wall, "events_per_s": st.events / wall,
                                  "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                                  "rounds": int(st.rounds), "gpu_busy_ms": st.busy_ms, "wall_ms": wall * 1e3,
                                  "peak_gib": st.peak_bytes / 2**30, "failed": int(sum(r.status != 0 for r in res.values()))}
        last = [res[k + 1] for k in range(count)]  # ids are 1.. in submission order
    t0 = time.perf_counter()
    lat, alone_ms = [], []
    for k in range(count):
        ts = time.perf_counter()
        with g.Network(int(N[k]), int(S[k]), seed=int(seeds[k]), drive_scale=float(D[k]), record_raster=False) as x:
            x.run(int(T[k]), g.ALG_AUTO)
            alone_ms.append(x.info().last_run_ms)
        lat.append((time.perf_counter() - ts) * 1e3)
    wall = time.perf_counter() - t0
    out["plain"] = {"req_per_s": count / wall, "p50_service_ms": float(np.percentile(lat, 50)),
                    "p99_service_ms": float(np.percentile(lat, 99)), "wall_ms": wall * 1e3,
                    "device_ms": float(sum(alone_ms)), "host_ms": wall * 1e3 - float(sum(alone_ms))}
    best = max(v["req_per_s"] for k, v in out.items() if k.startswith("lambda_"))
    out["speedup_vs_plain"] = best / out["plain"]["req_per_s"]
    out["breakdown"] = served_breakdown(N, T, last, np.array(lat), np.array(alone_ms), out["plain"]["wall_ms"])
    return out


def served_breakdown(N, T, res, plain_ms, alone_ms, plain_wall_ms, sms=152):
    """Per-request accounting of the last arrival rate's served run, binned by N x steps:
    device time alone on the whole GPU (the plain leg, autotuned scheme), device time of
    the request's steps in the mix and the same times its team's CTAs (SM-ms), creation and
    queueing.  The bound: the mix cannot finish before its SM time fills every SM, nor
    before the admission thread has created every network; plain wall / that bound is the
    best speed-up this mix allows in the batched geometry."""
    import numpy as np
    work = N.astype(float) * T
    edges = [0, 1e7, 1e8, 1e9, np.inf]
    bins = []
    for lo, hi in zip(edges[:-1], edges[1:]):
        m = (work >= lo) & (work < hi)
        if not m.any():
            continue
        sel = [r for r, k in zip(res, m) if k]
        bins.append({"N_x_steps": f"[{lo:.0e}, {hi:.0e})", "requests": int(m.sum()),
                     "alone_device_ms": float(alone_ms[m].sum()), "plain_wall_ms": float(plain_ms[m].sum()),
                     "mix_device_ms": float(sum(r.device_ms for r in sel)),
                     "mix_sm_ms": float(sum(r.sm_ms for r in sel)),
                     "mean_team": float(np.mean([r.team for r in sel])),
                     "create_ms": float(sum(r.create_ms for r in sel)),
                     "mean_queue_ms": float(np.mean([r.queue_ms for r in sel])),
                     "mean_latency_ms": float(np.mean([r.latency_ms for r in sel]))})
    sm_ms = float(sum(r.sm_ms for r in res))
    create_ms = float(sum(r.create_ms for r in res))
    longest = float(max(r.device_ms + r.create_ms for r in res))
    bound = max(sm_ms / sms, create_ms, longest)
    return {"bins": bins, "sm_ms": sm_ms, "create_ms": create_ms, "longest_request_ms": longest,
            "bound_ms": bound, "best_speedup_in_this_geometry": plain_wall_ms / bound}


def load_traffic(name, steps_per_launch):
    """DRAM bytes (read + written) per launch of the team kernel on this workload, from the
    committed ncu summary (a table row `| workload | steps per launch | bytes per launch |`),
    scaled to this launch's steps; None if the workload was not captured."""
    import re
    p = os.path.join(ROOT, "profiles", "k_team_dram_traffic.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        m = re.match(r"^\|\s*(\w+)\s*\|\s*(\d+)\s*\|\s*([0-9.eE+]+)\s*\|", line)
        if m and m.group(1) == name:
            return float(m.group(3)) * steps_per_launch / int(m.group(2))
    return None


def timed_leg(g, net, name, cfg, alg, a, pg, local, drive_override):
    """W warm-up runs, then K timed runs of T steps (CUDA events on the library's stream,
    clocks sampled meanwhile); returns the measured figures and the roofline of the step
    kernel (algorithmic bytes per launch over the mean launch time)."""
    n, nsyn, T, drive, seed = cfg
    for _ in range(a.warmup):
        net.run(T, alg)
    runs = []
    if pg:
        pg.barrier()
    with ClockSampler(local) as clk:
        w0 = time.perf_counter()
        for _ in range(a.steps):
            net.run(T, alg)
            inf = net.info()
            u, s = net.step_times()
            runs.append((inf.last_run_ms, inf.last_run_kernel_ms, inf.last_run_spikes, inf.last_run_launches,
                         float(u[-T:].sum()), float(s[-T:].sum()), inf.last_algorithm))
        wall = time.perf_counter() - w0
    if pg:
        pg.barrier()
    dev_ms = sum(r[0] for r in runs)
    kern_ms = sum(r[1] for r in runs)
    spikes = sum(r[2] for r in runs)
    launches = sum(r[3] for r in runs)
    events = spikes * nsyn
    peak, peak_kind = peaks()
    team, slice_ = net.geometry()
    last_alg = int(runs[-1][6])
    resident = last_alg == g.ALG_SKL and team > 0 and slice_ <= RESIDENT_SLICE
    deliv_bytes = events * 8
    upd_bytes = spikes * STAT_BYTES_PER_SPIKE + (0 if resident else n * T * a.steps * UPDATE_BYTES_PER_NEURON)
    n_launch = max(1, launches)
    achieved = (deliv_bytes + upd_bytes) / n_launch / (kern_ms / n_launch * 1e-3) / 1e9
    upd_ms = sum(r[4] for r in runs)
    deliv_ms = max(1e-9, sum(r[5] for r in runs) - upd_ms)
    if last_alg == g.ALG_SKL and team > 0:
        mapping = {0: ", segment runs", 1: ", eight-lane groups"}.get(net.delivery(), "")
        kname = (f"k_team (SKL team kernel: {team} CTAs x {net.block_threads()} threads, {slice_} neurons per CTA"
                 f"{mapping})")
    elif last_alg == g.ALG_SKL:
        kname = "k_persistent (SKL global-atomic kernel)"
    else:
        kname = f"k_update + k_deliver ({ALG_LABEL[last_alg]})"
    roofline = {"kernel": kname, "bound": "hbm",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": (load_traffic(name, T) if last_alg == g.ALG_SKL and team > 0 and not drive_override
                            else None),  # (the committed captures are of the workloads' own drive)
                "state_on_chip": resident,
                "algorithmic_bytes_per_launch": (deliv_bytes + upd_bytes) / n_launch,
                "launch_ms": kern_ms / n_launch,
                "delivery_phase": {"bytes": deliv_bytes, "ms": deliv_ms, "gbs": deliv_bytes / deliv_ms / 1e6,
                                   "frac": deliv_bytes / deliv_ms / 1e6 / peak},
                "update_phase": {"bytes": upd_bytes, "ms": upd_ms, "gbs": upd_bytes / max(upd_ms, 1e-9) / 1e6}}
    return {"dev_ms": dev_ms, "spikes": spikes, "events": events, "launches": launches, "wall": wall,
            "last_alg": last_alg, "roofline": roofline, "clocks": clk.summary()}


def large_leg(g, a, local, drives=(0.5, 2.0)):
    """The large single networks at their workloads' own drive, each on its own: N=10^6 x
    1000 and N=250,000 x 10,000, SKL (the autotuner's pick for both), with the roofline of
    that launch, its clocks and its DRAM traffic from the committed ncu summary; then the
    same networks at the other drive scales of the sweep (the quiet and the irregular
    regime), each a fresh network timed the same way."""
    out = {}
    for name in ("n1m", "n250k_s10k"):
        cfg = WORKLOADS[name]
        n, nsyn, T, drive, seed = cfg
        t0 = time.perf_counter()
        net = g.Network(n, nsyn, seed=seed, drive_scale=drive, record_raster=False)
        create_s = time.perf_counter() - t0
        r = timed_leg(g, net, name, cfg, g.ALG_SKL, a, None, local, False)
        net.close()
        out[name] = {"metric": "synaptic events/s", "value": r["events"] / (r["dev_ms"] * 1e-3), "unit": "events/s",
                     "ms_per_step": r["dev_ms"] / a.steps, "us_per_sim_step": r["dev_ms"] * 1e3 / (a.steps * T),
                     "steps": a.steps, "warmup": a.warmup, "firing_rate_hz": r["spikes"] / (n * T * a.steps) * 1e3,
                     "config": workload_config(name, cfg), "create_s": create_s, "roofline": r["roofline"],
                     "clocks": r["clocks"], "gpu_launches": int(r["launches"])}
        sweep = {}
        for d in drives:
            dcfg = (n, nsyn, T, d, seed)
            net = g.Network(n, nsyn, seed=seed, drive_scale=d, record_raster=False)
            r = timed_leg(g, net, name, dcfg, g.ALG_SKL, a, None, local, True)
            net.close()
            sweep[f"drive_{d:g}"] = {"value": r["events"] / (r["dev_ms"] * 1e-3), "unit": "events/s",
                                     "us_per_sim_step": r["dev_ms"] * 1e3 / (a.steps * T),
                                     "firing_rate_hz": r["spikes"] / (n * T * a.steps) * 1e3,
                                     "frac": r["roofline"]["frac"],
                                     "delivery_frac": r["roofline"]["delivery_phase"]["frac"],
                                     "kernel": r["roofline"]["kernel"], "clocks": r["clocks"]}
        out[name]["drive_sweep"] = sweep
    return out


def reference_gpu_leg(cfg, steps=1000):
    """The reference's own CUDA kernels (gpu4snn.cu compiled unmodified for sm_103a) on this
    GPU, on the same network's connectivity (the oracle's Philox rows, in draw order, as the
    reference keeps its rows), its drive mode matching the workload's gains, one run of
    `steps` steps per scheme after a warm-up run; "unavailable" when the cubin is absent."""
    n, nsyn, T, drive, seed = cfg
    modes = {0.5: 0, 1.0: 1, 1.5: 2}
    from oracle import g4s_oracle as O
    from oracle import refgpu as R
    why = R.unavailable()
    if why or drive not in modes:
        return {"unavailable": why or f"drive scale {drive} is none of the reference's modes"}
    if n * nsyn >= 2 ** 31:
        return {"unavailable": "N x Nsyn >= 2^31 overflows the reference's int synapse indices"}
    O.build()
    idx, w = O.conn_philox(O.make_desc(n, nsyn, seed))
    res = R.run(idx, w, steps=steps, schemes=(0, 1, 2, 3, 4), modes=(modes[drive],), seeds=(seed,), reps=2)
    out = {"kind": "reference CUDA kernels, gpu4snn.cu unmodified, -O3 for sm_103a (cubin), "
                   "driven by oracle/refgpu/g4s_refgpu.c", "mode": modes[drive], "steps": steps, "schemes": {}}
    for r in res:
        if r.get("rep") == 1:
            out["schemes"][R.SCHEMES[r["scheme"]]] = {
                "events_per_s": r["spikes"] * nsyn / (r["ms"] * 1e-3), "us_per_step": r["ms"] * 1e3 / steps,
                "grid": r["grid"], "block": r["block"]}
    best = max(out["schemes"].items(), key=lambda kv: kv[1]["events_per_s"])
    out["best"] = {"scheme": best[0], **best[1]}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="n100k")
    ap.add_argument("--drive", type=float, default=None,
                    help="drive scale in place of the workload's (0.5 quiet, 1 balanced, 1.5-2 irregular)")
    ap.add_argument("--algorithm", default="AUTO")
    ap.add_argument("--block-threads", type=int, default=0,
                    help="threads per CTA of the SKL team kernel, 1024 or 768 (0: default / autotuned)")
    ap.add_argument("--delivery", type=int, default=-1,
                    help="delivery mapping of a multi-CTA SKL team: -1 automatic, 0 segment runs, 1 eight lanes a spike")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--raster-budget-mb", type=int, default=0, help="device raster buffer per chunk (0: default)")
    ap.add_argument("--no-schemes", action="store_true", help="skip timing the five schemes one by one")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-ensemble leg")
    ap.add_argument("--batch-networks", type=int, default=256, help="networks of the batched ensemble")
    ap.add_argument("--served", default="50,200,1000",
                    help="comma-separated Poisson arrival rates (req/s) for the served leg ('' skips it)")
    ap.add_argument("--served-requests", type=int, default=200, help="requests per arrival rate")
    ap.add_argument("--no-large", action="store_true", help="skip the N=10^6 and 250k x 10k block")
    ap.add_argument("--no-reference-gpu", action="store_true", help="skip the reference-kernel block")
    a = ap.parse_args()
    if a.warmup < 3:
        a.warmup = 3
    ws, rank, local, pg = dist_setup()
    cfg = WORKLOADS[a.workload]
    drive_override = a.drive is not None and a.drive != cfg[3]
    if drive_override:
        cfg = cfg[:3] + (float(a.drive),) + cfg[4:]
    if a.impl == "reference":
        return run_reference(a, cfg, ws, rank, pg)

    import gpu4snn_gb300 as g
    from gpu4snn_gb300 import _lib
    n, nsyn, T, drive, seed = cfg
    seed = seed + rank
    _lib.check(g.load().g4s_set_device(local))
    alg = g.ALG_NAMES[a.algorithm.upper()] if not a.algorithm.isdigit() else int(a.algorithm)
    budget = a.raster_budget_mb << 20
    net = g.Network(n, nsyn, seed=seed, drive_scale=drive, record_raster=False, raster_budget_bytes=budget)
    if a.block_threads:
        net.set_block_threads(a.block_threads)
    if a.delivery != -1:
        net.set_geometry(0, a.delivery)
    schemes = None
    if not a.no_schemes:
        schemes = schemes_leg(g, net, nsyn, min(T, 2048))
    tuned = None
    if alg == g.ALG_AUTO:
        talg, tteam, tus = net.autotune(min(T, 200))
        tuned = {"algorithm": talg, "name": ALG_LABEL[talg], "team": tteam, "us_per_step": tus}
        net.run(8, alg)  # (applies the choice, so that its CTA size can be read back)
        tuned["block_threads"] = net.block_threads()
        tuned["delivery"] = {0: "segment runs", 1: "eight-lane groups"}.get(net.delivery(), "one CTA")
    r = timed_leg(g, net, a.workload, cfg, alg, a, pg, local, drive_override)
    t_max = reduce_max(pg, r["dev_ms"])
    ev_all = reduce_sum(pg, float(r["events"]))
    value = ev_all / (t_max * 1e-3)
    spikes, launches, wall, last_alg, roofline, clocks = (r["spikes"], r["launches"], r["wall"], r["last_alg"],
                                                          r["roofline"], r["clocks"])
    line = {"metric": "synaptic events/s", "value": value, "unit": "events/s", "n_gpus": ws, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": t_max / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic (seeded Philox network)",
            "config": workload_config(a.workload, cfg), "algorithm": ALG_LABEL[last_alg],
            "autotuned": tuned, "schemes": schemes,
            "firing_rate_hz": spikes / (n * T * a.steps) * 1000.0, "wall_s": wall,
            "roofline": roofline, "clocks": clocks, "gpu_launches": int(launches)}
    # end to end through the C ABI with host buffers
    if not a.no_e2e:
        idx_h, p_idx = _lib.pinned_empty((n, net.stride), "int32")
        w_h, p_w = _lib.pinned_empty((n, net.stride), "float32")
        idx_h[:], w_h[:] = net.tables()
        net.close()
        e2e_net = g.Network(n, nsyn, seed=seed, drive_scale=drive, record_raster=True)
        e2e_net.load_tables(idx_h, w_h)
        e2e_net.reset()
        e2e_net.run(T, alg)
        e_ev, e_wall, d2h = 0, 0.0, 0
        for _ in range(a.steps):
            t0 = time.perf_counter()
            e2e_net.load_tables(idx_h, w_h)
            e2e_net.reset()
            e2e_net.run(T, alg)
            rt, rid = e2e_net.raster()
            cnt = e2e_net.counts()
            e_wall += time.perf_counter() - t0
            e_ev += len(rt) * nsyn
            d2h = len(rt) * 4 + T * (4 + 8 + 16)
        k = a.steps
        e_wall = reduce_max(pg, e_wall)
        line["e2e"] = {"value": reduce_sum(pg, float(e_ev)) / e_wall, "unit": "events/s",
                       "h2d_bytes_per_step": int(2 * n * net.stride * 4), "d2h_bytes_per_step": int(d2h),
                       "steps": k, "path": "g4s_net_load_tables (pinned host) + g4s_net_reset + g4s_net_run "
                                           "(raster recorded) + g4s_net_raster"}
        e2e_net.close()
        _lib.pinned_free(p_idx)
        _lib.pinned_free(p_w)
    else:
        net.close()
    if rank == 0 and ws == 1 and not a.no_cpu:
        threads = os.cpu_count() or 1
        v, st, dt = cpu_port_rate(n, nsyn, seed, drive, threads, min_seconds=12.0, max_steps=2000,
                                  warm_steps=100)
        line["cpu_baseline"] = {"value": v, "unit": "events/s", "cores": threads, "kind": "port",
                                "sample": f"{st} simulation steps after 100 warm-up steps of the same network "
                                          f"({dt:.1f} s), oracle OpenMP port"}
    if rank == 0 and ws == 1 and not a.no_reference_gpu:
        line["reference_gpu"] = reference_gpu_leg(cfg)
        ref_best = line["reference_gpu"].get("best")
        if ref_best:
            line["reference_gpu"]["speedup_of_value"] = value / ref_best["events_per_s"]
    if rank == 0 and ws == 1 and not a.no_large:
        line["large"] = large_leg(g, a, local)
    if rank == 0 and ws == 1 and not a.no_batched:
        line["batched"] = batched_leg(g, a.batch_networks)
    if rank == 0 and ws == 1 and a.served:
        line["served"] = served_leg(g, a.served_requests, [float(x) for x in a.served.split(",")])
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
