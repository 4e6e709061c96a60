"""Benchmark: loop-cluster sweeps on one GB300 (MC sweeps*sites/s).

Workload (one step = one sweep of update + measurement, path_integral.C:355-864): S=1/2
Heisenberg antiferromagnet on a periodic 128x128 square lattice (16384 sites, 32768 bonds),
J = 1, beta = 64 (about 1.2 M operators), seed 7, iid random initial spins.  The chain is brought
near equilibrium (untimed) before the warm-up steps.  Between timed steps a 256 MiB device write
flushes the L2 cache (outside the timed brackets); each step is timed with CUDA events on the
engine's own stream.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 (torchrun) every rank runs its own independent replica chain (the path does not
shard; replicas only) and rank 0 prints the aggregate.  --impl reference times the CPU
loop-cluster update (the oracle's restatement of path_integral.C with the same random streams)
on this host's cores for the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "alps-looper_gb300"))
sys.path.insert(0, os.path.join(REPO, "tests"))

L_SIDE = 128
BETA = 64.0
SEED = 7
N_SITES = L_SIDE * L_SIDE
FLUSH_BYTES = 256 << 20
PRE_THERM = 256
METRIC = "MC sweeps*sites/s"
UNIT = "sweeps*sites/s"
WORKLOAD = ("square 128x128 S=1/2 Heisenberg AF, J=1, beta=64, periodic (16384 sites, "
            "32768 bonds, ~1.2M operators/sweep)")


def _rank_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _dist_init(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def _reduce_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _reduce_sum(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def _barrier(dist):
    if dist is not None:
        dist.barrier()


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.th.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def _traffic_from_profile():
    """DRAM bytes per sweep from the committed ncu summary, when present."""
    path = os.path.join(REPO, "profiles", "sweep_square128_b64.md")
    try:
        for ln in open(path):
            if ln.startswith("dram_bytes_per_sweep:"):
                return float(ln.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


def _params(lg, seed=SEED, sweeps=1 << 13, therm=1 << 10):
    return lg.make_params(LATTICE="square", L=L_SIDE, BETA=BETA, J=1.0, SEED=seed,
                          SWEEPS=sweeps, THERMALIZATION=therm, INITIAL_SPINS="random")


def cpu_port_rate(seconds=12.0, threads=1, state=None, warm=3):
    """Oracle (CPU restatement) sweeps*sites/s on this host for the bench workload."""
    import oracle_lib as orc
    chains = [orc.Oracle(2, L_SIDE, BETA, 1.0, 1.0, 0.0, seed=SEED + 1000 * i)
              for i in range(threads)]
    for o in chains:
        if state is not None:
            o.set_state(*state, 0)
        o.sweep(warm)
    done = [0] * threads
    stop = time.perf_counter() + seconds

    def work(i):
        while time.perf_counter() < stop:
            chains[i].sweep(1)
            done[i] += 1

    t0 = time.perf_counter()
    ths = [threading.Thread(target=work, args=(i,)) for i in range(threads)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    el = time.perf_counter() - t0
    for o in chains:
        o.close()
    return sum(done) * N_SITES / el, sum(done), el


def batched_params(lg, n=512, seed=99):
    """512 square-lattice Heisenberg AFs: L uniform in {8,12,...,64}, T log-uniform in
    [0.02, 2], seed 99 (the batched-chain workload)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    Ls = rng.choice(np.arange(8, 65, 4), size=n)
    Ts = np.exp(rng.uniform(math.log(0.02), math.log(2.0), size=n))
    return [lg.make_params(LATTICE="square", L=int(L), T=float(T), J=1.0, SEED=seed * 1000 + i,
                           SWEEPS=1 << 12, THERMALIZATION=1 << 10, INITIAL_SPINS="random")
            for i, (L, T) in enumerate(zip(Ls, Ts))]


def run_batched(lg, steps, therm, plain_sample=16):
    """Batched arena vs the plain path on the same chains (one chain per launch sequence)."""
    ps = batched_params(lg)
    sites = sum(p.L * p.L for p in ps)
    b = lg.Batch(ps)
    b.run(therm // 2)
    # launch shapes chosen by the autotuner on the arena's own (thermalization) sweeps
    shape, report = b.autotune(4, FLUSH_BYTES)
    b.run(therm - therm // 2)
    b.time_sweeps(3, FLUSH_BYTES)
    ms = b.time_sweeps(steps, FLUSH_BYTES)
    t_b = float(ms.sum()) / 1e3
    value_b = steps * sites / t_b
    # plain path: a sample of the same chains run alone, sweep by sweep
    idx = list(range(0, len(ps), max(1, len(ps) // plain_sample)))[:plain_sample]
    t_p, s_p = 0.0, 0
    for i in idx:
        w = lg.LoopWorker(ps[i])
        w.run(min(therm, 64))
        w.autotune(2, FLUSH_BYTES)  # the plain path at its own best launch shape
        m = w.time_sweeps(max(16, steps), FLUSH_BYTES)
        t_p += float(m.mean()) / 1e3
        s_p += ps[i].L * ps[i].L
        w.close()
    value_p = s_p / t_p
    b.close()
    return {"workload": "512 square Heisenberg AF chains, L uniform in {8..64}, T log-uniform "
                        "[0.02,2], seed 99 (%d sites)" % sites,
            "value": value_b, "unit": UNIT, "ms_per_sweep": t_b * 1e3 / steps,
            "steps": steps, "thermalization_sweeps": therm,
            "plain_value": value_p, "plain_sample_chains": len(idx),
            "speedup_vs_plain": value_b / value_p,
            "shape": shape, "autotune_candidates": report.count(" ms\n") - 1}


def replica_params(lg, n=64):
    """64 replicas of the S=1/2 XXZ model on a periodic 24^3 simple-cubic lattice (13824
    sites), Jxy = 1, Jz = 0.5, uniform field h = 0.3, beta = 8, seeds 1000..1063."""
    return [lg.make_params(LATTICE="cubic", L=24, BETA=8.0, Jxy=1.0, Jz=0.5, h=0.3,
                           SEED=1000 + i, SWEEPS=1 << 13, THERMALIZATION=1 << 10,
                           INITIAL_SPINS="random")
            for i in range(n)]


def run_replicas(lg, steps, therm, plain_sample=4):
    """The 64 field replicas in one arena vs the plain path on a sample of them."""
    ps = replica_params(lg)
    sites = sum(p.L ** 3 for p in ps)
    b = lg.Batch(ps)
    b.run(therm // 2)
    shape, _ = b.autotune(2, FLUSH_BYTES)
    b.run(therm - therm // 2)
    b.time_sweeps(3, FLUSH_BYTES)
    ms = b.time_sweeps(steps, FLUSH_BYTES)
    t_b = float(ms.sum()) / 1e3
    t_p, s_p = 0.0, 0
    for i in range(plain_sample):
        w = lg.LoopWorker(ps[i])
        w.run(min(therm, 64))
        w.autotune(2, FLUSH_BYTES)
        m = w.time_sweeps(max(8, steps), FLUSH_BYTES)
        t_p += float(m.mean()) / 1e3
        s_p += ps[i].L ** 3
        w.close()
    b.close()
    return {"workload": "64 replicas, XXZ Jxy=1 Jz=0.5 h=0.3 on a 24^3 cubic lattice, beta=8, "
                        "seeds 1000..1063 (%d sites)" % sites,
            "value": steps * sites / t_b, "unit": UNIT, "ms_per_sweep": t_b * 1e3 / steps,
            "steps": steps, "thermalization_sweeps": therm,
            "plain_value": s_p / t_p, "plain_sample_replicas": plain_sample,
            "speedup_vs_plain": (steps * sites / t_b) / (s_p / t_p), "shape": shape}


def served_requests(lg, n=4096, seed=2024):
    """The served stream: Poisson arrivals at 200/s; lattice uniform over {chain L in [32,4096],
    square L in [8,96], cubic L in [6,24]} (L rounded up to even: odd periodic lattices with an
    antiferromagnetic xy coupling have a sign problem), beta log-uniform in [0.5,64],
    Jz/Jxy uniform in [0.5,1.5] with Jxy = 1, h uniform in [0,0.5], SWEEPS in {2^10, 2^12}."""
    import numpy as np
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1 / 200.0, size=n))
    out = []
    for i in range(n):
        kind = int(rng.integers(0, 3))
        if kind == 0:
            lat, L = "chain", int(rng.integers(32, 4097))
        elif kind == 1:
            lat, L = "square", int(rng.integers(8, 97))
        else:
            lat, L = "cubic", int(rng.integers(6, 25))
        L += L % 2
        beta = math.exp(rng.uniform(math.log(0.5), math.log(64.0)))
        r = rng.uniform(0.5, 1.5)
        h = rng.uniform(0.0, 0.5)
        sw = int(rng.choice([1 << 10, 1 << 12]))
        out.append((float(arrivals[i]),
                    lg.make_params(LATTICE=lat, L=L, BETA=beta, Jxy=1.0, Jz=r, h=h, SWEEPS=sw,
                                   SEED=seed * 100000 + i, INITIAL_SPINS="random")))
    return out


def run_served(lg, n_requests, plain_sample=32, lanes=3):
    reqs = served_requests(lg)[:n_requests]
    srv = lg.Server(sweeps_per_tick=16, rebuild_interval_s=0.02, lanes=lanes)
    t0 = time.perf_counter()
    for t_arr, p in reqs:
        d = t0 + t_arr - time.perf_counter()
        if d > 0:
            time.sleep(d)
        srv.submit(p)
    srv.wait(3600)
    wall = time.perf_counter() - t0
    res = srv.poll()
    st = srv.stats()
    srv.close()
    ok = [r for r in res if r["status"] == 0]
    lat = sorted(r["t_finish"] - r["t_submit"] for r in ok)
    work = sum(r["sites"] * r["sweeps"] for r in ok)
    served = work / wall
    # plain path: the same requests one at a time (sampled; wall clock per sweep through lg_run)
    idx = list(range(0, len(reqs), max(1, len(reqs) // plain_sample)))[:plain_sample]
    t_plain, w_plain = 0.0, 0
    for i in idx:
        p = reqs[i][1]
        w = lg.LoopWorker(p)
        w.run(4)
        w.autotune(2)  # the plain path at its own best launch shape
        t1 = time.perf_counter()
        w.run(32)
        per = (time.perf_counter() - t1) / 32
        total_sweeps = p.sweeps + (p.sweeps >> 3)
        t_plain += per * total_sweeps
        w_plain += p.L ** p.lattice * total_sweeps
        w.close()
    plain = w_plain / t_plain
    q = lambda f: lat[min(len(lat) - 1, int(f * len(lat)))] if lat else None  # noqa: E731
    return {"workload": "served stream: first %d of 4096 Poisson requests (200/s, seed 2024)"
                        % len(reqs),
            "value": served, "unit": UNIT, "wall_s": wall, "completed": len(ok), "lanes": lanes,
            "rejected": int(st["rejected"]), "rebuilds": int(st["rebuilds"]),
            "latency_p50_s": q(0.50), "latency_p99_s": q(0.99),
            "plain_value": plain, "plain_sample_requests": len(idx),
            "speedup_vs_plain": served / plain}


def run_ours(args, dist, ws, rank, local):
    import looper_gb300 as lg
    lg.lib()
    w = lg.LoopWorker(_params(lg, seed=SEED + 7919 * rank))
    w.run(PRE_THERM // 2)
    if args.shape == "auto":
        # launch shape chosen by the autotuner on the chain's own pre-thermalization sweeps
        shape, _ = w.autotune(8, FLUSH_BYTES)
    else:
        w.shape = json.loads(args.shape)  # a fixed shape (e.g. to profile the tuned one)
        shape = w.shape
    w.run(PRE_THERM // 2)
    w.time_sweeps(max(3, args.warmup), FLUSH_BYTES)
    clk = Clocks(local) if rank == 0 else None
    if clk:
        clk.start()
    _barrier(dist)
    l0 = lg.kernel_launches()
    ms = w.time_sweeps(args.steps, FLUSH_BYTES)
    launches = lg.kernel_launches() - l0
    _barrier(dist)
    clocks = clk.stop() if clk else None
    total_ms = float(ms.sum())
    total_ms = _reduce_max(dist, total_ms)
    value = ws * args.steps * N_SITES / (total_ms / 1e3)
    # per-stage profile (events between launches) for the roofline
    prof, verts = w.profile_sweeps(16, FLUSH_BYTES)
    nv_mean = verts / 16.0
    sweep_ms = sum(prof.values()) / 16.0
    # algorithmic bytes per sweep: 64 per vertex (record read and write 24, leg links 8, parent
    # write and read 8, labels 12, estimator re-read 12) and 16 per site (spin read and write 8,
    # boundary fragment 4, site label 4)
    bytes_alg = 64.0 * nv_mean + 16.0 * N_SITES
    peak, peak_kind = _peaks()
    achieved = bytes_alg / (total_ms / args.steps / 1e3) / 1e9
    dom = max(prof, key=prof.get)
    shares = {k: round(v / sum(prof.values()), 4) for k, v in prof.items()}
    traffic = _traffic_from_profile()
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_kind": peak_kind, "scope": "one sweep (all kernels of the CUDA graph)",
                "algorithmic_bytes_per_sweep": int(bytes_alg),
                "dominant_kernel": dom, "dominant_share": shares[dom],
                "stage_ms_per_sweep": {k: round(v / 16.0, 5) for k, v in prof.items()},
                "profiled_sweep_ms": round(sweep_ms, 5)}
    # end to end through the public C ABI: create + run + observables, host wall clock
    t0 = time.perf_counter()
    e = lg.LoopWorker(_params(lg, seed=SEED + 31 + rank, sweeps=args.steps - args.steps // 2,
                              therm=args.steps // 2))
    e.run(args.steps)
    obs = e.observables()
    e2e_s = time.perf_counter() - t0
    e2e_s = _reduce_max(dist, e2e_s)
    e2e = {"value": ws * args.steps * N_SITES / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": round((2 * 32768 * 4 + 4 * 16384 * 4 + 16384) / args.steps, 1),
           "d2h_bytes_per_step": 32 * 8 + 32,
           "scope": "lg_create + lg_run(steps) + lg_observables from a cold start"}
    e.close()
    cpu = None
    if rank == 0 and args.cpu_seconds > 0:
        state = w.state()
        rate, n, el = cpu_port_rate(seconds=args.cpu_seconds, threads=1, state=state)
        cpu = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "%d sweeps of the same 128x128 beta=64 chain started from the GPU's "
                         "equilibrated state, %.1f s, 1 thread (CPU restatement of "
                         "path_integral.C in oracle/)" % (n, el)}
    w.close()
    batched = None
    if rank == 0 and args.batched_steps > 0:
        batched = run_batched(lg, args.batched_steps, args.batched_therm)
    replicas = None
    if rank == 0 and args.replica_steps > 0:
        replicas = run_replicas(lg, args.replica_steps, args.replica_therm)
    served = None
    if rank == 0 and args.served_requests > 0:
        served = run_served(lg, args.served_requests)
    if rank != 0:
        return None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64 (FP64 times on a 2^-52 grid)",
        "data": "synthetic (seeded Philox streams; iid random initial spins)",
        "config": {"workload": WORKLOAD, "lattice": "square", "L": L_SIDE, "beta": BETA,
                   "J": 1.0, "seed": SEED, "step": "one sweep",
                   "pre_thermalization_sweeps": PRE_THERM, "launch_shape": shape,
                   "l2": "flushed between steps (256 MiB device write, untimed)",
                   "parallelism": "replicas" if ws > 1 else "single chain"},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
        "clocks": clocks,
        "batched": batched,
        "replicas_field": replicas,
        "served": served,
        "observables": {"Energy Density": obs["Energy Density"][0],
                        "sweeps_measured": int(obs["count"]),
                        "note": "the e2e chain: cold start, %d thermalization sweeps" % (args.steps // 2)},
    }
    return out


def run_reference(args, dist, ws, rank, local):
    if rank != 0:
        return None
    threads = max(1, os.cpu_count() or 1)
    steps = max(1, min(args.steps, 16))
    import oracle_lib as orc
    chains = [orc.Oracle(2, L_SIDE, BETA, 1.0, 1.0, 0.0, seed=SEED + 1000 * i)
              for i in range(threads)]

    def work(i, n):
        chains[i].sweep(n)

    def par(n):
        ths = [threading.Thread(target=work, args=(i, n)) for i in range(threads)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()

    par(max(3, min(args.warmup, 4)))
    t0 = time.perf_counter()
    par(steps)
    el = time.perf_counter() - t0
    value = threads * steps * N_SITES / el
    for o in chains:
        o.close()
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp64 times", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "lattice": "square", "L": L_SIDE, "beta": BETA,
                   "step": "one sweep per thread"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d threads x %d sweeps after %d warm-up sweeps from a "
                                   "random start (the reference's path_integral binary needs "
                                   "ALPS and does not build here)" % (threads, steps,
                                                                      max(3, min(args.warmup, 4)))},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=512)
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--batched-steps", type=int, default=16)
    ap.add_argument("--batched-therm", type=int, default=128)
    ap.add_argument("--replica-steps", type=int, default=8)
    ap.add_argument("--replica-therm", type=int, default=32)
    ap.add_argument("--served-requests", type=int, default=256)
    ap.add_argument("--shape", default="auto",
                    help='launch shape of the headline chain: "auto" (autotuned) or a JSON dict '
                         'of lg_shape fields')
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    ws, rank, local = _rank_info()
    if ws > 1 and args.impl == "ours":
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = _dist_init(ws)
    if args.impl == "reference":
        out = run_reference(args, dist, ws, rank, local)
    else:
        out = run_ours(args, dist, ws, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
