"""Benchmark: loop-cluster sweeps on one GB300 (MC sweeps*sites/s).

Headline workload (one step = one sweep of update + measurement, path_integral.C:355-864): S=1/2
Heisenberg antiferromagnet on a periodic 128x128 square lattice (16384 sites, 32768 bonds),
J = 1, beta = 64 (about 1.2 M operators), seed 7, iid random initial spins.  The chain is brought
to equilibrium (untimed) before the warm-up steps.  Between timed steps a 256 MiB device write
flushes the L2 cache (outside the timed brackets); each step is timed with CUDA events on the
engine's own stream.

Beside it, in the same JSON line: the CPU-runnable chain workload (L=64, beta=10, seed 1234: the
plain GPU path, a batch of such chains, and the standalone restatement on the host cores), the
512-chain batched arena, the 64 field replicas and the 4096-request served stream.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 (torchrun) every rank runs its own independent replica chain (the path does not
shard; replicas only) and rank 0 prints the aggregate.  --impl reference times the CPU
loop-cluster update (the oracle's restatement of path_integral.C with the same random streams)
on this host's cores for the headline workload, each thread's chain equilibrated first.
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
    """nvidia-smi sampling (every 20 ms) around the timed region.  Each sample carries its host
    time, so that stop() can summarise the samples of a window: the warm-up steps (kept running
    for at least WARM_S seconds so that the clocks settle under load) and the timed steps."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    WARM_S = 0.3

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append((time.perf_counter(), ln.strip()))

    def wait_first(self, timeout=3.0):
        t = time.perf_counter() + timeout
        while self.proc is not None and not self.lines and time.perf_counter() < t:
            time.sleep(0.01)

    def stop(self, t0=None, t1=None):
        if self.proc is None:
            return None
        time.sleep(0.05)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.th.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ts, ln in self.lines:
            if t0 is not None and (ts < t0 or ts > t1 + 0.04):
                continue
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
                "reasons": sorted(reasons), "samples": len(sm),
                "window": "warm-up steps (>= %.1f s under load) and the timed steps" % self.WARM_S}


def cpu_model():
    """The host CPU's model name (lscpu), for every CPU figure."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


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
    """Oracle (CPU restatement) sweeps*sites/s and operators/s on this host for the headline
    workload; each thread's chain starts from `state` (or a random one) and runs `warm` untimed
    sweeps first."""
    import oracle_lib as orc
    chains = [orc.Oracle(2, L_SIDE, BETA, 1.0, 1.0, 0.0, seed=SEED + 1000 * i)
              for i in range(threads)]
    for o in chains:
        if state is not None:
            o.set_state(*state, 0)
        o.sweep(warm)
        o.clear_records()
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
    ops = sum(int(o.records()[:, 0].sum()) for o in chains)
    for o in chains:
        o.close()
    return {"rate": sum(done) * N_SITES / el, "sweeps": sum(done), "seconds": el,
            "operators_per_s": ops / el, "mean_operators": ops / max(1, sum(done))}


# ---- the CPU-runnable chain workload: S=1/2 Heisenberg AF chain, L=64, beta=10, seed 1234 ----
SMALL_L, SMALL_BETA, SMALL_SEED, SMALL_THERM, SMALL_SWEEPS = 64, 10.0, 1234, 1 << 12, 1 << 14


def _small_standalone(_):
    import oracle_lib as orc
    out, speed = orc.standalone(SMALL_L, 1.0 / SMALL_BETA, SMALL_SWEEPS, SMALL_SWEEPS >> 3)
    return speed


def run_small_chain(lg, batch_chains=1024, batch_steps=256):
    """The CPU-runnable chain workload on the plain GPU path (lg_create + lg_run of the whole
    2^12 + 2^14 sweeps + lg_observables, host wall clock), as a batch of such chains (one arena,
    device time), and on the host: the oracle's restatement of standalone/loop.C (which
    reproduces that program's output digit for digit: same draws, same arithmetic) with its
    options -l 64 -t 0.1 -n 16384, on one core and as one process per core."""
    import multiprocessing as mp
    p = lg.make_params(LATTICE="chain", L=SMALL_L, BETA=SMALL_BETA, J=1.0, SEED=SMALL_SEED,
                       SWEEPS=SMALL_SWEEPS, THERMALIZATION=SMALL_THERM, INITIAL_SPINS="random")
    t0 = time.perf_counter()
    w = lg.LoopWorker(p)
    w.run(SMALL_THERM + SMALL_SWEEPS)
    obs = w.observables()
    el = time.perf_counter() - t0
    w.close()
    plain = (SMALL_THERM + SMALL_SWEEPS) * SMALL_L / el
    ps = [lg.make_params(LATTICE="chain", L=SMALL_L, BETA=SMALL_BETA, J=1.0, SEED=SMALL_SEED + i,
                         SWEEPS=SMALL_SWEEPS, THERMALIZATION=SMALL_THERM, INITIAL_SPINS="random")
          for i in range(batch_chains)]
    b = lg.Batch(ps)
    b.run(64)
    b.time_sweeps(3)
    ms = b.time_sweeps(batch_steps)
    batched = batch_chains * SMALL_L * batch_steps / (float(ms.sum()) / 1e3)
    b.close()
    # host: one process, then one process per core (spawned: no GPU context is forked)
    speed1 = _small_standalone(0)
    cores = os.cpu_count() or 1
    with mp.get_context("spawn").Pool(cores) as pool:
        t1 = time.perf_counter()
        speeds = pool.map(_small_standalone, range(cores))
        el_all = time.perf_counter() - t1
    return {"workload": "S=1/2 Heisenberg AF chain, L=64, J=1, beta=10, seed 1234, 2^12 + 2^14 "
                        "sweeps, iid random initial spins",
            "plain": {"value": plain, "unit": UNIT, "seconds": el,
                      "scope": "lg_create + lg_run(2^12 + 2^14) + lg_observables, wall clock",
                      "energy_density": obs["Energy Density"][0],
                      "energy_density_err": obs["Energy Density"][1]},
            "batched": {"value": batched, "unit": UNIT, "chains": batch_chains,
                        "ms_per_sweep": float(ms.mean()), "steps": batch_steps,
                        "scope": "one arena of %d such chains (seeds 1234 + i), device time"
                                 % batch_chains},
            "cpu": {"value_1core": speed1 * SMALL_L, "value_all_cores": sum(speeds) * SMALL_L,
                    "unit": UNIT, "cores": cores, "cpu_model": cpu_model(), "kind": "port",
                    "program": "oracle restatement of standalone/loop.C, options -l 64 -t 0.1 "
                               "-n 16384 (its own thermalization n/8 = 2048, seed 29833, spins "
                               "all up)", "wall_s_all_cores": el_all}}


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


def _leg(fn, *a):
    """A supplementary measurement (small chain, batched, replicas, served): its failure is
    reported in its own entry of the line instead of ending the run."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001
        return {"error": "%s: %s" % (type(e).__name__, e)}


def run_served(lg, n_requests, plain_sample=32, lanes=3):
    """The served request stream (Poisson arrivals at 200/s) through lg_server_*, against the
    plain path on a sample of the same requests run alone from an equilibrated start."""
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
    svc = sorted(r["t_finish"] - r["t_start"] for r in ok)
    work = sum(r["sites"] * r["sweeps"] for r in ok)
    served = work / wall
    # plain path: the same requests one at a time (sampled): wall clock per sweep through lg_run
    # after max(64, THERMALIZATION / 4) equilibrating sweeps, times the request's sweeps
    idx = list(range(0, len(reqs), max(1, len(reqs) // plain_sample)))[:plain_sample]
    t_plain, w_plain = 0.0, 0
    for i in idx:
        p = reqs[i][1]
        w = lg.LoopWorker(p)
        w.run(max(64, (p.sweeps >> 3) // 4))
        w.autotune(2)  # the plain path at its own best launch shape
        t1 = time.perf_counter()
        w.run(32)
        per = (time.perf_counter() - t1) / 32
        total_sweeps = p.sweeps + (p.sweeps >> 3)
        t_plain += per * total_sweeps
        w_plain += p.L ** p.lattice * total_sweeps
        w.close()
    plain = w_plain / t_plain
    q = lambda v, f: v[min(len(v) - 1, int(f * len(v)))] if v else None  # noqa: E731
    return {"workload": "served stream: %d of the 4096 Poisson requests (200/s, seed 2024)"
                        % len(reqs),
            "value": served, "unit": UNIT, "wall_s": wall, "completed": len(ok), "lanes": lanes,
            "offered_rate_per_s": 200.0, "arrival_span_s": reqs[-1][0] if reqs else 0.0,
            "sustained_rate_per_s": len(ok) / wall,
            "rejected": int(st["rejected"]), "rebuilds": int(st["rebuilds"]),
            "latency_p50_s": q(lat, 0.50), "latency_p99_s": q(lat, 0.99),
            "service_p50_s": q(svc, 0.50), "service_p99_s": q(svc, 0.99),
            "latency_note": "completion minus submit time at the offered 200/s, queueing included; "
                            "service = completion minus admission",
            "plain_value": plain, "plain_sample_requests": len(idx),
            "speedup_vs_plain": served / plain}


def run_ours(args, dist, ws, rank, local):
    import looper_gb300 as lg
    lg.lib()
    w = lg.LoopWorker(_params(lg, seed=SEED + 7919 * rank))
    w.run(PRE_THERM // 2)
    if args.shape == "auto":
        # launch shape chosen by the autotuner on the chain's own pre-thermalization sweeps
        shape, report = w.autotune(8, args.flush_bytes)
        if rank == 0:
            sys.stderr.write(report)
    else:
        w.shape = json.loads(args.shape)  # a fixed shape (e.g. to profile the tuned one)
        shape = w.shape
    w.run(PRE_THERM // 2)
    blob = w.save()  # the equilibrated state the end-to-end run starts from
    clk = Clocks(local) if rank == 0 else None
    if clk:
        clk.start()
        clk.wait_first()
    t_warm = time.perf_counter()
    w.time_sweeps(max(3, args.warmup), args.flush_bytes)
    while time.perf_counter() - t_warm < Clocks.WARM_S:
        w.time_sweeps(8, args.flush_bytes)
    _barrier(dist)
    l0 = lg.kernel_launches()
    ms = w.time_sweeps(args.steps, args.flush_bytes)
    launches = lg.kernel_launches() - l0
    t_end = time.perf_counter()
    _barrier(dist)
    clocks = clk.stop(t_warm, t_end) if clk else None
    total_ms = float(ms.sum())
    total_ms = _reduce_max(dist, total_ms)
    value = ws * args.steps * N_SITES / (total_ms / 1e3)
    # per-stage profile (events between launches) for the roofline
    prof, verts = w.profile_sweeps(16, args.flush_bytes)
    nv_mean = verts / 16.0
    sweep_ms = sum(prof.values()) / 16.0
    # algorithmic bytes per sweep: 64 per vertex (record read and write 24, leg links 8, parent
    # write and read 8, labels 12, estimator re-read 12) and 16 per site (spin read and write 8,
    # boundary fragment 4, site label 4)
    bytes_alg = 64.0 * nv_mean + 16.0 * N_SITES
    peak, peak_kind = _peaks()
    step_s = total_ms / args.steps / 1e3
    achieved = bytes_alg / step_s / 1e9
    dom = max(prof, key=prof.get)
    shares = {k: round(v / sum(prof.values()), 4) for k, v in prof.items()}
    traffic = _traffic_from_profile()
    # the union-find stage's own share of the algorithmic bytes: leg links and parent write/read,
    # 16 per vertex
    un_s = prof.get("k_union", 0.0) / 16.0 / 1e3
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_kind": peak_kind, "scope": "one sweep (one launch of the sweep's CUDA graph)",
                "algorithmic_bytes_per_sweep": int(bytes_alg),
                "dominant_kernel": dom, "dominant_share": shares[dom],
                "union_achieved_gbs": round(16.0 * nv_mean / un_s / 1e9, 1) if un_s > 0 else None,
                "stage_ms_per_sweep": {k: round(v / 16.0, 5) for k, v in prof.items()},
                "profiled_sweep_ms": round(sweep_ms, 5),
                "operators_per_sweep": nv_mean, "operators_per_s": nv_mean / step_s}
    # end to end through the public C ABI, host buffers: lg_create, lg_load of the equilibrated
    # checkpoint (host -> device), lg_run(steps) (records back each chunk), lg_observables
    h0, d0 = lg.copy_bytes()
    t0 = time.perf_counter()
    e = lg.LoopWorker(_params(lg, seed=SEED + 31 + rank, sweeps=1 << 13, therm=0))
    t1 = time.perf_counter()
    e.load(blob)
    t2 = time.perf_counter()
    e.run(args.steps)
    t3 = time.perf_counter()
    obs = e.observables()
    e2e_s = time.perf_counter() - t0
    h1, d1 = lg.copy_bytes()
    split_ms = {"lg_create": (t1 - t0) * 1e3, "lg_load": (t2 - t1) * 1e3,
                "lg_run": (t3 - t2) * 1e3, "lg_observables": (t0 + e2e_s - t3) * 1e3}
    e.close()
    e2e_s = _reduce_max(dist, e2e_s)
    e_nop = obs["Number of Operators"][0]
    e2e = {"value": ws * args.steps * N_SITES / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": round((h1 - h0) / args.steps, 1),
           "d2h_bytes_per_step": round((d1 - d0) / args.steps, 1),
           "seconds": e2e_s, "split_ms": {k: round(v, 3) for k, v in split_ms.items()},
           "checkpoint_bytes": len(blob),
           "operators_per_sweep": e_nop, "operators_vs_device_timed": e_nop / nv_mean,
           "scope": "lg_create + lg_load(equilibrated checkpoint) + lg_run(steps) + "
                    "lg_observables, host wall clock; bytes counted by the library's copies"}
    cpu = None
    if rank == 0 and args.cpu_seconds > 0:
        state = w.state()
        r = cpu_port_rate(seconds=args.cpu_seconds, threads=1, state=state)
        cpu = {"value": r["rate"], "unit": UNIT, "cores": 1, "kind": "port",
               "cpu_model": cpu_model(), "operators_per_s": r["operators_per_s"],
               "mean_operators": r["mean_operators"],
               "sample": "%d sweeps of the same 128x128 beta=64 chain started from the GPU's "
                         "equilibrated state, %.1f s, 1 thread (CPU restatement of "
                         "path_integral.C in oracle/)" % (r["sweeps"], r["seconds"])}
    w.close()
    small_chain = _leg(run_small_chain, lg) if rank == 0 and args.small_chain else None
    batched = None
    if rank == 0 and args.batched_steps > 0:
        batched = _leg(run_batched, lg, args.batched_steps, args.batched_therm)
    replicas = None
    if rank == 0 and args.replica_steps > 0:
        replicas = _leg(run_replicas, lg, args.replica_steps, args.replica_therm)
    served = None
    if rank == 0 and args.served_requests > 0:
        served = _leg(run_served, lg, args.served_requests)
    if rank != 0:
        return None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "int64 (FP64 times on a 2^-52 grid; exponential gaps from float -ln U, U a "
                 "23-bit uniform refined by 23 more bits in its lowest bin)",
        "data": "synthetic (seeded Philox streams; iid random initial spins)",
        "config": {"workload": WORKLOAD, "lattice": "square", "L": L_SIDE, "beta": BETA,
                   "J": 1.0, "seed": SEED, "step": "one sweep",
                   "pre_thermalization_sweeps": PRE_THERM, "launch_shape": shape,
                   "l2": ("flushed between steps (%d MiB device write, untimed)" % (args.flush_bytes >> 20)
                          if args.flush_bytes else "NOT flushed between steps (a profiling aid; "
                          "not a valid timed number)"),
                   "parallelism": "replicas" if ws > 1 else "single chain"},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
        "clocks": clocks,
        "small_chain": small_chain,
        "batched": batched,
        "replicas_field": replicas,
        "served": served,
        "observables": {"Energy Density": obs["Energy Density"][0],
                        "sweeps_measured": int(obs["count"]),
                        "note": "the e2e chain, from the equilibrated checkpoint"},
    }
    return out


def run_reference(args, dist, ws, rank, local):
    """The CPU loop-cluster update (the oracle's restatement of path_integral.C, same random
    streams) on every host core: one chain per thread, each equilibrated by ref_warmup sweeps
    (the operator count settles within about 12 sweeps from a random start at this size), then
    exactly `steps` timed sweeps per thread."""
    if rank != 0:
        return None
    threads = max(1, os.cpu_count() or 1)
    steps = max(1, args.steps)
    warm = max(1, args.ref_warmup)
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

    par(warm)
    for o in chains:
        o.clear_records()
    t0 = time.perf_counter()
    par(steps)
    el = time.perf_counter() - t0
    ops = sum(int(o.records()[:, 0].sum()) for o in chains)
    value = threads * steps * N_SITES / el
    for o in chains:
        o.close()
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp64 times", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "lattice": "square", "L": L_SIDE, "beta": BETA,
                   "J": 1.0, "seed": SEED, "step": "one sweep",
                   "parallelism": "one chain per host thread (%d threads, seeds %d + 1000 i)"
                                  % (threads, SEED)},
        "operators_per_s": ops / el, "mean_operators": ops / (threads * steps),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "cpu_model": cpu_model(),
                         "sample": "%d threads x %d sweeps, each thread's chain equilibrated by %d "
                                   "sweeps from a random start (the reference's path_integral "
                                   "binary needs ALPS and does not build here)"
                                   % (threads, steps, warm)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=512)
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--small-chain", type=int, default=1,
                    help="run the CPU-runnable chain workload (L=64 chain, beta=10)")
    ap.add_argument("--batched-steps", type=int, default=16)
    ap.add_argument("--batched-therm", type=int, default=128)
    ap.add_argument("--replica-steps", type=int, default=8)
    ap.add_argument("--replica-therm", type=int, default=32)
    ap.add_argument("--served-requests", type=int, default=4096)
    ap.add_argument("--ref-warmup", type=int, default=16,
                    help="equilibrating sweeps per thread before the reference arm's timed ones")
    ap.add_argument("--flush-bytes", type=int, default=FLUSH_BYTES,
                    help="device bytes written between the headline's timed steps to flush the L2 "
                         "(0 only to compare DRAM traffic under a profiler)")
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
