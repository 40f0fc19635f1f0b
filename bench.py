"""Benchmark: node-days/s of the GPU ssm solver on the SEIR-with-events
workload (1,000,000 nodes x 365 days, 730k enter/exit and 182.5M external
transfer events), one JSON line on stdout.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--scale S] [--no-e2e] [--no-cpu] [--batch R] [--abc N]
                  [--serve-seconds T] [--serve-rate R]

Beside the plain run the line carries the batched forms: `batched` (R
replicates of the workload in one plan), `abc` (N uneven ABC proposals as
one batch with on-device distances, against one run per proposal),
`pfilter` (the 4,096-particle SISe particle filter) and `serve` (an
open-loop request trace through the serving loop, p50/p99 latency, against
serving the same trace one request at a time).
The secondary legs time the "next" paths on their own inputs:
`reductions` (prevalence and trajectory of the resident U), `event_sort`
(the schedule's ordering), `individual_events` (the individual-event
cleaner on a synthetic livestock register), `aem` (the all-events solver).

A step is one full run of the workload's horizon.  `value` times K steps of
siminf_gpu_plan_run with every input already resident in HBM (CUDA events on
the launching stream); `e2e` times K calls of the C ABI entry point
siminf_gpu_run_solver_ex with host buffers (planning, host->device copies,
solve, device->host copy of U inside the timed region).  The state (U alone
is 5.84 GB) is far larger than the 129 MB L2, so no flush is needed between
steps.  `--impl reference` times the reference algorithm on every host core
(the oracle's C port of the ssm solver with OpenMP, whose parity with the
reference's own sources is tested where those compile) on the same whole
workload, one run per step; the port, not those sources, because the
workload needs capped transfer sizes, which the reference does not have.
`cpu_baseline` is one such run inside this arm.  `untruncated` runs the
same generator with the destination power law left uncut, at a tenth of
the size, on the GPU and on the host cores: there one hub's chain of
transitions sets the length of every day.

With N > 1 (torchrun) every rank runs an independent replica of the
workload with its own seed (the path has no data exchange between
replicates); value = node-days of all ranks / max-over-ranks time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "node-days/s"
UNIT = "node-days/s"
# Algorithmic HBM bytes per node-day of this workload: one U column entry
# (4 compartments x 4 B) + events read (0.504 events per node-day x 36 B).
ALGO_BYTES_PER_NODE_DAY = 16 + 0.504 * 36
# DRAM traffic of one k_ssa_e1 launch (dram__bytes_read.sum +
# dram__bytes_write.sum) measured by ncu on this workload at its full node
# count (10^6 nodes, day 110 of a 120-day run: 93.3 MB read, 10.6 MB
# written), per node; another node count moves that much per node.
SSA_TRAFFIC_BYTES_PER_NODE = (93.299968e6 + 10.620928e6) / 1_000_000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=float, default=1.0,
                    help="fraction of the 1e6 nodes / 5e5 transfers per day (1.0 = full)")
    ap.add_argument("--days", type=int, default=365)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--batch", type=int, default=16,
                    help="replicates of the workload run as one batched plan (0/1: skip)")
    ap.add_argument("--batch-steps", type=int, default=2)
    ap.add_argument("--abc", type=int, default=256,
                    help="ABC proposals (uneven models) run as one batch and one by one (0: skip)")
    ap.add_argument("--pfilter", type=int, default=4096,
                    help="particles of the particle-filter workload (0: skip)")
    ap.add_argument("--serve-full", action="store_true",
                    help="serve the request mix at its stated sizes (plain path: first 10 s)")
    ap.add_argument("--abc-smc", type=int, default=0,
                    help="generations of the ABC-SMC run over uneven models (0: off)")
    ap.add_argument("--abc-smc-quantile", type=float, default=0.5,
                    help="quantile of the accepted distances that sets the next tolerance")
    ap.add_argument("--serve-seconds", type=float, default=5.0,
                    help="length of the open-loop serving trace (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="arrivals per second")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-scale", type=float, default=1.0,
                    help="workload fraction of the CPU baseline's run (1.0: the whole "
                         "workload, about 15 s on 16 cores)")
    ap.add_argument("--no-untruncated", dest="untruncated", action="store_false",
                    help="skip the run on the untruncated power-law graph")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.samples = []
        self.proc = None
        self.index = index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, name in enumerate(names):
                if len(s) > 4 + k and s[4 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def measured_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_baseline(scale, days, threads, seed=42, m=None):
    """The reference algorithm on the host cores: one run of the workload
    (the model m when given, else the workload at `scale` of its nodes and
    transfers); returns (node-days/s, transitions/s, seconds, kind, result)."""
    from siminf_gb300 import abi, workloads
    from oracle import oracle
    if m is None:
        m = workloads.seir_events(nodes=max(1, int(1_000_000 * scale)), days=days,
                                  transfers=max(1, int(500_000 * scale)))
    h = abi.build_args(m, seed)
    t0 = time.perf_counter()
    code, res = oracle.run(h, m.name, threads, cap_transfers=True)
    dt = time.perf_counter() - t0
    if code:
        raise RuntimeError("oracle failed with %d" % code)
    return res.node_days / dt, res.transitions / dt, dt, "port", res


def abc_bench(n, seed=11):
    """The ABC workload: n proposals over uneven models (node counts 100 to
    50,000, 60 to 365 days, events scaled to size), run as one batch with the
    prevalence distance on the device, and one run() per proposal."""
    from siminf_gb300 import workloads
    from siminf_gb300.run import run, run_batch
    models, seeds = workloads.abc_models(n, seed=seed)
    node_days = sum(m.Nn * len(m.tspan) for m in models)
    tmax = max(len(m.tspan) for m in models)
    target = np.linspace(0.0, 0.05, tmax)
    targets = [target[:len(m.tspan)] for m in models]
    run_batch(models, seeds, targets, cap_transfers=True)         # warm-up
    ts = []
    for _ in range(2):
        t0 = time.perf_counter()
        run_batch(models, seeds, targets, cap_transfers=True)
        ts.append(time.perf_counter() - t0)
    tb = min(ts)
    t0 = time.perf_counter()
    for m, sd in zip(models, seeds):
        run(m, seed=sd, cap_transfers=True)
    tp = time.perf_counter() - t0
    return {"models": n, "node_days": int(node_days), "value": node_days / tb, "unit": UNIT,
            "seconds": tb, "one_run_per_model_value": node_days / tp,
            "one_run_per_model_seconds": tp, "vs_one_run_per_model": tp / tb,
            "data": "synthetic ABC proposals: SEIR, node counts {100,1e3,1e4,5e4} w.p. "
                    "{.4,.3,.2,.1}, 60-365 days, events scaled to size, prior draws; "
                    "end to end through the C ABI (host buffers)"}


def sir_plain_bench(threads):
    """The small plain case: mparse SIR, 1,000 nodes of (S=99, I=5, R=0),
    beta=0.16, gamma=0.077, tspan 1:150, no events, seed 42; run() end to
    end against the oracle port on the host cores.  Latency-bound (one
    k_horizon launch); reported, not optimised for."""
    from siminf_gb300 import abi, workloads
    from siminf_gb300.run import run
    from oracle import oracle
    m = workloads.sir_plain()
    run(m, seed=42)
    ts = []
    for _ in range(5):
        t0 = time.perf_counter()
        r = run(m, seed=42)
        ts.append(time.perf_counter() - t0)
    dt = min(ts)
    node_days = m.Nn * len(m.tspan)
    h = abi.build_args(m, 42)
    t0 = time.perf_counter()
    code, res = oracle.run(h, m.name, threads)
    dc = time.perf_counter() - t0
    return {"nodes": m.Nn, "days": len(m.tspan), "value": node_days / dt, "unit": UNIT,
            "ms": dt * 1e3, "transitions": int(r.stats.transitions),
            "cpu_baseline": {"value": node_days / dc, "unit": UNIT, "ms": dc * 1e3,
                             "cores": threads, "kind": "port",
                             "sample": "the whole case"},
            "data": "synthetic SIR (mparse) 1,000 nodes x 150 days, end to end"}


def pfilter_bench(particles):
    """The particle-filter workload: SISe with phi, 500 nodes per particle,
    52 weekly Binomial(I, 0.8) observations from a ground-truth run (seed 7),
    per-particle upsilon and gamma; one filter pass through the C ABI."""
    from siminf_gb300 import workloads
    from siminf_gb300.run import pfilter
    m, gdata, t_obs, obs = workloads.sise_pfilter(nodes=500, particles=particles, weeks=52)
    pfilter(m, particles, t_obs, obs, 1, 0.8, seed=3, gdata=gdata)      # warm-up
    ts, res = [], None
    for _ in range(2):
        t0 = time.perf_counter()
        res = pfilter(m, particles, t_obs, obs, 1, 0.8, seed=3, gdata=gdata)
        ts.append(time.perf_counter() - t0)
    dt = min(ts)
    node_days = particles * m.Nn * int(t_obs[-1])
    return {"particles": particles, "nodes": m.Nn, "observations": len(t_obs),
            "node_days": int(node_days), "value": node_days / dt, "unit": UNIT,
            "seconds": dt, "loglik": res.loglik,
            "data": "synthetic SISe particle filter (phi pts), end to end through the C ABI"}


def serve_bench(seconds, rate, seed=5, full=False, plain_seconds=None):
    """Open-loop Poisson arrivals of a request mix (60% SIR runs, 100-20,000
    nodes log-uniform, 30-365 days; 30% particle filters on the SISe model,
    256-4,096 particles; 10% SEIR-with-events runs, 10,000-200,000 nodes)
    served by the request loop, and the same trace served one request at a
    time (the plain path).  By default particle filters use 40 nodes and 6
    weekly observations and SEIR runs 30 days so the trace stays inside a
    minute; full=True takes the stated sizes (500 nodes x 52 weeks, SEIR
    over 365 days), and the plain path then serves only the first
    plain_seconds of the trace."""
    from siminf_gb300 import model as M
    from siminf_gb300 import workloads
    from siminf_gb300.run import pfilter, run
    from siminf_gb300.serve import Server
    rng = np.random.default_rng(seed)
    pool_sir = []
    for _ in range(12):
        n = int(np.exp(rng.uniform(np.log(100), np.log(20000))))
        days = int(rng.integers(30, 366))
        u0 = {"S": np.full(n, 99), "I": np.full(n, 5), "R": np.zeros(n, int)}
        pool_sir.append(M.SIR_mparse(u0, np.arange(1, days + 1), 0.16, 0.077))
    pool_pf = []
    for k in range(4):
        pm, gdata, t_obs, obs = workloads.sise_pfilter(nodes=500 if full else 40, particles=4096,
                                                       weeks=52 if full else 6, seed=7 + k)
        pool_pf.append((pm, gdata, t_obs, obs))
    pool_seir = [workloads.seir_events_fast(n, 365 if full else 30, n // 2, rng)
                 for n in (10000, 60000, 200000)]
    trace, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            break
        r = rng.random()
        kind = "sir" if r < 0.6 else ("pf" if r < 0.9 else "seir")
        trace.append((t, kind, int(rng.integers(0, 1 << 30)),
                      int(rng.integers(256, 4097)) if kind == "pf" else 0,
                      int(rng.integers(0, 12 if kind == "sir" else
                                       (4 if kind == "pf" else 3)))))

    def node_days(kind, np_, k):
        if kind == "sir":
            return pool_sir[k].Nn * len(pool_sir[k].tspan)
        if kind == "pf":
            return np_ * pool_pf[k][0].Nn * int(pool_pf[k][2][-1])
        return pool_seir[k].Nn * len(pool_seir[k].tspan)

    total_nd = sum(node_days(kind, n_p, k) for _, kind, _, n_p, k in trace)

    def submit(srv, kind, sd, n_p, k):
        if kind == "sir":
            return srv.run(pool_sir[k], seed=sd)
        if kind == "pf":
            pm, gdata, t_obs, obs = pool_pf[k]
            return srv.pfilter(pm, n_p, t_obs, obs, 1, 0.8, seed=sd, gdata=gdata[:n_p])
        return srv.run(pool_seir[k], seed=sd, cap_transfers=True)

    srv = Server(slots=8, hbm_budget_bytes=150 * 10 ** 9)
    for kind, k in (("sir", 0), ("pf", 0), ("seir", 0)):
        srv.wait(submit(srv, kind, 1, 256, k))                     # warm-up
    # Finished requests are collected while the trace runs and their
    # outputs dropped (a SEIR request of 200,000 nodes x 365 days returns
    # 1.2 GB of U).  At the stated sizes the offered load is several times
    # what one GPU serves, so the backlog's result buffers are bounded: a
    # request whose arrival would take the outstanding U bytes above
    # max_backlog_bytes is submitted when enough earlier ones finish.
    # Latency is counted from the request's arrival time in the trace, so
    # that wait is part of it.
    def out_bytes(kind, k):
        if kind == "sir":
            return pool_sir[k].Nn * pool_sir[k].Nc * len(pool_sir[k].tspan) * 4
        if kind == "seir":
            return pool_seir[k].Nn * pool_seir[k].Nc * len(pool_seir[k].tspan) * 4
        return 0

    max_backlog_bytes = 16 * 10 ** 9
    t0 = time.perf_counter()
    live, lat = [], []
    backlog = [0]
    held_s = 0.0

    def reap():
        still = []
        for tk, at, t_sub, nb in live:
            if tk.finished:
                srv.wait(tk)                # raises on the request's error
                lat.append((t_sub - at) * 1e3 + tk.latency_ms)
                backlog[0] -= nb
                tk.holder = tk.model = None
                tk.keep = []
            else:
                still.append((tk, at, t_sub, nb))
        live[:] = still

    t_log = 0.0
    for at, kind, sd, n_p, k in trace:
        nb = out_bytes(kind, k)
        if full and at >= t_log:
            print("serve: t %.0f s of the trace, %d served, %d in flight, %.1f GB of results "
                  "held, %.0f s elapsed" % (at, len(lat), len(live), backlog[0] / 1e9,
                                            time.perf_counter() - t0),
                  file=sys.stderr, flush=True)
            t_log += 10.0
        while True:
            reap()
            now = time.perf_counter() - t0
            if at <= now and (backlog[0] + nb <= max_backlog_bytes or not live):
                break
            time.sleep(min(max(at - now, 0.0), 0.002) or 0.002)
        t_sub = time.perf_counter() - t0
        held_s = max(held_s, t_sub - at)
        backlog[0] += nb
        live.append((submit(srv, kind, sd, n_p, k), at, t_sub, nb))
    n_log = 0
    while live:
        reap()
        if full and len(lat) >= n_log:
            print("serve: trace submitted, %d served, %d in flight, %.0f s elapsed"
                  % (len(lat), len(live), time.perf_counter() - t0), file=sys.stderr, flush=True)
            n_log = len(lat) + 1000
        time.sleep(0.001)
    served_s = time.perf_counter() - t0
    lat = np.array(lat)
    srv.close()

    # plain path: the same trace, one request at a time on the caller's thread
    plain_trace = trace if plain_seconds is None else [x for x in trace if x[0] <= plain_seconds]
    plain_nd = sum(node_days(kind, n_p, k) for _, kind, _, n_p, k in plain_trace)
    if full:
        print("serve: served in %.0f s; plain path over %d requests" % (served_s, len(plain_trace)),
              file=sys.stderr, flush=True)
    t0 = time.perf_counter()
    plain_lat = []
    for at, kind, sd, n_p, k in plain_trace:
        now = time.perf_counter() - t0
        if at > now:
            time.sleep(at - now)
        if kind == "sir":
            run(pool_sir[k], seed=sd)
        elif kind == "pf":
            pm, gdata, t_obs, obs = pool_pf[k]
            pfilter(pm, n_p, t_obs, obs, 1, 0.8, seed=sd, gdata=gdata[:n_p])
        else:
            run(pool_seir[k], seed=sd, cap_transfers=True)
        plain_lat.append((time.perf_counter() - t0 - at) * 1e3)
    plain_s = time.perf_counter() - t0
    plain_lat = np.array(plain_lat)
    return {"requests": len(trace), "rate_per_s": rate, "trace_seconds": seconds,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "value": total_nd / served_s, "unit": UNIT, "seconds": served_s,
            "plain_p50_ms": float(np.percentile(plain_lat, 50)),
            "plain_p99_ms": float(np.percentile(plain_lat, 99)),
            "plain_value": plain_nd / plain_s, "plain_seconds": plain_s,
            "plain_requests": len(plain_trace),
            "slots": 8, "hbm_budget_bytes": 150 * 10 ** 9, "stated_sizes": bool(full),
            "max_backlog_bytes": max_backlog_bytes, "max_submit_delay_s": held_s,
            "node_days": int(total_nd),
            "data": "synthetic request mix, open-loop Poisson arrivals; latency from "
                    "submission to completion; plain = one request at a time"}


def abc_smc_bench(generations, n_particles=2048, seed=3, batch=512, quantile=0.5):
    """ABC-SMC over uneven models (config 4): particles' node counts from
    {100, 1e3, 1e4, 5e4} w.p. {.4, .3, .2, .1}, tspans U{60, 365}, events as
    the headline's scaled to size (a pool of 64 such structures, each
    proposal taking one with its own parameters and seed); priors beta ~
    U(0.05, 0.5), epsilon ~ U(0.1, 0.5), gamma ~ U(0.02, 0.2); distance: the
    L2 norm of daily prevalence I/N against one seeded target run (10,000
    nodes, 365 days, beta 0.16, epsilon 0.25, gamma 0.077, seed 7).  First
    tolerance from 2 n_particles prior draws, then the `quantile` rule (the median by default)
    (siminf_gb300/abc.py); proposals in batches of `batch` models (each
    model averages ~0.8M events, so a batch of 512 holds ~4e8)."""
    import copy
    from siminf_gb300 import abc, workloads
    from siminf_gb300 import model as M
    from siminf_gb300.run import run, run_batch
    rng = np.random.default_rng(seed)
    pool = []
    for _ in range(64):
        Nn = int(rng.choice((100, 1000, 10000, 50000), p=(0.4, 0.3, 0.2, 0.1)))
        T = int(rng.integers(60, 366))
        pool.append(workloads.seir_events_fast(Nn, T, max(1, Nn // 2), rng))
    truth = workloads.seir_events_fast(10000, 365, 5000, np.random.default_rng(7))
    r = run(truth, seed=7, cap_transfers=True)
    I = r.U[2::4].sum(axis=0).astype(float)         # rows: node * 4 + compartment
    N = r.U.sum(axis=0).astype(float)
    target = np.where(N > 0, I / np.maximum(N, 1.0), 0.0)

    def simulate(theta, g):
        models, seeds, targets = [], [], []
        for b, e, gm in theta:
            s = copy.copy(pool[int(g.integers(0, len(pool)))])
            s.ldata = M._rep_ldata(s.Nn, b, e, gm)
            models.append(s)
            seeds.append(int(g.integers(1, 2 ** 62)))
            targets.append(target[:len(s.tspan)])
        return models, seeds, targets

    priors = [abc.Prior("beta", "uniform", 0.05, 0.5), abc.Prior("epsilon", "uniform", 0.1, 0.5),
              abc.Prior("gamma", "uniform", 0.02, 0.2)]
    pm0, ps0, pt0 = simulate(abc.proposals(priors, 8, rng)[0], rng)
    run_batch(pm0, ps0, pt0, cap_transfers=True)             # warm-up
    t0 = time.perf_counter()
    gens = abc.abc_smc(simulate, priors, n_particles, generations, batch=batch,
                       n_init=2 * n_particles, seed=seed, verbose=True, quantile=quantile)
    dt = time.perf_counter() - t0
    nd = sum(g.node_days for g in gens)
    return {"generations": generations, "particles": n_particles, "batch": batch, "seconds": dt,
            "tolerance_quantile": quantile,
            "node_days": int(nd), "value": nd / dt, "unit": UNIT,
            "per_generation": [{"tolerance": g.tolerance, "proposals": g.nprop,
                                "ess": g.ess, "seconds": g.seconds,
                                "posterior_mean": [float(v) for v in
                                                   np.average(g.x, axis=0, weights=g.w)]}
                               for g in gens],
            "data": "config-4 ABC-SMC: synthetic uneven SEIR models with events, prior "
                    "proposals and SMC perturbations, distances on the device; end to end "
                    "through the C ABI (host buffers)"}


UNTRUNCATED_SCALE = 0.1


def untruncated_workload():
    """The headline generator with the destination power law left
    untruncated (exponent 2.1 on [1, inf)), at a tenth of the nodes and
    transfers: a few hubs collect most of the population and one node's
    chain of transitions sets the length of every day."""
    from siminf_gb300 import workloads
    return workloads.seir_events(nodes=int(1_000_000 * UNTRUNCATED_SCALE),
                                 transfers=int(500_000 * UNTRUNCATED_SCALE), cutoff=np.inf)


def untruncated_cpu(threads, m=None):
    m = m if m is not None else untruncated_workload()
    v, tr, dt, kind, res = cpu_baseline(UNTRUNCATED_SCALE, 365, threads, m=m)
    return {"value": v, "unit": UNIT, "ms": dt * 1e3, "cores": threads, "kind": kind,
            "transitions": int(res.transitions)}


def untruncated_bench(torch, C, stream, threads, cpu=True):
    """The untruncated graph on the GPU (resident plan, tuned as the
    headline) and on the host cores, with the run's critical path."""
    from siminf_gb300 import abi, native
    m = untruncated_workload()
    h = abi.build_args(m, 42)
    p = native.Plan(h, m.name, cap_transfers=True)
    s = C.c_void_p(stream.cuda_stream)
    p.run(s)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    p.run(s)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    dmax = p.day_max(s)
    nd = m.Nn * p.stats().days
    out = {"nodes": m.Nn, "days": 365, "transfers_per_day": int(500_000 * UNTRUNCATED_SCALE),
           "value": nd / (ms / 1e3), "unit": UNIT, "ms": ms,
           "critical_path_transitions": int(dmax.sum()),
           "us_per_critical_transition": ms * 1e3 / max(1, int(dmax.sum())),
           "graph": "destination weights power law 2.1 on [1, inf), no cutoff",
           "cpu_baseline": untruncated_cpu(threads, m) if cpu else None}
    p.close()
    return out


def workload_config(args, m, st_days, e2_waves=None):
    """The config object both arms print for the headline workload."""
    nodes = max(1, int(1_000_000 * args.scale))
    transfers = max(1, int(500_000 * args.scale))
    cfg = {"workload": "seir_events_%dx%d" % (nodes, args.days) if args.scale != 1.0
           else "seir_events_1e6x365",
           "nodes": nodes, "days": st_days, "transfers_per_day": transfers,
           "events": int(len(m.events["event"])), "cap_transfers": True,
           "graph": "uniform sources, destination weights power law 2.1 cut at sqrt(edges)"}
    if e2_waves is not None:
        cfg["e2_waves"] = e2_waves
    return cfg


def run_reference(args):
    """The reference arm: the reference algorithm (the oracle's C port of
    the ssm solver with OpenMP over nodes and the serial external-transfer
    phase, bit-identical to the reference's own sources where those
    compile) on every host core, on the same full workload as the GPU arm:
    one step is one whole run of the horizon.  A CPU run has nothing to
    warm up beyond its first (page faults, the thread pool), so at most one
    warm-up run is made whatever --warmup says, which keeps the arm within
    minutes at about 15 s per run on 16 cores."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    from oracle import oracle
    from siminf_gb300 import workloads
    oracle.build()
    nodes = max(1, int(1_000_000 * args.scale))
    transfers = max(1, int(500_000 * args.scale))
    m = workloads.seir_events(nodes=nodes, days=args.days, transfers=transfers)
    for _ in range(min(args.warmup, 1)):
        cpu_baseline(args.scale, args.days, threads, m=m)
    vals, trans, secs = [], [], []
    for _ in range(args.steps):
        v, tr, dt, kind, res = cpu_baseline(args.scale, args.days, threads, m=m)
        vals.append(v)
        trans.append(tr)
        secs.append(dt)
    ms = float(np.mean(secs)) * 1e3
    value = res.node_days / (ms / 1e3)
    sample = ("the whole workload (%d nodes, %d days, %d transfers/day), cap_transfers on, "
              "%d threads, one run per step" % (nodes, args.days, transfers, threads))
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": min(args.warmup, 1),
        "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32 state, f64 rates",
        "data": "synthetic",
        "config": workload_config(args, m, args.days),
        "transitions_per_s": float(np.mean(trans)),
        "transitions_per_step": int(res.transitions),
        "serial_e2_ms_per_step": res.seconds_e2 * 1e3,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "untruncated": dict(untruncated_cpu(threads),
                            graph="destination weights power law 2.1 on [1, inf), no cutoff",
                            nodes=int(1_000_000 * UNTRUNCATED_SCALE)),
    }
    print(json.dumps(out), flush=True)


def replica_seed(rank):
    """Each rank simulates its own replica of the workload with its own
    seed: the path has no exchange between replicates."""
    return 42 + rank


def max_over_ranks(x, torch, world, device):
    """The largest of every rank's x: a job's time is its slowest rank's."""
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, ms):
    """Whole-job throughput: the units of every rank over the slowest
    rank's time (ms)."""
    return units_per_rank * world / (ms / 1e3)


def run_ours(args):
    import ctypes as C
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from siminf_gb300 import abi, build, native, workloads
    build.build()
    nodes = max(1, int(1_000_000 * args.scale))
    transfers = max(1, int(500_000 * args.scale))
    seed = replica_seed(rank)
    t_gen = time.perf_counter()
    m = workloads.seir_events(nodes=nodes, days=args.days, transfers=transfers)
    t_gen = time.perf_counter() - t_gen
    holder = abi.build_args(m, seed)
    stream = torch.cuda.current_stream()
    plan = native.Plan(holder, m.name, cap_transfers=True)
    st = plan.stats()
    node_days = nodes * st.days
    # the library's autotuner picks the work queue's layout (heavy
    # threshold, one- or two-pass days) on the whole horizon: the epidemic
    # peaks after the first months, where the heavy part matters (results
    # do not depend on the layout)
    tune = plan.tune(probe_days=args.days, stream=C.c_void_p(stream.cuda_stream))
    autotune = tune_summary(tune)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        plan.run(C.c_void_p(stream.cuda_stream))
    barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            plan.run(C.c_void_p(stream.cuda_stream))
        ev1.record(stream)
        barrier()
    ms = ev0.elapsed_time(ev1)
    st = plan.stats()
    ms = max_over_ranks(ms, torch, world, "cuda")
    ms_step = ms / args.steps
    value = job_rate(node_days, world, ms_step)
    transitions_per_s = job_rate(st.transitions, world, ms_step)
    # dominant kernel: per-kernel device time from the library's own
    # per-launch events (one step), see roofline below; its launch counts
    # are the launches of one step
    prof = plan_kernel_profile(plan, C, stream)
    launches = sum(k["launches"] for k in (prof["kernels"] or {}).values())
    # the run's critical path: every day lasts at least as long as its
    # busiest node's chain of transitions (one recording run)
    critical = None
    if prof["kernels"] and "k_ssa_e1" in prof["kernels"]:
        dmax = plan.day_max(C.c_void_p(stream.cuda_stream))
        ssa_ms = prof["kernels"]["k_ssa_e1"]["ms"]
        critical = {"transitions": int(dmax.sum()), "k_ssa_e1_ms": ssa_ms,
                    "us_per_critical_transition": ssa_ms * 1e3 / max(1, int(dmax.sum())),
                    "note": "sum over days of the most transitions one node fired that "
                            "day; k_ssa_e1 time / that sum is the time per step of the "
                            "busiest chain, which GB300's FP64 latency (64 cycles per "
                            "dependent operation) bounds from below"}
    peak, peak_kind = measured_peaks()
    reductions = reduce_bench(plan, peak) if rank == 0 else None
    event_sort = events_bench(m, peak) if rank == 0 and world == 1 else None
    individual = (individual_bench(peak, os.cpu_count() or 1, cpu=not args.no_cpu)
                  if rank == 0 and world == 1 else None)
    # the aem leg's CPU sample stays at 5% of the workload: the oracle's
    # aem is a secondary baseline and a whole run would add half a minute
    aem = (aem_bench(m, node_days, torch, C, stream, os.cpu_count() or 1,
                     0.0 if args.no_cpu else min(args.cpu_scale, 0.05))
           if rank == 0 and world == 1 else None)

    # batched form: R replicates of the same workload in one device-resident
    # plan (the mssm layout), so one replicate's latency-bound tail overlaps
    # the others' work
    batched = None
    if args.batch > 1:
        mb = m.replicate(args.batch)
        hb = abi.build_args(mb, seed)
        pb = native.Plan(hb, mb.name, cap_transfers=True)
        # tuned over the whole horizon too: a 120-day probe ranks the heavy
        # thresholds the other way round from the year (threshold 8 ahead
        # on 120 days, 17% behind threshold 32 over 365)
        tune_b = tune_summary(pb.tune(probe_days=args.days,
                                      stream=C.c_void_p(stream.cuda_stream)))
        pb.run(C.c_void_p(stream.cuda_stream))
        barrier()
        b0 = torch.cuda.Event(enable_timing=True)
        b1 = torch.cuda.Event(enable_timing=True)
        b0.record(stream)
        for _ in range(args.batch_steps):
            pb.run(C.c_void_p(stream.cuda_stream))
        b1.record(stream)
        barrier()
        msb = b0.elapsed_time(b1) / args.batch_steps
        stb = pb.stats()
        vb = args.batch * node_days * world / (msb / 1e3)
        batched = {"replicates": args.batch, "value": vb, "unit": UNIT, "ms_per_step": msb,
                   "steps": args.batch_steps, "warmup": 1,
                   "transitions_per_s": stb.transitions * world / (msb / 1e3),
                   "vs_plain": vb / value, "autotune": tune_b,
                   "data": "%d replicates of the same synthetic workload in one plan "
                           "(mssm), inputs resident" % args.batch}
        pb.close()
        del hb, mb

    sir = sir_plain_bench(os.cpu_count() or 1) if rank == 0 and world == 1 else None
    abc = abc_bench(args.abc) if args.abc > 0 and rank == 0 and world == 1 else None
    pf = (pfilter_bench(args.pfilter)
          if args.pfilter > 0 and rank == 0 and world == 1 else None)
    serve = (serve_bench(args.serve_seconds, args.serve_rate, full=args.serve_full,
                         plain_seconds=10.0 if args.serve_full else None)
             if args.serve_seconds > 0 and rank == 0 and world == 1 else None)
    abc_smc = (abc_smc_bench(args.abc_smc, quantile=args.abc_smc_quantile)
               if args.abc_smc > 0 and rank == 0 and world == 1 else None)

    e2e = None
    if not args.no_e2e:
        opt = abi.Options(cap_transfers=1)
        dm = native.device_model(m.name)
        # pinned host copies of the step's inputs and outputs
        pin = pinned_holder(m, seed, torch)
        lib = native.lib()
        for _ in range(1):
            native.check(lib.siminf_gpu_run_solver_ex(C.cast(pin.ref(), C.c_void_p), dm.handle,
                                                      C.byref(opt)))
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            native.check(lib.siminf_gpu_run_solver_ex(C.cast(pin.ref(), C.c_void_p), dm.handle,
                                                      C.byref(opt)))
        barrier()
        dt = max_over_ranks((time.perf_counter() - t0) / args.steps, torch, world, "cuda")
        h2d = (m.u0.nbytes + sum(v.nbytes for v in m.events.values()) +
               m.ldata.nbytes)
        d2h = pin.U.nbytes
        e2e = {"value": job_rate(node_days, world, dt * 1e3), "unit": UNIT,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "ms_per_step": dt * 1e3}
        estats = native.last_stats()
        e2e["ms_upload"] = estats.ms_upload
        e2e["ms_plan"] = estats.ms_plan
        e2e["ms_solve"] = estats.ms_solve
        e2e["ms_download"] = estats.ms_download

    untrunc = (untruncated_bench(torch, C, stream, os.cpu_count() or 1, cpu=not args.no_cpu)
               if args.untruncated and rank == 0 and world == 1 else None)

    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        from oracle import oracle
        oracle.build()
        whole = args.cpu_scale >= 1.0
        v, tr, dt, kind, res = cpu_baseline(args.cpu_scale, args.days, os.cpu_count() or 1,
                                            m=m if whole else None)
        cpu = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": kind,
               "sample": ("one run of the whole workload, %.1f s" % dt if whole else
                          "SEIR with events at %.3g scale (%d nodes, %d days), %.1f s" %
                          (args.cpu_scale, int(1e6 * args.cpu_scale), args.days, dt)),
               "transitions_per_s": tr}

    if rank == 0:
        top = prof["top"]
        achieved = None
        if top and top["ms_per_launch"] > 0:
            bytes_per_launch = ALGO_BYTES_PER_NODE_DAY * top["node_days_per_launch"]
            achieved = bytes_per_launch / (top["ms_per_launch"] / 1e3) / 1e9
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32 state, f64 rates", "data": "synthetic",
            "config": dict(workload_config(args, m, st.days, st.e2_waves),
                           l2="state and U (5.8 GB) exceed the 129 MB L2; no flush",
                           parallelism="replicas x%d" % world),
            "transitions_per_s": transitions_per_s,
            "transitions_per_step": int(st.transitions),
            "gpu_launches": launches * args.steps,
            "clocks": clk.summary(),
            "roofline": {"bound": "hbm", "kernel": top["name"] if top else None,
                         "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None,
                         "traffic": (SSA_TRAFFIC_BYTES_PER_NODE * nodes
                                     if top and top["name"] == "k_ssa_e1" else None),
                         "traffic_unit": "bytes per launch",
                         "algorithmic_bytes_per_launch": (ALGO_BYTES_PER_NODE_DAY * nodes),
                         "peak_source": peak_kind,
                         "note": "algorithmic bytes = %.1f B/node-day x node-days per launch; "
                                 "traffic measured by ncu at 10^6 nodes (day 110 of 120); "
                                 "the SSA kernel is bound by its serial chain, not HBM"
                                 % ALGO_BYTES_PER_NODE_DAY},
            "kernels": prof["kernels"],
            "autotune": autotune,
            "critical_path": critical,
            "reductions": reductions,
            "event_sort": event_sort,
            "individual_events": individual,
            "aem": aem,
            "batched": batched,
            "sir_plain": sir,
            "abc_smc": abc_smc,
            "abc": abc,
            "pfilter": pf,
            "serve": serve,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "untruncated": untrunc,
            "t_generate_s": t_gen,
        }
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def pinned_holder(m, seed, torch):
    """ArgsHolder whose inputs (u0, ldata, the event arrays) and output U
    live in pinned host memory, as the e2e timing asks."""
    import ctypes as C
    from siminf_gb300 import abi
    h = abi.build_args(m, seed)
    a = h.args

    def pinned(src):
        t = torch.from_numpy(np.ascontiguousarray(src)).pin_memory()
        h.keep.append(t)
        return t.numpy()

    def repoint(field, n, dtype, ctype):
        arr = np.ctypeslib.as_array(getattr(a, field), shape=(n,)).view(dtype)
        arr = pinned(arr)
        setattr(a, field, arr.ctypes.data_as(C.POINTER(ctype)))
        return arr

    for k in ("event", "time", "node", "dest", "n", "select", "shift"):
        repoint(k, a.len, np.int32, C.c_int)
    repoint("proportion", a.len, np.float64, C.c_double)
    repoint("u0", m.Nn * m.Nc * m.replicates, np.int32, C.c_int)
    repoint("ldata", max(1, m.Nld * m.Nn), np.float64, C.c_double)
    h.U = pinned(h.U)
    a.U = h.U.ctypes.data_as(C.POINTER(C.c_int))
    return h


def reduce_bench(plan, peak, reps=5):
    """The trajectory consumers on the resident U of the headline run:
    level-1 prevalence (I ~ .) and the long-format trajectory of I over
    every node; kernel time (CUDA events), achieved HBM GB/s against the
    measured peak, and the whole call with the result's copy to the host."""
    from siminf_gb300.trajectory import _outputs, prevalence_device, trajectory_device
    dU, _, ncol = _outputs(plan)
    a = plan.holder.args
    out = {}
    runs = {"prevalence_level1": lambda: prevalence_device(dU, a.Nn, a.Nc, ncol, 0b0100,
                                                           0b1111, 1),
            "trajectory_I": lambda: trajectory_device(dU, a.Nn, a.Nc, ncol, [3])}
    for name, fn in runs.items():
        fn()
        best = None
        for _ in range(reps):
            _, st = fn()
            if best is None or st.ms_kernel < best.ms_kernel:
                best = st
        moved = best.bytes_read + best.bytes_written
        gbs = moved / (best.ms_kernel / 1e3) / 1e9
        out[name] = {"ms_kernel": best.ms_kernel, "ms_total": best.ms_total,
                     "bytes_read": best.bytes_read, "bytes_written": best.bytes_written,
                     "achieved_gbs": gbs, "peak_gbs": peak, "frac": gbs / peak,
                     "bound": "hbm"}
    return out


def events_bench(m, peak, frac=0.1, seed=3):
    """The event table's ordering (SimInf_events, R/SimInf_events.R:396)
    on the device: the first tenth of the headline schedule, shuffled, sorted
    by siminf_gpu_sort_events; against numpy's stable lexsort of the same
    table on one host core."""
    from siminf_gb300.events import COLUMNS, sort_events
    n = int(len(m.events["time"]) * frac)
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n)
    ev = {k: np.asarray(m.events[k])[:n][perm] for k in COLUMNS}
    sort_events(ev)
    best = None
    for _ in range(3):
        _, st = sort_events(ev, stats=True)
        if best is None or st.ms_kernel < best.ms_kernel:
            best = st
    t0 = time.perf_counter()
    order = np.lexsort((ev["select"], ev["event"], ev["time"]))
    _ = {k: v[order] for k, v in ev.items()}
    cpu_ms = (time.perf_counter() - t0) * 1e3
    moved = best.bytes_read + best.bytes_written
    gbs = moved / (best.ms_kernel / 1e3) / 1e9
    return {"events": n, "ms_kernel": best.ms_kernel, "ms_total": best.ms_total,
            "bytes_moved": moved, "achieved_gbs": gbs, "peak_gbs": peak, "frac": gbs / peak,
            "bound": "hbm",
            "cpu_baseline": {"ms": cpu_ms, "cores": 1, "kind": "numpy stable lexsort",
                             "sample": "the same %d shuffled events" % n},
            "data": "first tenth of the headline schedule, shuffled; the sort kernels "
                    "(ms_kernel) and the call with every column's copies (ms_total)"}


def individual_bench(peak, threads, cpu=True, n_ind=2_500_000, n_nodes=200_000, seed=7):
    """The individual-event cleaner (SimInf_individual_events,
    src/misc/SimInf_individual_events.c) on a synthetic livestock register
    of n_ind animals (about 9.2e6 events, 185 MB of int32 columns, above the
    L2) through siminf_gpu_individual_events; against the oracle's
    restatement on all host cores (OpenMP over individuals, as the
    reference's one task per individual)."""
    from siminf_gb300.individual import longest_paths
    from siminf_gb300.workloads import livestock_register
    cols = livestock_register(n_ind, n_nodes, seed)
    n = len(cols[0])
    keep = longest_paths(*cols)
    best = None
    for _ in range(3):
        _, st = longest_paths(*cols, stats=True)
        if best is None or st.ms_kernel < best.ms_kernel:
            best = st
    moved = best.bytes_read + best.bytes_written
    gbs = moved / (best.ms_kernel / 1e3) / 1e9
    out = {"events": n, "individuals": n_ind, "kept": int(keep.sum()),
           "events_per_s": n / (best.ms_kernel / 1e3),
           "events_per_s_e2e": n / (best.ms_total / 1e3),
           "ms_kernel": best.ms_kernel, "ms_total": best.ms_total, "bytes_moved": moved,
           "achieved_gbs": gbs, "peak_gbs": peak, "frac": gbs / peak,
           "bound": "latency of the per-individual search; frac is against HBM",
           "data": "synthetic livestock register (%d animals, %d holdings, seed %d); "
                   "the two kernels (ms_kernel) and the call with its copies of the five "
                   "columns and keep (ms_total)" % (n_ind, n_nodes, seed)}
    if cpu:
        from oracle import oracle
        oracle.build()
        t0 = time.perf_counter()
        want, _ = oracle.individual_events(*cols, threads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"events_per_s": n / dt, "ms": dt * 1e3, "cores": threads,
                               "kind": "port", "sample": "the same %d events" % n,
                               "identical": bool(np.array_equal(want, keep))}
    return out


def aem_bench(m, node_days, torch, C, stream, threads, cpu_scale, seed=42):
    """The all-events method (solver = 1, src/solvers/SimInf_solver_aem.c)
    on the same workload, resident, with the oracle's aem on the host cores
    over the CPU baseline's sample beside it."""
    from siminf_gb300 import abi, native, workloads
    h = abi.build_args(m, seed, solver=1)
    p = native.Plan(h, m.name, cap_transfers=True)
    p.run(C.c_void_p(stream.cuda_stream))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    p.run(C.c_void_p(stream.cuda_stream))
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    st = p.stats()
    p.close()
    out = {"value": node_days / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
           "transitions_per_s": st.transitions / (ms / 1e3),
           "data": "the headline workload under the aem solver, inputs resident"}
    if cpu_scale > 0:
        from oracle import oracle
        oracle.build()
        ms_ = workloads.seir_events(nodes=max(1, int(1_000_000 * cpu_scale)), days=365,
                                    transfers=max(1, int(500_000 * cpu_scale)))
        hc = abi.build_args(ms_, seed, solver=1)
        t0 = time.perf_counter()
        code, res = oracle.run(hc, ms_.name, threads, cap_transfers=True)
        dt = time.perf_counter() - t0
        if code == 0:
            out["cpu_baseline"] = {"value": res.node_days / dt, "unit": UNIT, "cores": threads,
                                   "kind": "port", "sample": "aem at %.3g scale, %.1f s"
                                   % (cpu_scale, dt)}
    return out


def tune_summary(tune):
    """The autotuner's candidates, probe times and choice."""
    k = tune.chosen
    return {"probe_days": tune.probe_days, "cached": bool(tune.cached),
            "candidates": [{"heavy_rate": tune.heavy_rate[i], "two_pass": tune.two_pass[i],
                            "ssa_variant": tune.ssa_variant[i],
                            "wave_block": tune.wave_block[i],
                            "heavy_lanes": tune.heavy_lanes[i] or 32, "ms": tune.ms[i]}
                           for i in range(tune.n_candidates)],
            "chosen_heavy_rate": tune.heavy_rate[k], "chosen_two_pass": tune.two_pass[k],
            "chosen_ssa_variant": tune.ssa_variant[k], "chosen_wave_block": tune.wave_block[k],
            "chosen_heavy_lanes": tune.heavy_lanes[k] or 32}


def plan_kernel_profile(plan, C, stream):
    """Per-phase device time of one step from the library's profiling run."""
    from siminf_gb300 import native
    lib = native.lib()
    if not hasattr(lib, "siminf_gpu_plan_profile"):
        return {"top": None, "kernels": None}
    prof = (C.c_double * 8)()
    cnt = (C.c_longlong * 8)()
    lib.siminf_gpu_plan_profile.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                                            C.POINTER(C.c_longlong)]
    lib.siminf_gpu_plan_profile.restype = C.c_int
    native.check(lib.siminf_gpu_plan_profile(plan.handle, C.c_void_p(stream.cuda_stream),
                                             prof, cnt))
    names = ["k_init", "k_ssa_e1", "k_e2_wave+k_e2_tail", "k_pts_store", "k_horizon", "k_quick"]
    kernels = {n: {"ms": prof[i], "launches": int(cnt[i])} for i, n in enumerate(names)
               if cnt[i] > 0}
    total = sum(k["ms"] for k in kernels.values()) or 1.0
    for k in kernels.values():
        k["share"] = k["ms"] / total
    top_name = max(kernels, key=lambda n: kernels[n]["ms"]) if kernels else None
    top = None
    if top_name:
        st = plan.stats()
        nodes = plan.holder.args.Nn * plan.holder.args.Nrep
        launches = kernels[top_name]["launches"]
        per_launch_nd = nodes * st.days / launches if top_name != "k_e2_wave+k_e2_tail" else 0
        top = {"name": top_name, "ms_per_launch": kernels[top_name]["ms"] / launches,
               "node_days_per_launch": per_launch_nd}
    return {"top": top, "kernels": kernels}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
