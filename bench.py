"""Throughput benchmark of the particle hot path on one GB300.

Default workload (N=1): the served job stream -- Poisson-arriving jobs
(exactly 50 % granular cooling gases of 100..200000 spheres, 25 % two-sphere
Hertz rebounds, 25 % LJ FCC melts of 500..100000 atoms; 1000..50000 steps
each) advanced by the continuous-batching server (mdg_server_*) in mixed
precision.  A "step" is one server pump: admission of the jobs that arrived,
one multi-step device launch (200 timesteps) over every resident job,
retirement of finished jobs.  The timed window is K pumps of the steady state
while jobs keep arriving (default pumps 10..90 of a 384-job stream arriving
at 4 per pump); value = particle-steps advanced inside it / CUDA-event time
on the server's stream.  Reported beside it: p50/p99 job latency (arrival to
retirement) over the whole trace once it drains, the window's saturation
(queued jobs, resident particles, GPU share), the precision form's error
statement, and the same jobs run one by one on the plain FP64 path.
--sweep runs the stream at several arrival rates and admission limits.

Other workloads (--workload): lj256k, lj864, dem500, gas200k, poly1m (one
system; a step is one timestep, L2 flushed before each), ens256 (256 gas
replicas in one batch context; a step is one timestep of all).

--impl reference times the CPU FP64 restatement of the reference's path (the
oracle) on the same workload with every host core.

Multi-GPU (--gpus N under torchrun): replicas only; every rank runs its own
copy of the workload; value = all ranks' particle-steps / max rank time.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_FLUSH = 512 << 20
FALLBACK_HBM_GBS = 6800.0


def workload(name, rsa=None):
    """(description, config, state maker) of a single-system workload;
    ``rsa``: the sphere generator of the gases (default the library's;
    False when only the description is wanted)."""
    from mddem_gb300 import config, inputs

    rsa = rsa or None

    if name == "lj256k":
        cfg = config.lj_fluid_config(box=67.06)
        return "LJ fluid 256000 atoms FCC rho=0.85 T=0.85 NH rc=2.5", cfg, lambda: inputs.lj_fcc(40, 67.06, 0.85, 0.85, seed=2024)
    if name == "lj864":
        cfg = config.lj_fluid_config(box=10.06)
        return "LJ fluid 864 atoms FCC rho=0.85 T=0.85 NH rc=2.5", cfg, lambda: inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=2024)
    if name == "lj500":
        cfg = config.lj_fluid_config(box=8.252)
        return ("LJ fluid 500 atoms FCC rho=0.89 T=1.0 NH rc=2.5 (few bins: warp-per-particle list build)", cfg,
                lambda: inputs.lj_fcc(5, 8.252, 500 / 8.252 ** 3, 1.0, seed=3))
    if name == "lj88k":
        L = (87808 / 0.884) ** (1.0 / 3.0)
        cfg = config.lj_fluid_config(box=L)
        return ("LJ fluid 87808 atoms FCC rho=0.884 T=1.0 NH rc=2.5 (warp-per-bin list build)", cfg,
                lambda: inputs.lj_fcc(28, L, 87808 / L ** 3, 1.0, seed=3))
    if name == "dem500":
        cfg = config.granular_gas_config()
        return "DEM granular gas 500 glass spheres r=1mm box 0.025", cfg, lambda: inputs.dem_granular_gas(500, seed=0)
    from mddem_gb300 import workloads as w

    if name == "gas200k":
        cfg = config.granular_gas_config(box=w.gas_box(200000, 0.15), dt=w.DT_GAS)
        return ("DEM granular gas 200000 glass spheres r=1mm solid fraction 0.15", cfg,
                lambda: w.gas(200000, phi=0.15, seed=2024, rsa=rsa)[1])
    if name == "gas138k":
        cfg = config.granular_gas_config(box=w.gas_box(138195, 0.05), dt=w.DT_GAS)
        return ("DEM granular gas 138195 glass spheres r=1mm solid fraction 0.05 (thread-per-particle list build)",
                cfg, lambda: w.gas(138195, phi=0.05, seed=3, rsa=rsa)[1])
    if name == "poly1m":
        cfg = w.polydisperse_config()
        return ("DEM polydisperse gas 1000000 glass spheres r~U[0.8,1.2]mm solid fraction 0.30 Maxwellian", cfg,
                lambda: w.polydisperse_gas(seed=2024, rsa=rsa)[1])
    raise SystemExit(f"unknown workload {name}")


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()  # the timed region starts once sampling has
            while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def mark(self):
        """Index of the next sample: bracket a window with two marks."""
        return len(self.lines)

    def summary(self, i0=0, i1=None):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines[i0:i1]
        if i0 and len(lines) < 2:  # window shorter than the sampling period
            lines = self.lines[max(0, i0 - 2):(i1 or len(self.lines)) + 2]
        for ln in lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for k, v in zip(names, p[3:7]):
                if v.lower() == "active":
                    reasons.add(k)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        for k in ("hbm_gbs", "hbm_GBs", "hbm"):
            if k in d:
                v = d[k]
                return float(v["value"] if isinstance(v, dict) else v), "measured"
    except (OSError, ValueError, KeyError, TypeError):
        pass
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


def cpu_baseline_sample(wl, max_seconds=15.0):
    """Single-core oracle on a bounded sample of the workload (steps until
    ~max_seconds of CPU time)."""
    from oracle.oracle import Oracle

    desc, cfg, make = workload(wl)
    st = make()
    o = Oracle(cfg.replace(precision="fp64"))
    o.load(st)
    o.step(1)  # first step includes the first full rebuild
    n = len(st["tag"])
    steps, t0 = 0, time.perf_counter()
    while True:
        o.step(1)
        steps += 1
        el = time.perf_counter() - t0
        if el > max_seconds or steps >= 200:
            break
    return {"value": n * steps / el, "unit": "particle-steps/s", "cores": 1, "kind": "port",
            "sample": f"{steps} timesteps of the same {n}-particle workload, single thread, after 1 warm-up step"}


REF_BUDGET = 40.0  # seconds of stepping per core in the reference arm


def _ref_fill(make_jobs, budget=REF_BUDGET, cap_ps=4e6):
    """Step jobs one after another on the oracle (the CPU FP64 restatement of
    the reference's path), each for up to its step count capped at cap_ps
    particle-steps after one warm-up step, cycling through the list until
    `budget` seconds of stepping are spent; setup is not timed.  The inputs
    are made without the library (the oracle's own sphere placement).
    Returns (particle-steps, seconds)."""
    from oracle.oracle import Oracle

    jobs = make_jobs()
    work = secs = 0.0
    k = 0
    while secs < budget and jobs:
        cfg, st, steps = jobs[k % len(jobs)]
        o = Oracle(cfg.replace(precision="fp64"))
        o.load(st)
        o.step(1)
        n = len(st["tag"])
        todo = max(1, min(int(steps), int(cap_ps // n)))
        t0 = time.perf_counter()
        done = 0
        while done < todo and secs + (time.perf_counter() - t0) < budget:
            o.step(1)
            done += 1
        secs += time.perf_counter() - t0
        work += n * done
        o.close()
        k += 1
    return work, secs


def _ref_single_jobs(wl):
    from oracle import oracle

    desc, cfg, make = workload(wl, rsa=oracle.rsa_spheres)
    return [(cfg, make(), 1 << 30)]


def _ref_serve_jobs(idx, njobs):
    import types

    from oracle import oracle

    trace = serve_trace(types.SimpleNamespace(jobs=njobs))
    out = []
    for k in idx:
        cfg, st = trace[k].make("fp64", "reference", rsa=oracle.rsa_spheres)
        out.append((cfg, st, trace[k].steps))
    return out


def _ref_ens_jobs(idx):
    from mddem_gb300 import workloads as w
    from oracle import oracle

    return [(c, s, 5000) for c, s in w.ensemble(precision="fp64", policy="reference", rsa=oracle.rsa_spheres,
                                                only=idx)]


def _ref_worker(args):
    kind, arg = args
    import functools

    if kind == "single":
        return _ref_fill(functools.partial(_ref_single_jobs, arg))
    if kind == "serve":
        return _ref_fill(functools.partial(_ref_serve_jobs, *arg))
    return _ref_fill(functools.partial(_ref_ens_jobs, arg))


def _ref_pool(tasks):
    """Run the reference workers, one per host core; the arm's rate is the sum
    of the per-core rates (each core steps for the same wall budget)."""
    import multiprocessing as mp

    with mp.get_context("spawn").Pool(len(tasks)) as pool:
        res = pool.map(_ref_worker, tasks)
    return sum(w_ / s_ for w_, s_ in res if s_ > 0), len(res)


def _ref_line(a, metric, val, cores, workload_desc, sample):
    return {
        "impl": "reference", "metric": metric, "value": val, "unit": "particle-steps/s",
        "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_desc, "precision": "fp64", "parallelism": f"{cores} host cores"},
        "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_reference_ensemble(a):
    cores = os.cpu_count() or 1
    parts = [list(range(c, 256, cores)) for c in range(cores)]
    val, used = _ref_pool([("ens", p) for p in parts if p])
    sample = (f"the 256 replicas dealt round-robin to {used} cores; each core steps its replicas in turn "
              f"(each up to 5000 steps or 4e6 particle-steps after 1 warm-up step) for {REF_BUDGET:g} s; "
              "value = sum of the per-core rates")
    print(json.dumps(_ref_line(a, "particle-steps/s", val, used, ENS_DESC, sample)), flush=True)


def run_reference_serve(a):
    trace = serve_trace(a)
    cores = os.cpu_count() or 1
    order = sorted(range(len(trace)), key=lambda k: trace[k].arrival)
    parts = [order[c::cores] for c in range(cores)]
    val, used = _ref_pool([("serve", (p, a.jobs)) for p in parts if p])
    sample = (f"the stream's jobs dealt round-robin to {used} cores; each core steps its jobs in turn "
              f"(each up to its step count or 4e6 particle-steps after 1 warm-up step) for {REF_BUDGET:g} s; "
              "value = sum of the per-core rates")
    print(json.dumps(_ref_line(a, "particle-steps/s served", val, used, serve_desc(trace, a), sample)), flush=True)


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if a.workload == "serve":
        return run_reference_serve(a)
    if a.workload == "ens256":
        return run_reference_ensemble(a)
    desc, _, _ = workload(a.workload, rsa=False)
    cores = os.cpu_count() or 1
    val, used = _ref_pool([("single", a.workload)] * cores)
    sample = (f"{used} independent copies of the workload, one per core, each stepping for {REF_BUDGET:g} s "
              "after 1 warm-up step; value = sum of the per-core rates")
    print(json.dumps(_ref_line(a, "particle-steps/s", val, used, desc, sample)), flush=True)


# ---------------------------------------------------------------------------
# served job stream
# ---------------------------------------------------------------------------
SERVE_PUMP = 200            # timesteps per pump (one bench step)
SERVE_JOBS = 384
SERVE_BACKLOG = 64          # jobs already queued when the stream starts
SERVE_RATE = 4.0            # Poisson arrivals per pump tick after the backlog
SERVE_BUDGET_GB = 96        # admission budget of resident jobs' device bytes (GB)
SERVE_SLOT_MULT = 2         # times the slot counts of workloads.SERVE_*_SLOTS
SERVE_WINDOW = 80           # timed pumps by default: the steady state while jobs keep arriving
SERVE_WARMUP = 10           # pumps of the stream before the timed window
SERVE_GROUPS = "split"      # slots per batch context (workloads.serve_groups): DEM, LJ <= 16384, LJ 100000
PLAIN_SAMPLE_STEPS = 200
# (jobs, backlog, arrivals per pump, budget GB, slot multiplier) of --sweep;
# each setting's arrivals last about as long as the timed window
SERVE_SWEEP = [(128, 32, 1.0, 96, 2), (224, 48, 2.0, 96, 2), (384, 64, 4.0, 96, 2), (704, 64, 8.0, 96, 2),
               (704, 64, 8.0, 192, 4)]


def reduce_over_ranks(dist, ms, work):
    """Job-wide figures of a replicas-only run: the slowest rank's time and the
    work of all ranks (a max and a sum over the ranks; no other exchange)."""
    if dist is None:
        return float(ms), float(work)
    import torch

    t = torch.tensor([ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    w = torch.tensor([work], dtype=torch.float64)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return float(t.item()), float(w.item())


def serve_trace(a):
    from mddem_gb300 import workloads as w

    trace = w.serve_trace(njobs=a.jobs, rate=getattr(a, "serve_rate", SERVE_RATE), seed=2024)
    scale = getattr(a, "job_steps_scale", 1.0)
    for j in trace:
        j.steps = max(1, int(round(j.steps * scale)))
    backlog = getattr(a, "backlog", SERVE_BACKLOG)
    t0 = trace[backlog].arrival if len(trace) > backlog else 0.0
    for k, j in enumerate(trace):  # the backlog arrives at tick 0, the rest keep their gaps
        j.arrival = 0.0 if k < backlog else j.arrival - t0 + 1.0
    return trace


def serve_desc(trace, a):
    kinds = {}
    for j in trace:
        kinds[j.kind] = kinds.get(j.kind, 0) + 1
    scale = getattr(a, "job_steps_scale", 1.0)
    return (f"served stream: {len(trace)} jobs ({kinds.get('gas', 0)} cooling gases N 100-200000, "
            f"{kinds.get('rebound', 0)} two-sphere rebounds, {kinds.get('lj', 0)} LJ FCC melts N 500-100000), "
            f"steps {1000 * scale:g}-{50000 * scale:g} log-uniform, {getattr(a, 'backlog', SERVE_BACKLOG)} queued "
            f"at start then Poisson {getattr(a, 'serve_rate', SERVE_RATE):g}/pump, {SERVE_PUMP} timesteps per pump")


def serve_server(a):
    """The job server of the served-stream workload: slot classes times
    a.slot_mult, admission budget a.budget_gb."""
    from mddem_gb300 import capi, workloads as w

    cfgs, caps = w.serve_slots(a.precision, a.policy, mult=getattr(a, "slot_mult", SERVE_SLOT_MULT))
    groups = w.serve_groups(cfgs, caps, getattr(a, "groups", SERVE_GROUPS))
    return capi.Server(cfgs, caps, int(getattr(a, "budget_gb", SERVE_BUDGET_GB) * (1 << 30)), groups=groups)


def state_bytes(st):
    import numpy as np

    return sum(v.nbytes for v in st.values() if isinstance(v, np.ndarray))


def replay(a, srv, trace, made, clk):
    """Submit each job at its arrival tick, pump until the stream drains.
    Pumps [warmup, warmup + steps) are the timed window (CUDA events on the
    server's stream); steps = 0: every pump from warmup until the drain.  Returns window and whole-run figures and job infos."""
    import torch

    order = sorted(range(len(trace)), key=lambda k: trace[k].arrival)
    # warm-up pumps of the stream itself; a stream shorter than that (small
    # cases for launch lists) keeps its last pumps timed
    est = int(max(j.arrival + j.steps / SERVE_PUMP for j in trace))
    warm = min(a.warmup, max(0, est - 2))
    stream = torch.cuda.ExternalStream(srv.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nxt, tick, infos, sid = 0, 0, {}, {}
    h2d = d2h = 0
    win = {}
    t_all = time.perf_counter()
    while True:
        while nxt < len(order) and trace[order[nxt]].arrival <= tick:
            k = order[nxt]
            cfg, st = made[k]
            sid[srv.submit(cfg, st, trace[k].steps)] = k
            h2d += state_bytes(st)
            nxt += 1
        if "s0" in win and "s1" not in win:
            # saturation: jobs waiting for admission and particles resident
            # at the start of each timed pump
            ss = srv.stats()
            win.setdefault("pend", []).append(ss["pending"])
            win.setdefault("res_n", []).append(sum(r["n"] for r in srv.resident()))
        if tick == warm:
            win.update(s0=srv.stats(), l0=srv.launches(), c0=clk.mark(), w0=time.perf_counter(), warm=warm)
            ss = srv.stats()
            win["pend"] = [ss["pending"]]
            win["res_n"] = [sum(r["n"] for r in srv.resident())]
            e0.record(stream)
        active, pending = srv.pump(SERVE_PUMP)
        tick += 1
        mid = warm + (a.steps // 2 if a.steps else min(10, max(0, est - warm) // 2))
        if tick >= mid and "mix" not in win:
            win["mix"] = [sid[r["id"]] for r in srv.resident()]
        drained = nxt == len(order) and active == 0 and pending == 0
        if "s0" in win and "s1" not in win and ((a.steps and tick == warm + a.steps) or drained):
            e1.record(stream)
            e1.synchronize()
            win.update(s1=srv.stats(), l1=srv.launches(), c1=clk.mark(), w1=time.perf_counter(),
                       ms=e0.elapsed_time(e1), pumps=tick - warm)
        for info in srv.poll():
            out = srv.fetch(info["id"])
            d2h += state_bytes(out)
            infos[sid[info["id"]]] = info
        if drained:
            break
    wall = time.perf_counter() - t_all
    return win, infos, {"wall_s": wall, "pumps": tick, "h2d": h2d, "d2h": d2h}


def saturation(win):
    """Whether the timed window ran saturated: jobs waiting for admission at
    the start of every timed pump means the admission limits (slots, HBM
    budget), not the arrivals, bounded the resident work; the GPU's share of
    the window is its CUDA-event time over the window's wall time."""
    import numpy as np

    pend = np.array(win.get("pend", [0]))
    res = np.array(win.get("res_n", [0]))
    wall_ms = (win["w1"] - win["w0"]) * 1e3
    return {"pumps_with_queue_frac": float(np.mean(pend > 0)), "queued_jobs_mean": float(pend.mean()),
            "resident_particles_mean": float(res.mean()), "resident_particles_max": int(res.max()),
            "gpu_busy_frac": float(win["ms"] / wall_ms) if wall_ms > 0 else None}


def plain_job_by_job(trace, made):
    """The same jobs on the plain FP64 path, one context per job, one after
    another: create + upload + steps + download.  Steps are timed on a sample
    of each job (up to PLAIN_SAMPLE_STEPS after one warm-up step) and scaled to
    the job's step count."""
    from mddem_gb300 import capi

    work = secs = 0.0
    for j, (cfg, st) in zip(trace, made):
        n = len(st["tag"])
        t0 = time.perf_counter()
        ctx = capi.Context(cfg.replace(precision="fp64"), n)
        ctx.upload(st)
        ctx.step(1)
        t1 = time.perf_counter()
        m = max(1, min(j.steps - 1, PLAIN_SAMPLE_STEPS))
        ctx.step(m)
        t2 = time.perf_counter()
        ctx.download()
        t3 = time.perf_counter()
        ctx.close()
        work += n * j.steps
        secs += (t1 - t0) + (t3 - t2) + (t2 - t1) * (j.steps - 1) / m + (t2 - t1) / m
    return {"value": work / secs, "unit": "particle-steps/s", "jobs": len(trace),
            "sample": f"each job's step time measured over up to {PLAIN_SAMPLE_STEPS} steps after 1 warm-up step, "
                      "scaled to its step count; setup, upload and download timed in full"}


# Compulsory DRAM bytes per particle of the per-particle kernels (each array
# touched once per launch; neighbours' rows assumed L2-resident), by kind and
# precision.  k_initial: v, f, x (+ mixed geometry copy and its build-time
# value for the rebuild test: DEM two-float 2 x 32, LJ fixed-point 2 x 16;
# fp64: build-time x) (+ DEM: omega, torque, quaternion) read, v, x (+ the
# geometry copy) (+ omega, quaternion) written.  k_final: f, v, m, x (+ omega,
# torque) read, v (+ omega) written.
INIT_BYTES = {("dem", "mixed"): 352, ("dem", "fp64"): 352, ("lj", "mixed"): 192, ("lj", "fp64"): 192}


def init_bytes(kind, prec, spinning=1.0):
    """k_initial / k_initial_mixed per particle: v, f, x read and v, x written;
    DEM adds omega and the torque read, omega written and the quaternion read
    and written; the mixed kernels also read and write the geometry copy and
    read its build copy.  The mixed DEM kernel leaves the quaternion of a
    sphere that has never spun (omega = 0: nothing to rotate) untouched, so its
    64 B count only for the `spinning` fraction."""
    b = INIT_BYTES[(kind, prec)]
    if (kind, prec) == ("dem", "mixed"):
        b += 64 * spinning
    return b


def spinning_fraction(states):
    """Share of DEM particles with nonzero angular velocity over `states`."""
    import numpy as np

    n = sum(len(st["tag"]) for st in states)
    k = sum(int(np.count_nonzero(np.any(st["omega"] != 0.0, axis=1))) for st in states)
    return k / max(1, n)
FINAL_BYTES = {"dem": 232, "lj": 136}


def rebuild_bytes(kind, nfull, contacts, prec="mixed"):
    """Per particle whose system rebuilds (every rebuild sorts by bin, as
    sort_atoms_by_bin): the bin of its position (32 read, 4 written), the
    counting sort's permutation entry (4 + 4), its state permuted once (read and
    written: x, v, m, cutoff, tag, type, image 104; DEM adds omega and q 64 and
    the history count 4 + 60 per contact), the geometry copies written
    (two-float x 32; mixed adds the build copy 32, mixed LJ the fixed-point
    positions 32), and the list build (two-float x 32, bin start and count 8,
    4 per row entry, row length 4)."""
    row = 104 + (64 + 4 + 60 * contacts if kind == "dem" else 0)
    geo = 32 + (32 if prec == "mixed" else 0) + (32 if (kind, prec) == ("lj", "mixed") else 0)
    return 36 + 8 + 2 * row + geo + 44 + 4 * nfull


def force_bytes(kind, nfull, contacts, prec="fp64"):
    """k_lj_* / k_dem_*: row length 4 + entries 4 each + own geometry (32; the
    mixed LJ kernel's fixed-point position 16) + force 32 written; DEM adds v
    and omega 64, torque 32, and per contact the partner tag and 7 spring
    values read and written (2 x 60)."""
    b = 4 + 4 * nfull + (16 if (kind, prec) == ("lj", "mixed") else 32) + 32
    if kind == "dem":
        b += 64 + 32 + 4 + 120 * contacts
    return b


def serve_mix(srv, trace, sid):
    """Particles, mean full-list row length and stored contacts per particle
    of the jobs resident now, by kind."""
    import numpy as np

    per = {}
    for r in srv.resident():
        kind = "lj" if trace[sid[r["id"]]].kind == "lj" else "dem"
        p = per.setdefault(kind, dict(n=0, pairs=0, contacts=0, jobs=0, spin=0))
        p["n"] += int(r["n"])
        p["jobs"] += 1
        p["pairs"] += len(srv.pairs_resident(r["slot"]))
        if kind == "dem":
            p["contacts"] += len(srv.history_resident(r["slot"])[0])
            w = srv.download_resident(r["slot"])["omega"]
            p["spin"] += int(np.count_nonzero(np.any(w != 0.0, axis=1)))
    return {k: dict(particles=p["n"], jobs=p["jobs"], avg_full_neighbors=2.0 * p["pairs"] / max(1, p["n"]),
                    contacts_per_particle=p["contacts"] / max(1, p["n"]),
                    spinning_fraction=p["spin"] / max(1, p["n"])) for k, p in per.items()}


def serve_samples(srv, trace, made, sid, per_kind=(("gas", 3), ("lj", 2), ("rebound", 1))):
    """States (with contact history) of the largest resident jobs of each kind,
    downloaded from the server's context: the sample the precision form's
    force error is stated on."""
    res = srv.resident()
    out = []
    for kind, m in per_kind:
        ks = sorted((r for r in res if trace[sid[r["id"]]].kind == kind), key=lambda r: -r["n"])[:m]
        for r in ks:
            cfg = made[sid[r["id"]]][0]
            st = srv.download_resident(r["slot"])
            hist = srv.history_resident(r["slot"]) if cfg.kind == "dem" else None
            out.append((kind, cfg, st, hist))
    return out


def precision_errors(samples):
    """Per-particle force (and torque) error of the mixed path against the
    plain FP64 path on each sampled job's current state (same state, same
    contact history, one force evaluation each), with the per-particle metric
    |F_mixed - F_fp64|_inf / max(|F_fp64|_inf, sum_pairs |f_pair|)."""
    from mddem_gb300 import capi, validate

    out = {"bound": 1e-5, "jobs": []}
    worst = {"force": 0.0, "torque": 0.0}
    for kind, cfg, st, hist in samples:
        res = {}
        for prec in ("fp64", "mixed"):
            c = capi.Context(cfg.replace(precision=prec), len(st["tag"]))
            c.upload(st)
            if hist is not None and len(hist[0]):
                c.set_history(*hist)
            c.force_only()
            res[prec] = (c.download(), c.pairs())
            c.close()
        e = validate.force_error(cfg, res["fp64"][0], res["mixed"][0], res["fp64"][1])
        out["jobs"].append({"kind": kind, "particles": len(st["tag"]), **e})
        for q in e:
            worst[q] = max(worst[q], e[q])
    out.update({"force_rel_max": worst["force"], "torque_rel_max": worst["torque"]})
    return out


def physics_errors():
    """Conserved / statistical quantities of the mixed path beside the plain
    FP64 path (whose LJ energy history equals the oracle's to 1e-6 of its
    drift, and whose Haff time is within 2 % of the oracle's, in the GPU
    test suite): LJ NVE energy drift over 2000 steps (864 atoms), and the
    Haff cooling time of a frictionless gas (2000 spheres, solid fraction
    0.2, e = 0.8, 40000 steps) with its kinetic-theory value."""
    from mddem_gb300 import capi, config, inputs, validate, workloads

    slopes = {}
    for prec in ("fp64", "mixed"):
        cfg = config.lj_fluid_config(nose_hoover=False, precision=prec)
        st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=3)
        c = capi.Context(cfg, len(st["tag"]))
        c.upload(st)
        slopes[prec] = validate.energy_drift(c)[1]
        c.close()
    tc = {}
    for prec in ("fp64", "mixed"):
        cfg, st = workloads.gas(2000, phi=0.2, restitution=0.8, friction=0.0, seed=11, precision=prec)
        c = capi.Context(cfg, 2000)
        c.upload(st)
        tc[prec], theory, _ = validate.haff(c, cfg, 2000, 0.8)
        c.close()
    return {"lj_energy_drift": {"mixed_per_step": slopes["mixed"], "fp64_per_step": slopes["fp64"],
                                "ratio": abs(slopes["mixed"]) / max(abs(slopes["fp64"]), 1e-300), "bound": 2.0},
            "haff_tc": {"mixed": tc["mixed"], "fp64": tc["fp64"], "kinetic_theory": theory,
                        "mixed_vs_fp64": tc["mixed"] / tc["fp64"] - 1.0, "fp64_vs_theory": tc["fp64"] / theory - 1.0,
                        "bounds": {"mixed_vs_fp64": 0.02, "fp64_vs_theory": 0.15}}}


# run lengths of the workloads' own error statements (the configs' run lengths)
LJ_RDF_STEPS = 100000       # 864 atoms; 10000 from 10^4 atoms on (a large melt's g(r) converges sooner)
LJ_RDF_FRAMES = 20
COOL_STEPS = {"dem500": 10000, "gas200k": 20000, "gas138k": 20000, "poly1m": 20000}


def lj_structure(cfg, st, steps=LJ_RDF_STEPS, frames=LJ_RDF_FRAMES):
    """g(r) of an NH LJ melt on the mixed and on the plain FP64 path, both
    from the same FCC state: `steps` steps, g averaged over `frames` frames of
    the second half; the reference's structure checks on each and the largest
    |g_mixed - g_fp64| over r < 3 sigma."""
    import numpy as np
    from mddem_gb300 import capi, validate

    out, gs = {}, {}
    nb, rmax = 200, 3.0
    for prec in ("fp64", "mixed"):
        c = capi.Context(cfg.replace(precision=prec), len(st["tag"]))
        c.upload(st)
        c.step(steps // 2)
        acc = []
        for _ in range(frames):
            c.step(steps // 2 // frames)
            acc.append(c.rdf(r_max=rmax, nbins=nb)[1])
        c.close()
        gs[prec] = np.mean(acc, axis=0)
        out[prec] = validate.rdf_checks((np.arange(nb) + 0.5) * rmax / nb, gs[prec])
    out["max_abs_diff"] = float(np.max(np.abs(gs["mixed"] - gs["fp64"])))
    out["steps"], out["frames"] = steps, frames
    return out


def workload_errors(name, cfg, make, ctx, sys_=None):
    """The precision form's error statement for a single-system workload (or
    the listed replicas of a batch): the per-particle force / torque error
    against the plain FP64 path on the state the timed steps left (with its
    contact history); for LJ the NVE energy drift over 2000 steps and g(r)
    after the NH run; for the gases the cooling fit over the workload's run
    length.  The plain FP64 path is the one the GPU parity tests hold to the
    oracle (1e-12 per force, identical pair sets and histories)."""
    from mddem_gb300 import capi, validate

    samples = []
    for q in (sys_ if sys_ is not None else [0]):
        c = cfg[q] if isinstance(cfg, list) else cfg
        samples.append((f"{name}[{q}]" if sys_ is not None else name, c, ctx.download(q),
                        ctx.history(q) if c.kind == "dem" else None))
    out = {"force": precision_errors(samples)}
    if isinstance(cfg, list):
        return out
    st = make()
    n = len(st["tag"])
    if cfg.kind == "lj":
        slopes = {}
        for prec in ("fp64", "mixed"):
            c = capi.Context(cfg.replace(precision=prec, nose_hoover=False), n)
            c.upload(st)
            slopes[prec] = validate.energy_drift(c)[1] / n
            c.close()
        out["lj_energy_drift"] = {"mixed_per_step_per_atom": slopes["mixed"], "fp64_per_step_per_atom": slopes["fp64"],
                                  "ratio": abs(slopes["mixed"]) / max(abs(slopes["fp64"]), 1e-300), "bound": 2.0,
                                  "steps": 2000, "ensemble": "NVE (thermostat off)"}
        out["rdf"] = lj_structure(cfg, st, steps=LJ_RDF_STEPS if n < 10000 else 10000)
    elif name in COOL_STEPS:
        steps = COOL_STEPS[name]
        res = {}
        for prec in ("fp64", "mixed"):
            c = capi.Context(cfg.replace(precision=prec), n)
            c.upload(st)
            res[prec] = validate.cooling(c, cfg.dt, steps, steps // 20)
            c.close()
        m = cfg.materials[0]
        mono = float(st["radius"].min()) == float(st["radius"].max())
        theory = (validate.haff_theory(n, cfg.box[0], float(st["radius"][0]), m.restitution, res["fp64"][2][0])
                  if mono else None)
        out["cooling"] = {"steps": steps, "tc_mixed": res["mixed"][0], "tc_fp64": res["fp64"][0],
                          "mixed_vs_fp64": res["mixed"][0] / res["fp64"][0] - 1.0,
                          "T_end_over_T0": {"mixed": res["mixed"][1], "fp64": res["fp64"][1]},
                          "frictionless_kinetic_theory_tc": theory, "bound_mixed_vs_fp64": 0.02,
                          "note": "T(t) = T0 / (1 + t/t_c)^2 fitted on 1/sqrt(T); frictional spheres, so kinetic "
                                  "theory (smooth spheres) is context only"}
    return out


def serve_phases(a, trace, made, at_tick, pumps=2):
    """Where the served step's time goes: the same stream replayed with
    ordinary pumps up to `at_tick` (the middle of the timed window), then
    `pumps` pumps whose timesteps run on the server's own context as
    single-step graphs with CUDA events between the phases (initial
    integration, rebuild pipeline, force, final integration), on the mix of
    jobs resident there.  Admission and retirement run as in a pump
    (mdg_server_pump with 0 steps before and after)."""
    import numpy as np
    from mddem_gb300 import capi, workloads as w

    srv = serve_server(a)
    order = sorted(range(len(trace)), key=lambda k: trace[k].arrival)
    nxt, tick, sid = 0, 0, {}
    rows, mix, samples, rebuilt, ctx_rows = [], None, [], {}, []
    while tick < at_tick + pumps:
        while nxt < len(order) and trace[order[nxt]].arrival <= tick:
            k = order[nxt]
            sid[srv.submit(*made[k], trace[k].steps)] = k
            nxt += 1
        if tick < at_tick:
            active, pending = srv.pump(SERVE_PUMP)
        else:
            srv.pump(0)
            if mix is None:
                mix = serve_mix(srv, trace, sid)
                samples = serve_samples(srv, trace, made, sid)
            # each context's timesteps, one context after the other; the
            # systems' build counters give the particles rebuilt
            per = []
            for c in srv.contexts():
                live = [q for q in range(c.nsys) if c.n[q]]
                nb0 = {q: c.thermo(q)["nbuilds"] for q in live}
                per.append(c.timed_steps(SERVE_PUMP))
                for q in live:
                    kind = c.configs[q].kind
                    rebuilt[kind] = rebuilt.get(kind, 0) + c.n[q] * (c.thermo(q)["nbuilds"] - nb0[q])
                t_c = per[-1][0]
                kinds = {c.configs[q].kind for q in live}
                ctx_rows.append({"kind": "+".join(sorted(kinds)), "particles": int(sum(c.n[q] for q in live)),
                                 "step_ms": float(t_c[:, 0].mean()),
                                 "phases_ms": {ph: float(t_c[:, 1 + i].mean())
                                               for i, ph in enumerate(("initial", "rebuild", "force", "final"))}})
            rows.append((sum(q[0] for q in per), sum(q[1] for q in per), np.max([q[2] for q in per], axis=0)))
            active, pending = srv.pump(0)
        for info in srv.poll():
            srv.fetch(info["id"])
        tick += 1
        if nxt == len(order) and active == 0 and pending == 0:
            break
    srv.close()
    if not rows:
        return None, None, []
    t = np.concatenate([r[0] for r in rows])
    kern = np.concatenate([r[1] for r in rows])
    rb = np.concatenate([r[2] for r in rows])
    names = ("initial", "rebuild", "force", "final")
    ph = {q: float(t[:, 1 + i].mean()) for i, q in enumerate(names)}
    return {"at_pump": at_tick, "timesteps": int(len(t)), "step_ms": float(t[:, 0].mean()), "phases_ms": ph,
            "rebuild_steps_frac": float(rb.mean()), "kernels_per_step": float(kern.mean()),
            "rebuilt_particles_per_step": {k: v / len(t) for k, v in rebuilt.items()},
            "per_context": ctx_rows}, mix, samples


def serve_roofline(a, phases, mix, served_rate):
    """Roofline of the served step from its phase split: each phase's
    algorithmic bytes (per-particle figures of the mix's kinds, see INIT_BYTES,
    FINAL_BYTES, force_bytes) over its CUDA-event time; the dominant phase is
    reported, plus the whole step's bytes per particle-step times the
    window's served rate."""
    prec = a.precision
    init_b = sum(m["particles"] * init_bytes(k, prec, m.get("spinning_fraction", 1.0)) for k, m in mix.items())
    fin_b = sum(m["particles"] * FINAL_BYTES[k] for k, m in mix.items())
    force_b = sum(m["particles"] * force_bytes(k, m["avg_full_neighbors"], m["contacts_per_particle"], prec)
                  for k, m in mix.items())
    rb_b = sum(v * rebuild_bytes(k, mix[k]["avg_full_neighbors"], mix[k]["contacts_per_particle"], prec)
               for k, v in phases.get("rebuilt_particles_per_step", {}).items() if k in mix)
    ph = phases["phases_ms"]
    cands = {"initial": (ph["initial"], init_b), "force": (ph["force"], force_b), "final": (ph["final"], fin_b),
             "rebuild": (ph["rebuild"], rb_b or None)}
    name = max(cands, key=lambda q: cands[q][0])
    ms, nbytes = cands[name]
    peak, src = peak_hbm()
    kernel = {"initial": f"k_initial_{prec}", "final": f"k_final_{prec}",
              "rebuild": "rebuild pipeline (bin sort, permutation, k_build)",
              "force": ("k_dem_screen + k_dem_contact + k_lj_mixed" if prec == "mixed" else "k_dem_fp64 + k_lj_fp64")}[name]
    step_b = init_b + fin_b + force_b + (rb_b or 0.0)
    bpps = step_b / sum(m["particles"] for m in mix.values())
    traffic = ncu_traffic(name + "/serve")
    per = ncu_traffic("rebuild_per_particle")
    if name == "rebuild" and per:
        # the pipeline's measured DRAM bytes per rebuilt particle (LJ 256k, gas
        # 200k) times the particles the mix rebuilt per step
        traffic = sum(v * per[k] for k, v in phases.get("rebuilt_particles_per_step", {}).items() if k in per)
    out = {"bound": "hbm", "kernel": kernel, "phase": name, "share": ms / phases["step_ms"],
           "achieved": nbytes / (ms / 1e3) / 1e9 if nbytes else None, "peak": peak, "unit": "GB/s",
           "peak_source": src, "traffic": traffic, "algorithmic_bytes_per_launch": nbytes,
           "launch_ms": ms,
           "phases": {q: {"ms": v[0], "share": v[0] / phases["step_ms"],
                          "algorithmic_bytes": v[1],
                          "frac": (v[1] / (v[0] / 1e3) / 1e9 / peak) if v[1] else None}
                      for q, v in cands.items()},
           "whole_step": {"bytes_per_particle_step": bpps, "served_particle_steps_per_s": served_rate,
                          "achieved": bpps * served_rate / 1e9, "frac": bpps * served_rate / 1e9 / peak,
                          "note": "the mix's algorithmic bytes per particle-step (integrators, force and the "
                                  "rebuilds it made) x the window's served rate, over the measured copy peak"},
           "attribution": phases, "mix": mix}
    out["frac"] = out["achieved"] / peak if out["achieved"] else None
    return out


def _oracle_job(cfg, st, steps_cap, budget):
    from oracle.oracle import Oracle

    o = Oracle(cfg.replace(precision="fp64"))
    o.load(st)
    o.step(1)
    n, done, t0 = len(st["tag"]), 0, time.perf_counter()
    while done < steps_cap and time.perf_counter() - t0 < budget:
        o.step(1)
        done += 1
    return n * done, time.perf_counter() - t0


def serve_cpu_sample(trace, made, budget=15.0):
    """The oracle (single thread) on the stream's jobs in arrival order, each
    for up to 2e6 particle-steps after one warm-up step, until `budget` s."""
    work = secs = 0.0
    used = 0
    for j, (cfg, st) in sorted(zip(trace, made), key=lambda q: q[0].arrival):
        if secs > budget:
            break
        w_, s_ = _oracle_job(cfg, st, max(1, min(j.steps, int(2e6 // j.n))), budget - secs + 1.0)
        work += w_
        secs += s_
        used += 1
    return {"value": work / secs, "unit": "particle-steps/s", "cores": 1, "kind": "port",
            "sample": f"first {used} jobs of the stream in arrival order, each up to 2e6 particle-steps "
                      "after 1 warm-up step, single thread"}


def bench_serve(a, world, rank, local, dist):
    import numpy as np
    from mddem_gb300 import build, capi, workloads as w

    build.build()
    trace = serve_trace(a)
    made = [j.make(a.precision, a.policy) for j in trace]
    srv = serve_server(a)
    if a.eager:
        for c in srv.contexts():
            c.set_graph_mode(0)
    # warm-up jobs (one of each kind), drained before the stream starts
    wsteps = 2 * SERVE_PUMP if a.job_steps_scale >= 1.0 else SERVE_PUMP // 4
    for j in (w.Job("gas", 300, wsteps, 0, dict(phi=0.1, e=0.9, seed=7)),
              w.Job("rebound", 2, wsteps, 0, dict(speed=1.0)),
              w.Job("lj", 500, wsteps, 0, dict(cells=5, rho=0.85, T=1.0, seed=7))):
        c, s = j.make(a.precision, a.policy)
        srv.submit(c, s, j.steps)
    while True:
        act, pen = srv.pump(SERVE_PUMP)
        for info in srv.poll():
            srv.fetch(info["id"])
        if not act and not pen:
            break
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        win, infos, run = replay(a, srv, trace, made, clk)
    ps = win["s1"]["particle_steps"] - win["s0"]["particle_steps"]
    ms = win["ms"]
    ms, ps = reduce_over_ranks(dist, ms, ps)
    lat = np.array([infos[k]["end_s"] - infos[k]["submit_s"] for k in sorted(infos)])
    failed = [k for k in infos if infos[k]["status"] != 0]
    total_ps = float(sum(j.n * j.steps for j in trace))
    line = {
        "metric": "particle-steps/s served", "value": ps / (ms / 1e3), "unit": "particle-steps/s",
        "n_gpus": world, "steps": win["pumps"], "warmup": win["warm"], "ms_per_step": ms / win["pumps"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if a.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": serve_desc(trace, a), "precision": a.precision, "rebuild_policy": a.policy,
                   "pump_timesteps": SERVE_PUMP,
                   "slots": {"dem": [[c, n * a.slot_mult] for c, n in w.SERVE_DEM_SLOTS],
                             "lj": [[c, n * a.slot_mult] for c, n in w.SERVE_LJ_SLOTS]},
                   "hbm_budget_bytes": int(a.budget_gb * (1 << 30)),
                   "slot_groups": f"{a.groups}: one batch context and stream per group; every context's "
                                  "multi-step launch is queued before any is waited on",
                   "plain_fp64_reference": "the same jobs one by one on the plain FP64 path; each job's step time "
                                           f"is sampled over up to {PLAIN_SAMPLE_STEPS} steps and scaled to its "
                                           "step count (setup, upload and download timed in full)",
                   "l2": "inputs larger than L2 (resident state of all jobs, > 129 MB)",
                   "parallelism": f"replicas x{world}"},
        "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                      "max": float(lat.max()), "jobs": int(len(lat)), "failed": len(failed)},
        "saturation": saturation(win),
        "trace": {"particle_steps": total_ps, "wall_s": run["wall_s"], "pumps": run["pumps"],
                  "host_split_s": {q: win["s1"][q] - win["s0"][q] for q in ("admit_s", "step_s", "retire_s")}},
        "gpu_launches": int(win["l1"] - win["l0"]),
        "clocks": clk.summary(win["c0"], win["c1"]),
        "e2e": {"value": total_ps / run["wall_s"], "unit": "particle-steps/s",
                "h2d_bytes_per_step": run["h2d"] / run["pumps"], "d2h_bytes_per_step": run["d2h"] / run["pumps"],
                "note": "whole stream through mdg_server_* with host buffers: submit, pumps, poll, fetch"},
    }
    srv.close()
    if rank == 0:
        phases, mix, samples = serve_phases(a, trace, made, win["warm"] + max(1, win["pumps"] // 2))
        if phases:
            line["roofline"] = serve_roofline(a, phases, mix, line["value"] / world)
        if a.precision == "mixed" and not a.no_error:
            line["error"] = {"served_jobs": precision_errors(samples), **physics_errors()}
        if not a.no_plain:
            line["plain_fp64_job_by_job"] = plain_job_by_job(trace, made)
            line["served_vs_plain"] = line["value"] / world / line["plain_fp64_job_by_job"]["value"]
        if not a.no_cpu_baseline:
            line["cpu_baseline"] = serve_cpu_sample(trace, made)
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def serve_sweep(a):
    """The served stream at each SERVE_SWEEP setting (jobs, backlog, arrival
    rate, HBM budget, slot multiplier): one JSON line per setting with the
    window's served rate, p50 / p99 latency and its saturation figures."""
    import numpy as np
    from mddem_gb300 import build

    build.build()
    for jobs, backlog, rate, budget, mult in SERVE_SWEEP:
        b = argparse.Namespace(**vars(a))
        b.jobs, b.backlog, b.serve_rate, b.budget_gb, b.slot_mult = jobs, backlog, rate, budget, mult
        trace = serve_trace(b)
        made = [j.make(b.precision, b.policy) for j in trace]
        srv = serve_server(b)
        with ClockSampler(0) as clk:
            win, infos, run = replay(b, srv, trace, made, clk)
        srv.close()
        ps = win["s1"]["particle_steps"] - win["s0"]["particle_steps"]
        lat = np.array([infos[k]["end_s"] - infos[k]["submit_s"] for k in sorted(infos)])
        print(json.dumps({"sweep": {"jobs": jobs, "backlog": backlog, "arrivals_per_pump": rate, "budget_gb": budget,
                                    "slot_mult": mult},
                          "value": ps / (win["ms"] / 1e3), "unit": "particle-steps/s", "pumps": win["pumps"],
                          "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
                          "saturation": saturation(win), "stream_wall_s": run["wall_s"],
                          "e2e": sum(j.n * j.steps for j in trace) / run["wall_s"],
                          "clocks": clk.summary(win["c0"], win["c1"])}), flush=True)


# ---------------------------------------------------------------------------
# replica ensemble in one batch context
# ---------------------------------------------------------------------------
ENS_DESC = ("ensemble: 256 periodic granular-gas replicas, N log-uniform [500, 50000], solid fraction U[0.1,0.3], "
            "restitution U[0.70,0.99], friction U[0,0.5], r = 1 mm, dt = 2.934e-7 s, one batch context")


def bench_ensemble(a, world, rank, local, dist):
    import numpy as np
    import torch
    from mddem_gb300 import build, capi, workloads as w

    build.build()
    ens = w.ensemble(precision=a.precision, policy=a.policy)
    cfgs = [e[0] for e in ens]
    sts = [e[1] for e in ens]
    n = sum(len(s["tag"]) for s in sts)
    ctx = capi.Context(cfgs, [len(s["tag"]) for s in sts])
    for q, s in enumerate(sts):
        ctx.upload(s, q)
    tune = ctx.autotune(steps=20) if not a.no_tune else None
    if a.eager:
        ctx.set_graph_mode(0)
    stream = torch.cuda.ExternalStream(ctx.stream())
    ctx.step(a.warmup)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ctx.launches()
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        c0 = clk.mark()
        e0.record(stream)
        ctx.step(a.steps)  # one launch: a device-side loop over the K steps
        e1.record(stream)
        e1.synchronize()
        c1 = clk.mark()
    ms = e0.elapsed_time(e1)
    l1 = ctx.launches()
    ms, work = reduce_over_ranks(dist, ms, float(n * a.steps))
    line = {
        "metric": "particle-steps/s", "value": work / (ms / 1e3), "unit": "particle-steps/s",
        "n_gpus": world, "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if a.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": ENS_DESC, "particles": n, "precision": a.precision, "rebuild_policy": a.policy,
                   "autotune": tune, "l2": "inputs larger than L2 (1.5 GB of particle state)",
                   "launch": "one CUDA-graph launch runs all K steps (device-side WHILE loop)",
                   "parallelism": f"replicas x{world}"},
        "gpu_launches": int(l1 - l0),
        "clocks": clk.summary(c0, c1),
    }
    if rank == 0:
        # per-kernel phases (eager launches, CUDA events) for the roofline
        ctx.set_graph_mode(0)
        t, _, _ = ctx.timed_steps(5, 0)
        ctx.set_graph_mode(0 if a.eager else 1)
        contacts = sum(len(ctx.history(q)[0]) for q in range(len(sts))) / n
        nfull = sum(2.0 * len(ctx.pairs(q)) for q in range(len(sts))) / n
        spin = spinning_fraction([ctx.download(q) for q in range(len(sts))])
        cands = {("k_initial_mixed" if a.precision == "mixed" else "k_initial"):
                     (float(t[:, 1].mean()), n * init_bytes("dem", a.precision, spin)),
                 ("k_dem_screen + k_dem_contact" if a.precision == "mixed" else "k_dem_fp64"):
                     (float(t[:, 3].mean()), n * force_bytes("dem", nfull, contacts, a.precision)),
                 ("k_final_mixed" if a.precision == "mixed" else "k_final"):
                     (float(t[:, 4].mean()), n * FINAL_BYTES["dem"])}
        name = max(cands, key=lambda q: cands[q][0])
        kms, nbytes = cands[name]
        peak, src = peak_hbm()
        ach = nbytes / (kms / 1e3) / 1e9
        line["roofline"] = {"bound": "hbm", "kernel": name, "achieved": ach, "peak": peak, "unit": "GB/s",
                            "frac": ach / peak, "peak_source": src, "traffic": ncu_traffic(name + "/ens256"),
                            "algorithmic_bytes_per_launch": nbytes, "launch_ms": kms, "spinning_fraction": spin,
                            "kernels_ms": {q: v[0] for q, v in cands.items()}}
        if a.precision == "mixed" and not a.no_error:
            sizes = [len(q["tag"]) for q in sts]
            pick = sorted(set(sorted(range(len(sts)), key=lambda q: -sizes[q])[:2]
                              + [min(range(len(sts)), key=lambda q: cfgs[q].materials[0].restitution),
                                 max(range(len(sts)), key=lambda q: cfgs[q].materials[0].friction)]))
            line["error"] = workload_errors("ens256", cfgs, None, ctx, pick)
        if not a.no_e2e:
            line["e2e"] = ensemble_e2e(cfgs, sts, a.steps)
        if not a.no_plain:
            line["plain_fp64_replica_by_replica"] = plain_replicas(cfgs, sts)
            line["batched_vs_plain"] = line["value"] / world / line["plain_fp64_replica_by_replica"]["value"]
        if not a.no_cpu_baseline:
            import types

            tr = [types.SimpleNamespace(n=len(s["tag"]), steps=5000, arrival=float(q)) for q, s in enumerate(sts)]
            line["cpu_baseline"] = serve_cpu_sample(tr, list(zip(cfgs, sts)))
            line["cpu_baseline"]["sample"] = line["cpu_baseline"]["sample"].replace("jobs of the stream", "replicas")
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def ensemble_e2e(cfgs, sts, steps):
    """Upload of every replica from host arrays, K steps (one launch), thermo
    read-back of every replica, download of every replica; wall clock."""
    from mddem_gb300 import capi

    ctx = capi.Context(cfgs, [len(s["tag"]) for s in sts])
    for q, s in enumerate(sts):
        ctx.upload(s, q)
    ctx.step(3)
    t0 = time.perf_counter()
    up = down = 0
    for q, s in enumerate(sts):
        ctx.upload(s, q)
        up += state_bytes(s)
    ctx.step(steps)
    for q in range(len(sts)):
        ctx.thermo(q)
        down += state_bytes(ctx.download(q)) + 8 * 16
    el = time.perf_counter() - t0
    ctx.close()
    n = sum(len(s["tag"]) for s in sts)
    return {"value": n * steps / el, "unit": "particle-steps/s", "h2d_bytes_per_step": up / steps,
            "d2h_bytes_per_step": down / steps}


def plain_replicas(cfgs, sts):
    """Every replica on the plain FP64 path, one context each, one after
    another (step time sampled over up to PLAIN_SAMPLE_STEPS steps, scaled to
    the replicas' 5000 steps)."""
    import types

    tr = [types.SimpleNamespace(n=len(s["tag"]), steps=5000) for s in sts]
    r = plain_job_by_job(tr, list(zip(cfgs, sts)))
    r["sample"] = r["sample"].replace("each job's", "each replica's") + "; 5000 steps per replica"
    return r


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 50; served stream: 80 pumps, 0 = every pump until it drains)")
    ap.add_argument("--warmup", type=int, default=None,
                    help="untimed steps first (default 5; served stream: 10 pumps)")
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--workload", default="serve")
    ap.add_argument("--jobs", type=int, default=SERVE_JOBS, help="jobs in the served stream")
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--policy", default="displacement")
    ap.add_argument("--tpp", type=int, default=0, help="threads per particle in the force kernel (0 = auto)")
    ap.add_argument("--eager", action="store_true", help="launch kernels one by one (for profilers)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (ensemble)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison (serve, ensemble)")
    ap.add_argument("--serve-rate", type=float, default=SERVE_RATE, help="served stream: Poisson arrivals per pump")
    ap.add_argument("--backlog", type=int, default=SERVE_BACKLOG, help="served stream: jobs queued at the start")
    ap.add_argument("--budget-gb", type=float, default=SERVE_BUDGET_GB, help="served stream: admission HBM budget")
    ap.add_argument("--slot-mult", type=int, default=SERVE_SLOT_MULT, help="served stream: slot count multiplier")
    ap.add_argument("--groups", default=SERVE_GROUPS, choices=("kind", "split", "size", "class"),
                    help="served stream: slots per batch context (one context and stream per group)")
    ap.add_argument("--no-error", action="store_true", help="skip the precision-form error block")
    ap.add_argument("--sweep", action="store_true",
                    help="served stream at each SERVE_SWEEP setting: throughput, latency and saturation per setting")
    ap.add_argument("--job-steps-scale", type=float, default=1.0,
                    help="scale the served jobs' step counts (small cases for launch lists)")
    a = ap.parse_args()
    a.steps_auto = a.steps is None and a.workload not in ("serve", "ens256")
    if a.steps is None:
        # ens256: the ensemble's 5000 steps per replica in one launch
        a.steps = SERVE_WINDOW if a.workload == "serve" else (5000 if a.workload == "ens256" else 50)
    if a.warmup is None:
        a.warmup = SERVE_WARMUP if a.workload == "serve" else 5
    a.warmup = max(3, a.warmup)
    if a.impl == "reference":
        return run_reference(a)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
        import torch.distributed as dist  # replicas only: a barrier and a max reduction, no data path

        dist.init_process_group("gloo")

    if a.workload == "serve" and a.sweep:
        return serve_sweep(a)
    if a.workload == "serve":
        return bench_serve(a, world, rank, local, dist)
    if a.workload == "ens256":
        return bench_ensemble(a, world, rank, local, dist)
    from mddem_gb300 import build, capi

    build.build()
    desc, cfg, make = workload(a.workload)
    cfg = cfg.replace(precision=a.precision, rebuild_policy=a.policy, threads_per_particle=a.tpp)
    t0 = time.perf_counter()
    st = make()
    host_setup = time.perf_counter() - t0
    n = len(st["tag"])
    ctx = capi.Context(cfg, n)
    ctx.upload(st)
    if a.eager:
        ctx.set_graph_mode(0)
    ctx.timed_steps(a.warmup, L2_FLUSH)
    if a.steps_auto:
        # long enough for the clock sampler (200 ms period) to see the region
        probe = float(ctx.timed_steps(5, L2_FLUSH)[0][:, 0].mean())
        a.steps = int(min(100000, max(a.steps, math.ceil(1500.0 / max(probe, 1e-3)))))
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        t, kernels, rebuilt = ctx.timed_steps(a.steps, L2_FLUSH)
    total_ms, work = reduce_over_ranks(dist, float(t[:, 0].sum()), float(n * a.steps))
    value = work / (total_ms / 1e3)
    th = ctx.thermo()
    nfull = th["max_neighbors"]
    pairs = len(ctx.pairs())
    nfull_avg = 2.0 * pairs / n
    force_ms = float(t[:, 3].mean())
    kind = cfg.kind
    contacts = len(ctx.history()[0]) / n if kind == "dem" else 0.0
    spin = spinning_fraction([ctx.download()]) if kind == "dem" else 0.0
    suffix = "mixed" if a.precision == "mixed" else "fp64"
    # the dominant per-particle kernel of the step: force, initial or final
    # integration (phases timed by CUDA events; rebuild steps averaged in)
    fname = {("dem", "mixed"): "k_dem_screen + k_dem_contact", ("dem", "fp64"): "k_dem_fp64",
             ("lj", "mixed"): "k_lj_mixed", ("lj", "fp64"): "k_lj_fp64"}[(kind, a.precision)]
    cands = {fname: (force_ms, force_bytes(kind, nfull_avg, contacts, a.precision)),
             ("k_initial_mixed" if a.precision == "mixed" else "k_initial"):
                 (float(t[:, 1].mean()), init_bytes(kind, a.precision, spin)),
             ("k_final_mixed" if a.precision == "mixed" else "k_final"):
                 (float(t[:, 4].mean()), FINAL_BYTES[kind])}
    kname = max(cands, key=lambda q: cands[q][0])
    kms, bpp = cands[kname]
    achieved = bpp * n / (kms / 1e3) / 1e9
    peak, src = peak_hbm()
    traffic = ncu_traffic(kname + "/" + a.workload) or (ncu_traffic(kname) if a.workload == "lj256k" else None)
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": total_ms / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if a.precision == "mixed" else "f64",
        "data": "synthetic",
        "config": {"workload": desc, "precision": a.precision, "rebuild_policy": a.policy, "particles": n,
                   "steps_rule": ("timed steps chosen to last >= 1.5 s (clock sampling)" if a.steps_auto
                                  else "as given"),
                   "l2": "flushed before every timed step (512 MB write)", "parallelism": f"replicas x{world}"},
        "phases_ms": {"initial": float(t[:, 1].mean()), "rebuild": float(t[:, 2].mean()), "force": force_ms,
                      "final": float(t[:, 4].mean())},
        "rebuild_steps": int(rebuilt.sum()),
        "gpu_launches": int(kernels.sum()),
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": src, "traffic": traffic,
                     "algorithmic_bytes_per_particle": bpp, "avg_full_neighbors": nfull_avg, "launch_ms": kms,
                     "spinning_fraction": spin,
                     "kernels_ms": {q: v[0] for q, v in cands.items()}},
        "clocks": clk.summary(),
    }
    if rank == 0:
        line["setup"] = setup_times(a.workload, cfg, st, host_setup)
    if rank == 0 and a.precision == "mixed" and not a.no_error:
        line["error"] = workload_errors(a.workload, cfg, make, ctx)
    if rank == 0 and not a.no_e2e:
        line["e2e"] = e2e(cfg, make, a.steps)
    if rank == 0 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(a.workload)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def setup_times(name, cfg, st, host_s):
    """Initial-condition set-up: the host generator the workload's inputs come
    from (shared with the reference arm) beside the device generator making a
    system of the same kind and size in a context (mdg_generate_fcc / _gas,
    wall clock of the call)."""
    from mddem_gb300 import capi, workloads as w

    out = {"host_generator_s": host_s}
    n = len(st["tag"])
    c = capi.Context(cfg, n)
    t0 = time.perf_counter()
    if cfg.kind == "lj":
        dens = n / float(cfg.box[0] * cfg.box[1] * cfg.box[2])
        c.generate_fcc(dens, 0.85 if name != "lj500" else 1.0, seed=2024)
        what = "FCC lattice with Gaussian velocities (mdg_generate_fcc)"
    else:
        rad = st["radius"]
        poly = float(rad.min()) != float(rad.max())
        c.generate_gas(n, w.POLY_R if poly else float(rad[0]), sep_factor=1.0 if poly else 1.1,
                       velocity="maxwell_rms" if poly else "speed", speed=0.5, seed=2024)
        what = "grid-parallel RSA and velocities (mdg_generate_gas)"
    out["device_generator_s"] = time.perf_counter() - t0
    out["device_generator"] = what
    c.close()
    return out


def e2e(cfg, make, steps):
    """End to end through the public C ABI with host buffers: upload of the
    host state, `steps` x (mdg_step(1) + mdg_thermo read-back), download of the
    final state; wall clock around all of it."""
    from mddem_gb300 import capi

    st = make()
    n = len(st["tag"])
    ctx = capi.Context(cfg, n)
    ctx.upload(st)
    ctx.step(3)
    t0 = time.perf_counter()
    ctx.upload(st)
    for _ in range(steps):
        ctx.step(1)
        ctx.thermo()
    out = ctx.download()
    el = time.perf_counter() - t0
    up = sum(st[k].nbytes for k in ("tag", "type", "pos", "vel", "mass", "cutoff_radius"))
    down = sum(v.nbytes for v in out.values())
    thermo_bytes = 8 * 16 + 8 * 16
    return {"value": n * steps / el, "unit": "particle-steps/s", "h2d_bytes_per_step": up / steps,
            "d2h_bytes_per_step": thermo_bytes + down / steps}


if __name__ == "__main__":
    main()
