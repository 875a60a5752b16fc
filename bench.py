"""Throughput benchmark: particle-steps/s of the hot path on one GB300.

Default workload (N=1): LJ fluid, 256,000 atoms (40^3 FCC cells, box 67.06,
rho* = 0.85, T* = 0.85), Nose-Hoover (T = 0.85, tau = 1), dt = 0.005, list
cutoff 2.8 (rc 2.5 x skin 1.12), mixed-precision forces (FP32 geometry and
arithmetic with Kahan sums, FP64 integration).  A "step" is one MD timestep
of the whole system.  Each timed step is bracketed by CUDA events on the
library's stream; L2 is flushed (512 MB write) before every step outside the
events.

--impl reference times the CPU FP64 restatement of the reference's path (the
oracle) on the same workload, one independent copy per host core.

Multi-GPU (--gpus N under torchrun): replicas only; every rank advances its
own copy of the workload; value = all ranks' particle-steps / max rank time.
"""
from __future__ import annotations

import argparse
import json
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


def workload(name):
    from mddem_gb300 import config, inputs

    if name == "lj256k":
        cfg = config.lj_fluid_config(box=67.06)
        return "LJ fluid 256000 atoms FCC rho=0.85 T=0.85 NH rc=2.5", cfg, lambda: inputs.lj_fcc(40, 67.06, 0.85, 0.85, seed=2024)
    if name == "lj864":
        cfg = config.lj_fluid_config(box=10.06)
        return "LJ fluid 864 atoms FCC rho=0.85 T=0.85 NH rc=2.5", cfg, lambda: inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=2024)
    if name == "dem500":
        cfg = config.granular_gas_config()
        return "DEM granular gas 500 glass spheres r=1mm box 0.025", cfg, lambda: inputs.dem_granular_gas(500, seed=0)
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

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
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


def force_bytes_per_particle(nfull, precision):
    """Algorithmic DRAM bytes per particle of one force launch: row length (4),
    the row's list entries (4 each), the particle's own geometry read once
    (fp64 row 32 B, or the two-float copy 32 B), and the force row written
    (32 B)."""
    return 4 + 4 * nfull + 32 + 32


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


def _ref_worker(args):
    wl, warm, steps, budget = args
    from oracle.oracle import Oracle

    desc, cfg, make = workload(wl)
    st = make()
    o = Oracle(cfg.replace(precision="fp64"))
    o.load(st)
    o.step(max(1, warm))
    t0 = time.perf_counter()
    done = 0
    for _ in range(steps):
        o.step(1)
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    return len(st["tag"]) * done, time.perf_counter() - t0, done


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp

    desc, cfg, make = workload(a.workload)
    cores = os.cpu_count() or 1
    ctxm = mp.get_context("spawn")
    budget = 60.0
    with ctxm.Pool(cores) as pool:
        res = pool.map(_ref_worker, [(a.workload, a.warmup, a.steps, budget)] * cores)
    total = sum(r[0] for r in res)
    wall = max(r[1] for r in res)
    val = total / wall
    line = {
        "impl": "reference", "metric": "particle-steps/s", "value": val, "unit": "particle-steps/s",
        "n_gpus": a.gpus, "steps": min(r[2] for r in res), "warmup": a.warmup, "ms_per_step": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "replicas": cores},
        "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} independent copies x {min(r[2] for r in res)} timesteps, one per core"},
        "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--workload", default="lj256k")
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--policy", default="displacement")
    ap.add_argument("--tpp", type=int, default=0, help="threads per particle in the force kernel (0 = auto)")
    ap.add_argument("--eager", action="store_true", help="launch kernels one by one (for profilers)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    a = ap.parse_args()
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

    from mddem_gb300 import build, capi

    build.build()
    desc, cfg, make = workload(a.workload)
    cfg = cfg.replace(precision=a.precision, rebuild_policy=a.policy, threads_per_particle=a.tpp)
    st = make()
    n = len(st["tag"])
    ctx = capi.Context(cfg, n)
    ctx.upload(st)
    if a.eager:
        ctx.set_graph_mode(0)
    ctx.timed_steps(a.warmup, L2_FLUSH)
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        t, kernels, rebuilt = ctx.timed_steps(a.steps, L2_FLUSH)
    total_ms = float(t[:, 0].sum())
    if dist:
        import torch

        tt = torch.tensor([total_ms], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms = float(tt.item())
    value = world * n * a.steps / (total_ms / 1e3)
    th = ctx.thermo()
    nfull = th["max_neighbors"]
    pairs = len(ctx.pairs())
    nfull_avg = 2.0 * pairs / n
    force_ms = float(t[:, 3].mean())
    bpp = force_bytes_per_particle(nfull_avg, a.precision)
    achieved = bpp * n / (force_ms / 1e3) / 1e9
    peak, src = peak_hbm()
    kname = "k_lj_mixed" if a.precision == "mixed" else "k_lj_fp64"
    traffic = ncu_traffic(kname)
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": total_ms / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if a.precision == "mixed" else "f64",
        "data": "synthetic",
        "config": {"workload": desc, "precision": a.precision, "rebuild_policy": a.policy, "particles": n,
                   "l2": "flushed before every timed step (512 MB write)", "parallelism": f"replicas x{world}"},
        "phases_ms": {"initial": float(t[:, 1].mean()), "rebuild": float(t[:, 2].mean()), "force": force_ms,
                      "final": float(t[:, 4].mean())},
        "rebuild_steps": int(rebuilt.sum()),
        "gpu_launches": int(kernels.sum()),
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": src, "traffic": traffic,
                     "algorithmic_bytes_per_particle": bpp, "avg_full_neighbors": nfull_avg},
        "clocks": clk.summary(),
    }
    if rank == 0 and not a.no_e2e:
        line["e2e"] = e2e(cfg, make, a.steps)
    if rank == 0 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(a.workload)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


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
