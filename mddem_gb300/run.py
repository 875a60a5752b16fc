"""Run a reference TOML config on the GPU path: ``python -m mddem_gb300.run config.toml``.

The host side of the reference's ``App`` for this path (examples/*/main.rs with
CorePlugins + GranularDefaultPlugins or LJDefaultPlugins): the TOML sections
the hot path reads (``config.from_toml``), the initial state from ``[lattice]``
(FCC, crates/md_lattice/src/lib.rs:232-471) or ``[[particles.insert]]``
(random insertion, crates/dem_atom/src/insert.rs:417-614: region = domain
inset by the radius or a block region, rejection at 1.1 (r_i + r_j), per-component Gaussian
velocities of std ``velocity`` plus ``velocity_x/y/z``; or ``source = "file"``
CSV, insert.rs:652-776), the timestep (``[run] dt``, else 0.15 Rayleigh time
of the smallest sphere, insert.rs:1392-1431, or 0.005 for a lattice), then
``[run] steps`` steps with a thermo line every ``[run] thermo`` steps,
``[measure]`` RDF / MSD sampling (md_measure) written at the end, and
``[restart]`` files in the reference's format every ``interval`` steps in
``<output dir>/restart`` (restart_base_dir, crates/mddem_print/src/lib.rs:
528-534); ``read = true`` resumes from the latest file there (read_restart,
lib.rs:1143-1260): state, forces, contact history and the step count.
The state lives on the GPU throughout; the host only sees thermo values and
the states it writes.
"""
from __future__ import annotations

import argparse
import math
import os
import sys
import time
import tomllib

import numpy as np

from . import capi, config, inputs, restart


class RunError(ValueError):
    pass


def _insert(doc, cfg, seed):
    blocks = doc.get("particles", {}).get("insert", [])
    if not blocks:
        raise RunError("a DEM config needs [[particles.insert]]")
    names = [m.name for m in cfg.materials]
    states = []
    for k, b in enumerate(blocks):
        if b.get("source", "random") == "file":
            if b.get("format", "csv") != "csv":
                raise RunError(f"insert source format {b.get('format')!r}: only csv is supported")
            states.append(inputs.read_csv(b["file"], density=float(b.get("density", 2500.0))))
            continue
        if "rate" in b:
            raise RunError("rate-based insertion is not supported")
        n = int(b["count"])
        rad = b["radius"]
        if isinstance(rad, dict):
            if rad.get("distribution") != "uniform":
                raise RunError(f"radius distribution {rad.get('distribution')!r}: fixed or uniform only")
            rmin, rmax = float(rad["min"]), float(rad["max"])
        else:
            rmin = rmax = float(rad)
        lo, hi, inset = cfg.box_lo, cfg.box_hi, True
        reg = b.get("region")
        if reg:
            # Region::Block: centres uniform inside [min, max], no inset (insert.rs:522-543)
            if reg.get("type") != "block":
                raise RunError(f"insertion region {reg.get('type')!r}: only block regions are supported")
            lo, hi, inset = tuple(map(float, reg["min"])), tuple(map(float, reg["max"])), False
        pos, r = capi.rsa_spheres(n, lo, hi, rmin, rmax, sep_factor=1.1, inset=inset, seed=seed + k)
        rng = np.random.default_rng(seed + 7919 * (k + 1))
        v = float(b.get("velocity", 0.0))
        vel = rng.normal(0.0, v, size=(n, 3)) if v > 0.0 else np.zeros((n, 3))
        vel += np.array([float(b.get("velocity_x", 0.0)), float(b.get("velocity_y", 0.0)),
                         float(b.get("velocity_z", 0.0))])
        mat = b.get("material", names[0])
        if mat not in names:
            raise RunError(f"material {mat!r} is not in [[dem.materials]]")
        st = inputs._dem_state(pos, vel, r, float(b["density"]), mtype=np.full(n, names.index(mat)))
        states.append(st)
    if len(states) == 1:
        return states[0]
    out = {}
    for key in states[0]:
        if isinstance(states[0][key], np.ndarray):
            out[key] = np.concatenate([s[key] for s in states])
    out["tag"] = np.arange(len(out["tag"]), dtype=np.uint32)
    return out


def _device_spec(doc, cfg, seed):
    """[gpu] generate = "device": the device generator call that makes the
    system (mdg_generate_fcc / mdg_generate_gas) instead of a host state; a
    granular config needs one random insertion block in the whole domain
    without directional velocity."""
    if cfg.kind == "lj":
        lat = doc.get("lattice")
        if not lat or lat.get("style", "fcc") != "fcc":
            raise RunError("an LJ config needs [lattice] style = \"fcc\"")
        rho = float(lat.get("density", 0.85))
        n = 4
        for d in range(3):
            n *= int(math.floor(cfg.box[d] / (4.0 / rho) ** (1.0 / 3.0)))
        return {"generate": "fcc", "n": n, "density": rho, "temperature": float(lat.get("temperature", 0.85)),
                "mass": float(lat.get("mass", 1.0)), "skin": float(lat.get("skin", 1.25)), "seed": seed,
                "type_fractions": lat.get("type_fractions"), "type_masses": lat.get("type_masses")}
    blocks = doc.get("particles", {}).get("insert", [])
    if len(blocks) != 1:
        raise RunError('generate = "device": one [[particles.insert]] block')
    b = blocks[0]
    if b.get("source", "random") != "random" or "rate" in b or "region" in b:
        raise RunError('generate = "device": random insertion in the whole domain only')
    if any(float(b.get(k, 0.0)) != 0.0 for k in ("velocity_x", "velocity_y", "velocity_z")):
        raise RunError('generate = "device": directional velocities are not supported')
    rad = b["radius"]
    rmin, rmax = (float(rad["min"]), float(rad["max"])) if isinstance(rad, dict) else (float(rad), float(rad))
    names = [m.name for m in cfg.materials]
    mat = b.get("material", names[0])
    if mat not in names:
        raise RunError(f"material {mat!r} is not in [[dem.materials]]")
    return {"generate": "gas", "n": int(b["count"]), "radius": (rmin, rmax), "density": float(b.get("density", 2500.0)),
            "sep_factor": 1.1, "velocity": "gaussian", "speed": float(b.get("velocity", 0.0)),
            "material": names.index(mat), "seed": seed}


def setup(text, seed=0, precision=None):
    """(config, initial state, run settings) from a reference TOML text; with
    [gpu] generate = "device" the state is the device generator's spec (a dict
    with "generate")."""
    doc = tomllib.loads(text)
    cfg = config.from_toml(text)
    if precision:
        cfg = cfg.replace(precision=precision)
    run = doc.get("run", {})
    if isinstance(run, list):
        run = run[0] if run else {}
    gen = doc.get("gpu", {}).get("generate", "host")
    if gen not in ("host", "device"):
        raise RunError(f"generate = {gen!r}: host or device")
    if gen == "device":
        st = _device_spec(doc, cfg, seed)
        if cfg.kind == "dem" and cfg.dt == 0.0:
            m = cfg.materials[0]
            cfg = cfg.replace(dt=config.rayleigh_dt(st["radius"][0], st["density"], m.youngs_mod, m.poisson_ratio))
    elif cfg.kind == "lj":
        lat = doc.get("lattice")
        if not lat or lat.get("style", "fcc") != "fcc":
            raise RunError("an LJ config needs [lattice] style = \"fcc\"")
        L = cfg.box[0]
        rho = float(lat.get("density", 0.85))
        ncell = int(math.floor(L / (4.0 / rho) ** (1.0 / 3.0)))
        extra = set(lat) - {"style", "density", "temperature", "mass", "skin", "type_fractions", "type_masses"}
        if extra:
            raise RunError(f"[lattice]: unknown key(s) {sorted(extra)}")
        st = inputs.lj_fcc(ncell, L, rho, float(lat.get("temperature", 0.85)), mass=float(lat.get("mass", 1.0)),
                           skin=float(lat.get("skin", 1.25)), seed=seed, lo=cfg.box_lo[0],
                           type_fractions=lat.get("type_fractions"), type_masses=lat.get("type_masses"))
        if cfg.lj_types > 1 and int(st["type"].max()) >= cfg.lj_types:
            raise RunError(f"[lattice] type_fractions give {int(st['type'].max()) + 1} types, [lj] types has "
                           f"{cfg.lj_types}")
    else:
        st = _insert(doc, cfg, seed)
        if cfg.dt == 0.0:
            m = cfg.materials[0]
            dens = np.asarray(st.get("density", np.full(len(st["tag"]), 2500.0)))
            cfg = cfg.replace(dt=config.rayleigh_dt(float(np.min(st["radius"])), float(np.max(dens)),
                                                    m.youngs_mod, m.poisson_ratio))
    extra = set(doc.get("restart", {})) - {"interval", "format", "read"}
    if extra:
        raise RunError(f"[restart]: unknown key(s) {sorted(extra)} (RestartConfig: interval, format, read)")
    settings = {
        "steps": int(run.get("steps", 1000)),
        "thermo": int(run.get("thermo", 100)),
        "measure": doc.get("measure", {}),
        "restart": doc.get("restart", {}),
        "output": doc.get("output", {}).get("dir", "output"),
    }
    return cfg, st, settings


def latest_restart(directory, fmt="bincode", rank=0):
    """The restart file with the highest step for `rank` and `fmt` in
    `directory`, or None (read_restart's scan, lib.rs:1163-1185)."""
    ext = "json" if fmt == "json" else "bin"
    suffix = f"_rank{rank}.{ext}"
    best = None
    try:
        names = os.listdir(directory)
    except OSError:
        return None
    for name in names:
        if name.startswith("restart_") and name.endswith(suffix):
            mid = name[len("restart_"):len(name) - len(suffix)]
            if mid.isdigit() and (best is None or int(mid) > best[0]):
                best = (int(mid), name)
    return os.path.join(directory, best[1]) if best else None


def thermo_line(step, t, kind):
    if kind == "lj":
        return (f"{step:10d} T {t['temp']:.6f} KE {t['ke']:.6e} PE {t['pe']:.6e} E {t['ke'] + t['pe']:.6e} "
                f"P {t['pressure']:.5f}")
    return (f"{step:10d} T_g {t['granular_temp']:.6e} T_rot {t['rot_temp']:.6e} KE {t['ke']:.6e} "
            f"|P| {t['momentum']:.3e}")


def run(text, seed=0, precision=None, steps=None, out=sys.stdout):
    cfg, st, s = setup(text, seed, precision)
    nsteps = s["steps"] if steps is None else steps
    rs = s["restart"]
    rst_dir = os.path.join(s["output"], "restart")
    base = 0
    src = latest_restart(rst_dir, rs.get("format", "bincode")) if rs and rs.get("read") else None
    if src:
        st, hist, base, _ = restart.read_restart(src)
        print(f"# Restart: reading from {src}", file=out)
    if "generate" in st:  # made on the device
        spec = dict(st)
        kind, n = spec.pop("generate"), spec.pop("n")
        ctx = capi.Context(cfg, n)
        if kind == "fcc":
            ctx.generate_fcc(**spec)
        else:
            ctx.generate_gas(n, **spec)
    else:
        n = len(st["tag"])
        ctx = capi.Context(cfg, n)
        ctx.upload(st)
    if src and hist is not None and len(hist[0]):
        ctx.set_history(*hist)
    meas = s["measure"]
    rdf_every = int(meas.get("rdf_interval", 0)) if cfg.kind == "lj" and meas else 0
    msd_every = int(meas.get("msd_interval", 0)) if cfg.kind == "lj" and meas else 0
    nbins, rmax = int(meas.get("rdf_bins", 200)), float(meas.get("rdf_cutoff", 3.0))
    rst_every = int(rs.get("interval", 0)) if rs else 0
    fmt = rs.get("format", "bincode") if rs else "bincode"
    if rst_every or rdf_every or msd_every:
        os.makedirs(s["output"], exist_ok=True)
    if rst_every:
        os.makedirs(rst_dir, exist_ok=True)
    g_sum, g_n, msd = None, 0, []
    if msd_every:
        ctx.msd_reset()
    marks = sorted({k for every in (s["thermo"], rdf_every, msd_every, rst_every) if every
                    for k in range(every, nsteps + 1, every)} | {nsteps})
    print(f"# {cfg.kind} N={n} dt={cfg.dt:.6e} steps={nsteps} precision={cfg.precision}", file=out)
    print(thermo_line(base, ctx.thermo(), cfg.kind), file=out)
    done, t0 = 0, time.perf_counter()
    for k in marks:
        ctx.step(k - done)  # one graph launch for all the steps up to the next mark
        done = k
        if s["thermo"] and k % s["thermo"] == 0 or k == nsteps:
            print(thermo_line(base + k, ctx.thermo(), cfg.kind), file=out)
        if rdf_every and k % rdf_every == 0:
            r, g, _ = ctx.rdf(r_max=rmax, nbins=nbins)
            g_sum = g if g_sum is None else g_sum + g
            g_n += 1
        if msd_every and k % msd_every == 0:
            msd.append((base + k, ctx.msd()))
        if rst_every and k % rst_every == 0:
            p = os.path.join(rst_dir, restart.restart_filename(base + k, 0, fmt))
            hist = ctx.history() if cfg.kind == "dem" else None
            restart.write_restart(p, ctx.download(), hist, step=base + k, dt=cfg.dt, fmt=fmt)
    el = time.perf_counter() - t0
    print(f"# {nsteps} steps in {el:.3f} s: {n * nsteps / max(el, 1e-9):.4e} particle-steps/s", file=out)
    if g_n:
        with open(os.path.join(s["output"], "rdf.txt"), "w") as f:
            for rr, gg in zip((np.arange(nbins) + 0.5) * rmax / nbins, g_sum / g_n):
                f.write(f"{rr:.6f} {gg:.6f}\n")
    if msd:
        with open(os.path.join(s["output"], "msd.txt"), "w") as f:
            for k, v in msd:
                f.write(f"{k} {v:.10e}\n")
    return ctx


def main(argv=None):
    ap = argparse.ArgumentParser(description="Run a reference TOML config on the GB300 hot path")
    ap.add_argument("config")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default=None)
    ap.add_argument("--steps", type=int, default=None)
    a = ap.parse_args(argv)
    with open(a.config, "rb") as f:
        text = f.read().decode()
    run(text, a.seed, a.precision, a.steps)


if __name__ == "__main__":
    main()
