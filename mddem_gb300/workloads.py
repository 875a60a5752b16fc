"""Seeded synthetic workloads at the sizes of the hot path's benchmark cases.

* ``gas``: periodic monodisperse glass-sphere granular gas (E = 8.7e9 Pa,
  nu = 0.3, e = 0.95, mu = 0.4, r = 1 mm, rho = 2500), speeds 0.5 m/s in
  uniform directions, dt = 0.1 Rayleigh time;
* ``polydisperse_gas``: 1e6 spheres, r ~ U[0.8, 1.2] mm, solid fraction 0.30,
  Maxwellian speeds of RMS 0.5 m/s, dt = 0.1 Rayleigh time of the smallest;
* ``ensemble``: 256 independent gas replicas, N log-uniform in [500, 50000],
  solid fraction U[0.1, 0.3], restitution U[0.70, 0.99], friction U[0, 0.5],
  advanced in one batch context;
* ``serve_trace``: a Poisson-arriving job stream, 50 % cooling gases
  (N log-uniform [100, 200000], solid fraction U[0.05, 0.3], e U[0.8, 0.99]),
  25 % two-sphere Hertz rebounds (approach speed U[0.1, 2] m/s), 25 % LJ FCC
  melts (N in [500, 100000], rho* U[0.8, 0.9], T* U[0.7, 1.2]); step counts
  log-uniform in [1000, 50000].

Placement of more than a few thousand spheres uses the native grid RSA.  Its
exclusion factor is the reference's 1.1 (insert.rs:523-555) where the
resulting effective solid fraction stays below 0.3, else 1.0 (plain
non-overlap): 1.1^3 x 0.3 = 0.40 lies above the random-sequential-addition
jamming limit (about 0.38).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import config, inputs

SPHERE_V = 4.0 / 3.0 * math.pi * 1e-9  # volume of a 1 mm sphere
DT_GAS = config.rayleigh_dt(1e-3, 2500.0, 8.7e9, 0.3, fraction=0.1)  # 2.934e-7 s


def gas_box(n, phi, mean_r3=1e-9):
    return (n * 4.0 / 3.0 * math.pi * mean_r3 / phi) ** (1.0 / 3.0)


def sep_for(phi):
    return 1.1 if phi * 1.1 ** 3 <= 0.3 else 1.0


def gas(n, phi=None, box=None, restitution=0.95, friction=0.4, seed=0, precision="mixed", policy="displacement",
        rsa=None):
    """Monodisperse granular gas of n spheres at solid fraction phi (or in a
    cube of side box)."""
    if box is None:
        box = gas_box(n, phi)
    phi = phi if phi is not None else n * SPHERE_V / box ** 3
    cfg = config.granular_gas_config(box=box, dt=DT_GAS, precision=precision, policy=policy)
    cfg.materials[0].restitution = float(restitution)
    cfg.materials[0].friction = float(friction)
    st = inputs.dem_granular_gas(n, box=box, seed=seed, sep_factor=sep_for(phi), native=True, rsa=rsa)
    return cfg, st


POLY_R = (0.8e-3, 1.2e-3)


def polydisperse_config(n=1_000_000, phi=0.30, precision="mixed", policy="displacement"):
    rmin, rmax = POLY_R
    mean_r3 = (rmax ** 4 - rmin ** 4) / (4.0 * (rmax - rmin))
    box = gas_box(n, phi, mean_r3)
    dt = config.rayleigh_dt(rmin, 2500.0, 8.7e9, 0.3, fraction=0.1)
    return config.granular_gas_config(box=box, dt=dt, precision=precision, policy=policy)


def polydisperse_gas(n=1_000_000, phi=0.30, seed=0, precision="mixed", policy="displacement", rsa=None):
    cfg = polydisperse_config(n, phi, precision, policy)
    st = inputs.dem_granular_gas(n, box=cfg.box[0], radius=POLY_R, seed=seed, sep_factor=1.0, maxwellian=True,
                                 native=True, rsa=rsa)
    return cfg, st


def ensemble(nrep=256, nmin=500, nmax=50000, seed=0, precision="mixed", policy="displacement", rsa=None,
             only=None):
    """Returns [(cfg, state)] for the replica ensemble (the replicas listed in
    ``only``, default all; each replica's parameters do not depend on which
    are built)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nrep):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        phi = rng.uniform(0.1, 0.3)
        e = rng.uniform(0.70, 0.99)
        mu = rng.uniform(0.0, 0.5)
        if only is not None and k not in only:
            continue
        out.append(gas(n, phi=phi, restitution=e, friction=mu, seed=seed * 100003 + k, precision=precision,
                       policy=policy, rsa=rsa))
    return out


@dataclass
class Job:
    kind: str          # "gas" | "rebound" | "lj"
    n: int
    steps: int
    arrival: float     # in pump ticks
    params: dict = field(default_factory=dict)

    def make(self, precision="mixed", policy="displacement", rsa=None):
        """(config, initial state); ``rsa``: the sphere generator for gases
        (default the library's, see inputs.dem_granular_gas)."""
        p = self.params
        if self.kind == "gas":
            return gas(self.n, phi=p["phi"], restitution=p["e"], seed=p["seed"], precision=precision, policy=policy,
                       rsa=rsa)
        if self.kind == "rebound":
            st = inputs.two_sphere_rebound(speed=p["speed"])
            cfg = config.granular_gas_config(box=st["box"], dt=DT_GAS, precision=precision, policy=policy)
            return cfg, st
        nc = p["cells"]
        a = (4.0 / p["rho"]) ** (1.0 / 3.0)
        box = (nc + 1e-6) * a
        cfg = config.lj_fluid_config(box=box, precision=precision, policy=policy)
        cfg = cfg.replace(nh_temperature=p["T"])
        st = inputs.lj_fcc(nc, box, p["rho"], p["T"], seed=p["seed"])
        return cfg, st


def serve_trace(njobs=64, rate=0.5, seed=0, smin=1000, smax=50000, mix=(0.5, 0.25, 0.25)):
    """Job stream; arrivals are a Poisson process of `rate` jobs per pump tick.
    The kinds (cooling gas, two-sphere rebound, LJ melt) come in the exact
    proportions `mix` (rounded), in a seeded random order."""
    rng = np.random.default_rng(seed)
    ngas = int(round(mix[0] * njobs))
    nreb = int(round(mix[1] * njobs))
    kinds = np.array(["gas"] * ngas + ["rebound"] * nreb + ["lj"] * (njobs - ngas - nreb))
    kinds = kinds[rng.permutation(njobs)]
    t = 0.0
    jobs = []
    for k in range(njobs):
        t += rng.exponential(1.0 / rate) if k else 0.0
        steps = int(round(math.exp(rng.uniform(math.log(smin), math.log(smax)))))
        kind = kinds[k]
        if kind == "gas":
            n = int(round(math.exp(rng.uniform(math.log(100), math.log(200000)))))
            jobs.append(Job("gas", n, steps, t, dict(phi=rng.uniform(0.05, 0.3), e=rng.uniform(0.8, 0.99),
                                                       seed=seed * 1000 + k)))
        elif kind == "rebound":
            jobs.append(Job("rebound", 2, steps, t, dict(speed=rng.uniform(0.1, 2.0))))
        else:
            n_target = math.exp(rng.uniform(math.log(500), math.log(100000)))
            nc = max(5, int(round((n_target / 4.0) ** (1.0 / 3.0))))
            jobs.append(Job("lj", 4 * nc ** 3, steps, t, dict(cells=nc, rho=rng.uniform(0.8, 0.9),
                                                                T=rng.uniform(0.7, 1.2), seed=seed * 1000 + k)))
    return jobs


# Server slot classes for the job stream: (capacity, count).  DEM slots hold
# the rebounds (2 spheres) and gases up to 200000 spheres, LJ slots the melts
# up to 4 x 29^3 = 97556 atoms.
SERVE_DEM_SLOTS = [(128, 32), (1024, 24), (8192, 16), (65536, 12), (200000, 8)]
SERVE_LJ_SLOTS = [(2048, 8), (16384, 8), (100000, 6)]


SERVE_SPLIT = {"lj": 16384, "dem": None}  # "split": the larger slots of a kind get their own context


def serve_groups(cfgs, caps, policy="kind", small=1024, split=None):
    """Per-slot group ids for capi.Server(groups=...): "kind" one batch
    context per particle kind; "split" as "kind", with the slots of a kind
    above its `split` capacity (default SERVE_SPLIT) in a context of their
    own; "size" the slots of capacity <= `small` apart from the larger ones
    of their kind; "class" one context per (kind, capacity)."""
    split = SERVE_SPLIT if split is None else split
    keys = []
    for c, cap in zip(cfgs, caps):
        if policy == "kind":
            keys.append(c.kind)
        elif policy == "split":
            lim = split.get(c.kind)
            keys.append((c.kind, lim is not None and cap > lim))
        elif policy == "size":
            keys.append((c.kind, cap <= small))
        elif policy == "class":
            keys.append((c.kind, cap))
        else:
            raise ValueError(f"unknown grouping {policy}")
    ids = {}
    return [ids.setdefault(k, len(ids)) for k in keys]


def serve_slots(precision="mixed", policy="displacement", mult=1):
    """(slot configs, slot capacities) for a job server over serve_trace;
    `mult` times the slot counts of SERVE_DEM_SLOTS / SERVE_LJ_SLOTS."""
    cfgs, caps = [], []
    for cap, cnt in SERVE_DEM_SLOTS:
        cfgs += [config.granular_gas_config(precision=precision, policy=policy)] * (cnt * mult)
        caps += [cap] * (cnt * mult)
    for cap, cnt in SERVE_LJ_SLOTS:
        cfgs += [config.lj_fluid_config(precision=precision, policy=policy)] * (cnt * mult)
        caps += [cap] * (cnt * mult)
    return cfgs, caps
