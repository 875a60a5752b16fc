"""Shared helpers for the parity tests (CPU oracle vs CUDA path)."""
from __future__ import annotations

import numpy as np


def by_tag(st, *fields):
    """Return the given fields reordered by particle tag."""
    o = np.argsort(st["tag"], kind="stable")
    return [np.asarray(st[f])[o] for f in fields]


def pair_set(pairs):
    """Half-list pairs as a set of (owner tag, partner tag)."""
    return set(map(tuple, np.asarray(pairs).tolist()))


from mddem_gb300.validate import lj_pair_force_scale, rel_err  # noqa: E402,F401  (shared with bench.py)


def overlapping_spheres(n, box, radius, seed, sep_factor=0.96, speed=0.5, omega=200.0, poly=None):
    """Dense sphere packing with small overlaps, random velocities and spins:
    exercises every term of the contact law in one force evaluation."""
    from mddem_gb300 import inputs

    rad = radius if poly is None else poly
    pos, r = inputs.random_spheres(n, box, rad, seed=seed, sep_factor=sep_factor, inset=False)
    rng = np.random.default_rng(seed + 11)
    vel = rng.normal(scale=speed, size=(n, 3))
    st = inputs._dem_state(pos, vel, r, 2500.0)
    st["omega"] = rng.normal(scale=omega, size=(n, 3))
    return st


def dem_pair_force_scale(st_by_tag, box, pairs, e_eff):
    """Per-tag sum of Hertz elastic normal-force magnitudes 4/3 E* sqrt(R*) d^1.5
    over the particle's contacts: the per-pair force scale of the DEM
    force-error metric.  ``st_by_tag``: dict with pos and radius indexed by tag."""
    from mddem_gb300 import validate

    return validate.dem_pair_force_scale(st_by_tag["pos"], st_by_tag["radius"], box, pairs, e_eff)
