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


def lj_pair_force_scale(pos, box, pairs, rc=2.5, eps=1.0, sigma=1.0, types=None, table=None):
    """Per-tag sum of |f_pair| over the particle's LJ pairs (the normaliser of
    the per-particle force-error metric).  ``pos`` indexed by tag; with
    ``types`` (by tag) and an n x n ``table`` of (eps, sigma, rc) triples the
    coefficients of each pair come from its two types."""
    n = pos.shape[0]
    p = np.asarray(pairs, dtype=np.int64)
    d = pos[p[:, 1]] - pos[p[:, 0]]
    L = np.asarray(box)
    d -= L * np.round(d / L)
    r2 = np.einsum("ij,ij->i", d, d)
    if table is not None:
        nt = int(round(len(table) ** 0.5))
        tab = np.asarray(table, dtype=np.float64).reshape(nt * nt, 3)
        c = tab[np.asarray(types)[p[:, 0]].astype(np.int64) * nt + np.asarray(types)[p[:, 1]]]
        eps, sigma, rc = c[:, 0], c[:, 1], c[:, 2]
    else:
        eps, sigma, rc = np.full(len(p), eps), np.full(len(p), sigma), np.full(len(p), rc)
    m = r2 < (rc * sigma) ** 2
    r2, eps, sigma = r2[m], eps[m], sigma[m]
    s6 = sigma ** 6
    inv2 = 1.0 / r2
    inv6 = inv2 ** 3
    f = np.abs(inv2 * inv6 * (48 * eps * s6 * s6 * inv6 - 24 * eps * s6)) * np.sqrt(r2)
    scale = np.zeros(n)
    np.add.at(scale, p[m, 0], f)
    np.add.at(scale, p[m, 1], f)
    return scale


def rel_err(a, b, scale, tiny=1e-300):
    """max over particles of |a - b|_inf / max(|b|_inf, scale, tiny)."""
    num = np.max(np.abs(a - b), axis=1)
    den = np.maximum(np.maximum(np.max(np.abs(b), axis=1), scale), tiny)
    return float(np.max(num / den))


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
    pos, rad = st_by_tag["pos"], st_by_tag["radius"]
    n = pos.shape[0]
    p = np.asarray(pairs, dtype=np.int64)
    scale = np.zeros(n)
    if len(p) == 0:
        return scale
    d = pos[p[:, 1]] - pos[p[:, 0]]
    L = np.asarray(box)
    d -= L * np.round(d / L)
    dist = np.sqrt(np.einsum("ij,ij->i", d, d))
    r1, r2 = rad[p[:, 0]], rad[p[:, 1]]
    delta = np.clip(r1 + r2 - dist, 0.0, None)
    reff = r1 * r2 / (r1 + r2)
    f = 4.0 / 3.0 * e_eff * np.sqrt(reff) * delta ** 1.5
    np.add.at(scale, p[:, 0], f)
    np.add.at(scale, p[:, 1], f)
    return scale
