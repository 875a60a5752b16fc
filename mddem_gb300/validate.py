"""Error statements of the precision form: the measurements the parity tests
and bench.py's error block share.

* per-particle force / torque error, |F_a - F_b|_inf / max(|F_b|_inf,
  sum_pairs |f_pair|, tiny), with the pair sum from the pair list: the Hertz
  elastic normal force 4/3 E* sqrt(R*) delta^1.5 for granular pairs, the LJ
  12-6 pair force for LJ pairs;
* total-energy drift: the slope of a linear fit of KE + PE against the step;
* Haff cooling (Haff 1983; kinetic theory as in the reference's
  examples/granular_gas_benchmark/haff_analysis.py:82-104): T(t) = T0 /
  (1 + t / t_c)^2 fitted on 1 / sqrt(T), and t_c of kinetic theory.

The functions take any object with the stepping interface of capi.Context
(step, force_only, thermo), so a GPU context and a CPU stand-in can be
measured by the same code.
"""
from __future__ import annotations

import math

import numpy as np


def rel_err(a, b, scale, tiny=1e-300):
    """max over particles of |a - b|_inf / max(|b|_inf, scale, tiny)."""
    num = np.max(np.abs(np.asarray(a) - np.asarray(b)), axis=1)
    den = np.maximum(np.maximum(np.max(np.abs(b), axis=1), scale), tiny)
    return float(np.max(num / den)) if len(num) else 0.0


def _min_image(d, box):
    L = np.asarray(box, dtype=np.float64)
    return d - L * np.round(d / L)


def lj_pair_force_scale(pos, box, pairs, rc=2.5, eps=1.0, sigma=1.0, types=None, table=None):
    """Per-particle sum of |f_pair| over the particle's LJ pairs; ``pos`` and
    ``types`` indexed like the pair list's entries (by tag); an n x n
    ``table`` of (eps, sigma, rc) per type pair when ``types`` is given."""
    n = pos.shape[0]
    p = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    scale = np.zeros(n)
    if len(p) == 0:
        return scale
    d = _min_image(pos[p[:, 1]] - pos[p[:, 0]], box)
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
    np.add.at(scale, p[m, 0], f)
    np.add.at(scale, p[m, 1], f)
    return scale


def dem_pair_force_scale(pos, radius, box, pairs, e_eff):
    """Per-particle sum of Hertz elastic normal-force magnitudes
    4/3 E* sqrt(R*) delta^1.5 over the particle's contacts (arrays indexed
    like the pair list's entries)."""
    n = pos.shape[0]
    p = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    scale = np.zeros(n)
    if len(p) == 0:
        return scale
    d = _min_image(pos[p[:, 1]] - pos[p[:, 0]], box)
    dist = np.sqrt(np.einsum("ij,ij->i", d, d))
    r1, r2 = radius[p[:, 0]], radius[p[:, 1]]
    delta = np.clip(r1 + r2 - dist, 0.0, None)
    f = 4.0 / 3.0 * e_eff * np.sqrt(r1 * r2 / (r1 + r2)) * delta ** 1.5
    np.add.at(scale, p[:, 0], f)
    np.add.at(scale, p[:, 1], f)
    return scale


def e_eff(youngs_mod=8.7e9, poisson_ratio=0.3):
    """Effective modulus of two equal materials, 1/E* = 2 (1 - nu^2) / E."""
    return 1.0 / (2.0 * (1.0 - poisson_ratio ** 2) / youngs_mod)


def by_tag(st, *fields):
    o = np.argsort(st["tag"], kind="stable")
    return [np.asarray(st[f])[o] for f in fields]


def force_error(cfg, ref_state, test_state, pairs):
    """Per-particle force (and, granular, torque) error of test_state against
    ref_state after a force evaluation of the same state; ``pairs`` is the
    reference's half list as (tag, tag).  Returns {"force": e, "torque": e}."""
    out = {}
    if cfg.kind == "dem":
        fa, ta, pos, rad = by_tag(ref_state, "force", "torque", "pos", "radius")
        fb, tb = by_tag(test_state, "force", "torque")
        m = cfg.materials[0]
        sc = dem_pair_force_scale(pos, rad, cfg.box, pairs, e_eff(m.youngs_mod, m.poisson_ratio))
        out["force"] = rel_err(fb, fa, sc)
        out["torque"] = rel_err(tb, ta, sc * rad)
    else:
        fa, pos = by_tag(ref_state, "force", "pos")
        (fb,) = by_tag(test_state, "force")
        sc = lj_pair_force_scale(pos, cfg.box, pairs, rc=cfg.lj_cutoff, eps=cfg.lj_epsilon, sigma=cfg.lj_sigma)
        out["force"] = rel_err(fb, fa, sc)
    return out


def energy_drift(sim, steps=2000, every=50):
    """(energies, slope per step) of KE + PE sampled every `every` steps."""
    sim.force_only()
    E = []
    for k in range(steps // every + 1):
        t = sim.thermo()
        E.append(t["ke"] + t["pe"])
        if k < steps // every:
            sim.step(every)
    E = np.array(E)
    return E, float(np.polyfit(np.arange(len(E)) * every, E, 1)[0])


def cooling(sim, dt, steps=40000, every=2000):
    """Granular temperature sampled every `every` steps: (t_c fitted on
    1/sqrt(T) = (1 + t/t_c) / sqrt(T0), T_end / T_0, the samples)."""
    T = []
    for k in range(steps // every + 1):
        T.append(sim.thermo()["granular_temp"])
        if k < steps // every:
            sim.step(every)
    T = np.array(T)
    t = np.arange(len(T)) * every * dt
    a, b = np.polyfit(t, 1.0 / np.sqrt(T), 1)
    return float(b / a), float(T[-1] / T[0]), T


def haff_theory(n, box, radius, restitution, T0):
    """t_c = 2 / (omega_0 sqrt(T0)) with omega_0 = 4/3 n d^2 g0 sqrt(pi)
    (1 - e^2) and the Carnahan-Starling g0 (monodisperse spheres)."""
    nd = n / box ** 3
    ph = nd * 4.0 / 3.0 * math.pi * radius ** 3
    g0 = (1.0 - ph / 2.0) / (1.0 - ph) ** 3
    om = 4.0 / 3.0 * nd * (2.0 * radius) ** 2 * g0 * math.sqrt(math.pi) * (1.0 - restitution ** 2)
    return float(2.0 / (om * math.sqrt(T0)))


def haff(sim, cfg, n, restitution, radius=1e-3, steps=40000, every=2000):
    """Haff cooling of a frictionless granular gas: (t_c fitted on
    1/sqrt(T) = (1 + t/t_c) / sqrt(T0), t_c of kinetic theory, T_end / T_0)."""
    tc, ratio, T = cooling(sim, cfg.dt, steps, every)
    return tc, haff_theory(n, cfg.box[0], radius, restitution, T[0]), ratio


def rdf_checks(r, g):
    """The LJ liquid structure checks of the reference's
    examples/lj_argon/validate.py:66-110: first peak position in
    [0.95, 1.15] sigma and height in [2.4, 3.5] (r in (0.8, 1.5)), mean g
    over r in (2.0, 2.8) within [0.7, 1.3]."""
    sel = (r > 0.8) & (r < 1.5)
    k = int(np.argmax(g[sel]))
    peak_r, peak_g = float(r[sel][k]), float(g[sel][k])
    far = float(np.mean(g[(r > 2.0) & (r < 2.8)]))
    return {"peak_r": peak_r, "peak_g": peak_g, "far_mean": far,
            "pass": bool(0.95 <= peak_r <= 1.15 and 2.4 <= peak_g <= 3.5 and 0.7 <= far <= 1.3)}
