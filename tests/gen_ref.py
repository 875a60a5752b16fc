"""CPU restatement of the device generators (mddem_gb300/csrc/mdg_generate.cu),
test infrastructure: the counter-based draws, the FCC lattice with its
velocity fix-up, sequential random sequential addition over the generator's
proposal stream, and the gas velocities.

The device RSA settles each batch of proposals so that its result equals the
sequential algorithm on the same stream; `rsa` here is that sequential
algorithm, one proposal after another, with the same floating-point
operations (centre in_lo + in_w u, minimum image d - L rint(d / L), squared
distance summed x, y, z, rejection when r^2 <= (sep (r_i + r_j))^2), so
centres and radii compare bit for bit.  Normals use numpy's sin/cos where the
device uses sincospi: velocities compare to ~1e-15 relative.
"""
from __future__ import annotations

import math

import numpy as np

GOLDEN = 0x9E3779B97F4A7C15
M64 = (1 << 64) - 1
STREAM_PLACE, STREAM_VEL = 1, 2


def _mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def draw(seed, stream, idx):
    """mdg_counter_draw over an index array."""
    key = int(_mix64(np.array([(seed + GOLDEN * (stream + 1)) & M64], dtype=np.uint64))[0])
    i = np.asarray(idx, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return _mix64(np.uint64(key) + np.uint64(GOLDEN) * (i + np.uint64(1)))


def uniform(h):
    return (np.asarray(h, dtype=np.uint64) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def normal3(seed, n):
    """(n, 3) standard normals: Box-Muller of draws (4i, 4i+1) and (4i+2, 4i+3)
    of the velocity stream, the fourth normal dropped."""
    i = np.arange(n, dtype=np.uint64) * np.uint64(4)
    out = np.empty((n, 3))
    for k, base in enumerate((i, i + np.uint64(2))):
        u1 = ((draw(seed, STREAM_VEL, base) >> np.uint64(11)).astype(np.float64) + 1.0) * 2.0 ** -53
        u2 = uniform(draw(seed, STREAM_VEL, base + np.uint64(1)))
        r = np.sqrt(-2.0 * np.log(u1))
        out[:, 2 * k] = r * np.cos(2.0 * math.pi * u2)
        if k == 0:
            out[:, 1] = r * np.sin(2.0 * math.pi * u2)
    return out


def fcc(box, density, temperature, mass=1.0, seed=0, lo=0.0, type_fractions=None, type_masses=None):
    """(pos, vel, types, masses) of mdg_generate_fcc in a cube of side box."""
    from mddem_gb300 import inputs

    nc = int(math.floor(box / math.cbrt(4.0 / density)))
    st = inputs.lj_fcc(nc, box, density, temperature, mass=mass, seed=0, lo=lo, type_fractions=type_fractions,
                       type_masses=type_masses)
    n = len(st["tag"])
    masses = st["mass"]
    v = normal3(seed, n) * np.sqrt(temperature / masses)[:, None]
    v -= v.sum(axis=0) / n
    ke = 0.5 * float(np.sum(masses * np.sum(v * v, axis=1)))
    cur = 2.0 * ke / (3.0 * n - 3.0)
    if cur > 1e-20:
        v *= math.sqrt(temperature / cur)
    return st["pos"], v, st["type"], masses


def rsa(n, box_lo, box_hi, rmin, rmax, sep, inset, seed, max_proposals=0, chunk=4096):
    """Sequential RSA over the generator's proposal stream: (centres (k, 3),
    radii (k,)) in acceptance order."""
    lo = np.asarray(box_lo, dtype=np.float64)
    hi = np.asarray(box_hi, dtype=np.float64)
    L = hi - lo
    in_lo = lo + (rmax if inset else 0.0)
    in_w = (hi - (rmax if inset else 0.0)) - in_lo
    limit = max_proposals or n * 20000
    P = np.empty((n, 3))
    R = np.empty(n)
    k = 0
    g0 = 0
    while k < n and g0 < limit:
        m = min(chunk, limit - g0)
        g = np.arange(g0, g0 + m, dtype=np.uint64) * np.uint64(4)
        u = [uniform(draw(seed, STREAM_PLACE, g + np.uint64(q))) for q in range(4)]
        cx = in_lo[0] + in_w[0] * u[0]
        cy = in_lo[1] + in_w[1] * u[1]
        cz = in_lo[2] + in_w[2] * u[2]
        cr = rmin + (rmax - rmin) * u[3] if rmax > rmin else np.full(m, rmin)
        for c in range(m):
            if k:
                d0 = P[:k, 0] - cx[c]
                d1 = P[:k, 1] - cy[c]
                d2 = P[:k, 2] - cz[c]
                d0 -= L[0] * np.rint(d0 / L[0])
                d1 -= L[1] * np.rint(d1 / L[1])
                d2 -= L[2] * np.rint(d2 / L[2])
                r2 = d0 * d0 + d1 * d1 + d2 * d2
                md = sep * (cr[c] + R[:k])
                if np.any(r2 <= md * md):
                    continue
            P[k] = (cx[c], cy[c], cz[c])
            R[k] = cr[c]
            k += 1
            if k == n:
                break
        g0 += m
    return P[:k], R[:k]


def gas_velocities(n, mode, speed, seed):
    """Velocities of mdg_generate_gas: "speed" (|v| = speed, isotropic),
    "maxwell_rms" (sigma speed / sqrt(3)) or "gaussian" (sigma speed)."""
    if mode == "speed":
        i = np.arange(n, dtype=np.uint64) * np.uint64(4)
        u1 = uniform(draw(seed, STREAM_VEL, i))
        u2 = uniform(draw(seed, STREAM_VEL, i + np.uint64(1)))
        z = 1.0 - 2.0 * u1
        s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
        return np.stack([speed * (s * np.cos(2 * math.pi * u2)), speed * (s * np.sin(2 * math.pi * u2)),
                         speed * z], axis=1)
    sg = speed / math.sqrt(3.0) if mode == "maxwell_rms" else speed
    return sg * normal3(seed, n)
