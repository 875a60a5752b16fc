"""Seeded initial-condition generators for the hot-path workloads.

The reference draws its initial conditions from an unseeded ``rand::rng()``
(DEM insertion, ``crates/dem_atom/src/insert.rs:446,541-571``; FCC velocities,
``crates/md_lattice/src/lib.rs:372-391``).  These generators restate the same
construction with a seeded numpy ``PCG64`` stream so that the CUDA path and the
oracle read identical states.  States can be written in the reference's CSV
particle format (``crates/dem_atom/src/insert.rs:652-776``: columns
x,y,z,radius,vx,vy,vz[,type]).

Every state is a plain dict of numpy arrays (SoA, float64 unless noted):
``tag`` (u32), ``type`` (u32), ``pos`` (n,3), ``vel`` (n,3), ``mass``,
``cutoff_radius``, and for DEM ``radius``, ``density``, ``inv_inertia``,
``omega`` (n,3), ``quat`` (n,4).
"""
from __future__ import annotations

import math

import numpy as np

PI = math.pi


def sphere_mass(density, radius):
    """Solid-sphere mass, ``density * 4.0 / 3.0 * PI * radius.powi(3)``
    (``crates/dem_atom/src/insert.rs:343``), same operation order."""
    r = np.asarray(radius, dtype=np.float64)
    return ((np.asarray(density, dtype=np.float64) * 4.0) / 3.0) * PI * ((r * r) * r)


def sphere_inv_inertia(mass, radius):
    """``1.0 / (0.4 * mass * radius * radius)`` (``insert.rs:349``)."""
    r = np.asarray(radius, dtype=np.float64)
    return 1.0 / (((0.4 * np.asarray(mass, dtype=np.float64)) * r) * r)


def _dem_state(pos, vel, radius, density, mtype=None):
    n = pos.shape[0]
    mass = sphere_mass(density, radius)
    return {
        "kind": "dem",
        "tag": np.arange(n, dtype=np.uint32),
        "type": np.zeros(n, np.uint32) if mtype is None else np.asarray(mtype, np.uint32),
        "pos": np.ascontiguousarray(pos, dtype=np.float64),
        "vel": np.ascontiguousarray(vel, dtype=np.float64),
        "mass": mass,
        "cutoff_radius": np.asarray(radius, dtype=np.float64).copy(),
        "radius": np.asarray(radius, dtype=np.float64).copy(),
        "density": np.full(n, float(density)),
        "inv_inertia": sphere_inv_inertia(mass, radius),
        "omega": np.zeros((n, 3)),
        "quat": np.tile(np.array([1.0, 0.0, 0.0, 0.0]), (n, 1)),
    }


def _min_image(d, L):
    return d - L * np.round(d / L)


def random_spheres(n, box, radius, seed=0, sep_factor=1.1, inset=True, max_attempts=None):
    """Seeded random sequential addition of non-overlapping spheres in a
    periodic cube.

    Restates the reference's rejection sampling (``insert.rs:523-571``):
    candidate centres uniform in the box inset by the largest radius, radius
    drawn per candidate, rejected when any existing sphere is within
    ``sep_factor * (r_i + r_j)`` under the minimum image.  A cell grid replaces
    the reference's O(N^2) scan (same accept/reject decisions).

    ``radius`` is a float (monodisperse) or ``(rmin, rmax)`` for a uniform
    distribution.  Returns (pos (n,3), radius (n,)).
    """
    rng = np.random.default_rng(seed)
    L = float(box)
    if isinstance(radius, (tuple, list)):
        rmin, rmax = float(radius[0]), float(radius[1])
    else:
        rmin = rmax = float(radius)
    lo = rmax if inset else 0.0
    hi = L - rmax if inset else L
    reach = sep_factor * 2.0 * rmax
    nc = max(1, int(L // reach))
    cell = L / nc
    grid: dict = {}
    pos = np.empty((n, 3))
    rad = np.empty(n)
    count = 0
    attempts = 0
    limit = max_attempts if max_attempts is not None else n * 20000
    batch = 256
    while count < n and attempts < limit:
        cand = lo + (hi - lo) * rng.random((batch, 3))
        crad = rmin + (rmax - rmin) * rng.random(batch) if rmax > rmin else np.full(batch, rmin)
        for c, cr in zip(cand, crad):
            attempts += 1
            ci = (np.floor(c / cell).astype(int)) % nc
            ok = True
            for dx in (-1, 0, 1):
                if not ok:
                    break
                for dy in (-1, 0, 1):
                    if not ok:
                        break
                    for dz in (-1, 0, 1):
                        key = ((ci[0] + dx) % nc, (ci[1] + dy) % nc, (ci[2] + dz) % nc)
                        lst = grid.get(key)
                        if not lst:
                            continue
                        idx = np.fromiter(lst, dtype=np.int64)
                        d = _min_image(pos[idx] - c, L)
                        md = (cr + rad[idx]) * sep_factor
                        if np.any(np.einsum("ij,ij->i", d, d) <= md * md):
                            ok = False
                            break
            if ok:
                pos[count] = c
                rad[count] = cr
                grid.setdefault(tuple(ci), []).append(count)
                count += 1
                if count == n:
                    break
    if count < n:
        raise RuntimeError(f"could only place {count}/{n} spheres in box {L}")
    return pos, rad


def isotropic_directions(rng, n):
    """Unit vectors uniform on the sphere."""
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def dem_granular_gas(n=500, box=0.025, radius=1e-3, density=2500.0, speed=0.5, seed=0,
                     sep_factor=1.1, maxwellian=False, native=False, rsa=None):
    """Granular-gas initial state: seeded non-overlapping spheres, speeds of
    magnitude ``speed`` in uniform random directions (or Maxwellian with RMS
    ``speed`` when ``maxwellian``), omega = 0, identity quaternions.

    ``native`` places the spheres with the library's grid RSA
    (``mdg_rsa_spheres``, same acceptance rule, its own random stream) --
    needed from about 1e4 spheres on; ``radius`` may be ``(rmin, rmax)``.
    ``rsa``, when given, is another generator with mdg_rsa_spheres'
    arguments (n, lo, hi, rmin, rmax, sep_factor, inset, seed) that places
    the same spheres."""
    if rsa is not None or native:
        rmin, rmax = (radius, radius) if not isinstance(radius, (tuple, list)) else radius
        if rsa is None:
            from . import capi

            rsa = capi.rsa_spheres
        gen = rsa
        pos, rad = gen(n, (0.0, 0.0, 0.0), (box, box, box), rmin, rmax, sep_factor, True, seed)
    else:
        pos, rad = random_spheres(n, box, radius, seed=seed, sep_factor=sep_factor)
    rng = np.random.default_rng(seed + 7919)
    if maxwellian:
        vel = rng.normal(scale=speed / math.sqrt(3.0), size=(n, 3))
    else:
        vel = speed * isotropic_directions(rng, n)
    return _dem_state(pos, vel, rad, density)


def two_sphere_rebound(radius=1e-3, speed=1.0, gap_frac=0.1, box_factor=12.0, density=2500.0):
    """Two spheres approaching head-on along x with relative speed ``speed``,
    initial surface gap ``gap_frac * radius``, centred in a periodic box of side
    ``box_factor * radius``."""
    L = box_factor * radius
    c = 0.5 * L
    half = radius + 0.5 * gap_frac * radius
    pos = np.array([[c - half, c, c], [c + half, c, c]])
    vel = np.array([[0.5 * speed, 0.0, 0.0], [-0.5 * speed, 0.0, 0.0]])
    st = _dem_state(pos, vel, np.full(2, radius), density)
    st["box"] = L
    return st


def lattice_types(n, type_fractions=None):
    """Atom types of fcc_insert's deterministic assignment
    (crates/md_lattice/src/lib.rs:291-327): atom k of n takes the first type
    whose cumulative fraction exceeds (k + 0.5) / n, else the last type."""
    fr = list(type_fractions) if type_fractions else [1.0]
    out = np.empty(n, np.uint32)
    for k in range(n):
        f = (k + 0.5) / n
        t = len(fr) - 1
        for q, thr in enumerate(fr):
            if f < thr:
                t = q
                break
        out[k] = t
    return out


def lj_fcc(n_cells=6, box=10.06, density=0.85, temperature=0.85, mass=1.0, skin=1.25, seed=0, lo=0.0,
           type_fractions=None, type_masses=None):
    """FCC lattice with Gaussian velocities, restating ``fcc_insert``
    (``crates/md_lattice/src/lib.rs:232-454``): lattice constant from
    ``(4/rho)^(1/3)``, unit cells stretched to tile the box, 4-atom basis in
    (ix, iy, iz, basis) order, velocities N(0, sqrt(T/m)) per component, COM
    velocity removed, then rescaled to exactly T with 3N-3 degrees of freedom.
    ``n_cells`` must equal floor(box / a_ideal).  ``type_fractions``
    (cumulative) and ``type_masses`` give the multi-type lattice: types by
    lattice_types, each atom's mass from its type (``mass`` past the list)."""
    a_ideal = (4.0 / density) ** (1.0 / 3.0)
    nx = int(math.floor(box / a_ideal))
    if nx != n_cells:
        raise ValueError(f"box {box} holds {nx} FCC cells at rho={density}, not {n_cells}")
    ax = box / nx
    basis = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])
    ii = np.arange(nx, dtype=np.float64)
    gx, gy, gz = np.meshgrid(ii, ii, ii, indexing="ij")
    cells = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1)
    pos = (cells[:, None, :] + basis[None, :, :]).reshape(-1, 3)
    pos = lo + pos * ax
    n = pos.shape[0]
    types = lattice_types(n, type_fractions)
    masses = np.full(n, float(mass))
    if type_masses:
        tm = [float(m) for m in type_masses]
        masses = np.array([tm[t] if t < len(tm) else float(mass) for t in types])
    rng = np.random.default_rng(seed)
    if type_masses:
        vel = rng.standard_normal(size=(n, 3)) * np.sqrt(temperature / masses)[:, None]
    else:
        vel = rng.normal(0.0, math.sqrt(temperature / mass), size=(n, 3))
    vel -= vel.sum(axis=0) / n
    ndof = 3.0 * n - 3.0
    ke = 0.5 * float(np.sum(masses * np.sum(vel * vel, axis=1)))
    cur = 2.0 * ke / ndof
    if cur > 1e-20:
        vel *= math.sqrt(temperature / cur)
    return {
        "kind": "lj",
        "tag": np.arange(n, dtype=np.uint32),
        "type": types,
        "pos": np.ascontiguousarray(pos),
        "vel": np.ascontiguousarray(vel),
        "mass": masses,
        "cutoff_radius": np.full(n, float(skin)),
        "box": float(box),
    }


def write_csv(path, state):
    """Write a DEM state in the reference's CSV particle format
    (x,y,z,radius,vx,vy,vz,type; header line skipped by the reader)."""
    with open(path, "w") as f:
        f.write("x,y,z,radius,vx,vy,vz,type\n")
        for p, r, v, t in zip(state["pos"], state["radius"], state["vel"], state["type"]):
            vals = [float(p[0]), float(p[1]), float(p[2]), float(r), float(v[0]), float(v[1]), float(v[2])]
            f.write(",".join(repr(x) for x in vals) + f",{int(t)}\n")


def read_csv(path, density=2500.0):
    """Read a reference-format CSV (x,y,z,radius,vx,vy,vz[,type])."""
    rows = []
    with open(path) as f:
        for ln, line in enumerate(f):
            s = line.strip()
            if not s or s.startswith("#"):
                continue
            if ln == 0 and s[0].isalpha():
                continue
            rows.append([float(x) for x in s.split(",")])
    a = np.array(rows)
    mtype = a[:, 7].astype(np.uint32) if a.shape[1] > 7 else None
    vel = a[:, 4:7] if a.shape[1] >= 7 else np.zeros((a.shape[0], 3))
    return _dem_state(a[:, 0:3], vel, a[:, 3], density, mtype)
