"""Configuration: the TOML sections the hot-path plugins read.

Field names and defaults follow the reference's config structs:
``[domain]`` (crates/mddem_core/src/domain.rs:46-78), ``[neighbor]``
(crates/mddem_core/src/neighbor.rs:44-80), ``[[dem.materials]]`` and ``[dem]``
(crates/dem_atom/src/lib.rs:78-158), ``[lj]`` (crates/md_lj/src/lib.rs:115-140),
``[thermostat]`` (crates/md_thermostat/src/lib.rs:85-97), ``[run] dt``, plus a
``[gpu]`` section for the GB300 path (precision, rebuild policy, capacities,
threads per particle).  Unknown keys are rejected like the reference's
``deny_unknown_fields``.
"""
from __future__ import annotations

import dataclasses
import math
import tomllib
from dataclasses import dataclass, field


class ConfigError(ValueError):
    """Invalid configuration (the reference exits with status 1)."""


@dataclass
class Material:
    name: str = "glass"
    youngs_mod: float = 8.7e9
    poisson_ratio: float = 0.3
    restitution: float = 0.95
    friction: float = 0.4
    rolling_friction: float = 0.0
    twisting_friction: float = 0.0
    cohesion_energy: float = 0.0
    surface_energy: float = 0.0
    kn: float = 0.0
    kt: float = 0.0
    rolling_stiffness: float = 0.0
    rolling_damping: float = 0.0
    twisting_stiffness: float = 0.0
    twisting_damping: float = 0.0


@dataclass
class Wall:
    """Plane wall ([[wall]], crates/dem_wall/src/lib.rs:171-262)."""
    point: tuple = (0.0, 0.0, 0.0)
    normal: tuple = (0.0, 0.0, 1.0)
    bound_lo: tuple = (-math.inf, -math.inf, -math.inf)
    bound_hi: tuple = (math.inf, math.inf, math.inf)
    velocity: tuple = (0.0, 0.0, 0.0)
    material: int = 0


@dataclass
class SimConfig:
    kind: str = "dem"                         # "dem" | "lj"
    box_lo: tuple = (0.0, 0.0, 0.0)
    box_hi: tuple = (1.0, 1.0, 1.0)
    dt: float = 0.0
    # [neighbor]
    skin_fraction: float = 1.0
    bin_size: float = 1.0
    every: int = 0
    check: bool = True
    sort_every: int = 1000
    newton: bool = True
    # [dem]
    materials: list = field(default_factory=lambda: [Material()])
    contact_model: str = "hertz"
    adhesion_model: str = "jkr"
    rolling_model: str = "constant"
    twisting_model: str = "constant"
    # [lj]
    lj_epsilon: float = 1.0
    lj_sigma: float = 1.0
    lj_cutoff: float = 2.5
    # [lj] multi-type mode: the number of types (0 = single type) and the
    # row-major n x n pair table of (epsilon, sigma, cutoff) triples
    lj_types: int = 0
    lj_pairs: tuple = ()
    # [thermostat]
    nose_hoover: bool = False
    nh_temperature: float = 0.85
    nh_coupling: float = 1.0
    virial: bool = False
    # [gpu]
    precision: str = "fp64"                   # "fp64" | "mixed"
    rebuild_policy: str = "reference"         # "reference" | "displacement"
    threads_per_particle: int = 0
    neighbor_capacity: int = 0
    history_capacity: int = 0
    langevin: bool = False
    lv_temperature: float = 0.85
    lv_damping: float = 1.0
    lv_seed: int = 12345
    fixed: tuple = (0, 0, 0)
    walls: list = field(default_factory=list)

    def replace(self, **kw) -> "SimConfig":
        return dataclasses.replace(self, **kw)

    @property
    def box(self):
        return tuple(h - l for l, h in zip(self.box_lo, self.box_hi))


_SECTIONS = {
    "domain": {"x_low", "x_high", "y_low", "y_high", "z_low", "z_high", "x_lo", "x_hi", "y_lo", "y_hi",
               "z_lo", "z_hi", "boundary_x", "boundary_y", "boundary_z", "shrink_wrap_padding"},
    "neighbor": {"skin_fraction", "bin_size", "every", "check", "sort_every", "newton"},
    "lj": {"epsilon", "sigma", "cutoff", "mixing", "types", "pair_coeffs"},
    "thermostat": {"temperature", "coupling", "group"},
    "langevin": {"temperature", "damping", "seed", "group"},
    "gpu": {"precision", "rebuild_policy", "threads_per_particle", "neighbor_capacity", "history_capacity",
            "virial", "generate"},
}
_MATERIAL_KEYS = {f.name for f in dataclasses.fields(Material)}
_WALL_KEYS = {"type", "point_x", "point_y", "point_z", "normal_x", "normal_y", "normal_z", "material", "name",
              "bound_x_low", "bound_x_high", "bound_y_low", "bound_y_high", "bound_z_low", "bound_z_high",
              "velocity", "oscillate", "servo", "axis", "center", "radius", "lo", "hi", "inside", "region",
              "temperature"}


def _check_keys(section: str, table: dict, allowed: set):
    extra = set(table) - allowed
    if extra:
        raise ConfigError(f"unknown field(s) {sorted(extra)} in [{section}]")


def from_toml(text: str, kind: str | None = None) -> SimConfig:
    """Parse a reference-style TOML config into a SimConfig.

    ``kind`` is inferred: ``[lj]`` or ``[lattice]`` -> LJ, ``[dem]`` -> DEM.
    """
    doc = tomllib.loads(text)
    c = SimConfig()
    if kind is None:
        kind = "lj" if ("lj" in doc or "lattice" in doc) else "dem"
    c.kind = kind
    dom = doc.get("domain", {})
    _check_keys("domain", dom, _SECTIONS["domain"])
    fixed = []
    for ax in ("x", "y", "z"):
        bt = dom.get(f"boundary_{ax}", "periodic")
        if bt not in ("periodic", "fixed"):
            raise ConfigError(f"boundary_{ax} = {bt!r}: the GPU path supports periodic and fixed boundaries")
        fixed.append(1 if bt == "fixed" else 0)
    c.fixed = tuple(fixed)
    lo = [float(dom.get(f"{a}_low", dom.get(f"{a}_lo", 0.0))) for a in "xyz"]
    hi = [float(dom.get(f"{a}_high", dom.get(f"{a}_hi", 1.0))) for a in "xyz"]
    c.box_lo, c.box_hi = tuple(lo), tuple(hi)
    nb = doc.get("neighbor", {})
    _check_keys("neighbor", nb, _SECTIONS["neighbor"])
    c.skin_fraction = float(nb.get("skin_fraction", 1.0))
    c.bin_size = float(nb.get("bin_size", 1.0))
    c.every = int(nb.get("every", 0))
    c.check = bool(nb.get("check", True))
    c.sort_every = int(nb.get("sort_every", 1000))
    c.newton = bool(nb.get("newton", True))
    run = doc.get("run", {})
    if isinstance(run, list):
        run = run[0] if run else {}
    c.dt = float(run.get("dt", 0.0))
    if kind == "dem":
        dem = doc.get("dem", {})
        mats = []
        for m in dem.get("materials", []) or []:
            _check_keys("dem.materials", m, _MATERIAL_KEYS)
            mats.append(Material(**m))
        if not mats:
            raise ConfigError("[[dem.materials]] requires at least one material")
        c.materials = mats
        c.walls = []
        for w in doc.get("wall", []) or []:
            _check_keys("wall", w, _WALL_KEYS)
            if w.get("type", "plane") != "plane":
                raise ConfigError(f"wall type {w.get('type')!r}: the GPU path supports plane walls only")
            if w.get("oscillate") or w.get("servo"):
                raise ConfigError("oscillating and servo walls are not supported by the GPU path")
            if w.get("temperature") is not None:
                raise ConfigError("wall heat transfer is not supported by the GPU path")
            names = [m.name for m in mats]
            if w.get("material") not in names:
                raise ConfigError(f"wall material {w.get('material')!r} is not in [[dem.materials]]")
            c.walls.append(Wall(
                point=tuple(float(w.get(f"point_{a}", 0.0)) for a in "xyz"),
                normal=tuple(float(w.get(f"normal_{a}", 0.0)) for a in "xyz"),
                bound_lo=tuple(float(w.get(f"bound_{a}_low", -math.inf)) for a in "xyz"),
                bound_hi=tuple(float(w.get(f"bound_{a}_high", math.inf)) for a in "xyz"),
                velocity=tuple(float(x) for x in (w.get("velocity") or (0.0, 0.0, 0.0))),
                material=names.index(w["material"])))
        c.contact_model = dem.get("contact_model", "hertz")
        c.adhesion_model = dem.get("adhesion_model", "jkr")
        c.rolling_model = dem.get("rolling_model", "constant")
        c.twisting_model = dem.get("twisting_model", "constant")
    else:
        lj = doc.get("lj", {})
        _check_keys("lj", lj, _SECTIONS["lj"])
        c.lj_epsilon = float(lj.get("epsilon", 1.0))
        c.lj_sigma = float(lj.get("sigma", 1.0))
        c.lj_cutoff = float(lj.get("cutoff", 2.5))
        if lj.get("types") is not None:
            types = []
            for t in lj["types"]:
                _check_keys("lj.types", t, {"epsilon", "sigma"})
                if "epsilon" not in t or "sigma" not in t:
                    raise ConfigError("[[lj.types]] needs epsilon and sigma")
                types.append((float(t["epsilon"]), float(t["sigma"])))
            overrides = []
            for o in lj.get("pair_coeffs") or ():
                _check_keys("lj.pair_coeffs", o, {"types", "epsilon", "sigma", "cutoff"})
                if "types" not in o or "epsilon" not in o or "sigma" not in o or len(o["types"]) != 2:
                    raise ConfigError("[[lj.pair_coeffs]] needs types = [a, b], epsilon and sigma")
                overrides.append((int(o["types"][0]), int(o["types"][1]), float(o["epsilon"]), float(o["sigma"]),
                                  None if o.get("cutoff") is None else float(o["cutoff"])))
            if not types:
                raise ConfigError("[lj] types is empty")
            table = lj_pair_table(types, c.lj_cutoff, lj.get("mixing"), overrides)
            if len(types) == 1:
                # one type: lj_force reads the 1 x 1 table
                c.lj_epsilon, c.lj_sigma, c.lj_cutoff = table[0]
            else:
                c.lj_types, c.lj_pairs = len(types), table
        if c.dt == 0.0:
            c.dt = 0.005  # lattice_set_dt (crates/md_lattice/src/lib.rs:461-471)
        th = doc.get("thermostat")
        if th is not None:
            _check_keys("thermostat", th, _SECTIONS["thermostat"])
            if th.get("group"):
                raise ConfigError("thermostat groups are not supported by the GPU path")
            c.nose_hoover = True
            c.nh_temperature = float(th.get("temperature", 0.85))
            c.nh_coupling = float(th.get("coupling", 1.0))
    lv = doc.get("langevin")
    if lv is not None:
        _check_keys("langevin", lv, _SECTIONS["langevin"])
        if lv.get("group"):
            raise ConfigError("thermostat groups are not supported by the GPU path")
        c.langevin = True
        c.lv_temperature = float(lv.get("temperature", 0.85))
        c.lv_damping = float(lv.get("damping", 1.0))
        c.lv_seed = int(lv.get("seed", 12345))
    gpu = doc.get("gpu", {})
    _check_keys("gpu", gpu, _SECTIONS["gpu"])
    for k in ("precision", "rebuild_policy", "threads_per_particle", "neighbor_capacity", "history_capacity",
              "virial"):
        if k in gpu:
            setattr(c, k, gpu[k])
    return c


def lj_pair_table(types, cutoff=2.5, mixing=None, overrides=()):
    """The LJ pair table of build_lj_pair_table (crates/md_lj/src/lib.rs:
    334-384) as a row-major tuple of (epsilon, sigma, cutoff) for n x n type
    pairs: `types` is [(epsilon, sigma), ...]; cross pairs mix by
    sqrt(e_i e_j), sqrt(s_i s_j) ("geometric", the default and any other
    name) or by (e_i + e_j) / 2, (s_i + s_j) / 2 ("arithmetic"), all at the
    global `cutoff` (units of sigma); then each override (a, b, epsilon,
    sigma, cutoff or None for the global one) replaces pair (a, b) and (b, a)
    in order, as PairCoeffTable::set does."""
    n = len(types)
    arith = mixing == "arithmetic"
    tab = [[None] * n for _ in range(n)]
    for i in range(n):
        for j in range(i, n):
            (ei, si), (ej, sj) = types[i], types[j]
            eps = (ei + ej) / 2.0 if arith else math.sqrt(ei * ej)
            sig = (si + sj) / 2.0 if arith else math.sqrt(si * sj)
            tab[i][j] = tab[j][i] = (float(eps), float(sig), float(cutoff))
    for a, b, eps, sig, cut in overrides:
        if not (0 <= a < n and 0 <= b < n):
            raise ConfigError(f"[[lj.pair_coeffs]] types = [{a}, {b}]: only {n} types")
        tab[a][b] = tab[b][a] = (float(eps), float(sig), float(cutoff if cut is None else cut))
    return tuple(x for row in tab for x in row)


def rayleigh_dt(radius, density, youngs_mod, poisson_ratio, fraction=0.15):
    """Rayleigh-wave timestep (calculate_delta_time, crates/dem_atom/src/insert.rs:1392-1431):
    ``T_R = PI * r / alpha * sqrt(rho / G)``, ``alpha = 0.1631 nu + 0.876605``,
    ``G = E / (2 (1 + nu))``; returns ``fraction * min T_R``."""
    g = youngs_mod / (2.0 * (1.0 + poisson_ratio))
    alpha = 0.1631 * poisson_ratio + 0.876605
    r = min(radius) if hasattr(radius, "__iter__") else radius
    return fraction * (math.pi * r / alpha * math.sqrt(density / g))


def granular_gas_config(box=0.025, dt=None, precision="fp64", policy="reference", **kw) -> SimConfig:
    """Periodic glass-sphere granular gas: E=8.7e9, nu=0.3, e=0.95, mu=0.4,
    bin 0.005, skin_fraction 1.1, dt = 0.1 T_R(1 mm) unless given."""
    if dt is None:
        dt = rayleigh_dt(1e-3, 2500.0, 8.7e9, 0.3, fraction=0.1)
    c = SimConfig(kind="dem", box_lo=(0.0, 0.0, 0.0), box_hi=(box, box, box), dt=dt, skin_fraction=1.1,
                  bin_size=0.005, materials=[Material()], precision=precision, rebuild_policy=policy)
    return c.replace(**kw) if kw else c


def lj_fluid_config(box=10.06, precision="fp64", policy="reference", nose_hoover=True, **kw) -> SimConfig:
    """LJ fluid in reduced units: eps = sigma = 1, rc = 2.5, lattice skin 1.25
    with skin_fraction 1.12 (list cutoff 2.8), NH at T = 0.85, tau = 1,
    dt = 0.005."""
    c = SimConfig(kind="lj", box_lo=(0.0, 0.0, 0.0), box_hi=(box, box, box), dt=0.005, skin_fraction=1.12,
                  bin_size=1.0, lj_epsilon=1.0, lj_sigma=1.0, lj_cutoff=2.5, nose_hoover=nose_hoover,
                  nh_temperature=0.85, nh_coupling=1.0, precision=precision, rebuild_policy=policy)
    return c.replace(**kw) if kw else c
