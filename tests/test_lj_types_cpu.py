"""Multi-type LJ on CPU: the pair table of build_lj_pair_table
(md_lj/src/lib.rs:334-384; geometric or arithmetic mixing at the global
cutoff, then [[lj.pair_coeffs]] overrides, symmetric as PairCoeffTable::set
makes it), its TOML form, the lattice's type assignment and per-type masses
(fcc_insert, md_lattice/src/lib.rs:291-347), and the oracle's per-pair
lookup (pair_table.get(ti, tj) in lj_force, lib.rs:488-633) and equimolar
tail corrections (setup_lj_tails, lib.rs:397-465), checked against closed
forms of those formulas."""
import math

import numpy as np
import pytest

TYPES = [(1.0, 1.0), (0.5, 0.88)]
# pair cutoffs (sigma x cutoff) 2.5, 0.94 x 2.4 = 2.256 and 0.88 x 2.5 = 2.2 sit
# between the FCC shells of the density-0.85 lattice (2.05, 2.37, 2.65), so
# the fp32 cutoff test of the mixed path meets no pair at its edge
OVERRIDE = [(0, 1, 0.8, 0.94, 2.4)]

LJ_TYPES_TOML = """
[domain]
x_high = 10.06
y_high = 10.06
z_high = 10.06

[neighbor]
skin_fraction = 1.12
bin_size = 1.0

[run]
steps = 100
thermo = 50

[lj]
cutoff = 2.5
mixing = "geometric"

[[lj.types]]
epsilon = 1.0
sigma = 1.0

[[lj.types]]
epsilon = 0.5
sigma = 0.88

[[lj.pair_coeffs]]
types = [0, 1]
epsilon = 0.8
sigma = 0.94
cutoff = 2.4

[lattice]
style = "fcc"
density = 0.85
temperature = 0.85
type_fractions = [0.5, 1.0]
type_masses = [1.0, 1.5]
"""


def two_type_config(**kw):
    from mddem_gb300 import config

    table = config.lj_pair_table(TYPES, 2.5, None, OVERRIDE)
    return config.lj_fluid_config(nose_hoover=False).replace(lj_types=2, lj_pairs=table, **kw)


def f_pair(r, eps, sig):
    """|F(r)| of LJ 12-6 with lj1 = 48 eps sigma^12, lj2 = 24 eps sigma^6."""
    s6 = sig ** 6
    return (48 * eps * s6 * s6 / r ** 13) - (24 * eps * s6 / r ** 7)


def test_pair_table_geometric_arithmetic_and_overrides():
    from mddem_gb300 import config

    t = config.lj_pair_table([(1.0, 1.0), (0.25, 0.81)], 2.5)
    assert t == ((1.0, 1.0, 2.5), (0.5, 0.9, 2.5), (0.5, 0.9, 2.5), (0.25, 0.81, 2.5))
    t = config.lj_pair_table([(1.0, 1.0), (0.5, 0.8)], 2.5, "arithmetic")
    assert t == ((1.0, 1.0, 2.5), (0.75, 0.9, 2.5), (0.75, 0.9, 2.5), (0.5, 0.8, 2.5))
    # any name but "arithmetic" mixes geometrically, as the reference's match arm does
    assert config.lj_pair_table([(1.0, 1.0), (0.25, 0.81)], 2.5, "lorentz") == \
        config.lj_pair_table([(1.0, 1.0), (0.25, 0.81)], 2.5)
    # overrides replace both (a, b) and (b, a), in order; no cutoff = the global one
    t = config.lj_pair_table([(1.0, 1.0)] * 3, 2.5, None, [(2, 0, 0.3, 0.7, None), (2, 0, 0.4, 0.6, 3.0),
                                                           (1, 1, 0.9, 1.1, 2.0)])
    assert t[2 * 3 + 0] == t[0 * 3 + 2] == (0.4, 0.6, 3.0)
    assert t[1 * 3 + 1] == (0.9, 1.1, 2.0)
    assert t[0] == (1.0, 1.0, 2.5)
    with pytest.raises(config.ConfigError, match="only 2 types"):
        config.lj_pair_table(TYPES, 2.5, None, [(0, 2, 1.0, 1.0, None)])


def test_toml_types_and_pair_coeffs():
    from mddem_gb300 import config

    cfg = config.from_toml(LJ_TYPES_TOML)
    assert cfg.lj_types == 2
    assert cfg.lj_pairs == config.lj_pair_table(TYPES, 2.5, "geometric", OVERRIDE)
    assert cfg.lj_pairs[1] == (0.8, 0.94, 2.4)
    # one entry in types: the single-type path with the table's (0, 0) pair
    one = LJ_TYPES_TOML.split("[[lj.types]]")[0] + "[[lj.types]]\nepsilon = 0.7\nsigma = 1.1\n\n[lattice]\n"
    c1 = config.from_toml(one)
    assert c1.lj_types == 0 and (c1.lj_epsilon, c1.lj_sigma, c1.lj_cutoff) == (0.7, 1.1, 2.5)


@pytest.mark.parametrize("edit,msg", [
    (("sigma = 0.88\n", "sigma = 0.88\nradius = 1\n"), "unknown"),
    (("epsilon = 0.5\nsigma = 0.88\n", "epsilon = 0.5\n"), "needs epsilon and sigma"),
    (("types = [0, 1]", "types = [0, 2]"), "only 2 types"),
    (("types = [0, 1]", "types = [0]"), "types = \\[a, b\\]"),
])
def test_toml_errors(edit, msg):
    from mddem_gb300 import config

    with pytest.raises(config.ConfigError, match=msg):
        config.from_toml(LJ_TYPES_TOML.replace(*edit))


def test_lattice_types_and_masses():
    from mddem_gb300 import inputs

    t = inputs.lattice_types(864, [0.8, 1.0])
    assert np.bincount(t).tolist() == [691, 173]
    assert t[:691].max() == 0 and t[691:].min() == 1  # by index, (k + 0.5) / n against the thresholds
    # fractions that stop short of 1: the rest take the last type
    assert np.bincount(inputs.lattice_types(100, [0.25, 0.5])).tolist() == [25, 75]
    assert inputs.lattice_types(10).tolist() == [0] * 10
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=3, type_fractions=[0.5, 1.0], type_masses=[1.0, 1.5])
    assert np.array_equal(st["mass"], np.where(st["type"] == 0, 1.0, 1.5))
    m, v = st["mass"], st["vel"]
    n = len(m)
    assert np.allclose(np.sum(v, axis=0), 0.0, atol=1e-12)
    assert np.sum(m[:, None] * v * v) / (3 * n - 3) == pytest.approx(0.85, rel=1e-12)
    # masses past type_masses fall back to `mass`
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=3, mass=3.0, type_fractions=[0.5, 1.0], type_masses=[2.0])
    assert sorted(set(st["mass"].tolist())) == [2.0, 3.0]
    # single type: the same state as before the multi-type arguments existed
    a = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=3)
    assert np.all(a["type"] == 0) and np.all(a["mass"] == 1.0)


def test_runner_setup_builds_the_typed_lattice():
    from mddem_gb300 import run

    cfg, st, _ = run.setup(LJ_TYPES_TOML)
    assert cfg.lj_types == 2 and len(st["tag"]) == 864
    assert np.bincount(st["type"]).tolist() == [432, 432]
    assert np.array_equal(st["mass"], np.where(st["type"] == 0, 1.0, 1.5))
    bad = LJ_TYPES_TOML.replace("type_fractions = [0.5, 1.0]", "type_fractions = [0.3, 0.6, 1.0]")
    with pytest.raises(run.RunError, match="types"):
        run.setup(bad)
    with pytest.raises(run.RunError, match="unknown"):
        run.setup(LJ_TYPES_TOML.replace('style = "fcc"', 'style = "fcc"\nbasis = 2'))


@pytest.mark.parametrize("ti,tj,r,want_zero", [
    (0, 0, 1.12, False), (1, 1, 1.0, False), (0, 1, 1.05, False),
    (0, 1, 2.3, True),    # beyond the (0, 1) override's cutoff 0.94 * 2.4 = 2.256
    (1, 1, 2.1, False),   # inside the (1, 1) cutoff 0.88 * 2.5 = 2.2
    (0, 0, 2.45, False),
])
def test_oracle_pair_force_by_type(ti, tj, r, want_zero):
    from mddem_gb300 import config
    from oracle.oracle import Oracle

    cfg = two_type_config()
    st = {"tag": np.array([0, 1], np.uint32), "type": np.array([ti, tj], np.uint32),
          "pos": np.array([[4.0, 5.0, 5.0], [4.0 + r, 5.0, 5.0]]), "vel": np.zeros((2, 3)),
          "mass": np.ones(2), "cutoff_radius": np.full(2, 1.25)}
    o = Oracle(cfg)
    o.load(st)
    o.force_only()
    f = o.state()["force"]
    e, s, _ = config.lj_pair_table(TYPES, 2.5, None, OVERRIDE)[ti * 2 + tj]
    want = 0.0 if want_zero else f_pair(r, e, s)
    # the force on atom 0 points away from atom 1 when repulsive
    assert f[0, 0] == pytest.approx(-want, rel=1e-12, abs=1e-300)
    assert f[1, 0] == pytest.approx(want, rel=1e-12, abs=1e-300)
    assert np.all(f[:, 1:] == 0.0)


def test_oracle_tails_equimolar_sum():
    from oracle.oracle import Oracle

    from mddem_gb300 import config, inputs

    cfg = two_type_config()
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=3, type_fractions=[0.5, 1.0])
    o = Oracle(cfg)
    o.load(st)
    e, p = o.lj_tails()
    n, v = 864.0, 10.06 ** 3
    rho = n / v
    we = wp = 0.0
    for eps, sig, rc_s in config.lj_pair_table(TYPES, 2.5, None, OVERRIDE):
        rc = rc_s * sig
        s3 = sig ** 3
        we += 0.25 * (8.0 / 3.0) * math.pi * n * rho * eps * s3 * (s3 ** 3 / (3 * rc ** 9) - s3 / rc ** 3)
        wp += 0.25 * (16.0 / 3.0) * math.pi * rho * rho * eps * s3 * (2 * s3 ** 3 / (3 * rc ** 9) - s3 / rc ** 3)
    assert e == pytest.approx(we, rel=1e-13) and p == pytest.approx(wp, rel=1e-13)


def test_oracle_force_is_the_gradient_of_its_energy():
    """Per-type masses and pair coefficients in a disordered two-type fluid:
    the force on a particle is minus the central difference of the pair
    energy the oracle sums (no pair crosses its cutoff within the step)."""
    from oracle.oracle import Oracle

    from mddem_gb300 import inputs

    cfg = two_type_config()
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.7, seed=11, type_fractions=[0.5, 1.0], type_masses=[1.0, 1.5])
    st["pos"] = st["pos"] + np.random.default_rng(4).normal(scale=0.08, size=st["pos"].shape)

    def energy_and_force(pos):
        o = Oracle(cfg)
        o.load(dict(st, pos=pos))
        o.force_only()
        return o.thermo()["pe"], o.state()

    _, s0 = energy_and_force(st["pos"])
    f0 = s0["force"][np.argsort(s0["tag"])]
    h = 1e-6
    for k in (0, 431, 432, 863):
        for d in range(3):
            up, dn = st["pos"].copy(), st["pos"].copy()
            up[k, d] += h
            dn[k, d] -= h
            num = -(energy_and_force(up)[0] - energy_and_force(dn)[0]) / (2 * h)
            assert num == pytest.approx(f0[k, d], rel=1e-5, abs=1e-6), (k, d)


@pytest.mark.parametrize("ti,tj,r", [(0, 0, 1.12), (0, 1, 1.3), (1, 1, 0.95), (0, 1, 2.3), (0, 1, 2.2)])
def test_oracle_pair_energy_by_type(ti, tj, r):
    from mddem_gb300 import config
    from oracle.oracle import Oracle

    cfg = two_type_config()
    st = {"tag": np.array([0, 1], np.uint32), "type": np.array([ti, tj], np.uint32),
          "pos": np.array([[4.0, 5.0, 5.0], [4.0 + r, 5.0, 5.0]]), "vel": np.zeros((2, 3)),
          "mass": np.ones(2), "cutoff_radius": np.full(2, 1.25)}
    o = Oracle(cfg)
    o.load(st)
    o.force_only()
    e, s, rc = config.lj_pair_table(TYPES, 2.5, None, OVERRIDE)[ti * 2 + tj]
    want = 4 * e * ((s / r) ** 12 - (s / r) ** 6) if r < rc * s else 0.0
    assert o.thermo()["pe"] == pytest.approx(want, rel=1e-12, abs=1e-300)
