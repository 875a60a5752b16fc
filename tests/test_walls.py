"""Plane walls and fixed boundaries (dem_wall, domain.rs boundary_x/y/z).

CPU: the oracle's sphere-wall rebound against Hertz theory with the bounds of
the reference's rebound benchmark (examples/bench_hertz_rebound/validate.py:
COR within 3 % for e >= 0.7, contact time and peak overlap within 10 % for
e >= 0.85); a fixed axis has no periodic images; a particle leaving a fixed
axis is reported; a moving wall's force after one step equals the closed form
of wall_contact_force; [[wall]] TOML parsing.

GPU (through the C ABI): the same rebound on both precisions, equal to the
oracle's; single-step force/torque parity in a box with walls on two fixed
axes (fp64: 1e-12 of the largest force; mixed: 1e-5 per particle against the
fp64 path); 100-step trajectories (positions within 1e-12 of the box length);
a constant-velocity wall; the lost-particle status.
"""
import math

import numpy as np
import pytest

from helpers import by_tag, pair_set, rel_err

R, RHO, E, NU, COR, V0 = 0.005, 2500.0, 70e9, 0.22, 0.9, 1.0
L = 0.012


def rebound_config(precision="fp64"):
    """One 5 mm glass sphere above the floor wall z = 0 of a fixed box
    (E = 70 GPa, nu = 0.22, e = 0.9, no friction), dt = 0.15 Rayleigh time."""
    from mddem_gb300 import config

    m = config.Material(name="glass", youngs_mod=E, poisson_ratio=NU, restitution=COR, friction=0.0)
    return config.SimConfig(kind="dem", box_lo=(-0.01, -0.01, 0.0), box_hi=(0.01, 0.01, 0.1),
                            dt=config.rayleigh_dt(R, RHO, E, NU), skin_fraction=1.1, bin_size=0.015, every=1,
                            materials=[m], fixed=(1, 1, 1), precision=precision,
                            walls=[config.Wall(point=(0.0, 0.0, 0.0), normal=(0.0, 0.0, 1.0), material=0)])


def rebound_state():
    from mddem_gb300 import inputs

    return inputs._dem_state(np.array([[0.0, 0.0, R + 2e-4]]), np.array([[0.0, 0.0, -V0]]), np.array([R]), RHO)


def track_rebound(step, read, max_steps=5000):
    """The reference's rebound tracker (bench_hertz_rebound/main.rs:70-112),
    after every step: impact velocity = v_z on the step before first contact,
    contact from the first step with r - z > 0 to the first without, peak
    overlap, rebound velocity.  Returns (cor, contact steps, peak overlap)."""
    was, prev, k0, peak = False, 0.0, 0, 0.0
    for k in range(1, max_steps + 1):
        step()
        z, vz = read()
        ov = R - z
        if not was and ov <= 0.0:
            prev = vz
        elif not was:
            was, k0, peak = True, k, ov
        elif ov > 0.0:
            peak = max(peak, ov)
        else:
            return -vz / prev, k - k0, peak
    raise AssertionError("no rebound")


def hertz_theory():
    e_star = E / (2.0 * (1.0 - NU * NU))
    m = 4.0 / 3.0 * math.pi * R ** 3 * RHO
    tc = 2.87 * (m * m / (R * e_star * e_star * V0)) ** 0.2
    dmax = (15.0 * m * V0 * V0 / (16.0 * math.sqrt(R) * e_star)) ** 0.4
    return tc, dmax


def check_rebound(cor, nsteps, peak, dt):
    tc, dmax = hertz_theory()
    assert abs(cor - COR) / COR <= 0.03
    assert abs(nsteps * dt - tc) / tc <= 0.10
    assert abs(peak - dmax) / dmax <= 0.10


def oracle_rebound():
    from oracle.oracle import Oracle

    cfg = rebound_config()
    o = Oracle(cfg)
    o.load(rebound_state())

    def read():
        s = o.state()
        return s["pos"][0, 2], s["vel"][0, 2]

    return track_rebound(lambda: o.step(1), read), cfg.dt


def test_oracle_hertz_rebound():
    (cor, nsteps, peak), dt = oracle_rebound()
    check_rebound(cor, nsteps, peak, dt)


def test_oracle_fixed_axis_has_no_periodic_images():
    """Two spheres overlapping only across the z faces: a pair with periodic z,
    no pair and no force with fixed z (comm_setup gives a fixed axis no
    neighbor on one rank, comm.rs:226-250)."""
    from mddem_gb300 import config, inputs
    from oracle.oracle import Oracle

    r = 5e-4
    pos = np.array([[0.006, 0.006, 0.4 * r], [0.006, 0.006, L - 0.4 * r], [0.003, 0.003, 0.006]])
    st = inputs._dem_state(pos, np.zeros((3, 3)), np.full(3, r), RHO)
    for fixed, npairs in (((0, 0, 0), 1), ((0, 0, 1), 0)):
        cfg = config.granular_gas_config(box=L, dt=1e-7, fixed=fixed)
        o = Oracle(cfg)
        o.load(st)
        o.force_only()
        assert len(o.pairs()) == npairs
        f = o.state()["force"]
        assert (np.abs(f[:2, 2]).max() > 0) == (npairs == 1)


def test_oracle_particle_leaving_fixed_axis_is_an_error():
    from mddem_gb300 import config, inputs
    from oracle.oracle import Oracle

    r = 5e-4
    pos = np.array([[0.006, 0.006, 2 * r], [0.003, 0.003, 0.006]])
    st = inputs._dem_state(pos, np.array([[0.0, 0.0, -100.0], [0.0, 0.0, 0.0]]), np.full(2, r), RHO)
    o = Oracle(config.granular_gas_config(box=L, dt=1e-7, fixed=(0, 0, 1)))
    o.load(st)
    with pytest.raises(RuntimeError, match="error 12"):
        o.step(200)


def moving_wall_force(dt, vw=0.01):
    """Closed form of wall_contact_force (lib.rs:848-944) for a sphere at rest
    touching the floor, after the floor moved once by vw * dt toward it."""
    from mddem_gb300 import config

    e_star = E / (2.0 * (1.0 - NU * NU))
    m = 4.0 / 3.0 * math.pi * R ** 3 * RHO
    log_e = math.log(COR)
    beta = -log_e / math.sqrt(math.pi ** 2 + log_e ** 2)
    delta = vw * dt
    sdr = math.sqrt(delta * R)
    s_n, k_n = 2.0 * e_star * sdr, 4.0 / 3.0 * e_star * sdr
    v_n = 0.0 - vw
    sqrt_5_3 = 0.9128709291752768  # dem_atom/src/lib.rs:63 (the value is sqrt(5/6))
    f = k_n * delta - 2.0 * beta * sqrt_5_3 * math.sqrt(s_n * m) * v_n
    cfg = rebound_config()
    cfg.walls[0] = config.Wall(point=(0.0, 0.0, 0.0), normal=(0.0, 0.0, 2.0), velocity=(0.0, 0.0, vw))
    return cfg, f


def resting_state():
    from mddem_gb300 import inputs

    return inputs._dem_state(np.array([[0.0, 0.0, R]]), np.zeros((1, 3)), np.array([R]), RHO)


def test_oracle_moving_wall_force():
    from oracle.oracle import Oracle

    cfg, f = moving_wall_force(rebound_config().dt)
    o = Oracle(cfg)
    o.load(resting_state())
    o.step(1)
    fz = o.state()["force"][0]
    assert fz[2] == pytest.approx(f, rel=1e-9) and f > 0
    assert fz[0] == 0.0 and fz[1] == 0.0


WALL_TOML = """
[domain]
x_low = -0.01
x_high = 0.01
y_low = -0.01
y_high = 0.01
z_low = 0.0
z_high = 0.1
boundary_x = "fixed"
boundary_y = "periodic"
boundary_z = "fixed"

[neighbor]
skin_fraction = 1.1
bin_size = 0.015

[[dem.materials]]
name = "glass"
youngs_mod = 70.0e9
poisson_ratio = 0.22
restitution = 0.9
friction = 0.0

[[dem.materials]]
name = "steel"
youngs_mod = 200.0e9
poisson_ratio = 0.3
restitution = 0.8
friction = 0.3

[[wall]]
normal_z = 1.0
material = "glass"

[[wall]]
point_z = 0.1
normal_z = -1.0
bound_x_low = -0.005
bound_x_high = 0.005
velocity = [0.0, 0.0, -0.5]
material = "steel"
"""


def test_toml_wall_sections():
    from mddem_gb300 import config

    c = config.from_toml(WALL_TOML)
    assert c.fixed == (1, 0, 1) and len(c.walls) == 2
    a, b = c.walls
    assert a.point == (0.0, 0.0, 0.0) and a.normal == (0.0, 0.0, 1.0) and a.material == 0
    assert a.bound_lo == (-math.inf,) * 3 and a.velocity == (0.0, 0.0, 0.0)
    assert b.point == (0.0, 0.0, 0.1) and b.material == 1 and b.velocity == (0.0, 0.0, -0.5)
    assert b.bound_lo[0] == -0.005 and b.bound_hi[0] == 0.005 and b.bound_hi[1] == math.inf
    with pytest.raises(config.ConfigError):  # unknown material
        config.from_toml(WALL_TOML.replace('material = "steel"', 'material = "brass"'))
    with pytest.raises(config.ConfigError):  # only plane walls on the GPU path
        config.from_toml(WALL_TOML.replace("[[wall]]\nnormal_z = 1.0", '[[wall]]\ntype = "cylinder"\nnormal_z = 1.0'))
    with pytest.raises(config.ConfigError):  # unknown key
        config.from_toml(WALL_TOML.replace("normal_z = 1.0", "normal_z = 1.0\nspring = 2.0"))


# ---------------------------------------------------------------------------
# GPU, through the C ABI


def _ctx(cfg, st):
    from mddem_gb300 import capi

    ctx = capi.Context(cfg, len(st["tag"]))
    ctx.upload(st)
    return ctx


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_hertz_rebound(gpu_lib, precision):
    ctx = _ctx(rebound_config(precision), rebound_state())

    def read():
        s = ctx.download()
        return s["pos"][0, 2], s["vel"][0, 2]

    cor, nsteps, peak = track_rebound(lambda: ctx.step(1), read)
    (ocor, onsteps, opeak), dt = oracle_rebound()
    check_rebound(cor, nsteps, peak, dt)
    assert nsteps == onsteps
    assert cor == pytest.approx(ocor, rel=1e-9) and peak == pytest.approx(opeak, rel=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_moving_wall_force(gpu_lib, precision):
    cfg, f = moving_wall_force(rebound_config().dt)
    ctx = _ctx(cfg.replace(precision=precision), resting_state())
    ctx.force_only()  # no wall move outside a step
    assert np.all(ctx.download()["force"][0] == 0.0)
    ctx.step(1)
    fz = ctx.download()["force"][0]
    assert fz[2] == pytest.approx(f, rel=1e-9)


def walled_config(precision="fp64", g_frac=0.2, **mat):
    """Periodic y; fixed x and z with four walls g_frac r inside the faces: the
    x-low wall bounded to y < L/2, the z-high wall of a second material moving
    along its normal."""
    from mddem_gb300 import config

    r = 5e-4
    m0 = config.Material(name="glass", youngs_mod=8.7e9, poisson_ratio=0.3, restitution=0.95, friction=0.4, **mat)
    m1 = config.Material(name="steel", youngs_mod=2e11, poisson_ratio=0.3, restitution=0.8, friction=0.3, **mat)
    g = g_frac * r
    walls = [
        config.Wall(point=(g, 0, 0), normal=(1, 0, 0), bound_hi=(math.inf, L / 2, math.inf), material=0),
        config.Wall(point=(L - g, 0, 0), normal=(-1, 0, 0), material=1),
        config.Wall(point=(0, 0, g), normal=(0, 0, 1), material=0),
        config.Wall(point=(0, 0, L - g), normal=(0, 0, -3), velocity=(0.0, 0.2, -0.05), material=1),
    ]
    return config.granular_gas_config(box=L, dt=1e-7, precision=precision, fixed=(1, 0, 1), walls=walls,
                                      materials=[m0, m1])


def walled_state(seed, n=900):
    from mddem_gb300 import inputs

    r = 5e-4
    pos, rad = inputs.random_spheres(n, L, r, seed=seed, sep_factor=0.96, inset=True)
    rng = np.random.default_rng(seed + 5)
    st = inputs._dem_state(pos, rng.normal(scale=0.5, size=(n, 3)), rad, RHO)
    st["omega"] = rng.normal(scale=200.0, size=(n, 3))
    st["type"] = (rng.random(n) < 0.3).astype(st["type"].dtype)
    return st


def _wall_contacts(st, g=0.2 * 5e-4):
    p, r = st["pos"], st["radius"]
    return int(np.sum(p[:, 0] - g < r) + np.sum(L - g - p[:, 0] < r) + np.sum(p[:, 2] - g < r)
               + np.sum(L - g - p[:, 2] < r))


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [dict(), dict(twisting_friction=0.05), dict(surface_energy=0.05),
                                     dict(cohesion_energy=500.0)])
def test_gpu_walled_force_parity(gpu_lib, variant):
    from oracle.oracle import Oracle

    cfg = walled_config(**variant)
    st = walled_state(seed=3)
    assert _wall_contacts(st) > 50
    ctx = _ctx(cfg, st)
    o = Oracle(cfg)
    o.load(st)
    ctx.force_only()
    o.force_only()
    assert pair_set(ctx.pairs()) == pair_set(o.pairs())
    g, r = ctx.download(), o.state()
    gf, gt = by_tag(g, "force", "torque")
    # per particle against max(|F_ref|, sum of its pair and wall force magnitudes)
    r["fscale"], r["tscale"] = o.pair_scale()
    rf, rt, fs, ts = by_tag(r, "force", "torque", "fscale", "tscale")
    assert rel_err(gf, rf, fs) <= 1e-12
    assert rel_err(gt, rt, ts) <= 1e-12
    # mixed: 1e-5 per particle against the fp64 path
    m = _ctx(cfg.replace(precision="mixed"), st)
    m.force_only()
    mf, mt = by_tag(m.download(), "force", "torque")
    scale = np.max(np.abs(gf), axis=1) + 1e-3 * np.max(np.abs(gf))
    assert rel_err(mf, gf, scale) <= 1e-5


@pytest.mark.gpu
def test_gpu_walled_100_steps_trajectory(gpu_lib):
    from oracle.oracle import Oracle

    cfg = walled_config(g_frac=0.05, twisting_friction=0.05)  # wall forces like the pair forces
    st = walled_state(seed=6)
    assert _wall_contacts(st, 0.05 * 5e-4) > 5
    ctx = _ctx(cfg, st)
    o = Oracle(cfg)
    o.load(st)
    ctx.step(100)
    o.step(100)
    gpos, gw = by_tag(ctx.download(), "pos", "omega")
    rpos, rw = by_tag(o.state(), "pos", "omega")
    assert np.max(np.abs(gpos - rpos)) <= 1e-12 * L
    assert np.max(np.abs(gw - rw)) <= 1e-9 * np.max(np.abs(rw))
    assert pair_set(ctx.history()[0]) == pair_set(o.history()[0])
    assert ctx.thermo()["nbuilds"] == o.thermo()["nbuilds"]
    m = _ctx(cfg.replace(precision="mixed"), st)
    m.step(100)
    (mpos,) = by_tag(m.download(), "pos")
    # 30 % steel particles (E 23x glass) make pair forces, and with them the
    # 1e-5 relative fp32 force error, larger than in the glass-only gas
    assert np.max(np.abs(mpos - gpos)) <= 1e-8 * L


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_particle_leaving_fixed_axis_is_an_error(gpu_lib, precision):
    from mddem_gb300 import capi, config, inputs

    r = 5e-4
    pos = np.array([[0.006, 0.006, 2 * r], [0.003, 0.003, 0.006]])
    st = inputs._dem_state(pos, np.array([[0.0, 0.0, -100.0], [0.0, 0.0, 0.0]]), np.full(2, r), RHO)
    ctx = _ctx(config.granular_gas_config(box=L, dt=1e-7, fixed=(0, 0, 1), precision=precision), st)
    with pytest.raises(capi.MdgError) as e:
        ctx.step(200)
    assert e.value.status == 12


REBOUND_TOML = WALL_TOML.replace('boundary_y = "periodic"', 'boundary_y = "fixed"').split("[[wall]]")[0] + """
[[particles.insert]]
material = "glass"
count = 1
radius = 0.005
density = 2500.0
velocity_z = -1.0
region = { type = "block", min = [-0.001, -0.001, 0.0052], max = [0.001, 0.001, 0.0053] }

[[wall]]
normal_z = 1.0
material = "glass"

[run]
steps = 1000
thermo = 100
"""


def test_runner_setup_block_region_and_walls():
    from mddem_gb300 import config, run

    cfg, st, s = run.setup(REBOUND_TOML, seed=2)
    assert cfg.fixed == (1, 1, 1) and len(cfg.walls) == 1 and s["steps"] == 1000
    assert cfg.dt == pytest.approx(config.rayleigh_dt(R, RHO, E, NU))
    p = st["pos"][0]
    assert -0.001 <= p[0] <= 0.001 and -0.001 <= p[1] <= 0.001 and 0.0052 <= p[2] <= 0.0053
    assert np.array_equal(st["vel"][0], [0.0, 0.0, -1.0])


@pytest.mark.gpu
def test_runner_rebound_config(gpu_lib, tmp_path):
    """The rebound config through the TOML runner: the sphere bounces off the
    floor wall and leaves upward at about e * v0."""
    import io

    from mddem_gb300 import run

    out = io.StringIO()
    ctx = run.run(REBOUND_TOML, seed=2, out=out)
    v = ctx.download()["vel"][0]
    assert v[2] == pytest.approx(COR * V0, rel=0.03)
    assert "1000 steps" in out.getvalue()


def _one_sphere_force(z, w=(0.0, 0.0, 0.0), v=(0.0, 0.0, 0.0), **mat):
    """Oracle force and torque on one 5 mm sphere at height z above the floor
    wall (one force evaluation)."""
    from mddem_gb300 import config, inputs
    from oracle.oracle import Oracle

    cfg = rebound_config()
    m = config.Material(name="glass", youngs_mod=E, poisson_ratio=NU, restitution=COR, friction=0.0, **mat)
    cfg = cfg.replace(materials=[m])
    st = inputs._dem_state(np.array([[0.0, 0.0, z]]), np.array([v]), np.array([R]), RHO)
    st["omega"] = np.array([w], dtype=float)
    o = Oracle(cfg)
    o.load(st)
    o.force_only()
    s = o.state()
    return s["force"][0], s["torque"][0]


def test_oracle_wall_hertz_force_closed_form():
    """Elastic part at rest: 4/3 E* sqrt(R delta) delta along the normal, with
    E* of the same material on both sides (wall_contact_force, lib.rs:905-944)."""
    delta = 1e-5
    f, t = _one_sphere_force(R - delta)
    e_star = E / (2.0 * (1.0 - NU * NU))
    assert f[2] == pytest.approx(4.0 / 3.0 * e_star * math.sqrt(R * delta) * delta, rel=1e-12)
    assert f[0] == 0.0 and f[1] == 0.0 and np.all(t == 0.0)
    f_far, _ = _one_sphere_force(R + 1e-6)  # out of contact, no adhesion: nothing
    assert np.all(f_far == 0.0)


def test_oracle_wall_twisting_torque_opposes_spin():
    """A sphere pressed on the floor and spinning about the normal feels
    -sign(omega_n) mu_tw |F_n| R about the normal (lib.rs:947-962)."""
    delta, mu_tw = 1e-5, 0.05
    for wz in (30.0, -30.0):
        f, t = _one_sphere_force(R - delta, w=(0.0, 0.0, wz), twisting_friction=mu_tw)
        assert t[2] == pytest.approx(-math.copysign(1.0, wz) * mu_tw * abs(f[2]) * R, rel=1e-12)
        assert t[0] == 0.0 and t[1] == 0.0


def test_oracle_wall_jkr_adhesion_only_range():
    """JKR: inside the pull-off distance but not touching, the wall pulls with
    1.5 pi gamma R (lib.rs:929-934); beyond it, nothing."""
    gamma = 0.05
    e_star = E / (2.0 * (1.0 - NU * NU))
    pull = (math.pi ** 2 * gamma ** 2 * R / (4.0 * e_star ** 2)) ** (1.0 / 3.0)
    f, _ = _one_sphere_force(R + 0.5 * pull, surface_energy=gamma)
    assert f[2] == pytest.approx(-1.5 * math.pi * gamma * R, rel=1e-12)
    f2, _ = _one_sphere_force(R + 2.0 * pull, surface_energy=gamma)
    assert np.all(f2 == 0.0)


def test_oracle_elastic_rebound_keeps_the_energy():
    """e = 1 (no damping): the sphere leaves with its impact speed, to the
    Verlet error of ~46 contact steps."""
    from mddem_gb300 import config
    from oracle.oracle import Oracle

    cfg = rebound_config()
    cfg = cfg.replace(materials=[config.Material(name="glass", youngs_mod=E, poisson_ratio=NU, restitution=1.0,
                                                 friction=0.0)])
    o = Oracle(cfg)
    o.load(rebound_state())

    def read():
        s = o.state()
        return s["pos"][0, 2], s["vel"][0, 2]

    cor, _, _ = track_rebound(lambda: o.step(1), read)
    assert cor == pytest.approx(1.0, abs=2e-3)
