"""GPU parity: CUDA path (through the C ABI) vs the CPU FP64 oracle.

Tolerances (stated here, as the bar of the FP64 path):
  * neighbour pair sets and contact-history keys: identical;
  * single-step forces and torques: per particle
    |F_gpu - F_ref|_inf / max(|F_ref|_inf, sum_pairs |f_pair|, tiny) <= 1e-12;
  * contact-history values: <= 1e-12 relative to the largest spring;
  * 100-step trajectories: positions within 1e-10 of the box length for the
    chaotic LJ melt and 1e-12 for the granular gas.
"""
import numpy as np
import pytest

from helpers import by_tag, lj_pair_force_scale, overlapping_spheres, pair_set, rel_err

pytestmark = pytest.mark.gpu


def _ctx(cfg, st):
    from mddem_gb300 import capi

    ctx = capi.Context(cfg, len(st["tag"]))
    ctx.upload(st)
    return ctx


def _oracle(cfg, st):
    from oracle.oracle import Oracle

    o = Oracle(cfg)
    o.load(st)
    return o


def test_lj_force_only_parity(gpu_lib):
    from mddem_gb300 import config, inputs

    cfg = config.lj_fluid_config()
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=5)
    rng = np.random.default_rng(0)
    st["pos"] = st["pos"] + rng.normal(scale=0.05, size=st["pos"].shape)  # off-lattice
    ctx = _ctx(cfg, st)
    ctx.force_only()
    g = ctx.download()
    gp = ctx.pairs()
    o = _oracle(cfg, st)
    o.force_only()
    r = o.state()
    rp = o.pairs()
    assert pair_set(gp) == pair_set(rp)
    assert len(gp) == len(rp)
    (gf,) = by_tag(g, "force")
    rf, rpos = by_tag(r, "force", "pos")
    scale = lj_pair_force_scale(rpos, cfg.box, rp)
    assert rel_err(gf, rf, scale) <= 1e-12
    assert abs(ctx.thermo()["pe"] - o.thermo()["pe"]) <= 1e-12 * abs(o.thermo()["pe"])


def test_lj_100_steps_nose_hoover(gpu_lib):
    from mddem_gb300 import config, inputs

    cfg = config.lj_fluid_config()
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=7)
    ctx = _ctx(cfg, st)
    o = _oracle(cfg, st)
    ctx.step(100)
    o.step(100)
    g = ctx.download()
    r = o.state()
    gpos, gvel = by_tag(g, "pos", "vel")
    rpos, rvel = by_tag(r, "pos", "vel")
    assert np.max(np.abs(gpos - rpos)) <= 1e-10 * 10.06
    assert np.max(np.abs(gvel - rvel)) <= 1e-9
    tg, tr = ctx.thermo(), o.thermo()
    for k in ("ke", "pe"):
        assert abs(tg[k] - tr[k]) <= 1e-10 * abs(tr[k]), k
    assert abs(tg["p_xi"] - tr["p_xi"]) <= 1e-8 * max(1.0, abs(tr["p_xi"]))
    assert tg["nbuilds"] == tr["nbuilds"]


def _dem_cfg(**kw):
    from mddem_gb300 import config

    return config.granular_gas_config(box=0.012, dt=1e-7, **kw)


def _dem_state(seed=1, n=900):
    return overlapping_spheres(n, 0.012, 5e-4, seed=seed)


def _check_dem_force_parity(cfg, st, hist=True):
    ctx = _ctx(cfg, st)
    o = _oracle(cfg, st)
    if hist:
        # seed the spring history of every owner pair with random springs
        o.force_only()
        keys, vals = o.history()
        rng = np.random.default_rng(3)
        vals = rng.normal(scale=1e-6, size=vals.shape)
        o2 = _oracle(cfg, st)
        o2.set_history(keys, vals)
        ctx.set_history(keys, vals)
        o = o2
    ctx.force_only()
    o.force_only()
    g = ctx.download()
    r = o.state()
    assert pair_set(ctx.pairs()) == pair_set(o.pairs())
    gf, gt = by_tag(g, "force", "torque")
    # per particle: |F_gpu - F_ref|_inf / max(|F_ref|_inf, sum_pairs |f_pair|)
    # (and the same with torques), the sums from the oracle's pair loop
    r["fscale"], r["tscale"] = o.pair_scale()
    rf, rt, fs, ts = by_tag(r, "force", "torque", "fscale", "tscale")
    assert rel_err(gf, rf, fs) <= 1e-12
    assert rel_err(gt, rt, ts) <= 1e-12
    gk, gv = ctx.history()
    rk, rv = o.history()
    assert pair_set(gk) == pair_set(rk)
    gd = {tuple(k): v for k, v in zip(gk.tolist(), gv)}
    vmax = max(1e-300, float(np.max(np.abs(rv)))) if len(rv) else 1.0
    for k, v in zip(rk.tolist(), rv):
        assert np.max(np.abs(gd[tuple(k)] - v)) <= 1e-12 * vmax
    return len(rk)


def test_dem_hertz_force_history_parity(gpu_lib):
    n = _check_dem_force_parity(_dem_cfg(), _dem_state())
    assert n > 100


@pytest.mark.parametrize("variant", [
    dict(contact_model="hooke"),
    dict(rolling=0.05, twisting=0.03),
    dict(rolling=0.05, twisting=0.03, rolling_model="sds", twisting_model="sds"),
    dict(surface_energy=0.05),
    dict(surface_energy=0.05, adhesion_model="dmt"),
    dict(cohesion_energy=500.0),
])
def test_dem_contact_variants(gpu_lib, variant):
    from mddem_gb300.config import Material

    m = Material()
    v = dict(variant)
    if v.pop("contact_model", None) == "hooke":
        m.kn, m.kt = 2e5, 5e4
        cfg = _dem_cfg(contact_model="hooke")
    else:
        cfg = _dem_cfg()
    m.rolling_friction = v.pop("rolling", 0.0)
    m.twisting_friction = v.pop("twisting", 0.0)
    m.surface_energy = v.pop("surface_energy", 0.0)
    m.cohesion_energy = v.pop("cohesion_energy", 0.0)
    if v.get("rolling_model") == "sds":
        m.rolling_stiffness, m.rolling_damping = 1e-4, 1e-7
        m.twisting_stiffness, m.twisting_damping = 1e-4, 1e-7
    cfg = cfg.replace(materials=[m], **v)
    _check_dem_force_parity(cfg, _dem_state(seed=2))


def test_dem_100_steps_trajectory(gpu_lib):
    cfg = _dem_cfg()
    st = _dem_state(seed=4)
    ctx = _ctx(cfg, st)
    o = _oracle(cfg, st)
    ctx.step(100)
    o.step(100)
    g = ctx.download()
    r = o.state()
    gpos, gw, gq = by_tag(g, "pos", "omega", "quat")
    rpos, rw, rq = by_tag(r, "pos", "omega", "quat")
    assert np.max(np.abs(gpos - rpos)) <= 1e-12 * 0.012
    assert np.max(np.abs(gw - rw)) <= 1e-9 * np.max(np.abs(rw))
    assert np.max(np.abs(gq - rq)) <= 1e-12
    assert pair_set(ctx.history()[0]) == pair_set(o.history()[0])
    assert ctx.thermo()["nbuilds"] == o.thermo()["nbuilds"]


def test_mixed_lj_force_error(gpu_lib):
    from mddem_gb300 import config, inputs

    cfg64 = config.lj_fluid_config()
    cfgmx = config.lj_fluid_config(precision="mixed")
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=5)
    rng = np.random.default_rng(0)
    st["pos"] = st["pos"] + rng.normal(scale=0.05, size=st["pos"].shape)
    a = _ctx(cfg64, st)
    b = _ctx(cfgmx, st)
    a.force_only()
    b.force_only()
    ga, gb = a.download(), b.download()
    fa, pa = by_tag(ga, "force", "pos")
    (fb,) = by_tag(gb, "force")
    scale = lj_pair_force_scale(pa, cfg64.box, a.pairs())
    err = rel_err(fb, fa, scale)
    assert err <= 1e-5, err


def test_batch_equals_single(gpu_lib):
    from mddem_gb300 import capi, config, inputs

    c1 = config.lj_fluid_config()
    s1 = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=11)
    c2 = _dem_cfg()
    s2 = _dem_state(seed=6, n=600)
    alone = []
    for c, s in ((c1, s1), (c2, s2)):
        ctx = _ctx(c, s)
        ctx.step(20)
        alone.append(ctx.download())
    b = capi.Context([c1, c2], [len(s1["tag"]), len(s2["tag"])])
    b.upload(s1, 0)
    b.upload(s2, 1)
    b.step(20)
    for k in range(2):
        g = b.download(k)
        for f in ("pos", "vel"):
            (x,) = by_tag(g, f)
            (y,) = by_tag(alone[k], f)
            assert np.array_equal(x, y), (k, f)


def test_mixed_dem_force_error(gpu_lib):
    """Precision form, DEM: fp32 geometry/force with double-float overlap and
    fp64 springs vs the fp64 path; per-particle force and torque error <= 1e-5
    relative to max(|F|, sum of pair forces)."""
    from helpers import dem_pair_force_scale

    st = _dem_state(seed=8)
    c64 = _dem_cfg()
    cmx = _dem_cfg(precision="mixed")
    o = _oracle(c64, st)
    o.force_only()
    keys, vals = o.history()
    rng = np.random.default_rng(9)
    vals = rng.normal(scale=1e-6, size=vals.shape)
    a, b = _ctx(c64, st), _ctx(cmx, st)
    a.set_history(keys, vals)
    b.set_history(keys, vals)
    a.force_only()
    b.force_only()
    ga, gb = a.download(), b.download()
    fa, ta, pa, ra = by_tag(ga, "force", "torque", "pos", "radius")
    fb, tb = by_tag(gb, "force", "torque")
    E, nu = 8.7e9, 0.3
    e_eff = 1.0 / (2 * (1 - nu * nu) / E)
    scale = dem_pair_force_scale({"pos": pa, "radius": ra}, c64.box, a.pairs(), e_eff)
    assert np.max(scale) > 0
    assert rel_err(fb, fa, scale) <= 1e-5
    assert rel_err(tb, ta, scale * ra) <= 1e-5
    ka, va = a.history()
    kb, vb = b.history()
    assert pair_set(ka) == pair_set(kb)
    db = {tuple(k): v for k, v in zip(kb.tolist(), vb)}
    vmax = float(np.max(np.abs(va)))
    for k, v in zip(ka.tolist(), va):
        assert np.max(np.abs(db[tuple(k)] - v)) <= 1e-5 * vmax


def test_mixed_dem_trajectory_close_to_fp64(gpu_lib):
    st = _dem_state(seed=10)
    a = _ctx(_dem_cfg(), st)
    b = _ctx(_dem_cfg(precision="mixed"), st)
    a.step(100)
    b.step(100)
    pa, qa, wa = by_tag(a.download(), "pos", "quat", "omega")
    pb, qb, wb = by_tag(b.download(), "pos", "quat", "omega")
    assert np.max(np.abs(pa - pb)) <= 1e-9 * 0.012
    # fp32 rotation increment: about 1e-7 x angle/2 per step on q
    assert np.max(np.abs(qa - qb)) <= 1e-8
    assert np.max(np.abs(wa - wb)) <= 1e-5 * np.max(np.abs(wa))
    ta, tb = a.thermo(), b.thermo()
    assert abs(ta["ke"] - tb["ke"]) <= 1e-5 * ta["ke"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_non_finite_state_reports_nan(gpu_lib, precision):
    """Two LJ atoms at the same point: r = 0 makes the pair force non-finite;
    the step returns MDG_ERR_NAN and the system's status word keeps the bit."""
    from mddem_gb300 import capi, config

    st = {"tag": np.arange(3, dtype=np.uint32), "type": np.zeros(3, np.uint32),
          "pos": np.array([[5.0, 5.0, 5.0], [5.0, 5.0, 5.0], [7.0, 7.0, 7.0]]), "vel": np.zeros((3, 3)),
          "mass": np.ones(3), "cutoff_radius": np.full(3, 1.25)}
    cfg = config.lj_fluid_config(box=12.0, nose_hoover=False, precision=precision)
    ctx = capi.Context(cfg, 3)
    ctx.upload(st)
    with pytest.raises(capi.MdgError) as e:
        ctx.step(2)
    assert e.value.status == 6  # MDG_ERR_NAN
    assert ctx.status() != 0


def test_fused_multistep_equals_unfused(gpu_lib):
    """The multi-step graph of a mixed context fuses each step's final half
    with the next step's initial half (one pass over the particle arrays); the
    result must be bitwise the eager launches' (separate initial and final
    kernels): a thermostatted LJ melt and two DEM gases in one batch, one gas
    with a step budget that ends inside a launch, over several launches."""
    from mddem_gb300 import capi, config, inputs

    cfgs = [config.lj_fluid_config(precision="mixed", policy="displacement"),
            config.granular_gas_config(box=0.02, dt=2e-7, precision="mixed", policy="displacement"),
            config.granular_gas_config(box=0.012, dt=1e-7, precision="mixed")]
    sts = [inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=31), inputs.dem_granular_gas(400, box=0.02, seed=32),
           _dem_state(seed=33, n=600)]
    out = []
    for graph in (1, 0):
        c = capi.Context(cfgs, [len(s["tag"]) for s in sts])
        for k, s in enumerate(sts):
            c.upload(s, k)
        c.set_graph_mode(graph)
        c.set_remaining(23, 1)
        for n in (1, 17, 40, 5):
            c.step(n)
        out.append([c.download(k) for k in range(3)] + [[c.thermo(k) for k in range(3)]])
    for k in range(3):
        for f in ("pos", "vel") + (("omega", "quat") if k else ()):
            (a,) = by_tag(out[0][k], f)
            (b,) = by_tag(out[1][k], f)
            assert np.array_equal(a, b), (k, f)
    for ta, tb in zip(out[0][3], out[1][3]):
        assert ta["step"] == tb["step"] and ta["nbuilds"] == tb["nbuilds"] and ta["p_xi"] == tb["p_xi"]
    assert out[0][3][1]["step"] == 23


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_dilute_gas_list_parity(gpu_lib, precision):
    """A dilute gas (about 2 spheres per bin, list built with a thread per
    particle) gives the oracle's pair set and forces, at the first build and
    after 600 steps with rebuilds."""
    from mddem_gb300 import workloads as w

    cfg, st = w.gas(4000, phi=0.08, seed=5, precision=precision, policy="reference")
    cfg = cfg.replace(dt=1e-6)
    ctx = _ctx(cfg, st)
    o = _oracle(cfg.replace(precision="fp64"), st)
    ctx.force_only()
    o.force_only()
    assert pair_set(ctx.pairs()) == pair_set(o.pairs())
    ctx.step(600)
    o.step(600)
    assert ctx.thermo()["nbuilds"] >= 3
    if precision == "fp64":
        assert ctx.thermo()["nbuilds"] == o.thermo()["nbuilds"]
        assert pair_set(ctx.pairs()) == pair_set(o.pairs())
        gpos, = by_tag(ctx.download(), "pos")
        rpos, = by_tag(o.state(), "pos")
        assert np.max(np.abs(gpos - rpos)) <= 1e-12 * cfg.box[0]


@pytest.mark.parametrize("newton", [True, False])
def test_mixed_lj_virial(gpu_lib, newton):
    """Precision form with a virial: the mixed LJ kernel's per-particle
    virials (fp32 per lane, summed in fp64) give the plain path's virial and
    pressure to 2e-6 of the virial's largest component on an off-lattice
    melt; after 30 steps (trajectories differ by the force error) to 1e-4."""
    from mddem_gb300 import config, inputs

    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=12)
    rng = np.random.default_rng(4)
    st["pos"] = st["pos"] + rng.normal(scale=0.05, size=st["pos"].shape)
    base = config.lj_fluid_config(virial=True, newton=newton)
    a = _ctx(base, st)
    b = _ctx(base.replace(precision="mixed"), st)
    for step in (0, 30):
        if step:
            a.step(step)
            b.step(step)
        else:
            a.force_only()
            b.force_only()
        tol = 1e-4 if step else 2e-6
        ta, tb = a.thermo(), b.thermo()
        wa, wb = np.array(ta["virial"]), np.array(tb["virial"])
        assert np.max(np.abs(wa)) > 0
        assert np.max(np.abs(wb - wa)) <= tol * np.max(np.abs(wa))
        # virial pressure terms -tr(W) / 3V (+ the same tail correction)
        pa = ta["pressure"] - 864 / 10.06 ** 3 * ta["temp"]
        pb = tb["pressure"] - 864 / 10.06 ** 3 * tb["temp"]
        assert abs(pb - pa) <= tol * np.max(np.abs(wa)) / 10.06 ** 3


def test_mixed_dem_virial(gpu_lib):
    """Precision form, DEM with a virial (contact.rs:559-569): the mixed
    contact pass's owner-side sums of d_a f_b (fp32 pair terms, fp64 sums)
    give the plain path's virial to 1e-5 of its largest component after one
    force evaluation with seeded springs, and to 1e-4 after 30 steps."""
    st = _dem_state(seed=27)
    c64 = _dem_cfg(virial=True)
    o = _oracle(c64, st)
    o.force_only()
    keys, vals = o.history()
    vals = np.random.default_rng(28).normal(scale=1e-6, size=vals.shape)
    a, b = _ctx(c64, st), _ctx(c64.replace(precision="mixed"), st)
    a.set_history(keys, vals)
    b.set_history(keys, vals)
    a.force_only()
    b.force_only()
    wa, wb = np.array(a.thermo()["virial"]), np.array(b.thermo()["virial"])
    assert np.max(np.abs(wa)) > 0
    assert np.max(np.abs(wb - wa)) <= 1e-5 * np.max(np.abs(wa))
    a2, b2 = _ctx(c64, st), _ctx(c64.replace(precision="mixed"), st)
    a2.step(30)
    b2.step(30)
    wa, wb = np.array(a2.thermo()["virial"]), np.array(b2.thermo()["virial"])
    assert np.max(np.abs(wb - wa)) <= 1e-4 * np.max(np.abs(wa))


def test_mixed_dem_grazing_contacts_in_a_large_box(gpu_lib):
    """Pairs overlapping by 1e-8 m (5e-6 of the radius sum) scattered through
    a 0.25 m box, where the lo parts of the two-float positions reach ~1e-8 m:
    the mixed path screens on the full two-float separation and keeps the
    dl^2 term of the squared distance, so every pair acts, with the fp64
    path's force to 1e-5."""
    from mddem_gb300 import config, inputs

    rng = np.random.default_rng(30)
    L, r, npair = 0.25, 1e-3, 200
    a = rng.uniform(0.01, L - 0.01, size=(npair, 3))
    u = rng.normal(size=(npair, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    b = a + u * (2 * r - 1e-8)
    pos = np.empty((2 * npair, 3))
    pos[0::2], pos[1::2] = a, b
    st = inputs._dem_state(pos, np.zeros((2 * npair, 3)), np.full(2 * npair, r), 2500.0)
    cfg = config.granular_gas_config(box=L, dt=1e-7)
    c64, cmx = _ctx(cfg, st), _ctx(cfg.replace(precision="mixed"), st)
    c64.force_only()
    cmx.force_only()
    (f64,) = by_tag(c64.download(), "force")
    (fmx,) = by_tag(cmx.download(), "force")
    mag = np.linalg.norm(f64, axis=1)
    assert np.all(mag > 0)
    assert rel_err(fmx, f64, mag) <= 1e-5


@pytest.mark.parametrize("dr", [-1e-9, 1e-9, -3e-7, 3e-7])
def test_mixed_lj_pairs_at_the_cutoff_count_like_fp64(gpu_lib, dr):
    """The LJ force is cut off without a shift (a jump of f(rc) at rc): a pair
    within fp32 rounding of the cutoff must be counted by the mixed path
    exactly when the FP64 path counts it, or its particles' force error is
    ~1e-3.  Two atoms at rc + dr, along x and along a diagonal through a
    periodic face."""
    import numpy as np

    from mddem_gb300 import capi, config

    cfg = config.lj_fluid_config(nose_hoover=False)
    rc = cfg.lj_cutoff * cfg.lj_sigma
    L = cfg.box[0]
    for a, u in (((5.0, 5.0, 5.0), (1.0, 0.0, 0.0)), ((L - 0.7, 3.1, 2.2), (0.6, 0.64, 0.48))):
        u = np.asarray(u) / np.linalg.norm(u)
        pa = np.asarray(a)
        pb = (pa + (rc + dr) * u) % L
        st = {"tag": np.arange(2, dtype=np.uint32), "type": np.zeros(2, np.uint32),
              "pos": np.array([pa, pb]), "vel": np.zeros((2, 3)), "mass": np.ones(2),
              "cutoff_radius": np.full(2, 1.25)}
        f = {}
        for prec in ("fp64", "mixed"):
            c = capi.Context(cfg.replace(precision=prec), 2)
            c.upload(st)
            c.force_only()
            f[prec] = c.download()["force"]
            c.close()
        inside = bool(np.any(f["fp64"] != 0.0))
        assert inside == (dr < 0.0)
        if inside:
            assert np.max(np.abs(f["mixed"] - f["fp64"])) <= 1e-5 * np.max(np.abs(f["fp64"])), (a, dr)
        else:
            assert not np.any(f["mixed"] != 0.0), (a, dr)
