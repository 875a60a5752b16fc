"""GPU parity on the paths the smaller tests do not reach, against the FP64
oracle (per-particle metric |F_gpu - F_ref|_inf / max(|F_ref|_inf,
sum_pairs |f_pair|) <= 1e-12, with sum_pairs |f_pair| from the oracle's own
pair loop; the same for torques):

  * every list-build mode (warp per bin, warp per particle, thread per
    particle) on one LJ fluid of 256,000 atoms, where the automatic choice is
    a warp per bin, and on a polydisperse gas: pair sets identical to the
    oracle's half list (owner rule included), forces at 1e-12;
  * a polydisperse DEM packing, r ~ U[0.8, 1.2] mm at solid fraction 0.3
    (50,000 spheres): the size-dependent list cutoff (s_i + s_j)^2 skin^2
    (neighbor.rs:1024-1025), unequal torque arms (contact.rs:402-408),
    R* and m_r of unequal partners; force, torque and history at 1e-12 and a
    100-step trajectory within 1e-12 of the box;
  * the displacement rebuild policy (positions unwrapped between builds,
    periodic images in the list) against the oracle's reference policy:
    100-step trajectories equal modulo the box (DEM 1e-12, LJ 1e-10 of L);
  * per-replica material tables in one batch (restitution and friction per
    replica, as in the 256-replica ensemble) against one oracle per replica;
  * the virial (virial.rs:61-68) of the plain path: LJ and DEM values
    against the oracle's at 1e-12 after one force evaluation.
"""
import numpy as np
import pytest

from helpers import by_tag, overlapping_spheres, pair_set, rel_err

pytestmark = pytest.mark.gpu

POLY_R = (0.8e-3, 1.2e-3)


def pair_codes(pairs):
    """Sorted uint64 codes owner << 32 | partner of a half list (fast set
    equality for lists of millions of pairs)."""
    p = np.asarray(pairs, dtype=np.uint64).reshape(-1, 2)
    return np.sort((p[:, 0] << np.uint64(32)) | p[:, 1])


def _oracle(cfg, st):
    from oracle.oracle import Oracle

    o = Oracle(cfg.replace(precision="fp64"))
    o.load(st)
    return o


def _ctx(cfg, st, mode=-1):
    from mddem_gb300 import capi

    ctx = capi.Context(cfg, len(st["tag"]))
    if mode >= 0:
        ctx.build_mode(mode)
    ctx.upload(st)
    return ctx


def _ref_forces(o):
    """Oracle forces, torques and the per-particle pair scales, by tag."""
    r = o.state()
    fs, ts = o.pair_scale()
    r["fscale"], r["tscale"] = fs, ts
    keys = ["force", "fscale"] + (["torque", "tscale"] if "torque" in r else [])
    return dict(zip(keys, by_tag(r, *keys)))


def _check_forces(ctx, ref, tol=1e-12):
    g = ctx.download()
    if "torque" in ref:
        gf, gt = by_tag(g, "force", "torque")
        assert rel_err(gt, ref["torque"], ref["tscale"]) <= tol
    else:
        (gf,) = by_tag(g, "force")
    assert rel_err(gf, ref["force"], ref["fscale"]) <= tol


def test_build_modes_lj_256k(gpu_lib):
    """LJ fluid, 256,000 atoms (40^3 FCC cells, box 67.06): 12,167 bins, so the
    automatic mode is a warp per bin; the two other modes are forced on the
    same system.  Every mode gives the oracle's pair set and forces."""
    from mddem_gb300 import config, inputs

    cfg = config.lj_fluid_config(box=67.06)
    st = inputs.lj_fcc(40, 67.06, 0.85, 0.85, seed=21)
    st["pos"] = st["pos"] + np.random.default_rng(21).normal(scale=0.03, size=st["pos"].shape)
    o = _oracle(cfg, st)
    o.force_only()
    ref_pairs = pair_codes(o.pairs())
    ref = _ref_forces(o)
    assert len(ref_pairs) > 9_000_000
    for mode in (-1, 0, 1, 2):
        ctx = _ctx(cfg, st, mode)
        ctx.force_only()
        assert np.array_equal(pair_codes(ctx.pairs()), ref_pairs), mode
        _check_forces(ctx, ref)
        ctx.close()


def _poly_state(n=50_000, seed=5):
    """Polydisperse packing with small overlaps (centres at least 0.96
    (r_i + r_j) apart, placed by the library's seeded grid RSA), random
    velocities and spins."""
    from mddem_gb300 import capi, inputs, workloads as w

    cfg = w.polydisperse_config(n=n, phi=0.30, precision="fp64", policy="reference")
    L = cfg.box[0]
    pos, rad = capi.rsa_spheres(n, (0.0, 0.0, 0.0), (L, L, L), POLY_R[0], POLY_R[1], sep_factor=0.96,
                                inset=False, seed=seed)
    rng = np.random.default_rng(seed + 11)
    st = inputs._dem_state(pos, rng.normal(scale=0.5, size=(n, 3)), rad, 2500.0)
    st["omega"] = rng.normal(scale=300.0, size=(n, 3))
    return cfg, st


def _check_history(ctx, o, tol=1e-12):
    gk, gv = ctx.history()
    rk, rv = o.history()
    assert np.array_equal(pair_codes(gk), pair_codes(rk))
    vmax = max(1e-300, float(np.max(np.abs(rv)))) if len(rv) else 1.0
    go = np.lexsort((gk[:, 1], gk[:, 0]))
    ro = np.lexsort((rk[:, 1], rk[:, 0]))
    assert np.max(np.abs(gv[go] - rv[ro])) <= tol * vmax


def test_polydisperse_dem_parity(gpu_lib):
    """Unequal radii: pair set, per-particle force and torque at 1e-12,
    history keys identical and values at 1e-12 after one force evaluation
    with seeded springs; 100 steps: positions within 1e-12 of the box,
    angular velocities within 1e-9, the same contact keys."""
    cfg, st = _poly_state()
    r = st["radius"]
    assert r.min() >= POLY_R[0] and r.max() <= POLY_R[1] and r.max() / r.min() > 1.4
    o = _oracle(cfg, st)
    o.force_only()
    keys, _ = o.history()
    assert len(keys) > 5_000
    vals = np.random.default_rng(7).normal(scale=1e-6, size=(len(keys), 7))
    o = _oracle(cfg, st)
    o.set_history(keys, vals)
    o.force_only()
    ctx = _ctx(cfg, st)
    ctx.set_history(keys, vals)
    ctx.force_only()
    assert np.array_equal(pair_codes(ctx.pairs()), pair_codes(o.pairs()))
    _check_forces(ctx, _ref_forces(o))
    _check_history(ctx, o)
    ctx.close()

    ctx = _ctx(cfg, st)
    o = _oracle(cfg, st)
    ctx.step(100)
    o.step(100)
    gp, gw = by_tag(ctx.download(), "pos", "omega")
    rp, rw = by_tag(o.state(), "pos", "omega")
    assert np.max(np.abs(gp - rp)) <= 1e-12 * cfg.box[0]
    assert np.max(np.abs(gw - rw)) <= 1e-9 * np.max(np.abs(rw))
    assert np.array_equal(pair_codes(ctx.history()[0]), pair_codes(o.history()[0]))
    assert ctx.thermo()["nbuilds"] == o.thermo()["nbuilds"]


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_build_modes_polydisperse(gpu_lib, mode):
    """The size-dependent list cutoff in every build mode: pair set and
    forces of the polydisperse packing (20,000 spheres)."""
    cfg, st = _poly_state(n=20_000, seed=9)
    o = _oracle(cfg, st)
    o.force_only()
    ctx = _ctx(cfg, st, mode)
    ctx.force_only()
    assert np.array_equal(pair_codes(ctx.pairs()), pair_codes(o.pairs()))
    _check_forces(ctx, _ref_forces(o))


def _unwrapped(st, box):
    pos, img = by_tag(st, "pos", "image")
    return pos + img * np.asarray(box)


def test_displacement_policy_dem(gpu_lib):
    """FP64 granular gas, displacement policy (rebuild on displacement only,
    unwrapped positions) vs the oracle's reference policy over 100 steps:
    positions equal modulo the box, unwrapped positions equal, same contact
    keys."""
    from mddem_gb300 import config

    cfg = config.granular_gas_config(box=0.012, dt=1e-7, policy="displacement")
    st = overlapping_spheres(900, 0.012, 5e-4, seed=14, speed=2.0)
    ctx = _ctx(cfg, st)
    o = _oracle(cfg.replace(rebuild_policy="reference"), st)
    ctx.step(100)
    o.step(100)
    g, r = ctx.download(), o.state()
    (gp,), (rp,) = by_tag(g, "pos"), by_tag(r, "pos")
    d = gp - rp
    d -= 0.012 * np.round(d / 0.012)
    assert np.max(np.abs(d)) <= 1e-12 * 0.012
    assert np.max(np.abs(_unwrapped(g, cfg.box) - _unwrapped(r, cfg.box))) <= 1e-12 * 0.012
    assert pair_set(ctx.history()[0]) == pair_set(o.history()[0])


def test_displacement_policy_lj(gpu_lib):
    """FP64 LJ melt with Nose-Hoover, displacement policy vs the oracle over
    100 steps: positions modulo the box within 1e-10 of L, kinetic and
    potential energy within 1e-10."""
    from mddem_gb300 import config, inputs

    cfg = config.lj_fluid_config(policy="displacement")
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=17)
    ctx = _ctx(cfg, st)
    o = _oracle(cfg.replace(rebuild_policy="reference"), st)
    ctx.step(100)
    o.step(100)
    g, r = ctx.download(), o.state()
    (gp,), (rp,) = by_tag(g, "pos"), by_tag(r, "pos")
    d = gp - rp
    d -= 10.06 * np.round(d / 10.06)
    assert np.max(np.abs(d)) <= 1e-10 * 10.06
    assert np.max(np.abs(_unwrapped(g, cfg.box) - _unwrapped(r, cfg.box))) <= 1e-10 * 10.06
    tg, tr = ctx.thermo(), o.thermo()
    for k in ("ke", "pe"):
        assert abs(tg[k] - tr[k]) <= 1e-10 * abs(tr[k]), k


def test_per_replica_materials_in_one_batch(gpu_lib):
    """Four granular replicas with their own restitution and friction (the
    ensemble's per-replica material tables) in one batch context: each
    replica's forces, torques and history equal its own oracle's at 1e-12,
    and after 100 steps its positions are within 1e-12 of the box."""
    from mddem_gb300 import capi, config
    from mddem_gb300.config import Material

    cfgs, sts = [], []
    for k, (e, mu) in enumerate([(0.70, 0.0), (0.80, 0.2), (0.90, 0.35), (0.99, 0.5)]):
        m = Material()
        m.restitution, m.friction = e, mu
        cfgs.append(config.granular_gas_config(box=0.012, dt=1e-7, materials=[m]))
        sts.append(overlapping_spheres(500 + 100 * k, 0.012, 5e-4, seed=40 + k))
    b = capi.Context(cfgs, [len(s["tag"]) for s in sts])
    for k, s in enumerate(sts):
        b.upload(s, k)
    b.force_only()
    ors = []
    for k, (c, s) in enumerate(zip(cfgs, sts)):
        o = _oracle(c, s)
        o.force_only()
        ors.append(o)
        g = b.download(k)
        ref = _ref_forces(o)
        gf, gt = by_tag(g, "force", "torque")
        assert rel_err(gf, ref["force"], ref["fscale"]) <= 1e-12, k
        assert rel_err(gt, ref["torque"], ref["tscale"]) <= 1e-12, k
        gk, gv = b.history(k)
        rk, rv = o.history()
        assert pair_set(gk) == pair_set(rk), k
    b2 = capi.Context(cfgs, [len(s["tag"]) for s in sts])
    for k, s in enumerate(sts):
        b2.upload(s, k)
    b2.step(100)
    for k, (c, s) in enumerate(zip(cfgs, sts)):
        o = _oracle(c, s)
        o.step(100)
        (gp,) = by_tag(b2.download(k), "pos")
        (rp,) = by_tag(o.state(), "pos")
        assert np.max(np.abs(gp - rp)) <= 1e-12 * 0.012, k


def test_plain_virial_lj(gpu_lib):
    """Plain-path LJ virial (newton on and off) equals the oracle's after one
    force evaluation (1e-12 of its largest component) and after 30 NH steps
    (1e-9)."""
    from mddem_gb300 import config, inputs

    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=23)
    st["pos"] = st["pos"] + np.random.default_rng(23).normal(scale=0.05, size=st["pos"].shape)
    for newton in (True, False):
        cfg = config.lj_fluid_config(virial=True, newton=newton)
        ctx = _ctx(cfg, st)
        o = _oracle(cfg, st)
        ctx.force_only()
        o.force_only()
        wg, wr = np.array(ctx.thermo()["virial"]), np.array(o.thermo()["virial"])
        assert np.max(np.abs(wr)) > 0
        assert np.max(np.abs(wg - wr)) <= 1e-12 * np.max(np.abs(wr)), newton
        ctx2, o2 = _ctx(cfg, st), _oracle(cfg, st)
        ctx2.step(30)
        o2.step(30)
        wg, wr = np.array(ctx2.thermo()["virial"]), np.array(o2.thermo()["virial"])
        assert np.max(np.abs(wg - wr)) <= 1e-9 * np.max(np.abs(wr)), newton


def test_plain_virial_dem(gpu_lib):
    """Plain-path DEM virial (contact.rs:559-569: normal plus tangential pair
    force against the separation) equals the oracle's after one force
    evaluation with seeded springs, at 1e-12 of its largest component."""
    from mddem_gb300 import config

    cfg = config.granular_gas_config(box=0.012, dt=1e-7, virial=True)
    st = overlapping_spheres(900, 0.012, 5e-4, seed=25)
    o = _oracle(cfg, st)
    o.force_only()
    keys, _ = o.history()
    vals = np.random.default_rng(5).normal(scale=1e-6, size=(len(keys), 7))
    o = _oracle(cfg, st)
    o.set_history(keys, vals)
    o.force_only()
    ctx = _ctx(cfg, st)
    ctx.set_history(keys, vals)
    ctx.force_only()
    wg, wr = np.array(ctx.thermo()["virial"]), np.array(o.thermo()["virial"])
    assert np.max(np.abs(wr)) > 0
    assert np.max(np.abs(wg - wr)) <= 1e-12 * np.max(np.abs(wr))
