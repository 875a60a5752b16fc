"""Multi-type LJ on the device (pair_table.get(ti, tj) in lj_force,
md_lj/src/lib.rs:488-633) against the FP64 oracle, on a two-type lattice
fluid with per-type masses, a geometric cross pair replaced by a
[[lj.pair_coeffs]] override with its own cutoff:

  * fp64: the same pair set, per-particle forces within 1e-12 of the pair
    scale, the pair energy within 1e-12, a 100-step Nose-Hoover trajectory
    within 1e-10 of the box length, tail corrections equal to 1e-14;
  * mixed: forces within 1e-5 of the fp64 path (the precision form's bound);
  * a single-type system batched with a multi-type one keeps its own
    coefficients: its force launch then runs the typed kernel instantiation,
    whose table entries hold the same coefficients, so after 20 steps its
    positions equal those of it run alone bit for bit (both precisions;
    measured on GB300);
  * a particle type outside the table is refused at upload.
"""
import numpy as np
import pytest

from helpers import by_tag, lj_pair_force_scale, pair_set, rel_err
from test_lj_types_cpu import two_type_config

pytestmark = pytest.mark.gpu


def _state(seed=5, noise=0.05):
    from mddem_gb300 import inputs

    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=seed, type_fractions=[0.5, 1.0], type_masses=[1.0, 1.5])
    st["pos"] = st["pos"] + np.random.default_rng(seed).normal(scale=noise, size=st["pos"].shape)
    return st


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


def test_fp64_force_parity(gpu_lib):
    cfg = two_type_config()
    st = _state()
    ctx = _ctx(cfg, st)
    ctx.force_only()
    g, gp = ctx.download(), ctx.pairs()
    o = _oracle(cfg, st)
    o.force_only()
    r, rp = o.state(), o.pairs()
    assert pair_set(gp) == pair_set(rp)
    (gf,) = by_tag(g, "force")
    rf, rpos, rtype = by_tag(r, "force", "pos", "type")
    scale = lj_pair_force_scale(rpos, cfg.box, rp, types=rtype, table=cfg.lj_pairs)
    assert rel_err(gf, rf, scale) <= 1e-12
    assert abs(ctx.thermo()["pe"] - o.thermo()["pe"]) <= 1e-12 * abs(o.thermo()["pe"])


def test_fp64_100_steps_nose_hoover(gpu_lib):
    cfg = two_type_config(nose_hoover=True)
    st = _state(seed=7, noise=0.0)
    ctx = _ctx(cfg, st)
    o = _oracle(cfg, st)
    ctx.step(100)
    o.step(100)
    gpos, gvel = by_tag(ctx.download(), "pos", "vel")
    rpos, rvel = by_tag(o.state(), "pos", "vel")
    assert np.max(np.abs(gpos - rpos)) <= 1e-10 * 10.06
    assert np.max(np.abs(gvel - rvel)) <= 1e-9
    tg, tr = ctx.thermo(), o.thermo()
    for k in ("ke", "pe"):
        assert abs(tg[k] - tr[k]) <= 1e-10 * abs(tr[k]), k
    assert tg["nbuilds"] == tr["nbuilds"]
    e, p = o.lj_tails()
    assert tg["e_tail"] == pytest.approx(e, rel=1e-14) and tg["p_tail"] == pytest.approx(p, rel=1e-14)


def test_mixed_force_error(gpu_lib):
    st = _state()
    a = _ctx(two_type_config(), st)
    b = _ctx(two_type_config(precision="mixed"), st)
    a.force_only()
    b.force_only()
    ga, gb = a.download(), b.download()
    fa, pa, ta = by_tag(ga, "force", "pos", "type")
    (fb,) = by_tag(gb, "force")
    scale = lj_pair_force_scale(pa, (10.06,) * 3, a.pairs(), types=ta, table=two_type_config().lj_pairs)
    err = rel_err(fb, fa, scale)
    assert err <= 1e-5, err


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_single_type_system_batched_with_a_typed_one(gpu_lib, precision):
    from mddem_gb300 import capi, config, inputs

    c1 = config.lj_fluid_config(precision=precision)
    s1 = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=11)
    c2 = two_type_config(precision=precision)
    s2 = _state(seed=3)
    alone = _ctx(c1, s1)
    alone.step(20)
    b = capi.Context([c1, c2], [len(s1["tag"]), len(s2["tag"])])
    b.upload(s1, 0)
    b.upload(s2, 1)
    b.step(20)
    (x,) = by_tag(b.download(0), "pos")
    (y,) = by_tag(alone.download(), "pos")
    assert np.array_equal(x, y)
    o = _oracle(c2, s2)
    o.step(20)
    (gx,) = by_tag(b.download(1), "pos")
    (rx,) = by_tag(o.state(), "pos")
    assert np.max(np.abs(gx - rx)) <= (1e-10 if precision == "fp64" else 1e-4) * 10.06


def test_type_outside_the_table_is_refused(gpu_lib):
    from mddem_gb300 import capi

    st = _state()
    st["type"] = st["type"].copy()
    st["type"][17] = 2
    ctx = capi.Context(two_type_config(), len(st["tag"]))
    with pytest.raises(capi.MdgError):
        ctx.upload(st)
