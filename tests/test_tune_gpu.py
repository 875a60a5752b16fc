"""Autotuner (mdg_autotune): it leaves the uploaded state exactly as it was,
picks values from its candidate sets, never reports a slower configuration
than the one it started from, refuses once a system has stepped, and a run
under the chosen parameters agrees with an untuned run (the knobs change
summation order only)."""
import numpy as np
import pytest

from helpers import by_tag

pytestmark = pytest.mark.gpu


def _batch():
    from mddem_gb300 import config, inputs

    c1 = config.lj_fluid_config(precision="mixed", policy="displacement")
    s1 = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=3)
    c2 = config.granular_gas_config(box=0.02, dt=2e-7, precision="mixed", policy="displacement")
    s2 = inputs.dem_granular_gas(400, box=0.02, seed=4)
    return [c1, c2], [s1, s2]


def test_autotune_keeps_state_and_picks_candidates(gpu_lib):
    from mddem_gb300 import capi

    cfgs, sts = _batch()
    ctx = capi.Context(cfgs, [len(s["tag"]) for s in sts])
    for k, s in enumerate(sts):
        ctx.upload(s, k)
    r = ctx.autotune(steps=20)
    assert r["tpp"] in (1, 2, 4, 8)
    assert r["skin_fraction"][0] in (1.05, 1.1, 1.2, 1.35, 1.5)
    assert r["skin_fraction"][1] in (1.08, 1.12, 1.2, 1.3, 1.4)
    assert r["bin_factor"][0] >= 1.0 and r["bin_factor"][1] >= 1.0
    assert 0 < r["ms_after"] <= r["ms_before"]
    assert r["trials"] >= 10
    for k, s in enumerate(sts):
        assert ctx.thermo(k)["step"] == 0
        g = ctx.download(k)
        for f in ("pos", "vel"):
            (x,) = by_tag(g, f)
            assert np.array_equal(x, s[f][np.argsort(s["tag"])]), f
    # untuned reference run of the same batch
    ref = capi.Context(cfgs, [len(s["tag"]) for s in sts])
    for k, s in enumerate(sts):
        ref.upload(s, k)
    ctx.step(50)
    ref.step(50)
    # positions compared under the minimum image: a different skin wraps
    # particles into the box at different rebuild steps.  The LJ force is cut
    # off without a shift: the two runs' rounding-level position differences
    # can put a pair that sits at rc on different sides of it in one step, a
    # kick of f(rc) dt (about 2e-4 in velocity, ~1e-5 sigma after 25 steps),
    # so the LJ bound is 1e-4 sigma; the granular forces are continuous
    for k, box, tol in ((0, 10.06, 1e-4), (1, 0.02, 1e-9 * 0.02)):
        (pa,) = by_tag(ctx.download(k), "pos")
        (pb,) = by_tag(ref.download(k), "pos")
        d = pa - pb
        d -= box * np.round(d / box)
        assert np.max(np.abs(d)) <= tol, k  # rounding-level divergence only


def test_autotune_refuses_after_stepping(gpu_lib):
    from mddem_gb300 import capi

    cfgs, sts = _batch()
    ctx = capi.Context(cfgs[:1], [len(sts[0]["tag"])])
    ctx.upload(sts[0])
    ctx.step(2)
    with pytest.raises(capi.MdgError) as e:
        ctx.autotune(steps=10)
    assert e.value.status == 10  # MDG_ERR_STATE
