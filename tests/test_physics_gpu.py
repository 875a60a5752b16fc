"""Conserved and statistical quantities, GPU paths against the oracle and the
reference's own validation bounds.

* LJ NVE energy (864 atoms, rc 2.5 unshifted, 2000 steps): the plain FP64
  path's energy history matches the oracle's (1e-6 of the drift), and the
  mixed path's linear energy drift is within 2x the oracle's.
* LJ NH melt (864 atoms, T* = rho* = 0.85, mixed): g(r) first peak at
  0.95-1.15 sigma with height 2.4-3.5 and g -> 1 (0.7-1.3) at 2-2.8 sigma,
  the bounds of examples/lj_argon/validate.py:66-110; D* from the MSD slope
  over 20 tau in [0.030, 0.050] (the reference quotes 0.041 over 100k steps;
  wider here for 864 atoms and a short run).
* Haff cooling (2000 frictionless spheres, solid fraction 0.2, e = 0.8,
  40000 steps): T(t) = T0 / (1 + t/t_c)^2 fitted on 1/sqrt(T); t_c of both
  GPU paths within 2 % of the oracle's and within 15 % of the kinetic-theory
  value of examples/granular_gas_benchmark/haff_analysis.py:82-104.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lj_energy(backend, prec, steps=2000, every=50):
    from mddem_gb300 import capi, config, inputs, validate

    cfg = config.lj_fluid_config(nose_hoover=False, precision=prec)
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=3)
    if backend == "oracle":
        from oracle.oracle import Oracle

        o = Oracle(cfg.replace(precision="fp64"))
        o.load(st)
    else:
        o = capi.Context(cfg, len(st["tag"]))
        o.upload(st)
    return validate.energy_drift(o, steps, every)


def test_lj_energy_drift(gpu_lib):
    Eo, so = _lj_energy("oracle", "fp64")
    Ef, sf = _lj_energy("gpu", "fp64")
    Em, sm = _lj_energy("gpu", "mixed")
    dev_o = np.max(np.abs(Eo - Eo[0]))
    assert np.max(np.abs(Ef - Eo)) <= 1e-6 * dev_o
    assert abs(sm) <= 2.0 * abs(so)


def test_lj_structure_and_diffusion(gpu_lib):
    from mddem_gb300 import capi, config, inputs

    cfg = config.lj_fluid_config(precision="mixed")
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=4)
    c = capi.Context(cfg, 864)
    c.upload(st)
    c.step(4000)
    c.msd_reset()
    gs = []
    for k in range(40):
        c.step(100)
        gs.append(c.rdf(r_max=3.0, nbins=200)[1])
        if k == 9:
            m1 = c.msd()
    m2 = c.msd()
    r = (np.arange(200) + 0.5) * 0.015
    g = np.mean(gs, axis=0)
    sel = (r > 0.8) & (r < 1.5)
    assert 0.95 <= r[sel][np.argmax(g[sel])] <= 1.15
    assert 2.4 <= g[sel].max() <= 3.5
    assert 0.7 <= g[(r > 2.0) & (r < 2.8)].mean() <= 1.3
    d = (m2 - m1) / (6.0 * 3000 * 0.005)
    assert 0.030 <= d <= 0.050, d


def _haff(backend, prec, n=2000, phi=0.2, e=0.8, steps=40000, every=2000):
    from mddem_gb300 import capi, validate, workloads

    cfg, st = workloads.gas(n, phi=phi, restitution=e, friction=0.0, seed=11, precision=prec)
    if backend == "oracle":
        from oracle.oracle import Oracle

        o = Oracle(cfg.replace(precision="fp64", rebuild_policy="reference"))
        o.load(st)
    else:
        o = capi.Context(cfg, n)
        o.upload(st)
    return validate.haff(o, cfg, n, e, steps=steps, every=every)


def test_haff_cooling(gpu_lib):
    tco, theory, ro = _haff("oracle", "fp64")
    for prec in ("fp64", "mixed"):
        tc, _, rg = _haff("gpu", prec)
        assert abs(tc / tco - 1.0) <= 0.02, (prec, tc, tco)
        assert abs(rg / ro - 1.0) <= 0.02, (prec, rg, ro)
    assert abs(tco / theory - 1.0) <= 0.15, (tco, theory)
    assert ro < 0.6  # it cooled: about a 1/(1 + t/t_c)^2 drop to ~0.48
