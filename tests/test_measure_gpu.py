"""Measurement kernels (md_measure/src/lib.rs) on the GPU.

* RDF pair counts equal a numpy restatement of the reference's single-rank
  loop (lib.rs:379-400: i < j, minimum image by one conditional shift,
  r^2 = dx dx + dy dy + dz dz, bin = sqrt(r^2) / dr truncated) on the same
  positions -- exact integer counts;
* g(r) of an ideal gas is 1 within its counting noise;
* MSD (x + image L against the positions at reset) and the rotational
  temperature and pressure of mdg_thermo match host formulas (1e-12).
"""
import numpy as np
import pytest

from helpers import by_tag, overlapping_spheres

pytestmark = pytest.mark.gpu


def _rdf_counts_ref(pos, L, r_max, nbins):
    n = len(pos)
    i, j = np.triu_indices(n, 1)
    out = np.zeros(nbins, np.int64)
    dr = r_max / nbins
    cut2 = r_max * r_max
    d = [pos[j, a] - pos[i, a] for a in range(3)]
    for a in range(3):
        h = L[a] * 0.5
        d[a] = np.where(d[a] > h, d[a] - L[a], np.where(d[a] < -h, d[a] + L[a], d[a]))
    r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2]
    m = (r2 < cut2) & (r2 >= 1e-20)
    b = (np.sqrt(r2[m]) / dr).astype(np.int64)
    b = b[b < nbins]
    np.add.at(out, b, 1)
    return out


def test_rdf_counts_equal_reference_loop(gpu_lib):
    from mddem_gb300 import capi, config, inputs

    cfg = config.lj_fluid_config()
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=5)
    st["pos"] = st["pos"] + np.random.default_rng(0).normal(scale=0.05, size=st["pos"].shape)
    ctx = capi.Context(cfg, len(st["tag"]))
    ctx.upload(st)
    (pos,) = by_tag(ctx.download(), "pos")
    for r_max, nbins in ((3.0, 200), (4.9, 37)):
        _, _, counts = ctx.rdf(r_max=r_max, nbins=nbins)
        ref = _rdf_counts_ref(pos, [10.06] * 3, r_max, nbins)
        assert np.array_equal(counts.astype(np.int64), ref), (r_max, nbins)
        assert counts.sum() > 0


def test_rdf_ideal_gas_is_one(gpu_lib):
    from mddem_gb300 import capi, config

    n, L = 6000, 20.0
    rng = np.random.default_rng(7)
    st = {"tag": np.arange(n, dtype=np.uint32), "type": np.zeros(n, np.uint32), "pos": rng.uniform(0, L, (n, 3)),
          "vel": np.zeros((n, 3)), "mass": np.ones(n), "cutoff_radius": np.full(n, 1.25)}
    cfg = config.lj_fluid_config(box=L, nose_hoover=False)
    ctx = capi.Context(cfg, n)
    ctx.upload(st)
    r, g, counts = ctx.rdf(r_max=3.0, nbins=30)
    sel = r >= 1.0
    expected = counts[sel] / g[sel]  # ideal counts per bin
    assert np.all(np.abs(g[sel] - 1.0) <= 5.0 / np.sqrt(expected))
    assert abs(np.mean(g[sel]) - 1.0) < 0.02


def test_msd_rot_temp_pressure(gpu_lib):
    from mddem_gb300 import capi, config, inputs

    # MSD on an LJ melt (particles cross the box and carry image flags)
    cfg = config.lj_fluid_config(virial=True)
    st = inputs.lj_fcc(6, 10.06, 0.85, 1.2, seed=9)
    ctx = capi.Context(cfg, len(st["tag"]))
    ctx.upload(st)
    ctx.step(5)
    ctx.msd_reset()
    assert ctx.msd() == 0.0
    p0, i0 = by_tag(ctx.download(), "pos", "image")
    ctx.step(200)
    p1, i1 = by_tag(ctx.download(), "pos", "image")
    u0 = p0 + i0 * 10.06
    u1 = p1 + i1 * 10.06
    ref = float(np.mean(np.sum((u1 - u0) ** 2, axis=1)))
    assert np.any(i1 != i0)
    assert abs(ctx.msd() - ref) <= 1e-12 * max(ref, 1e-300) + 1e-15
    # pressure: rho T - tr(W) / 3V + P_tail
    t = ctx.thermo()
    v = 10.06 ** 3
    pref = len(st["tag"]) / v * t["temp"] - sum(t["virial"][:3]) / (3 * v) + t["p_tail"]
    assert abs(t["pressure"] - pref) <= 1e-12 * abs(pref)
    # rotational temperature of spinning spheres
    dcfg = config.granular_gas_config(box=0.012, dt=1e-7)
    ds = overlapping_spheres(400, 0.012, 5e-4, seed=2)
    dc = capi.Context(dcfg, 400)
    dc.upload(ds)
    dc.step(3)
    g = dc.download()
    m, r, w = g["mass"], g["radius"], g["omega"]
    trot = np.sum(0.4 * m * r * r * np.sum(w * w, axis=1)) / (3 * np.sum(m))
    assert abs(dc.thermo()["rot_temp"] - trot) <= 1e-12 * trot
