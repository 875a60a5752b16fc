"""Seeded initial conditions made on the device (mdg_generate_fcc,
mdg_generate_gas) against their CPU restatement (tests/gen_ref.py) and the
host generators:

* FCC: positions, types and masses equal inputs.lj_fcc (the fcc_insert
  restatement) bit for bit; velocities equal the restated counter stream after
  the mean is removed and T is fixed (to 1e-13 of sigma); zero momentum, T
  exact; at 256000 atoms the components pass a Kolmogorov-Smirnov test
  against N(0, sqrt(T/m));
* gas: centres and radii equal sequential RSA over the same proposal stream
  bit for bit (monodisperse and polydisperse, dilute and at solid fraction
  0.3, where batches need several settling sweeps); masses and inertias as
  insert.rs:343-349; velocities as restated;
* 10^6 polydisperse spheres at solid fraction 0.3 (the large polydisperse
  workload's placement): no pair closer than sep (r_i + r_j), uniform in
  space and radius, and the same nearest-neighbour statistics as the host
  RSA at 2 x 10^5 spheres;
* a generated system steps exactly like the same state uploaded from the host.
"""
import math
import time

import numpy as np
import pytest

import gen_ref
from helpers import by_tag

pytestmark = pytest.mark.gpu


def _lj_ctx(box, n, **kw):
    from mddem_gb300 import capi, config

    return capi.Context(config.lj_fluid_config(box=box, **kw), n)


def test_fcc_matches_fcc_insert(gpu_lib):
    ctx = _lj_ctx(10.06, 864)
    assert ctx.generate_fcc(0.85, 0.85, seed=5) == 864
    st = ctx.download()
    pos, vel, typ, mass, cut = by_tag(st, "pos", "vel", "type", "mass", "cutoff_radius")
    rp, rv, rt, rm = gen_ref.fcc(10.06, 0.85, 0.85, seed=5)
    assert np.array_equal(pos, rp)
    assert np.array_equal(typ, rt) and np.array_equal(mass, rm)
    assert np.all(cut == 1.25)
    sigma = math.sqrt(0.85)
    assert np.max(np.abs(vel - rv)) <= 1e-13 * sigma
    assert np.all(np.abs(vel.sum(axis=0)) <= 1e-12 * 864 * sigma)
    ke = 0.5 * float(np.sum(mass * np.sum(vel * vel, axis=1)))
    assert abs(2.0 * ke / (3 * 864 - 3) / 0.85 - 1.0) < 1e-13
    ctx.close()


def test_fcc_two_types(gpu_lib):
    from mddem_gb300 import capi
    from test_lj_types_cpu import two_type_config

    cfg = two_type_config()
    ctx = capi.Context(cfg, 864)
    ctx.generate_fcc(0.85, 0.85, seed=2, type_fractions=[0.5, 1.0], type_masses=[1.0, 1.5])
    st = ctx.download()
    pos, vel, typ, mass = by_tag(st, "pos", "vel", "type", "mass")
    rp, rv, rt, rm = gen_ref.fcc(10.06, 0.85, 0.85, seed=2, type_fractions=[0.5, 1.0], type_masses=[1.0, 1.5])
    assert np.array_equal(pos, rp) and np.array_equal(typ, rt) and np.array_equal(mass, rm)
    assert np.max(np.abs(vel - rv)) <= 1e-13
    ctx.close()


def test_fcc_256k_velocity_statistics(gpu_lib):
    stats = pytest.importorskip("scipy.stats")
    ctx = _lj_ctx(67.06, 256000, precision="mixed")
    t0 = time.perf_counter()
    n = ctx.generate_fcc(0.85, 0.85, seed=2024)
    setup = time.perf_counter() - t0
    assert n == 256000
    st = ctx.download()
    vel, mass = by_tag(st, "vel", "mass")
    _, rv, _, _ = gen_ref.fcc(67.06, 0.85, 0.85, seed=2024)
    assert np.max(np.abs(vel - rv)) <= 1e-12
    z = vel / math.sqrt(0.85)
    for d in range(3):
        assert stats.kstest(z[:, d], "norm").statistic < 1.95 / math.sqrt(n)
    print(f"fcc 256000 atoms generated on the device in {setup * 1e3:.1f} ms")
    ctx.close()


def test_generated_lattice_steps_like_its_upload(gpu_lib):
    for prec in ("fp64", "mixed"):
        a = _lj_ctx(10.06, 864, precision=prec)
        a.generate_fcc(0.85, 0.85, seed=9)
        b = _lj_ctx(10.06, 864, precision=prec)
        b.upload(a.download())
        a.step(50)
        b.step(50)
        sa, sb = a.download(), b.download()
        for f in ("pos", "vel"):
            assert np.array_equal(by_tag(sa, f)[0], by_tag(sb, f)[0]), (prec, f)
        a.close()
        b.close()


GAS_CASES = [
    # n, box, (rmin, rmax), sep, velocity mode
    (500, 0.025, (1e-3, 1e-3), 1.1, "speed"),            # the 500-sphere granular gas
    (1500, 0.035, (0.8e-3, 1.2e-3), 1.0, "maxwell_rms"),  # polydisperse, dilute
    (4000, 0.0382, (1e-3, 1e-3), 1.0, "gaussian"),       # solid fraction 0.3
]


@pytest.mark.parametrize("n,box,radius,sep,vmode", GAS_CASES)
def test_gas_matches_sequential_rsa(gpu_lib, n, box, radius, sep, vmode):
    from mddem_gb300 import capi, config, inputs

    cfg = config.granular_gas_config(box=box)
    ctx = capi.Context(cfg, n)
    assert ctx.generate_gas(n, radius, sep_factor=sep, velocity=vmode, speed=0.5, seed=17) == n
    st = ctx.download()
    pos, rad, vel, mass, inv_i, omg, quat, cut = by_tag(st, "pos", "radius", "vel", "mass", "inv_inertia", "omega",
                                                        "quat", "cutoff_radius")
    rp, rr = gen_ref.rsa(n, (0.0,) * 3, (box,) * 3, radius[0], radius[1], sep, True, seed=17)
    assert len(rp) == n
    assert np.array_equal(pos, rp) and np.array_equal(rad, rr)
    assert np.array_equal(cut, rr)
    assert np.array_equal(mass, inputs.sphere_mass(2500.0, rr))
    assert np.array_equal(inv_i, inputs.sphere_inv_inertia(mass, rr))
    assert not omg.any() and np.all(quat == [1.0, 0.0, 0.0, 0.0])
    rv = gen_ref.gas_velocities(n, vmode, 0.5, seed=17)
    assert np.max(np.abs(vel - rv)) <= 1e-14
    if vmode == "speed":
        assert np.allclose(np.linalg.norm(vel, axis=1), 0.5, rtol=1e-14, atol=0)
    ctx.close()


def _no_overlap(pos, rad, box, sep, spatial):
    tree = spatial.cKDTree(pos, boxsize=box)
    pairs = tree.query_pairs(sep * 2.0 * rad.max(), output_type="ndarray")
    d = pos[pairs[:, 1]] - pos[pairs[:, 0]]
    d -= box * np.rint(d / box)
    r = np.sqrt((d * d).sum(axis=1))
    return bool(np.all(r > sep * (rad[pairs[:, 0]] + rad[pairs[:, 1]])))


def _nn_mean(pos, box, spatial):
    tree = spatial.cKDTree(pos, boxsize=box)
    return float(tree.query(pos, k=2)[0][:, 1].mean())


def test_polydisperse_million_statistics(gpu_lib):
    spatial = pytest.importorskip("scipy.spatial")
    stats = pytest.importorskip("scipy.stats")
    from mddem_gb300 import capi, workloads

    cfg = workloads.polydisperse_config()
    L = cfg.box[0]
    n = 1_000_000
    ctx = capi.Context(cfg, n)
    t0 = time.perf_counter()
    ctx.generate_gas(n, workloads.POLY_R, sep_factor=1.0, velocity="maxwell_rms", speed=0.5, seed=2024)
    setup = time.perf_counter() - t0
    st = ctx.download()
    pos, rad, vel = by_tag(st, "pos", "radius", "vel")
    rmin, rmax = workloads.POLY_R
    assert pos.min() >= rmax and pos.max() <= L - rmax
    assert _no_overlap(pos, rad, L, 1.0, spatial)
    # uniform in space: 8 x 8 x 8 cells, chi-square at 1e-4
    h, _ = np.histogramdd(pos, bins=8, range=[(0, L)] * 3)
    chi2 = float(((h - n / 512) ** 2 / (n / 512)).sum())
    assert stats.chi2.sf(chi2, 511) > 1e-4, chi2
    # radius distribution uniform on [rmin, rmax]... of the accepted spheres:
    # RSA favours small spheres late, so only the range and a mild tilt are checked
    assert rad.min() >= rmin and rad.max() <= rmax
    assert abs(rad.mean() / (0.5 * (rmin + rmax)) - 1.0) < 0.05
    rms = float(np.sqrt(np.mean(np.sum(vel * vel, axis=1))))
    assert abs(rms / 0.5 - 1.0) < 0.01
    print(f"10^6 polydisperse spheres (solid fraction 0.30) placed on the device in {setup:.2f} s")
    ctx.close()


def test_device_and_host_rsa_statistics_agree(gpu_lib):
    spatial = pytest.importorskip("scipy.spatial")
    from mddem_gb300 import capi, workloads

    n = 200_000
    cfg = workloads.polydisperse_config(n=n)
    L = cfg.box[0]
    ctx = capi.Context(cfg, n)
    ctx.generate_gas(n, workloads.POLY_R, sep_factor=1.0, velocity="maxwell_rms", speed=0.5, seed=3)
    pd, rd = by_tag(ctx.download(), "pos", "radius")
    ph, rh = capi.rsa_spheres(n, (0.0,) * 3, (L,) * 3, *workloads.POLY_R, sep_factor=1.0, inset=True, seed=3)
    assert abs(_nn_mean(pd, L, spatial) / _nn_mean(ph, L, spatial) - 1.0) < 0.005
    assert abs(rd.mean() / rh.mean() - 1.0) < 0.005
    ctx.close()


def test_generators_refuse_bad_requests(gpu_lib):
    from mddem_gb300 import capi, config

    dem = capi.Context(config.granular_gas_config(box=0.01), 4000)
    with pytest.raises(capi.MdgError) as e:  # cannot fit: the proposal budget runs out
        dem.generate_gas(4000, 1e-3, max_proposals=200000)
    assert e.value.status == 9  # MDG_ERR_ARG
    with pytest.raises(capi.MdgError):  # a DEM system has no lattice
        dem.generate_fcc(0.85, 0.85)
    with pytest.raises(capi.MdgError):  # never armed: stepping is out of order
        dem.step(1)
    dem.close()
    lj = _lj_ctx(10.06, 100)
    with pytest.raises(capi.MdgError):  # 864 atoms do not fit 100 slots
        lj.generate_fcc(0.85, 0.85)
    with pytest.raises(capi.MdgError):
        lj.generate_gas(10, 1e-3)
    lj.close()
