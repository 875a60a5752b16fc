"""CPU checks of the drop-in boundary: the library builds and exports every
entry point include/mdg.h declares; configuration parsing follows the
reference's TOML sections (unknown keys rejected like deny_unknown_fields)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from mddem_gb300 import build, capi

    build.build()
    return capi.load()


def header_symbols():
    with open(os.path.join(ROOT, "include", "mdg.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mdg_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_expected_entry_points():
    from mddem_gb300 import capi

    syms = header_symbols()
    assert syms == sorted(capi.EXPORTS)


def test_library_exports_every_header_symbol(lib):
    for s in header_symbols():
        assert hasattr(lib, s), s


def test_status_strings(lib):
    assert lib.mdg_status_string(0) == b"ok"
    assert b"overlap" in lib.mdg_status_string(5)
    assert lib.mdg_abi_version() == 1


def test_create_without_device_reports_nodevice(lib):
    from mddem_gb300 import capi, config

    n = ctypes.c_int(-1)
    if lib.mdg_device_count(ctypes.byref(n)) == 0 and n.value > 0:
        pytest.skip("a CUDA device is present")
    with pytest.raises(capi.MdgError) as e:
        capi.Context(config.lj_fluid_config(), 10)
    assert e.value.status == 11


def test_invalid_config_rejected_before_device(lib):
    from mddem_gb300 import capi, config

    bad = config.lj_fluid_config().replace(dt=-1.0)
    with pytest.raises(capi.MdgError) as e:
        capi.Context(bad, 10)
    assert e.value.status == 1


def test_lj_pair_table_validated_before_device(lib):
    """mdg_create checks the multi-type table before it looks for a device: an
    asymmetric table, a non-positive sigma or cutoff, or a missing table is
    MDG_ERR_CONFIG (1); a valid one gets as far as the device check."""
    from mddem_gb300 import capi, config

    n = ctypes.c_int(-1)
    if lib.mdg_device_count(ctypes.byref(n)) == 0 and n.value > 0:
        pytest.skip("a CUDA device is present")
    good = config.lj_pair_table([(1.0, 1.0), (0.5, 0.88)], 2.5)
    base = config.lj_fluid_config().replace(lj_types=2, lj_pairs=good)
    with pytest.raises(capi.MdgError) as e:
        capi.Context(base, 10)
    assert e.value.status == 11  # valid: MDG_ERR_NODEVICE here
    asym = list(good)
    asym[1] = (0.7, 0.94, 2.5)
    bad_sigma = list(good)
    bad_sigma[3] = (0.5, 0.0, 2.5)
    bad_cut = list(good)
    bad_cut[0] = (1.0, 1.0, -1.0)
    for table in (tuple(asym), tuple(bad_sigma), tuple(bad_cut)):
        with pytest.raises(capi.MdgError) as e:
            capi.Context(base.replace(lj_pairs=table), 10)
        assert e.value.status == 1
    cc, keep = capi.to_c_config(base)
    cc.lj_pairs = ctypes.cast(None, ctypes.POINTER(capi.LJPair))
    h = ctypes.c_void_p()
    assert lib.mdg_create(ctypes.byref(cc), 10, ctypes.byref(h)) == 1


REF_DEM_TOML = """
[domain]
x_low = 0.0
x_high = 0.025
y_low = 0.0
y_high = 0.025
z_low = 0.0
z_high = 0.025
boundary_x = "periodic"
boundary_y = "periodic"
boundary_z = "periodic"

[neighbor]
skin_fraction = 1.1
bin_size = 0.005

[run]
dt = 2.934e-7

[[dem.materials]]
name = "glass"
youngs_mod = 8.7e9
poisson_ratio = 0.3
restitution = 0.95
friction = 0.4
"""

REF_LJ_TOML = """
[domain]
x_high = 10.06
y_high = 10.06
z_high = 10.06

[neighbor]
skin_fraction = 1.12
bin_size = 1.0

[lj]
epsilon = 1.0
sigma = 1.0
cutoff = 2.5

[lattice]
density = 0.85

[thermostat]
temperature = 0.85
coupling = 1.0

[gpu]
precision = "mixed"
"""


def test_toml_dem_sections():
    from mddem_gb300 import from_toml

    c = from_toml(REF_DEM_TOML)
    assert c.kind == "dem" and c.box == pytest.approx((0.025, 0.025, 0.025))
    assert c.skin_fraction == 1.1 and c.bin_size == 0.005 and c.dt == 2.934e-7
    assert c.every == 0 and c.check and c.sort_every == 1000 and c.newton  # reference defaults
    m = c.materials[0]
    assert (m.youngs_mod, m.poisson_ratio, m.restitution, m.friction) == (8.7e9, 0.3, 0.95, 0.4)
    assert m.rolling_friction == 0.0 and c.contact_model == "hertz"


def test_toml_lj_sections():
    from mddem_gb300 import from_toml

    c = from_toml(REF_LJ_TOML)
    assert c.kind == "lj" and c.dt == 0.005  # lattice_set_dt
    assert c.nose_hoover and c.nh_temperature == 0.85 and c.precision == "mixed"


def test_toml_unknown_field_rejected():
    from mddem_gb300 import ConfigError, from_toml

    with pytest.raises(ConfigError):
        from_toml(REF_DEM_TOML.replace("bin_size = 0.005", "bin_size = 0.005\nbogus = 1"))
    with pytest.raises(ConfigError):
        from_toml(REF_DEM_TOML.replace('boundary_x = "periodic"', 'boundary_x = "shrink_wrap"'))
    assert from_toml(REF_DEM_TOML.replace('boundary_x = "periodic"', 'boundary_x = "fixed"')).fixed == (1, 0, 0)


def test_rayleigh_dt_matches_reference_formula():
    from mddem_gb300 import config

    dt = config.rayleigh_dt(1e-3, 2500.0, 8.7e9, 0.3, fraction=0.1)
    assert dt == pytest.approx(2.934e-7, rel=1e-3)


def test_generators_are_seeded_and_non_overlapping():
    from mddem_gb300 import inputs

    a = inputs.dem_granular_gas(200, seed=3)
    b = inputs.dem_granular_gas(200, seed=3)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])
    p = a["pos"]
    d = p[:, None, :] - p[None, :, :]
    d -= 0.025 * np.round(d / 0.025)
    r = np.sqrt((d ** 2).sum(-1)) + np.eye(len(p))
    assert r.min() > 1.1 * 2e-3
    assert np.allclose(np.linalg.norm(a["vel"], axis=1), 0.5)
    lj = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=1)
    assert len(lj["tag"]) == 864
    v = lj["vel"]
    assert np.allclose(v.sum(axis=0), 0.0, atol=1e-12)
    assert 0.5 * (v ** 2).sum() * 2 / (3 * 864 - 3) == pytest.approx(0.85, rel=1e-12)


def test_csv_roundtrip(tmp_path):
    from mddem_gb300 import inputs

    a = inputs.dem_granular_gas(50, seed=1)
    p = tmp_path / "p.csv"
    inputs.write_csv(p, a)
    b = inputs.read_csv(p)
    for k in ("pos", "vel", "radius", "mass", "inv_inertia"):
        assert np.array_equal(a[k], b[k]), k


def test_rsa_spheres_seeded_and_non_overlapping(lib):
    """mdg_rsa_spheres: same seed, same spheres; every pair under the minimum
    image keeps sep_factor * (r_i + r_j); radii within [rmin, rmax]; centres
    inset by rmax."""
    from mddem_gb300 import capi

    L = 0.03
    a = capi.rsa_spheres(1500, (0, 0, 0), (L, L, L), 0.8e-3, 1.2e-3, sep_factor=1.1, seed=7)
    b = capi.rsa_spheres(1500, (0, 0, 0), (L, L, L), 0.8e-3, 1.2e-3, sep_factor=1.1, seed=7)
    c = capi.rsa_spheres(1500, (0, 0, 0), (L, L, L), 0.8e-3, 1.2e-3, sep_factor=1.1, seed=8)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.array_equal(a[0], c[0])
    pos, rad = a
    assert rad.min() >= 0.8e-3 and rad.max() <= 1.2e-3
    assert pos.min() >= 1.2e-3 and pos.max() <= L - 1.2e-3
    d = pos[:, None, :] - pos[None, :, :]
    d -= L * np.round(d / L)
    r = np.sqrt(np.einsum("ijk,ijk->ij", d, d))
    np.fill_diagonal(r, np.inf)
    assert np.all(r > 1.1 * (rad[:, None] + rad[None, :]))


def test_rsa_spheres_reports_unplaceable(lib):
    from mddem_gb300 import capi

    with pytest.raises(capi.MdgError):  # solid fraction far above the RSA limit
        capi.rsa_spheres(5000, (0, 0, 0), (0.02, 0.02, 0.02), 1e-3, 1e-3, sep_factor=1.0, seed=1,
                         max_attempts=200000)


def test_toml_langevin_section():
    from mddem_gb300 import config

    txt = """
[domain]
x_high = 10.06
y_high = 10.06
z_high = 10.06
[lattice]
density = 0.85
[langevin]
temperature = 1.1
damping = 0.5
seed = 9
"""
    c = config.from_toml(txt)
    assert c.langevin and c.lv_temperature == 1.1 and c.lv_damping == 0.5 and c.lv_seed == 9
    with pytest.raises(config.ConfigError):
        config.from_toml(txt.replace("seed = 9", "seed = 9\nfriction = 1.0"))


def test_grouped_server_refuses_a_group_of_two_kinds(lib):
    """A slot group shares one batch context, so it must hold one particle
    kind; the check runs before any device work."""
    from mddem_gb300 import capi, config

    with pytest.raises(capi.MdgError) as e:
        capi.Server([config.granular_gas_config(), config.lj_fluid_config()], [100, 100], 1 << 30, groups=[0, 0])
    assert e.value.status == 1  # MDG_ERR_CONFIG
