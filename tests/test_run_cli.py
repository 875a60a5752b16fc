"""The TOML runner (python -m mddem_gb300.run): reference-format configs
(the sections of examples/lj_argon/config.toml and
examples/granular_gas_benchmark/run_debug.toml) give the same initial state
as the generators, and a GPU run prints thermo lines and writes restart and
measurement files."""
import io
import math

import numpy as np
import pytest

LJ = """
[domain]
x_low = 0.0
x_high = 10.06
y_low = 0.0
y_high = 10.06
z_low = 0.0
z_high = 10.06
boundary_x = "periodic"
boundary_y = "periodic"
boundary_z = "periodic"
[neighbor]
skin_fraction = 1.12
bin_size = 1.0
[lattice]
style = "fcc"
density = 0.85
temperature = 0.85
mass = 1.0
skin = 1.25
[lj]
epsilon = 1.0
sigma = 1.0
cutoff = 2.5
[thermostat]
temperature = 0.85
coupling = 1.0
[run]
steps = 300
thermo = 100
[measure]
rdf_bins = 100
rdf_cutoff = 3.0
rdf_interval = 100
msd_interval = 50
"""

DEM = """
[comm]
processors_x = 1
[neighbor]
skin_fraction = 1.1
bin_size = 0.005
every = 1
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
[[dem.materials]]
name = "glass"
youngs_mod = 8.7e9
poisson_ratio = 0.3
restitution = 0.95
friction = 0.4
[[particles.insert]]
material = "glass"
count = 500
radius = 0.001
density = 2500.0
velocity = 0.5
[run]
thermo = 200
steps = 400
[restart]
interval = 200
format = "bincode"
"""


def test_setup_lj_matches_generator():
    from mddem_gb300 import inputs, run

    cfg, st, s = run.setup(LJ, seed=5)
    ref = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=5)
    assert cfg.kind == "lj" and cfg.nose_hoover and cfg.dt == 0.005 and cfg.skin_fraction == 1.12
    assert np.array_equal(st["pos"], ref["pos"]) and np.array_equal(st["vel"], ref["vel"])
    assert s["steps"] == 300 and s["thermo"] == 100 and s["measure"]["rdf_bins"] == 100


def test_setup_dem_insertion_rules():
    from mddem_gb300 import config, run

    cfg, st, s = run.setup(DEM, seed=2)
    n = len(st["tag"])
    assert cfg.kind == "dem" and n == 500 and cfg.every == 1
    r = st["radius"]
    assert np.all(r == 0.001)
    assert st["pos"].min() >= 0.001 and st["pos"].max() <= 0.025 - 0.001  # region inset by r
    d = st["pos"][:, None, :] - st["pos"][None, :, :]
    d -= 0.025 * np.round(d / 0.025)
    dist = np.sqrt((d * d).sum(-1)) + np.eye(n)
    assert dist.min() > 1.1 * 0.002
    # per-component Gaussian velocities of std 0.5 (insert.rs:591-597)
    assert abs(st["vel"].std() - 0.5) < 0.05
    assert math.isclose(cfg.dt, config.rayleigh_dt(0.001, 2500.0, 8.7e9, 0.3))


@pytest.mark.gpu
def test_runner_runs_both_kinds(gpu_lib, tmp_path):
    from mddem_gb300 import restart, run

    out = io.StringIO()
    lj = LJ + f'\n[output]\ndir = "{tmp_path / "lj"}"\n'
    run.run(lj, out=out)
    lines = [x for x in out.getvalue().splitlines() if not x.startswith("#")]
    assert len(lines) == 4  # steps 0, 100, 200, 300
    assert 0.5 < float(lines[-1].split()[2]) < 1.2  # thermostatted T
    g = np.loadtxt(tmp_path / "lj" / "rdf.txt")
    assert 2.0 < g[:, 1].max() < 4.0
    assert (tmp_path / "lj" / "msd.txt").exists()
    out = io.StringIO()
    dem = DEM + f'\n[output]\ndir = "{tmp_path / "dem"}"\n'
    run.run(dem, out=out, precision="mixed")
    # the reference's restart directory: <output dir>/restart
    st, hist, step, dt = restart.read_restart(tmp_path / "dem" / "restart" / "restart_400_rank0.bin")
    assert step == 400 and len(st["tag"]) == 500
    assert (tmp_path / "dem" / "restart" / "restart_200_rank0.bin").exists()
    # [restart] read = true resumes from the latest file and numbers on from it
    out = io.StringIO()
    run.run(dem.replace('format = "bincode"', 'format = "bincode"\nread = true'), out=out, precision="mixed")
    lines = [x for x in out.getvalue().splitlines() if not x.startswith("#")]
    assert [int(x.split()[0]) for x in lines] == [400, 600, 800]
    assert "Restart: reading from" in out.getvalue()
    st2, _, step2, _ = restart.read_restart(tmp_path / "dem" / "restart" / "restart_800_rank0.bin")
    assert step2 == 800 and len(st2["tag"]) == 500


def test_latest_restart_picks_the_highest_step(tmp_path):
    from mddem_gb300 import run

    for name in ("restart_200_rank0.bin", "restart_1000_rank0.bin", "restart_900_rank0.bin",
                 "restart_5000_rank1.bin", "restart_7000_rank0.json", "notes.txt"):
        (tmp_path / name).write_bytes(b"")
    assert run.latest_restart(tmp_path).endswith("restart_1000_rank0.bin")
    assert run.latest_restart(tmp_path, "json").endswith("restart_7000_rank0.json")
    assert run.latest_restart(tmp_path, rank=1).endswith("restart_5000_rank1.bin")
    assert run.latest_restart(tmp_path / "missing") is None


def test_restart_section_rejects_unknown_keys():
    from mddem_gb300 import run

    with pytest.raises(run.RunError, match="unknown key"):
        run.setup(DEM.replace("[restart]\n", "[restart]\nevery = 3\n"))
