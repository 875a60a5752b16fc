"""The C++ host above the C ABI (mddem_gb300/csrc/host: TOML reader, App and
plugins, `mdg_run`) on CPU: `mdg_run --check` resolves the reference's TOML
sections into the same device configuration as the Python binding
(config.from_toml + capi.to_c_config) and the same initial state as the
Python runner's setup (positions from the seeded insertion / FCC lattice), and
a configuration error exits with status 1 and a message, like the
reference."""
import json
import math
import os
import subprocess

import numpy as np
import pytest

from test_lj_types_cpu import LJ_TYPES_TOML

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

GAS = """
[domain]
x_high = 0.025
y_high = 0.025
z_high = 0.025

[neighbor]
skin_fraction = 1.1
bin_size = 0.005

[run]
dt = 2.934e-7
steps = 500
thermo = 100

[dem]
contact_model = "hertz"
rolling_model = "sds"

[[dem.materials]]
name = "glass"
youngs_mod = 8.7e9
poisson_ratio = 0.3
restitution = 0.95
friction = 0.4
rolling_friction = 0.02

[[dem.materials]]
name = "steel"
youngs_mod = 2.0e11
poisson_ratio = 0.3
restitution = 0.8
friction = 0.3

[[particles.insert]]
material = "glass"
count = 300
radius = 0.001
density = 2500.0
velocity = 0.3

[[particles.insert]]
material = "steel"
count = 100
radius = { distribution = "uniform", min = 0.0008, max = 0.0012 }
density = 7800.0

[gpu]
precision = "mixed"
rebuild_policy = "displacement"
history_capacity = 16
"""

REBOUND = """
[domain]
x_low = -0.01
x_high = 0.01
y_low = -0.01
y_high = 0.01
z_low = 0.0
z_high = 0.1
boundary_x = "fixed"
boundary_y = "fixed"
boundary_z = "fixed"

[neighbor]
skin_fraction = 1.1
bin_size = 0.015
every = 1

[[dem.materials]]
name = "glass"
youngs_mod = 70.0e9
poisson_ratio = 0.22
restitution = 0.9
friction = 0.0

[[particles.insert]]
material = "glass"
count = 1
radius = 0.005
density = 2500.0
velocity_z = -1.0
region = { type = "block", min = [-0.001, -0.001, 0.007], max = [0.001, 0.001, 0.008] }

[[wall]]
point_z = 0.0
normal_z = 1.0
material = "glass"

[[wall]]
point_z = 0.1
normal_z = -1.0
bound_x_low = -0.005
velocity = [0.0, 0.0, -0.5]
material = "glass"

[run]
steps = 20000
"""

LJ = """
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
temperature = 1.1

[thermostat]
temperature = 0.85
coupling = 1.0

[gpu]
precision = "mixed"
virial = true
"""

LANGEVIN = LJ.replace("""[thermostat]
temperature = 0.85
coupling = 1.0
""", """[langevin]
temperature = 1.2
damping = 0.5
seed = 99
""")


@pytest.fixture(scope="module")
def runner():
    from mddem_gb300 import build

    build.build()
    return os.path.join(ROOT, "mddem_gb300", "_lib", "mdg_run")


def _run(runner, tmp_path, text, *args):
    p = tmp_path / "config.toml"
    p.write_text(text)
    return subprocess.run([runner, str(p), *args], capture_output=True, text=True, timeout=120)


def _num(x):
    return {"inf": math.inf, "-inf": -math.inf}.get(x, x) if isinstance(x, str) else x


@pytest.mark.parametrize("text", [GAS, REBOUND, LJ, LANGEVIN, LJ_TYPES_TOML],
                         ids=["gas", "rebound", "lj", "langevin", "lj_types"])
def test_check_matches_python_binding(runner, tmp_path, text):
    from mddem_gb300 import capi, run

    r = _run(runner, tmp_path, text, "--check")
    assert r.returncode == 0, r.stderr
    got = json.loads(r.stdout)
    cfg, st, s = run.setup(text, seed=0)
    cc, _keep = capi.to_c_config(cfg)
    for f in ("kind", "precision", "every", "check", "sort_every", "newton", "n_materials", "contact_model",
              "adhesion_model", "rolling_model", "twisting_model", "nose_hoover", "virial", "rebuild_policy",
              "threads_per_particle", "neighbor_capacity", "history_capacity", "langevin", "lv_seed"):
        assert got[f] == getattr(cc, f), f
    for f in ("dt", "skin_fraction", "bin_size", "lj_epsilon", "lj_sigma", "lj_cutoff", "nh_temperature",
              "nh_coupling", "lv_temperature", "lv_damping"):
        assert got[f] == getattr(cc, f), f
    assert got["box_lo"] == list(cc.box_lo) and got["box_hi"] == list(cc.box_hi)
    assert got["fixed"] == list(cc.fixed)
    for k in range(cc.n_materials):
        want = [getattr(cc.materials[k], f) for f, _ in capi.Material._fields_]
        assert got["materials"][k] == want
    assert len(got["walls"]) == cc.n_walls
    for k, w in enumerate(got["walls"]):
        for f in ("point", "normal", "bound_lo", "bound_hi", "velocity"):
            assert [_num(x) for x in w[f]] == list(getattr(cc.walls[k], f)), f
        assert w["material"] == cc.walls[k].material
    assert got["n_lj_types"] == cc.n_lj_types
    assert got["lj_pairs"] == [[cc.lj_pairs[k].epsilon, cc.lj_pairs[k].sigma, cc.lj_pairs[k].cutoff]
                               for k in range(cc.n_lj_types ** 2 if cc.n_lj_types > 1 else 0)]
    assert got["type_sum"] == int(np.sum(st["type"]))
    assert got["steps"] == s["steps"] and got["thermo"] == s["thermo"]
    # the initial state: same particles at the same places (velocities come
    # from each host's own seeded generator)
    assert got["n"] == len(st["tag"])
    assert np.allclose(got["pos_sum"], np.sum(st["pos"], axis=0), rtol=1e-12, atol=0)
    assert got["mass_sum"] == pytest.approx(float(np.sum(st["mass"])), rel=1e-12)
    if "radius" in st:
        assert got["radius_sum"] == pytest.approx(float(np.sum(st["radius"])), rel=1e-12)


@pytest.mark.parametrize("edit,msg", [
    (("bin_size = 0.005", "bin_size = 0.005\nbogus = 1"), "unknown field"),
    (("[gpu]", "[gpu]\nwarp = 2"), "unknown field"),
    (('rolling_model = "sds"', 'rolling_model = "spring"'), "rolling_model"),
    (('name = "steel"', 'name = "brass"'), "not in [[dem.materials]]"),
    (("count = 300", "count = 300\nrate = 1.0"), "rate-based"),
    (("[domain]", '[domain]\nboundary_y = "shrink_wrap"'), "boundary_y"),
])
def test_config_errors_exit_1(runner, tmp_path, edit, msg):
    r = _run(runner, tmp_path, GAS.replace(*edit), "--check")
    assert r.returncode == 1
    assert msg in r.stderr


def test_toml_syntax_error_names_the_line(runner, tmp_path):
    r = _run(runner, tmp_path, GAS.replace("[neighbor]", "[neighbor"), "--check")
    assert r.returncode == 1 and "line" in r.stderr


def test_cli_overrides(runner, tmp_path):
    r = _run(runner, tmp_path, LJ, "--check", "--steps", "77", "--precision", "fp64")
    got = json.loads(r.stdout)
    assert got["steps"] == 77 and got["precision"] == 0
    assert _run(runner, tmp_path, LJ, "--precision", "half").returncode == 1


def test_run_without_a_device_reports_it(runner, tmp_path):
    from mddem_gb300 import capi

    n = capi.load()
    import ctypes

    c = ctypes.c_int(0)
    n.mdg_device_count(ctypes.byref(c))
    if c.value > 0:
        pytest.skip("a CUDA device is present")
    r = _run(runner, tmp_path, LJ)
    assert r.returncode == 1 and "no CUDA device" in r.stderr


TOML_FORMS = """
# comments, literal and escaped strings, dotted keys, inline tables and
# arrays across lines, integers with separators, exponents
dem.contact_model = "hooke"

[domain]
x_low = -0.01   # trailing comment
x_high = +0.01
y_low = -1e-2
y_high = 1E-2
z_low = 0
z_high = 0.1
boundary_x = 'fixed'
"boundary_y" = "fixed"
boundary_z = "f\\u0069xed"

[neighbor]
skin_fraction = 1.1
bin_size = 0.015
every = 1_0
sort_every = 1_000

[[dem.materials]]
name = 'gl"ass'
youngs_mod = 70_000_000_000.0
poisson_ratio = 0.22
restitution = 0.9
friction = 0.0
kn = 2e5
kt = 5e4

[[particles.insert]]
material = 'gl"ass'
count = 3
radius = 0.002
density = 2500
region = { type = "block", min = [-0.005, -0.005, 0.01], max = [
    0.005,
    0.005,  # still the same array
    0.02,
] }

[[wall]]
normal_z = 1
velocity = [ 0.0, 0.0,
             0.25 ]
material = 'gl"ass'
"""


def test_toml_forms_read_like_tomllib(runner, tmp_path):
    from mddem_gb300 import capi, run

    r = _run(runner, tmp_path, TOML_FORMS, "--check")
    assert r.returncode == 0, r.stderr
    got = json.loads(r.stdout)
    cfg, st, s = run.setup(TOML_FORMS, seed=0)
    cc, _keep = capi.to_c_config(cfg)
    assert got["box_lo"] == list(cc.box_lo) and got["box_hi"] == list(cc.box_hi)
    assert got["fixed"] == [1, 1, 1] == list(cc.fixed)
    assert got["every"] == 10 and got["sort_every"] == 1000
    assert got["contact_model"] == 1 == cc.contact_model
    assert got["materials"][0] == [getattr(cc.materials[0], f) for f, _ in capi.Material._fields_]
    assert [_num(x) for x in got["walls"][0]["velocity"]] == [0.0, 0.0, 0.25]
    assert got["n"] == 3 and np.allclose(got["pos_sum"], np.sum(st["pos"], axis=0), rtol=1e-12, atol=0)


@pytest.mark.parametrize("bad", [
    "[domain]\nx_low = 1\nx_low = 2\n",          # duplicate key
    "[domain]\nx_low = \"open\n",                 # unterminated string
    "[domain]\nx_low = [1, 2\n",                  # unterminated array
    "[domain]\nx_low = 1 2\n",                    # junk after a value
    "[domain]\nx_low = \"\\q\"\n",                # bad escape
])
def test_toml_errors(runner, tmp_path, bad):
    r = _run(runner, tmp_path, bad + "[lj]\n[lattice]\n", "--check")
    assert r.returncode == 1 and "line" in r.stderr


@pytest.mark.parametrize("text", [GAS, LJ], ids=["gas", "lj"])
def test_restart_file_from_the_cpp_host(runner, tmp_path, text):
    """`mdg_run --check --write-restart` writes the initial state in the
    reference's bincode RestartData: the Python reader gets back the Python
    runner's particles, and the Python writer re-encodes it to the same bytes."""
    from mddem_gb300 import restart, run

    path = tmp_path / "restart_0_rank0.bin"
    r = _run(runner, tmp_path, text, "--check", "--write-restart", str(path))
    assert r.returncode == 0, r.stderr
    st, hist, step, dt = restart.read_restart(path)
    cfg, ref, _ = run.setup(text, seed=0)
    assert step == 0 and dt == cfg.dt
    assert np.array_equal(st["tag"], ref["tag"]) and np.array_equal(st["type"], ref["type"])
    assert np.array_equal(st["pos"], ref["pos"])
    assert np.array_equal(st["mass"], ref["mass"]) and np.array_equal(st["cutoff_radius"], ref["cutoff_radius"])
    if cfg.kind == "dem":
        assert np.array_equal(st["radius"], ref["radius"]) and np.array_equal(st["density"], ref["density"])
        assert np.array_equal(st["inv_inertia"], ref["inv_inertia"])
        assert hist is not None and len(hist[0]) == 0
    again = tmp_path / "again.bin"
    restart.write_restart(again, st, hist, step=step, dt=dt)
    assert again.read_bytes() == path.read_bytes()
    # the JSON form of the same state reads back to the same values
    jpath = tmp_path / "restart_0_rank0.json"
    r = _run(runner, tmp_path, text, "--check", "--write-restart", str(jpath))
    assert r.returncode == 0, r.stderr
    js, jh, jstep, jdt = restart.read_restart(jpath)
    assert (jstep, jdt) == (step, dt)
    for k in st:
        assert np.array_equal(js[k], st[k]), k
    assert (jh is None) == (hist is None)


@pytest.fixture(scope="module")
def fake_runner(runner, tmp_path_factory):
    """mdg_run next to a CPU stand-in of the library (tests/fake_mdg.cpp): the
    host's run path without a GPU."""
    import shutil

    d = tmp_path_factory.mktemp("fake")
    src = os.path.join(ROOT, "tests", "fake_mdg.cpp")
    subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(ROOT, "include"), src, "-o",
                    str(d / "libmddem_gb300.so")], check=True)
    shutil.copy(runner, d / "mdg_run")
    return str(d / "mdg_run")


def test_run_path_with_outputs_and_restarts(fake_runner, tmp_path):
    from mddem_gb300 import restart

    text = GAS.replace("steps = 500\nthermo = 100", "steps = 300\nthermo = 100") + "\n[restart]\ninterval = 100\n"
    p = tmp_path / "config.toml"
    p.write_text(text)
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if not l.startswith("#")]
    assert [int(l.split()[0]) for l in lines] == [0, 100, 200, 300]
    # one launch per output interval, not per step
    assert r.stderr.count("fake: step 100") == 3 and "fake: upload n=400 force=0" in r.stderr
    a = restart.read_restart(tmp_path / "output" / "restart" / "restart_100_rank0.bin")
    b = restart.read_restart(tmp_path / "output" / "restart" / "restart_200_rank0.bin")
    assert a[2] == 100 and b[2] == 200 and len(a[0]["tag"]) == 400
    assert np.allclose(b[0]["pos"] - a[0]["pos"], a[0]["vel"] * 2.934e-7 * 100, rtol=1e-9, atol=1e-15)
    assert np.array_equal(a[0]["density"][:300], np.full(300, 2500.0))
    assert np.array_equal(a[0]["density"][300:], np.full(100, 7800.0))
    keys, vals = a[1]
    assert keys.tolist() == [[0, 1]] and np.allclose(vals, [[0.5 * (q + 1) for q in range(7)]])


def test_run_path_resumes_from_the_latest_restart(fake_runner, tmp_path):
    """`[restart] read = true` (read_restart, mddem_print/src/lib.rs:1152-1251):
    the latest file in output/restart replaces the inserted state, the step
    counter continues from its step, and its forces, torques and contact
    history go to the device with the upload."""
    from mddem_gb300 import restart

    text = GAS.replace("steps = 500\nthermo = 100", "steps = 300\nthermo = 100") + "\n[restart]\ninterval = 100\n"
    p = tmp_path / "config.toml"
    p.write_text(text)
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    # mark the newest file so the resume can be told from a fresh insertion
    src = tmp_path / "output" / "restart" / "restart_300_rank0.bin"
    st, hist, step, dt = restart.read_restart(src)
    st["force"] = np.arange(st["pos"].size, dtype=float).reshape(-1, 3)
    st["torque"] = -st["force"]
    hist = (np.array([[3, 7], [5, 9]], np.uint32), np.arange(14, dtype=float).reshape(2, 7))
    restart.write_restart(src, st, hist, step=step, dt=dt)

    p.write_text(text.replace("steps = 300", "steps = 200") + "read = true\n")
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "# Restart: reading from output/restart/restart_300_rank0.bin" in r.stdout
    lines = [l for l in r.stdout.splitlines() if not l.startswith("#")]
    assert [int(l.split()[0]) for l in lines] == [300, 400, 500]
    assert "fake: upload n=400 force=1 torque=1" in r.stderr and "fake: set_history n=2" in r.stderr
    c = restart.read_restart(tmp_path / "output" / "restart" / "restart_500_rank0.bin")
    assert c[2] == 500
    assert np.allclose(c[0]["pos"] - st["pos"], st["vel"] * 2.934e-7 * 200, rtol=1e-9, atol=1e-15)
    for f in ("tag", "type", "mass", "radius", "density", "force", "torque", "quat"):
        assert np.array_equal(c[0][f], st[f]), f
    assert c[1][0].tolist() == [[3, 7], [5, 9]] and np.array_equal(c[1][1], hist[1])


def test_resume_without_files_runs_from_the_inserted_state(fake_runner, tmp_path):
    p = tmp_path / "config.toml"
    p.write_text(GAS.replace("steps = 500", "steps = 100") + "\n[restart]\nread = true\n")
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "# Restart: no restart files found in output/restart" in r.stdout
    assert [int(l.split()[0]) for l in r.stdout.splitlines() if not l.startswith("#")] == [0, 100]


def test_run_path_lj_measurements(fake_runner, tmp_path):
    text = LJ + "\n[run]\nsteps = 200\nthermo = 100\n\n[measure]\nrdf_interval = 50\nmsd_interval = 50\nrdf_bins = 30\n"
    p = tmp_path / "config.toml"
    p.write_text(text)
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if not l.startswith("#")]
    assert [int(l.split()[0]) for l in lines] == [0, 100, 200]
    assert r.stderr.count("fake: step 50") == 4  # measurement marks every 50 steps
    rdf = np.loadtxt(tmp_path / "output" / "rdf.txt")
    assert rdf.shape == (30, 2)
    msd = np.loadtxt(tmp_path / "output" / "msd.txt")
    assert msd[:, 0].tolist() == [50, 100, 150, 200] and msd[:, 1].tolist() == [50, 100, 150, 200]


def test_crlf_config_reads_the_same(runner, tmp_path):
    a = _run(runner, tmp_path, GAS, "--check")
    p = tmp_path / "crlf.toml"
    p.write_bytes(GAS.replace("\n", "\r\n").encode())
    b = subprocess.run([runner, str(p), "--check"], capture_output=True, text=True, timeout=60)
    assert a.returncode == 0 and b.returncode == 0, b.stderr
    assert json.loads(a.stdout) == json.loads(b.stdout)


@pytest.mark.parametrize("edit,msg", [
    (("sigma = 0.88\n", "sigma = 0.88\nradius = 1\n"), "unknown field"),
    (("epsilon = 0.5\nsigma = 0.88\n", "epsilon = 0.5\n"), "needs epsilon and sigma"),
    (("types = [0, 1]", "types = [0, 2]"), "only 2 types"),
    (("type_fractions = [0.5, 1.0]", "type_fractions = [0.3, 0.6, 1.0]"), "more types"),
    (('style = "fcc"', 'style = "fcc"\nbasis = 2'), "unknown field"),
])
def test_lj_types_errors_exit_1(runner, tmp_path, edit, msg):
    r = _run(runner, tmp_path, LJ_TYPES_TOML.replace(*edit), "--check")
    assert r.returncode == 1
    assert msg in r.stderr


def test_run_path_passes_the_lj_pair_table(fake_runner, tmp_path):
    """The C++ host hands the device the [lj] types table it built (the same
    numbers as config.lj_pair_table) and the lattice's typed particles."""
    from mddem_gb300 import config

    p = tmp_path / "config.toml"
    p.write_text(LJ_TYPES_TOML)
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "lj_types=2" in r.stderr and "fake: upload n=864" in r.stderr
    got = [tuple(float(x) for x in l.split()[3:]) for l in r.stderr.splitlines() if l.startswith("fake: lj_pair")]
    assert tuple(got) == config.from_toml(LJ_TYPES_TOML).lj_pairs


def test_run_path_json_restarts_and_resume(fake_runner, tmp_path):
    """[restart] format = "json": the C++ host writes restart_{step}_rank0.json
    (serde_json's field set), and read = true resumes from the latest of them,
    contact history included."""
    from mddem_gb300 import restart

    text = GAS.replace("steps = 500\nthermo = 100", "steps = 200\nthermo = 100") + \
        '\n[restart]\ninterval = 100\nformat = "json"\n'
    p = tmp_path / "config.toml"
    p.write_text(text)
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    d = tmp_path / "output" / "restart"
    assert sorted(x.name for x in d.iterdir()) == ["restart_100_rank0.json", "restart_200_rank0.json"]
    st, hist, step, _ = restart.read_restart(d / "restart_200_rank0.json")
    assert step == 200 and len(st["tag"]) == 400 and hist[0].tolist() == [[0, 1]]
    # the Python writer's JSON (json.dumps spacing and number forms) reads the same
    restart.write_restart(d / "restart_200_rank0.json", st, hist, step=step, dt=2.934e-7, fmt="json")
    p.write_text(text + "read = true\n")
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "reading from output/restart/restart_200_rank0.json" in r.stdout
    assert [int(l.split()[0]) for l in r.stdout.splitlines() if not l.startswith("#")] == [200, 300, 400]
    assert "fake: set_history n=1" in r.stderr
    st4, _, step4, _ = restart.read_restart(d / "restart_400_rank0.json")
    assert step4 == 400
    assert np.allclose(st4["pos"] - st["pos"], st["vel"] * 2.934e-7 * 200, rtol=1e-9, atol=1e-15)


@pytest.mark.parametrize("fmt", ["bincode", "json"])
def test_resume_from_a_damaged_file_is_an_error(fake_runner, tmp_path, fmt):
    """A truncated restart file stops the run with a message (exit 1), as the
    reference's read_restart does on a deserialisation error."""
    text = GAS.replace("steps = 500\nthermo = 100", "steps = 100\nthermo = 100") + \
        f'\n[restart]\ninterval = 100\nformat = "{fmt}"\n'
    p = tmp_path / "config.toml"
    p.write_text(text)
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    f = tmp_path / "output" / "restart" / ("restart_100_rank0." + ("json" if fmt == "json" else "bin"))
    f.write_bytes(f.read_bytes()[:-7])
    p.write_text(text + "read = true\n")
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 1 and "restart" in r.stderr, (r.returncode, r.stderr)


@pytest.mark.parametrize("count", [-1.0, 2.5, float("nan"), 1e30])
def test_resume_with_a_damaged_history_count_is_an_error(fake_runner, tmp_path, count):
    """A contact-history count that is negative, fractional, NaN or larger
    than the buffer stops the resume with a message (exit 1) in the C++ host
    and a ValueError in the Python reader, instead of a conversion of the
    stored double to a count."""
    from mddem_gb300 import restart

    text = GAS.replace("steps = 500\nthermo = 100", "steps = 100\nthermo = 100") + "\n[restart]\ninterval = 100\n"
    p = tmp_path / "config.toml"
    p.write_text(text)
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    f = tmp_path / "output" / "restart" / "restart_100_rank0.bin"
    st, hist, step, dt = restart.read_restart(f)
    fields = restart.restart_fields(st, hist, step, dt)
    fields["atom_data_buffers"][1][0] = count
    f.write_bytes(restart._bincode(fields))
    with pytest.raises(ValueError, match="contact-history"):
        restart.read_restart(f)
    p.write_text(text + "read = true\n")
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 1 and "contact-history" in r.stderr, (r.returncode, r.stderr)


GAS_DEVICE = """
[domain]
x_high = 0.025
y_high = 0.025
z_high = 0.025

[neighbor]
skin_fraction = 1.1
bin_size = 0.005

[run]
steps = 200

[[dem.materials]]
name = "glass"
youngs_mod = 8.7e9
poisson_ratio = 0.3
restitution = 0.95
friction = 0.4

[[particles.insert]]
material = "glass"
count = 500
radius = { distribution = "uniform", min = 0.0008, max = 0.0012 }
density = 2500.0
velocity = 0.3

[gpu]
generate = "device"
"""


@pytest.mark.parametrize("text,n", [(GAS_DEVICE, 500), (LJ.replace("[gpu]", '[gpu]\ngenerate = "device"'), None)],
                         ids=["gas", "lj"])
def test_device_generation_resolves_alike(runner, tmp_path, text, n):
    """[gpu] generate = "device": both hosts register the device generator
    (mdg_generate_gas / mdg_generate_fcc) instead of a host state, with the same
    particle count and the same dt (granular: from the smallest radius the
    block allows)."""
    from mddem_gb300 import run

    if "[gpu]" not in text:
        text += '\n[gpu]\ngenerate = "device"\n'
    r = _run(runner, tmp_path, text, "--check")
    assert r.returncode == 0, r.stderr
    got = json.loads(r.stdout)
    cfg, st, _ = run.setup(text, seed=0)
    assert st["generate"] in ("gas", "fcc")
    assert got["generate"] == "device" and got["n"] == st["n"]
    if n:
        assert st["n"] == n
    assert got["dt"] == cfg.dt


@pytest.mark.parametrize("edit,msg", [
    (('generate = "device"', 'generate = "gpu"'), "host or device"),
    (("velocity = 0.3", "velocity = 0.3\nvelocity_x = 0.1"), "velocity_x"),
    (("density = 2500.0", 'density = 2500.0\nregion = { type = "block", min = [0, 0, 0], max = [0.01, 0.01, 0.01] }'),
     "whole domain"),
])
def test_device_generation_refusals(runner, tmp_path, edit, msg):
    from mddem_gb300 import run

    text = GAS_DEVICE.replace(*edit)
    r = _run(runner, tmp_path, text, "--check")
    assert r.returncode == 1 and msg in r.stderr, r.stderr
    with pytest.raises(run.RunError):
        run.setup(text, seed=0)


def test_device_generation_failure_exits_1(fake_runner, tmp_path):
    """[gpu] generate = "device" with a library whose generator fails (the CPU
    stand-in has no device): the context is created for the generator's count,
    the failure is reported as a configuration error and the run exits 1."""
    p = tmp_path / "config.toml"
    p.write_text(GAS_DEVICE)
    r = subprocess.run([fake_runner, str(p)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 1
    assert "fake: create kind=0 capacity=500" in r.stderr
    assert "device generator" in r.stderr
