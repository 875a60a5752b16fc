"""The C++ host (`mdg_run`) driving the device: an LJ melt prints its thermo
lines at the print interval, and a glass sphere dropped on a wall through the
config's [[wall]], fixed boundaries and block insertion region leaves with
e^2 of its kinetic energy (restitution 0.9); its [restart] files read back."""
import os
import re
import subprocess

import pytest

from test_host_cpu import GAS_DEVICE, LJ, REBOUND

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(tmp_path, text, *args):
    from mddem_gb300 import build

    build.build()
    p = tmp_path / "config.toml"
    p.write_text(text)
    exe = os.path.join(ROOT, "mddem_gb300", "_lib", "mdg_run")
    return subprocess.run([exe, str(p), *args], capture_output=True, text=True, timeout=300, cwd=tmp_path)


def test_mdg_run_lj(gpu_lib, tmp_path):
    r = _run(tmp_path, LJ + "\n[run]\nsteps = 100\nthermo = 50\n")
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if not l.startswith("#")]
    steps = [int(l.split()[0]) for l in lines]
    assert steps == [0, 50, 100]
    temps = [float(re.search(r" T (\S+)", l).group(1)) for l in lines]
    assert all(0.3 < t < 3.0 for t in temps)


def test_mdg_run_wall_rebound(gpu_lib, tmp_path):
    from mddem_gb300 import restart

    r = _run(tmp_path, REBOUND + "\n[restart]\ninterval = 3000\n", "--steps", "6000")
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if not l.startswith("#")]
    ke = [float(re.search(r" KE (\S+)", l).group(1)) for l in lines]
    assert int(lines[-1].split()[0]) == 6000
    assert ke[-1] / ke[0] == pytest.approx(0.9 ** 2, rel=0.04)
    # restart files of the running system, read by the Python reader
    st, hist, step, dt = restart.read_restart(tmp_path / "output" / "restart" / "restart_6000_rank0.bin")
    assert step == 6000 and len(st["tag"]) == 1 and hist is not None
    assert st["vel"][0, 2] == pytest.approx(0.9, rel=0.04)
    assert (tmp_path / "output" / "restart" / "restart_3000_rank0.bin").exists()


def test_device_generated_configs_run_alike(gpu_lib, tmp_path, monkeypatch):
    """[gpu] generate = "device": both hosts make the same system on the
    device (same generator, same seed), so the C++ host's thermo lines equal
    the Python runner's, and a restart file written by the C++ host holds the
    generated particles."""
    import io

    from mddem_gb300 import restart, run

    monkeypatch.chdir(tmp_path)  # the Python runner writes its output directory here too
    gas = GAS_DEVICE.replace("[run]\nsteps = 200\n", "[run]\nsteps = 200\nthermo = 100\n\n[restart]\ninterval = 200\n")
    lj = LJ.replace("[gpu]", '[gpu]\ngenerate = "device"') + "\n[run]\nsteps = 100\nthermo = 50\n"
    for text in (gas, lj):
        r = _run(tmp_path, text)
        assert r.returncode == 0, r.stderr
        assert "generated on the device" in r.stdout
        cpp = [l for l in r.stdout.splitlines() if not l.startswith("#")]
        buf = io.StringIO()
        run.run(text, out=buf)
        py = [l for l in buf.getvalue().splitlines() if not l.startswith("#")]
        assert cpp == py
    st, _, step, _ = restart.read_restart(tmp_path / "output" / "restart" / "restart_200_rank0.bin")
    assert step == 200 and len(st["tag"]) == 500
