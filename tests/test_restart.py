"""Restart files in the reference's format (RestartData, bincode 1.3 default
options / serde_json; crates/mddem_print/src/lib.rs:297-376, 1050-1066).

CPU: the bincode byte layout of a one-atom file restated field by field from
the format (little-endian, fixed-width integers, u64 length before every
sequence); DEM state + contact history round trips in both formats; JSON
field names.  GPU: a run restarted from a file written mid-way continues the
uninterrupted run."""
import json
import struct

import numpy as np
import pytest

from helpers import by_tag, overlapping_spheres


def _lj_one():
    return {"tag": np.array([3], np.uint32), "type": np.array([0], np.uint32),
            "pos": np.array([[1.0, 2.0, 3.0]]), "vel": np.array([[0.5, -0.25, 0.125]]),
            "force": np.array([[4.0, 5.0, 6.0]]), "mass": np.array([1.0]), "cutoff_radius": np.array([1.25])}


def test_bincode_layout_one_atom(tmp_path):
    from mddem_gb300 import restart

    p = tmp_path / restart.restart_filename(7)
    restart.write_restart(p, _lj_one(), step=7, dt=0.005)
    b = p.read_bytes()
    u64 = lambda v: struct.pack("<Q", v)
    f64s = lambda *v: u64(len(v)) + struct.pack("<" + "d" * len(v), *v)
    exp = (u64(1) + u64(7) + struct.pack("<d", 0.005)
           + u64(1) + struct.pack("<I", 3) + u64(1) + struct.pack("<I", 0)
           + f64s(1.0) + f64s(2.0) + f64s(3.0) + f64s(0.5) + f64s(-0.25) + f64s(0.125)
           + f64s(4.0) + f64s(5.0) + f64s(6.0) + f64s(1.0) + f64s(1.25)
           + u64(0)                      # atom_data_buffers: none for LJ
           + u64(0) * 9                  # legacy omega/torque/ang_mom x/y/z
           + u64(0))                     # legacy quaternion
    assert b == exp
    assert p.name == "restart_7_rank0.bin"


@pytest.mark.parametrize("fmt", ["bincode", "json"])
def test_dem_round_trip_with_history(tmp_path, fmt):
    from mddem_gb300 import restart

    st = overlapping_spheres(50, 0.012, 5e-4, seed=3)
    st["force"] = np.random.default_rng(1).normal(size=(50, 3))
    st["torque"] = np.random.default_rng(2).normal(size=(50, 3))
    keys = np.array([[0, 5], [0, 9], [7, 2], [49, 1]], np.uint32)
    vals = np.random.default_rng(3).normal(scale=1e-6, size=(4, 7))
    p = tmp_path / restart.restart_filename(120, fmt=fmt)
    restart.write_restart(p, st, (keys, vals), step=120, dt=1e-7, fmt=fmt)
    got, hist, step, dt = restart.read_restart(p)
    assert step == 120 and dt == 1e-7
    for k in ("tag", "type", "pos", "vel", "force", "mass", "cutoff_radius", "radius", "inv_inertia", "omega",
              "torque", "quat", "density"):
        assert np.array_equal(np.asarray(got[k]), np.asarray(st[k])), k
    order = np.lexsort((keys[:, 1], keys[:, 0]))
    gorder = np.lexsort((hist[0][:, 1], hist[0][:, 0]))
    assert np.array_equal(hist[0][gorder], keys[order])
    assert np.array_equal(hist[1][gorder], vals[order])


def test_json_field_names(tmp_path):
    from mddem_gb300 import restart

    p = tmp_path / "r.json"
    restart.write_restart(p, _lj_one(), step=1, dt=0.005, fmt="json")
    d = json.loads(p.read_text())
    assert list(d) == ["natoms", "total_cycle", "dt", "tag", "atom_type", "pos_x", "pos_y", "pos_z", "vel_x",
                       "vel_y", "vel_z", "force_x", "force_y", "force_z", "mass", "cutoff_radius",
                       "atom_data_buffers", "omega_x", "omega_y", "omega_z", "torque_x", "torque_y", "torque_z",
                       "ang_mom_x", "ang_mom_y", "ang_mom_z", "quaternion"]


@pytest.mark.gpu
def test_restart_continues_the_run(gpu_lib, tmp_path):
    """30 steps, restart file (state + contact history), 30 more steps in a
    fresh context vs 60 uninterrupted steps (plain FP64 path): positions
    within 1e-12 of the box (the restarted run rebuilds its list at once, as
    the reference does after reading a restart, so sums run in another
    order), identical contact-history keys."""
    from mddem_gb300 import capi, config, restart

    cfg = config.granular_gas_config(box=0.012, dt=1e-7)
    st = overlapping_spheres(600, 0.012, 5e-4, seed=41)
    a = capi.Context(cfg, 600)
    a.upload(st)
    a.step(30)
    p = tmp_path / restart.restart_filename(30)
    restart.write_restart(p, a.download(), a.history(), step=30, dt=cfg.dt)
    a.step(30)
    got, hist, step, _ = restart.read_restart(p)
    assert step == 30
    b = capi.Context(cfg, 600)
    b.upload(got)
    b.set_history(*hist)
    b.step(30)
    pa, = by_tag(a.download(), "pos")
    pb, = by_tag(b.download(), "pos")
    d = pa - pb
    d -= 0.012 * np.round(d / 0.012)  # the two runs may wrap a particle at different steps
    assert np.max(np.abs(d)) <= 1e-12 * 0.012
    ka, kb = a.history()[0], b.history()[0]
    assert set(map(tuple, ka.tolist())) == set(map(tuple, kb.tolist()))
