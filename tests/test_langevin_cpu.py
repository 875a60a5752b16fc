"""Langevin in the oracle (langevin_force, md_thermostat/src/lib.rs:529-581):
the force F -= gamma m v, F += sqrt(2 gamma m kT / dt) N(0,1) at PostForce,
with N(0,1) from the counter-based stream keyed by (seed, step, tag,
component) that the device uses.  Checked: the draws equal a Python
restatement of that stream (one free particle, one step), the stream is
reproducible and seed dependent, and an LJ fluid relaxes to the bath
temperature."""
import math

import numpy as np
import pytest

M64 = (1 << 64) - 1


def _mix(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def _uniform(seed, step, tag, draw):
    h = _mix((seed + _mix((step * 0x9E3779B97F4A7C15 + _mix(((tag << 3) + draw) & M64)) & M64)) & M64)
    return (h >> 11) * 2.0 ** -53


def lv_normal(seed, step, tag, k):
    u1, u2 = _uniform(seed, step, tag, 2 * k), _uniform(seed, step, tag, 2 * k + 1)
    return math.sqrt(-2.0 * math.log(max(u1, 1e-300))) * math.cos(6.283185307179586 * u2)


def _free_particle(seed):
    from mddem_gb300 import config
    from oracle.oracle import Oracle

    cfg = config.lj_fluid_config(box=10.0, nose_hoover=False).replace(langevin=True, lv_temperature=1.3,
                                                                      lv_damping=0.7, lv_seed=seed)
    st = {"tag": np.array([5], np.uint32), "type": np.zeros(1, np.uint32), "pos": np.array([[5.0, 5.0, 5.0]]),
          "vel": np.zeros((1, 3)), "mass": np.array([2.0]), "cutoff_radius": np.array([1.25])}
    o = Oracle(cfg)
    o.load(st)
    o.step(1)
    return cfg, o.state()["vel"][0]


def test_oracle_draws_follow_the_counter_based_stream():
    seed = 424242
    cfg, v1 = _free_particle(seed)
    # at rest with no pair force: v(dt) = dt / (2 m) * sqrt(2 gamma m kT / dt) * N
    rc = math.sqrt(2.0 * 0.7 * 2.0 * 1.3 / cfg.dt)
    want = [0.5 * cfg.dt / 2.0 * rc * lv_normal(seed, 0, 5, k) for k in range(3)]
    assert np.allclose(v1, want, rtol=1e-13, atol=0)


def test_oracle_stream_reproducible_and_seeded():
    _, a = _free_particle(7)
    _, b = _free_particle(7)
    _, c = _free_particle(8)
    assert np.array_equal(a, b) and not np.array_equal(a, c)


def test_oracle_lj_relaxes_to_the_bath_temperature():
    from mddem_gb300 import config, inputs
    from oracle.oracle import Oracle

    cfg = config.lj_fluid_config(nose_hoover=False).replace(langevin=True, lv_temperature=1.2, lv_damping=2.0,
                                                            lv_seed=3)
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.6, seed=5)
    o = Oracle(cfg)
    o.load(st)
    o.step(600)
    temps = []
    for _ in range(20):
        o.step(25)
        temps.append(o.thermo()["temp"])
    assert np.mean(temps) == pytest.approx(1.2, rel=0.05)
