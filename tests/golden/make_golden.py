"""Generate the golden fixtures used by tests/test_kat.py.

The reference (Rust) cannot be built or run here, so its known-answer tests
are carried over as data: each fixture below restates the construction of
one reference unit test and the analytic value it asserts.

  bin30.json      -- crates/mddem_core/src/neighbor.rs:1187-1266: 30 atoms at
                     (sin(0.31 i) 1.5 + 2, cos(0.67 i) 1.5 + 2, sin(0.97 i) 1.5 + 2),
                     cutoff radius 0.3, skin_fraction 1.0, bin_size 0.5, box 4.0;
                     expected: every brute-force pair (|r| < r_i + r_j) is listed.
  two_sphere.json -- crates/dem_granular/src/contact.rs:2214-2360, 1267-1323,
                     1996-2049, 2452-2497 and crates/mddem_test_utils/src/lib.rs:126-175:
                     glass (E 8.7e9, nu 0.3, e 0.95, mu 0.4), r = 1 mm,
                     density 2500, analytic Hertz / JKR / DMT forces.
  verlet.json     -- crates/mddem_verlet/src/lib.rs:160-185 and
                     crates/dem_granular/src/rotational.rs:109-145.

Run from the repository root: ``python tests/golden/make_golden.py``.
"""
import json
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def bin30():
    n, r = 30, 0.3
    pos = [[math.sin(i * 0.31) * 1.5 + 2.0, math.cos(i * 0.67) * 1.5 + 2.0, math.sin(i * 0.97) * 1.5 + 2.0]
           for i in range(n)]
    pairs = []
    for i in range(n):
        for j in range(i + 1, n):
            d = math.sqrt(sum((pos[j][k] - pos[i][k]) ** 2 for k in range(3)))
            if d < (r + r) * 1.0:
                pairs.append([i, j])
    return {"source": "crates/mddem_core/src/neighbor.rs:1187-1266", "box": 4.0, "radius": r,
            "skin_fraction": 1.0, "bin_size": 0.5, "pos": pos, "brute_force_pairs": pairs}


def two_sphere():
    E, nu, radius = 8.7e9, 0.3, 1e-3
    e_eff = 1.0 / ((1.0 - nu * nu) / E + (1.0 - nu * nu) / E)
    r_eff = radius / 2.0
    delta = 5e-5
    hertz = (4.0 / 3.0) * e_eff * math.sqrt(r_eff) * delta ** 1.5
    gamma = 1.0
    return {
        "source": "crates/dem_granular/src/contact.rs:2214-2360,1267-1323,1996-2049,2452-2497",
        "material": {"youngs_mod": E, "poisson_ratio": nu, "restitution": 0.95, "friction": 0.4},
        "radius": radius, "density": 2500.0, "dt": 1e-7,
        "hertz": {"delta": delta, "force": hertz, "rel_tol": 1e-10},
        "scaling_deltas": [1e-5, 2e-5, 4e-5, 6e-5, 8e-5], "scaling_rel_tol": 0.01,
        "jkr": {"gamma": gamma, "gap": 1e-9, "force": 1.5 * math.pi * gamma * r_eff, "rel_tol": 1e-6},
        "dmt": {"gamma": gamma, "overlap": 1e-12, "force": 2.0 * math.pi * gamma * r_eff, "rel_tol": 1e-3},
        "newton3": {"sep": 0.0019, "vel": [[0.1, 0.2, -0.1], [-0.3, 0.1, 0.05]],
                    "omega": [[10.0, 20.0, -5.0], [-15.0, 5.0, 10.0]], "abs_tol": 1e-10},
        "momentum": {"sep": 0.00195, "dt": 1e-8, "steps": 100, "vel": [[0.1, 0.05, -0.02], [-0.05, 0.03, 0.01]],
                     "abs_tol": 1e-12},
    }


def verlet():
    radius, density, dt = 1e-3, 2500.0, 1e-7
    mass = density * 4.0 / 3.0 * math.pi * radius ** 3
    inertia = 0.4 * mass * radius * radius
    return {
        "source": "crates/mddem_verlet/src/lib.rs:160-185; crates/dem_granular/src/rotational.rs:109-145",
        "translation": {"dt": 0.01, "mass": 1.0, "v0": 1.0, "f0": 2.0, "v1": 1.01, "x1": 0.0101, "abs_tol": 1e-10},
        "rotation": {"dt": dt, "radius": radius, "torque_z": 1.0, "omega_z": 0.5 * dt * 1.0 / inertia, "abs_tol": 1e-20},
    }


if __name__ == "__main__":
    for name, fn in (("bin30.json", bin30), ("two_sphere.json", two_sphere), ("verlet.json", verlet)):
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(fn(), f, indent=1)
        print("wrote", name)
