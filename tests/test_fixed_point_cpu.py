"""The mixed LJ kernel's 32-bit fixed-point geometry, restated in numpy: a
coordinate is stored as u = round((x - lo) 2^32 / L) mod 2^32 (the kernel's
fixed_pos), a separation is (float32)(int32)(u_j - u_i) * float32(L / 2^32)
(fixed_sep).  The wrapped integer difference must give the minimum-image
separation, also for particles that drifted outside the box since the last
wrap, to within L 2^-32 (half a unit of quantisation per coordinate) +
2^-22 |d| (the int->float rounding, the rounded float scale and the product's
rounding, 2^-24 each), the bound the kernel's error budget assumes."""
import numpy as np


def fixed_pos(x, lo, L):
    return (np.rint((x - lo) * (2.0 ** 32 / L)).astype(np.int64) & 0xFFFFFFFF).astype(np.uint32)


def fixed_sep(uj, ui, L):
    d = (uj.astype(np.int64) - ui.astype(np.int64)) & 0xFFFFFFFF
    d = np.where(d >= 2 ** 31, d - 2 ** 32, d).astype(np.int32)
    return d.astype(np.float32) * np.float32(L / 2.0 ** 32)


def min_image(d, L):
    return d - L * np.round(d / L)


def test_fixed_point_separation_is_minimum_image_within_bound():
    rng = np.random.default_rng(7)
    for L, lo in ((67.06, 0.0), (10.06, -5.03), (1000.0, 250.0)):
        n = 200000
        xi = lo + rng.uniform(-0.02 * L, 1.02 * L, n)  # some drifted past the faces
        d_true = rng.uniform(-2.8, 2.8, n)  # list-cutoff separations
        xj = xi + d_true
        # partner stored through its own wrapped coordinate when it crossed a face
        xj_w = np.where(xj >= lo + L, xj - L, np.where(xj < lo, xj + L, xj))
        got = fixed_sep(fixed_pos(xj_w, lo, L), fixed_pos(xi, lo, L), L).astype(np.float64)
        want = min_image(xj_w - xi, L)
        err = np.abs(got - want)
        bound = L * 2.0 ** -32 + 2.0 ** -22 * np.abs(want)
        assert np.all(err <= bound), float(np.max(err / bound))
        assert np.allclose(want, d_true, atol=1e-9 * L)


def test_fixed_point_force_error_under_mixed_bound():
    """LJ 12-6 pair force from fixed-point separations vs fp64 over r in
    [0.85, 2.5] sigma, per pair relative to the size of its repulsive plus
    attractive parts (the force itself vanishes at 2^(1/6) sigma): well under
    the 1e-5 the mixed path states (the fp32 force arithmetic adds a few 1e-7)."""
    rng = np.random.default_rng(3)
    L = 67.06
    n = 100000
    xi = rng.uniform(0, L, (n, 3))
    r = rng.uniform(0.85, 2.5, n)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    xj = np.mod(xi + r[:, None] * u, L)
    d64 = min_image(xj - xi, L)
    d32 = np.stack([fixed_sep(fixed_pos(xj[:, k], 0.0, L), fixed_pos(xi[:, k], 0.0, L), L) for k in range(3)], 1)

    def fpair(d):
        r2 = np.sum(d.astype(np.float64) ** 2, axis=1)
        r6 = r2 ** -3
        return (48.0 * r6 * r6 - 24.0 * r6) / r2

    f64 = fpair(d64)[:, None] * d64
    f32 = fpair(d32)[:, None] * d32.astype(np.float64)
    r2 = np.sum(d64 ** 2, axis=1)
    r6 = r2 ** -3
    parts = (48.0 * r6 * r6 + 24.0 * r6) / np.sqrt(r2)
    rel = np.linalg.norm(f32 - f64, axis=1) / parts
    assert np.max(rel) < 2e-6
