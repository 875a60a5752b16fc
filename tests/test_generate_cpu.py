"""The device generators' counter-based stream and its CPU restatement, on the
CPU: the library's host copy of the draw (mdg_counter_draw, the same inline
function the kernels use) equals tests/gen_ref.py's numpy restatement, and the
sequential RSA restatement places non-overlapping spheres in the inset box
and keeps its proposal order."""
import numpy as np
import pytest

import gen_ref


@pytest.fixture(scope="module")
def lib():
    from mddem_gb300 import build, capi

    build.build()
    return capi.load()


def test_counter_draw_matches_the_restatement(lib):
    from mddem_gb300 import capi

    rng = np.random.default_rng(0)
    for seed in (0, 1, 2 ** 63 + 5, int(rng.integers(0, 2 ** 62))):
        for stream in (1, 2, 7):
            idx = np.concatenate([np.arange(8), rng.integers(0, 2 ** 40, 8)]).astype(np.uint64)
            ref = gen_ref.draw(seed, stream, idx)
            got = [capi.counter_draw(seed, stream, int(i)) for i in idx]
            assert [int(x) for x in ref] == got


def test_uniform_and_normal_statistics():
    u = gen_ref.uniform(gen_ref.draw(3, 1, np.arange(200000)))
    assert 0.0 <= u.min() and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 3e-3
    z = gen_ref.normal3(3, 100000)
    assert np.all(np.abs(z.mean(axis=0)) < 0.02)
    assert np.all(np.abs(z.std(axis=0) - 1.0) < 0.02)


@pytest.mark.parametrize("rmin,rmax,sep", [(1e-3, 1e-3, 1.1), (0.8e-3, 1.2e-3, 1.0)])
def test_sequential_rsa_restatement(rmin, rmax, sep):
    L = 0.03
    P, R = gen_ref.rsa(600, (0.0,) * 3, (L,) * 3, rmin, rmax, sep, True, seed=4, max_proposals=200000)
    assert len(P) == 600
    assert P.min() >= rmax and P.max() <= L - rmax
    assert R.min() >= rmin and R.max() <= rmax
    d = P[:, None, :] - P[None, :, :]
    d -= L * np.rint(d / L)
    r = np.sqrt((d * d).sum(axis=2))
    np.fill_diagonal(r, np.inf)
    assert np.all(r > sep * (R[:, None] + R[None, :]) * (1 - 1e-12))
    # a second call, same stream: same spheres
    P2, R2 = gen_ref.rsa(600, (0.0,) * 3, (L,) * 3, rmin, rmax, sep, True, seed=4, max_proposals=200000)
    assert np.array_equal(P, P2) and np.array_equal(R, R2)
