"""The benchmark's synthetic workloads on CPU: the served stream is a fixed,
seeded trace with the job mix the served-stream config describes (half
cooling gases of 100-200000 spheres, a quarter two-sphere rebounds, a quarter
LJ melts of 500-100000 atoms, 1000-50000 steps), every job fits a slot class,
and job states are reproducible."""
import numpy as np


def test_serve_trace_is_seeded_and_has_the_stated_mix():
    from mddem_gb300 import workloads as w

    a = w.serve_trace(njobs=128, rate=2.0, seed=2024)
    b = w.serve_trace(njobs=128, rate=2.0, seed=2024)
    assert [(j.kind, j.n, j.steps, j.arrival) for j in a] == [(j.kind, j.n, j.steps, j.arrival) for j in b]
    kinds = [j.kind for j in a]
    assert (kinds.count("gas"), kinds.count("rebound"), kinds.count("lj")) == (64, 32, 32)  # exactly 50/25/25
    assert all(1000 <= j.steps <= 50000 for j in a)
    assert all(100 <= j.n <= 200000 for j in a if j.kind == "gas")
    assert all(j.n == 2 for j in a if j.kind == "rebound")
    assert all(500 <= j.n <= 4 * 29 ** 3 for j in a if j.kind == "lj")
    arr = [j.arrival for j in a]
    assert arr == sorted(arr) and arr[0] == 0.0


def test_every_job_fits_a_slot_class():
    from mddem_gb300 import workloads as w

    dem_cap = max(c for c, _ in w.SERVE_DEM_SLOTS)
    lj_cap = max(c for c, _ in w.SERVE_LJ_SLOTS)
    for j in w.serve_trace(njobs=128, rate=2.0, seed=2024):
        assert j.n <= (lj_cap if j.kind == "lj" else dem_cap)
    for mult in (1, 2):
        cfgs, caps = w.serve_slots("mixed", mult=mult)
        assert len(cfgs) == len(caps) == mult * (sum(c for _, c in w.SERVE_DEM_SLOTS) +
                                                 sum(c for _, c in w.SERVE_LJ_SLOTS))
        assert all(c.precision == "mixed" for c in cfgs)


def test_job_states_are_reproducible():
    from mddem_gb300 import workloads as w

    trace = w.serve_trace(njobs=12, rate=2.0, seed=5)
    for j in trace:
        if j.n > 5000:
            continue
        c1, s1 = j.make("mixed", "displacement")
        c2, s2 = j.make("mixed", "displacement")
        assert len(s1["tag"]) == j.n
        assert np.array_equal(s1["pos"], s2["pos"]) and np.array_equal(s1["vel"], s2["vel"])
        assert c1 == c2


def test_oracle_rsa_places_the_library_spheres():
    """The oracle's seeded sphere placement (inputs of the CPU arm, made
    without the library) gives exactly the library's spheres: mono- and
    polydisperse, inset and periodic, several seeds."""
    import numpy as np

    from mddem_gb300 import build, capi
    from oracle import oracle

    build.build()
    oracle.build()
    for n, box, rmin, rmax, sep, inset, seed in [(500, 0.025, 1e-3, 1e-3, 1.1, True, 0),
                                                  (3000, 0.04, 0.8e-3, 1.2e-3, 1.0, False, 7),
                                                  (20000, 0.08, 1e-3, 1e-3, 1.1, True, 12345)]:
        a = capi.rsa_spheres(n, (0.0,) * 3, (box,) * 3, rmin, rmax, sep, inset, seed)
        b = oracle.rsa_spheres(n, (0.0,) * 3, (box,) * 3, rmin, rmax, sep, inset, seed)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_serve_groups_place_slots_by_kind_and_size():
    """The bench's "split" grouping: one context for the gases, one for the LJ
    slots up to 16384 atoms, one for the larger LJ slots; "kind" two; a
    group never mixes kinds."""
    from mddem_gb300 import workloads as w

    cfgs, caps = w.serve_slots("mixed", "displacement", mult=2)
    for policy, want in (("kind", 2), ("split", 3), ("class", 8)):
        g = w.serve_groups(cfgs, caps, policy)
        assert len(set(g)) == want, policy
        for k in set(g):
            assert len({c.kind for c, gg in zip(cfgs, g) if gg == k}) == 1
    g = w.serve_groups(cfgs, caps, "split")
    small = {gg for c, cap, gg in zip(cfgs, caps, g) if c.kind == "lj" and cap <= 16384}
    large = {gg for c, cap, gg in zip(cfgs, caps, g) if c.kind == "lj" and cap > 16384}
    assert len(small) == 1 and len(large) == 1 and small != large
