"""Batching and serving forms on the GPU.

* per-system step budgets inside one multi-step launch: a system with a
  budget of k steps ends exactly where a standalone k-step run ends;
* serving: jobs of both kinds and different sizes are queued, admitted into
  typed slots as slots and HBM budget free up, advanced together on the device,
  retired, and every job's final state equals the same job run alone
  (identical kernels and per-system arithmetic: bitwise);
* slot reuse: a slot reconfigured for a new job carries nothing over.
"""
import numpy as np
import pytest

from helpers import by_tag

pytestmark = pytest.mark.gpu


def _alone(cfg, st, steps):
    from mddem_gb300 import capi

    with capi.Context(cfg, len(st["tag"])) as c:
        c.upload(st)
        c.step(steps)
        return c.download()


def _same(a, b, fields=("pos", "vel")):
    for f in fields:
        (x,) = by_tag(a, f)
        (y,) = by_tag(b, f)
        if not np.array_equal(x, y):
            return False
    return True


def test_step_budgets_freeze_systems(gpu_lib):
    from mddem_gb300 import capi, config, inputs

    c1 = config.lj_fluid_config()
    s1 = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=21)
    c2 = config.granular_gas_config(box=0.02, dt=2e-7)
    s2 = inputs.dem_granular_gas(400, box=0.02, seed=22)
    b = capi.Context([c1, c2], [864, 400])
    b.upload(s1, 0)
    b.upload(s2, 1)
    b.set_remaining(13, 0)
    b.set_remaining(37, 1)
    b.step(50)
    assert b.remaining(0) == 0 and b.remaining(1) == 0
    assert b.thermo(0)["step"] == 13 and b.thermo(1)["step"] == 37
    assert _same(b.download(0), _alone(c1, s1, 13))
    assert _same(b.download(1), _alone(c2, s2, 37), ("pos", "vel", "omega"))


def _jobs(precision):
    from mddem_gb300 import config, inputs

    jobs = []
    for k, (n, steps) in enumerate([(300, 40), (900, 120), (1500, 80), (600, 60)]):
        box = (n * 4.19e-9 / 0.15) ** (1 / 3)
        cfg = config.granular_gas_config(box=box, dt=2e-7, precision=precision)
        cfg.materials[0].restitution = 0.8 + 0.05 * k
        jobs.append((cfg, inputs.dem_granular_gas(n, box=box, seed=30 + k), steps))
    for k, (nc, box, steps) in enumerate([(6, 10.06, 70), (5, 8.4, 150)]):
        cfg = config.lj_fluid_config(box=box, precision=precision)
        jobs.append((cfg, inputs.lj_fcc(nc, box, 0.85, 0.85 + 0.1 * k, seed=40 + k), steps))
    return jobs


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_server_results_equal_alone(gpu_lib, precision):
    from mddem_gb300 import capi, config

    jobs = _jobs(precision)
    slots = [config.granular_gas_config(precision=precision)] * 2 + [config.lj_fluid_config(precision=precision)] * 2
    caps = [2000, 2000, 1000, 1000]
    # budget for about two resident DEM jobs: forces queueing and slot reuse
    srv = capi.Server(slots, caps, hbm_budget=16 << 20)
    ids = [srv.submit(c, s, n) for c, s, n in jobs[:3]]
    srv.pump(25)
    # diagnostics view of the server's contexts: resident slots download
    res = srv.resident()
    assert res
    for r in res:
        assert len(srv.download_resident(r["slot"])["tag"]) == r["n"]
    assert srv.stats()["contexts"] == 2  # one per particle kind
    ids += [srv.submit(c, s, n) for c, s, n in jobs[3:]]
    done = {}
    for _ in range(1000):
        active, pending = srv.pump(25)
        for info in srv.poll():
            done[info["id"]] = info
        if active == 0 and pending == 0:
            break
    done.update({i["id"]: i for i in srv.poll()})
    assert sorted(done) == sorted(ids)
    for jid, (cfg, st, steps) in zip(ids, jobs):
        info = done[jid]
        assert info["status"] == 0 and info["steps"] == steps
        assert info["submit_s"] <= info["start_s"] <= info["end_s"]
        got = srv.fetch(jid)
        ref = _alone(cfg, st, steps)
        f = ("pos", "vel", "omega") if cfg.kind == "dem" else ("pos", "vel")
        assert _same(got, ref, f), (jid, cfg.kind, len(st["tag"]))
    srv.close()


def test_grouped_server_results_equal_alone(gpu_lib):
    """Every slot in its own context (mdg_server_create_grouped): four
    contexts on four streams, all launched before any is waited on; each job
    still ends bitwise where it ends alone."""
    from mddem_gb300 import capi, config

    jobs = _jobs("mixed")
    slots = [config.granular_gas_config(precision="mixed")] * 2 + [config.lj_fluid_config(precision="mixed")] * 2
    srv = capi.Server(slots, [2000, 2000, 1000, 1000], hbm_budget=1 << 30, groups=[0, 1, 2, 3])
    assert srv.stats()["contexts"] == 4
    ids = [srv.submit(c, s, n) for c, s, n in jobs]
    done = {}
    for _ in range(1000):
        active, pending = srv.pump(25)
        done.update({i["id"]: i for i in srv.poll()})
        if active == 0 and pending == 0:
            break
    assert sorted(done) == sorted(ids)
    for jid, (cfg, st, steps) in zip(ids, jobs):
        f = ("pos", "vel", "omega") if cfg.kind == "dem" else ("pos", "vel")
        assert _same(srv.fetch(jid), _alone(cfg, st, steps), f), jid
    srv.close()


def test_server_rejects_jobs_without_a_slot(gpu_lib):
    from mddem_gb300 import capi, config, inputs

    srv = capi.Server([config.granular_gas_config()], [200], hbm_budget=1 << 30)
    st = inputs.dem_granular_gas(500, seed=1)
    with pytest.raises(capi.MdgError) as e:
        srv.submit(config.granular_gas_config(), st, 10)
    assert e.value.status == 4  # MDG_ERR_BUDGET
    srv.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_server_walled_and_typed_jobs(gpu_lib, precision):
    """Jobs whose configs point at arrays (plane walls on fixed axes, a
    multi-type LJ pair table) are served from the server's own copies: the
    caller's arrays are gone by admission.  Every job, the single-type LJ
    job sharing the context with the typed one included (its force launch
    then runs the typed instantiation, same coefficients, same arithmetic),
    ends bitwise where it ends alone."""
    import gc

    from test_lj_types_gpu import _state as typed_state
    from test_lj_types_cpu import two_type_config
    from test_walls import walled_config, walled_state

    from mddem_gb300 import capi, config, inputs

    jobs = [(walled_config(precision=precision, g_frac=0.05), walled_state(seed=6), 60),
            (config.lj_fluid_config(precision=precision), inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=44), 50),
            (two_type_config(precision=precision), typed_state(seed=8), 70)]
    slots = [config.granular_gas_config(precision=precision), config.lj_fluid_config(precision=precision),
             config.lj_fluid_config(precision=precision)]
    srv = capi.Server(slots, [1000, 1000, 1000], hbm_budget=1 << 30)
    ids = [srv.submit(c, s, n) for c, s, n in jobs]
    gc.collect()
    done = {}
    for _ in range(1000):
        active, pending = srv.pump(20)
        for info in srv.poll():
            done[info["id"]] = info
        if active == 0 and pending == 0:
            break
    done.update({i["id"]: i for i in srv.poll()})
    for k, (jid, (cfg, st, steps)) in enumerate(zip(ids, jobs)):
        assert done[jid]["status"] == 0 and done[jid]["steps"] == steps
        got, ref = srv.fetch(jid), _alone(cfg, st, steps)
        assert _same(got, ref, ("pos", "vel", "omega") if cfg.kind == "dem" else ("pos", "vel")), k
    srv.close()


def test_stream_priority_keeps_results(gpu_lib):
    """mdg_set_stream_priority moves a context to a new stream of another
    priority: the same steps give the same bits, and it is refused while a
    launch is in flight."""
    from mddem_gb300 import capi, config, inputs

    cfg = config.lj_fluid_config(precision="mixed")
    st = inputs.lj_fcc(6, 10.06, 0.85, 0.85, seed=61)
    ref = _alone(cfg, st, 60)
    with capi.Context(cfg, len(st["tag"])) as c:
        c.stream_priority(-5)
        c.upload(st)
        c.step(30)
        c.stream_priority(0)
        c.step(30)
        assert _same(c.download(), ref)
        assert c.lib.mdg_step_async(c.h, 10) == 0
        assert c.lib.mdg_set_stream_priority(c.h, -1) == 10  # MDG_ERR_STATE
        assert c.lib.mdg_step_wait(c.h) == 0
