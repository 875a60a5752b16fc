"""The replicas-only multi-rank path of bench.py on CPU: two gloo ranks on
127.0.0.1 reduce their timings and work the way the GPU bench does (the max
of the ranks' times, the sum of their work), and the reference arm runs on
rank 0 only."""
import os
import socket
import subprocess
import sys
import types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = """
import os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
r = dist.get_rank()
ms, work = bench.reduce_over_ranks(dist, 10.0 + 3.0 * r, 100.0 * (r + 1))
dist.barrier()
dist.destroy_process_group()
print("RESULT", r, ms, work, flush=True)
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reduce_time_and_work():
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    outs = []
    try:
        for p in procs:
            out, _ = p.communicate(timeout=180)
            assert p.returncode == 0, out
            outs.append(out)
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    res = sorted(tuple(l.split()[1:]) for o in outs for l in o.splitlines() if l.startswith("RESULT"))
    assert [int(r[0]) for r in res] == [0, 1]
    for r in res:
        assert float(r[1]) == 13.0  # slowest rank's time
        assert float(r[2]) == 300.0  # work of both ranks


def test_single_rank_reduce_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.reduce_over_ranks(None, 12.5, 7.0) == (12.5, 7.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    a = types.SimpleNamespace(workload="serve", warmup=3, steps=0, gpus=2)
    assert bench.run_reference(a) is None
    assert capsys.readouterr().out == ""


def test_reference_arm_inputs_do_not_load_the_library():
    """The reference arm makes its jobs' inputs with the oracle's own sphere
    placement: building a stretch of the served stream's jobs and stepping
    them maps the oracle's library and never libmddem_gb300.so."""
    import subprocess
    import sys

    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import bench\n"
        "bench.REF_BUDGET = 0.5\n"
        "w, s = bench._ref_worker(('serve', (list(range(0, 16)), 16)))\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert w > 0 and s > 0\n"
        "assert 'libmdg_oracle' in maps\n"
        "assert 'libmddem_gb300' not in maps, 'library mapped'\n"
        "print('ok')\n" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-2000:]
