"""mdg_granular_temp_noalloc: the thermo reduction for callers that cannot
allocate device memory (their host keeps every byte of the GPU in its own pool,
or their step loop must not risk an allocation's device synchronisation).

The caller owns the input and output buffers (here: torch CUDA tensors); the
entry point's only scratch is a static device array inside the library.  The
results must match the context-based mdg_thermo on the same state, within the
1e-12 relative tolerance of the fp64 reductions (the two use different block
sizes, hence a different summation order), on two calls in a row.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, vel, mass, out, n, torch):
    stream = torch.cuda.current_stream().cuda_stream
    return lib.mdg_granular_temp_noalloc(ctypes.c_void_p(vel.data_ptr()), ctypes.c_void_p(mass.data_ptr()),
                                         ctypes.c_size_t(n), ctypes.c_void_p(out.data_ptr()),
                                         ctypes.c_void_p(stream))


def _reference(state):
    """mdg_thermo (context path) on the same particles."""
    from mddem_gb300 import capi, config

    cfg = config.granular_gas_config(box=0.05)
    with capi.Context(cfg, len(state["tag"])) as ctx:
        ctx.upload(state)
        t = ctx.thermo()
    return np.array([t["granular_temp"], t["ke"], t["momentum"]])


def test_noalloc_granular_temp_matches_thermo(gpu_lib):
    torch = pytest.importorskip("torch")
    from mddem_gb300 import inputs

    lib = gpu_lib
    st = inputs.dem_granular_gas(6000, box=0.05, seed=5)
    st["vel"] = st["vel"] + np.array([0.03, -0.02, 0.01])  # non-zero mean velocity
    n = len(st["tag"])
    vel = torch.tensor(st["vel"], dtype=torch.float64, device="cuda").contiguous()
    mass = torch.tensor(st["mass"], dtype=torch.float64, device="cuda").contiguous()
    out = torch.full((3,), float("nan"), dtype=torch.float64, device="cuda")
    want = _reference(st)
    scale = np.array([want[0], want[1], float(np.sum(st["mass"][:, None] * np.abs(st["vel"])))])
    for _ in range(2):  # the shared scratch must give the same answer on a repeat call
        out.fill_(float("nan"))
        assert _call(lib, vel, mass, out, n, torch) == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.all(np.abs(got - want) <= 1e-12 * scale), (got, want)

    # a different state through the same scratch: no leftovers from the last call
    st2 = dict(st)
    st2["vel"] = 0.5 * st["vel"][::-1].copy()
    vel2 = torch.tensor(st2["vel"], dtype=torch.float64, device="cuda").contiguous()
    want2 = _reference(st2)
    assert _call(lib, vel2, mass, out, n, torch) == 0
    torch.cuda.synchronize()
    got2 = out.cpu().numpy()
    scale2 = np.array([want2[0], want2[1], float(np.sum(st2["mass"][:, None] * np.abs(st2["vel"])))])
    assert np.all(np.abs(got2 - want2) <= 1e-12 * scale2), (got2, want2)


def test_noalloc_rejects_sizes_beyond_the_scratch(gpu_lib):
    torch = pytest.importorskip("torch")
    lib = gpu_lib
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    assert _call(lib, buf, buf, out, 1_048_577, torch) == 9  # MDG_ERR_ARG, nothing launched
    assert _call(lib, buf, buf, out, 0, torch) == 9
