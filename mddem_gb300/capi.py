"""ctypes binding of the C ABI in include/mdg.h.

This is the Python face of the drop-in boundary: each method maps to one
``extern "C"`` entry point of libmddem_gb300.so.  The library must be built
(``mddem_gb300.build.build()``); there is no CPU fallback, and every call
raises ``MdgError`` on a non-zero status.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .config import SimConfig

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmddem_gb300.so")

MDG_OK = 0
STATUS_NAMES = {
    0: "MDG_OK", 1: "MDG_ERR_CONFIG", 2: "MDG_ERR_CUDA", 3: "MDG_ERR_OOM", 4: "MDG_ERR_BUDGET",
    5: "MDG_ERR_OVERLAP_LIMIT", 6: "MDG_ERR_NAN", 7: "MDG_ERR_LIST_OVERFLOW", 8: "MDG_ERR_TIMEOUT",
    9: "MDG_ERR_ARG", 10: "MDG_ERR_STATE", 11: "MDG_ERR_NODEVICE", 12: "MDG_ERR_LOST",
}

# every symbol include/mdg.h declares
EXPORTS = [
    "mdg_abi_version", "mdg_status_string", "mdg_device_count", "mdg_create", "mdg_batch_create", "mdg_destroy",
    "mdg_num_systems", "mdg_upload_state", "mdg_download_state", "mdg_set_history", "mdg_get_history",
    "mdg_step", "mdg_step_async", "mdg_step_wait", "mdg_force_only", "mdg_get_pairs", "mdg_thermo", "mdg_synchronize", "mdg_kernel_launches",
    "mdg_set_graph_mode", "mdg_timed_steps", "mdg_granular_temp_noalloc", "mdg_set_remaining",
    "mdg_get_remaining", "mdg_get_status", "mdg_configure_system", "mdg_server_create", "mdg_server_create_grouped", "mdg_server_destroy",
    "mdg_server_submit", "mdg_server_pump", "mdg_server_poll", "mdg_server_fetch", "mdg_server_context",
    "mdg_server_slot_context",
    "mdg_rsa_spheres", "mdg_counter_draw", "mdg_set_stream_priority", "mdg_generate_fcc", "mdg_generate_gas", "mdg_get_progress", "mdg_get_stream", "mdg_server_stats",
    "mdg_server_resident", "mdg_get_config", "mdg_set_threads_per_particle", "mdg_get_threads_per_particle",
    "mdg_set_build_mode", "mdg_autotune", "mdg_rdf", "mdg_msd_reset", "mdg_msd",
]


class MdgError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__(f"{what}: {STATUS_NAMES.get(status, status)}")


class Material(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "youngs_mod", "poisson_ratio", "restitution", "friction", "rolling_friction", "twisting_friction",
        "cohesion_energy", "surface_energy", "kn", "kt", "rolling_stiffness", "rolling_damping",
        "twisting_stiffness", "twisting_damping")]


class Wall(C.Structure):
    _fields_ = [("point", C.c_double * 3), ("normal", C.c_double * 3), ("bound_lo", C.c_double * 3),
                ("bound_hi", C.c_double * 3), ("velocity", C.c_double * 3), ("material", C.c_int)]


class LJPair(C.Structure):
    _fields_ = [("epsilon", C.c_double), ("sigma", C.c_double), ("cutoff", C.c_double)]


class Config(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("precision", C.c_int),
        ("box_lo", C.c_double * 3), ("box_hi", C.c_double * 3), ("dt", C.c_double),
        ("skin_fraction", C.c_double), ("bin_size", C.c_double),
        ("every", C.c_int), ("check", C.c_int), ("sort_every", C.c_int), ("newton", C.c_int),
        ("n_materials", C.c_int), ("materials", C.POINTER(Material)),
        ("contact_model", C.c_int), ("adhesion_model", C.c_int), ("rolling_model", C.c_int),
        ("twisting_model", C.c_int),
        ("lj_epsilon", C.c_double), ("lj_sigma", C.c_double), ("lj_cutoff", C.c_double),
        ("nose_hoover", C.c_int), ("nh_temperature", C.c_double), ("nh_coupling", C.c_double),
        ("virial", C.c_int),
        ("rebuild_policy", C.c_int), ("threads_per_particle", C.c_int), ("neighbor_capacity", C.c_int),
        ("history_capacity", C.c_int),
        ("langevin", C.c_int), ("lv_temperature", C.c_double), ("lv_damping", C.c_double), ("lv_seed", C.c_uint64),
        ("fixed", C.c_int * 3), ("n_walls", C.c_int), ("walls", C.POINTER(Wall)),
        ("n_lj_types", C.c_int), ("lj_pairs", C.POINTER(LJPair)),
    ]


class StateView(C.Structure):
    _fields_ = [
        ("n", C.c_size_t),
        ("tag", C.POINTER(C.c_uint32)), ("type", C.POINTER(C.c_uint32)),
        ("pos", C.POINTER(C.c_double)), ("vel", C.POINTER(C.c_double)), ("force", C.POINTER(C.c_double)),
        ("mass", C.POINTER(C.c_double)), ("cutoff_radius", C.POINTER(C.c_double)),
        ("image", C.POINTER(C.c_int32)),
        ("radius", C.POINTER(C.c_double)), ("inv_inertia", C.POINTER(C.c_double)),
        ("omega", C.POINTER(C.c_double)), ("torque", C.POINTER(C.c_double)), ("quat", C.POINTER(C.c_double)),
    ]


class Thermo(C.Structure):
    _fields_ = [
        ("ke", C.c_double), ("pe", C.c_double), ("temp", C.c_double), ("p_xi", C.c_double),
        ("granular_temp", C.c_double), ("momentum", C.c_double), ("virial", C.c_double * 6),
        ("step", C.c_int64), ("nbuilds", C.c_int64), ("n", C.c_int64), ("status", C.c_int32),
        ("max_neighbors", C.c_int32), ("e_tail", C.c_double), ("p_tail", C.c_double),
        ("rot_temp", C.c_double), ("pressure", C.c_double),
    ]


class JobInfo(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int32), ("slot", C.c_int32), ("steps", C.c_int64),
                ("n", C.c_int64), ("submit_s", C.c_double), ("start_s", C.c_double), ("end_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("particle_steps", C.c_double), ("pumps", C.c_int64), ("retired", C.c_int64),
                ("resident", C.c_int32), ("pending", C.c_int32), ("hbm_used", C.c_size_t), ("time_s", C.c_double),
                ("admit_s", C.c_double), ("step_s", C.c_double), ("retire_s", C.c_double),
                ("launches", C.c_int64), ("contexts", C.c_int32)]


GEN_MAX_TYPES = 8
VEL_MODES = {"speed": 0, "maxwell_rms": 1, "gaussian": 2}


class FccSpec(C.Structure):
    _fields_ = [("density", C.c_double), ("temperature", C.c_double), ("mass", C.c_double), ("skin", C.c_double),
                ("seed", C.c_uint64), ("n_types", C.c_int32), ("type_fractions", C.c_double * GEN_MAX_TYPES),
                ("type_masses", C.c_double * GEN_MAX_TYPES)]


class GasSpec(C.Structure):
    _fields_ = [("n", C.c_size_t), ("rmin", C.c_double), ("rmax", C.c_double), ("density", C.c_double),
                ("sep_factor", C.c_double), ("inset", C.c_int32), ("velocity_mode", C.c_int32),
                ("speed", C.c_double), ("material", C.c_uint32), ("seed", C.c_uint64),
                ("max_proposals", C.c_uint64)]


class TuneOpts(C.Structure):
    _fields_ = [("steps", C.c_int), ("tune_tpp", C.c_int), ("tune_skin", C.c_int), ("tune_bin", C.c_int)]


class TuneResult(C.Structure):
    _fields_ = [("tpp", C.c_int), ("skin_fraction", C.c_double * 2), ("bin_factor", C.c_double * 2),
                ("ms_before", C.c_double), ("ms_after", C.c_double), ("trials", C.c_int)]


class StepTiming(C.Structure):
    _fields_ = [("step_ms", C.c_double), ("phase_ms", C.c_double * 4), ("kernels", C.c_int32),
                ("rebuilt", C.c_int32)]


_lib = None


def load(path: str = LIB_PATH):
    """Load libmddem_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the CUDA extension with mddem_gb300.build.build()")
    lib = C.CDLL(path)
    P = C.POINTER
    lib.mdg_abi_version.restype = C.c_int
    lib.mdg_status_string.restype = C.c_char_p
    lib.mdg_status_string.argtypes = [C.c_int]
    lib.mdg_device_count.argtypes = [P(C.c_int)]
    lib.mdg_create.argtypes = [P(Config), C.c_size_t, P(C.c_void_p)]
    lib.mdg_batch_create.argtypes = [P(Config), P(C.c_size_t), C.c_int, P(C.c_void_p)]
    lib.mdg_destroy.argtypes = [C.c_void_p]
    lib.mdg_destroy.restype = None
    lib.mdg_num_systems.argtypes = [C.c_void_p]
    lib.mdg_upload_state.argtypes = [C.c_void_p, C.c_int, P(StateView)]
    lib.mdg_download_state.argtypes = [C.c_void_p, C.c_int, P(StateView)]
    lib.mdg_set_history.argtypes = [C.c_void_p, C.c_int, C.c_size_t, P(C.c_uint32), P(C.c_double)]
    lib.mdg_get_history.argtypes = [C.c_void_p, C.c_int, P(C.c_uint32), P(C.c_double), C.c_size_t,
                                    P(C.c_size_t)]
    lib.mdg_step.argtypes = [C.c_void_p, C.c_int64]
    lib.mdg_force_only.argtypes = [C.c_void_p]
    lib.mdg_get_pairs.argtypes = [C.c_void_p, C.c_int, P(C.c_uint32), C.c_size_t, P(C.c_size_t)]
    lib.mdg_thermo.argtypes = [C.c_void_p, C.c_int, P(Thermo)]
    lib.mdg_synchronize.argtypes = [C.c_void_p]
    lib.mdg_kernel_launches.argtypes = [C.c_void_p]
    lib.mdg_kernel_launches.restype = C.c_int64
    lib.mdg_set_graph_mode.argtypes = [C.c_void_p, C.c_int]
    lib.mdg_timed_steps.argtypes = [C.c_void_p, C.c_int64, C.c_size_t, C.POINTER(StepTiming)]
    lib.mdg_set_remaining.argtypes = [C.c_void_p, C.c_int, C.c_int64]
    lib.mdg_get_remaining.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int64)]
    lib.mdg_get_status.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int32)]
    lib.mdg_configure_system.argtypes = [C.c_void_p, C.c_int, C.POINTER(Config)]
    lib.mdg_server_create.argtypes = [C.POINTER(Config), C.POINTER(C.c_size_t), C.c_int, C.c_size_t,
                                      C.POINTER(C.c_void_p)]
    lib.mdg_server_create_grouped.argtypes = [C.POINTER(Config), C.POINTER(C.c_size_t), C.POINTER(C.c_int), C.c_int,
                                              C.c_size_t, C.POINTER(C.c_void_p)]
    lib.mdg_server_destroy.argtypes = [C.c_void_p]
    lib.mdg_server_destroy.restype = None
    lib.mdg_server_submit.argtypes = [C.c_void_p, C.POINTER(Config), C.POINTER(StateView), C.c_int64,
                                      C.POINTER(C.c_int64)]
    lib.mdg_server_pump.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.mdg_server_poll.argtypes = [C.c_void_p, C.POINTER(JobInfo), C.c_int, C.POINTER(C.c_int)]
    lib.mdg_server_fetch.argtypes = [C.c_void_p, C.c_int64, C.POINTER(StateView)]
    lib.mdg_server_context.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    lib.mdg_server_slot_context.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_int)]
    lib.mdg_step_async.argtypes = [C.c_void_p, C.c_int64]
    lib.mdg_step_wait.argtypes = [C.c_void_p]
    lib.mdg_get_progress.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
    lib.mdg_rdf.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_uint64)]
    lib.mdg_msd_reset.argtypes = [C.c_void_p, C.c_int]
    lib.mdg_msd.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    lib.mdg_set_threads_per_particle.argtypes = [C.c_void_p, C.c_int]
    lib.mdg_get_threads_per_particle.argtypes = [C.c_void_p]
    lib.mdg_set_build_mode.argtypes = [C.c_void_p, C.c_int]
    lib.mdg_autotune.argtypes = [C.c_void_p, C.POINTER(TuneOpts), C.POINTER(TuneResult)]
    lib.mdg_server_resident.argtypes = [C.c_void_p, C.POINTER(JobInfo), C.c_int, C.POINTER(C.c_int)]
    lib.mdg_server_stats.argtypes = [C.c_void_p, C.POINTER(ServerStats)]
    lib.mdg_get_stream.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    lib.mdg_rsa_spheres.argtypes = [C.c_size_t, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double,
                                    C.c_double, C.c_double, C.c_int, C.c_uint64, C.c_uint64,
                                    C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_size_t)]
    lib.mdg_set_stream_priority.argtypes = [C.c_void_p, C.c_int]
    lib.mdg_counter_draw.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64]
    lib.mdg_counter_draw.restype = C.c_uint64
    lib.mdg_generate_fcc.argtypes = [C.c_void_p, C.c_int, C.POINTER(FccSpec), C.POINTER(C.c_size_t)]
    lib.mdg_generate_gas.argtypes = [C.c_void_p, C.c_int, C.POINTER(GasSpec), C.POINTER(C.c_size_t)]
    lib.mdg_granular_temp_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
    _lib = lib
    return lib


def _check(status, what):
    if status != MDG_OK:
        raise MdgError(status, what)


def _ptr(a, ct):
    return None if a is None else a.ctypes.data_as(C.POINTER(ct))


_KIND = {"dem": 0, "lj": 1}
_PREC = {"fp64": 0, "mixed": 1}
_POLICY = {"reference": 0, "displacement": 1}


def to_c_config(c: SimConfig):
    """Fill the C struct; returns (Config, keepalive) - keep both alive."""
    mats = (Material * max(1, len(c.materials)))()
    for k, m in enumerate(c.materials):
        for f, _ in Material._fields_:
            setattr(mats[k], f, float(getattr(m, f)))
    cc = Config()
    cc.kind = _KIND[c.kind]
    cc.precision = _PREC[c.precision]
    cc.box_lo[:] = [float(x) for x in c.box_lo]
    cc.box_hi[:] = [float(x) for x in c.box_hi]
    cc.dt = float(c.dt)
    cc.skin_fraction = float(c.skin_fraction)
    cc.bin_size = float(c.bin_size)
    cc.every, cc.check, cc.sort_every, cc.newton = int(c.every), int(c.check), int(c.sort_every), int(c.newton)
    cc.n_materials = len(c.materials) if c.kind == "dem" else 0
    cc.materials = C.cast(mats, C.POINTER(Material))
    cc.contact_model = {"hertz": 0, "hooke": 1}[c.contact_model]
    cc.adhesion_model = {"jkr": 0, "dmt": 1}[c.adhesion_model]
    cc.rolling_model = {"constant": 0, "sds": 1}[c.rolling_model]
    cc.twisting_model = {"constant": 0, "sds": 1}[c.twisting_model]
    cc.lj_epsilon, cc.lj_sigma, cc.lj_cutoff = float(c.lj_epsilon), float(c.lj_sigma), float(c.lj_cutoff)
    cc.nose_hoover = int(c.nose_hoover)
    cc.nh_temperature, cc.nh_coupling = float(c.nh_temperature), float(c.nh_coupling)
    cc.virial = int(c.virial)
    cc.rebuild_policy = _POLICY[c.rebuild_policy]
    cc.threads_per_particle = int(c.threads_per_particle)
    cc.neighbor_capacity = int(c.neighbor_capacity)
    cc.history_capacity = int(c.history_capacity)
    cc.langevin = int(c.langevin)
    cc.lv_temperature, cc.lv_damping, cc.lv_seed = float(c.lv_temperature), float(c.lv_damping), int(c.lv_seed)
    cc.fixed[:] = [int(x) for x in c.fixed]
    walls = (Wall * max(1, len(c.walls)))()
    for k, w in enumerate(c.walls):
        walls[k].point[:] = [float(x) for x in w.point]
        walls[k].normal[:] = [float(x) for x in w.normal]
        walls[k].bound_lo[:] = [float(x) for x in w.bound_lo]
        walls[k].bound_hi[:] = [float(x) for x in w.bound_hi]
        walls[k].velocity[:] = [float(x) for x in w.velocity]
        walls[k].material = int(w.material)
    cc.n_walls = len(c.walls)
    cc.walls = C.cast(walls, C.POINTER(Wall))
    nt = int(c.lj_types) if c.kind == "lj" else 0
    ljp = (LJPair * max(1, nt * nt))()
    if nt > 1:
        for k, (e, s, rc) in enumerate(c.lj_pairs):
            ljp[k].epsilon, ljp[k].sigma, ljp[k].cutoff = float(e), float(s), float(rc)
    cc.n_lj_types = nt
    cc.lj_pairs = C.cast(ljp, C.POINTER(LJPair))
    return cc, (mats, walls, ljp)


def _upload_view(state):
    """StateView over a state dict (keeps the arrays alive in the returned dict)."""
    n = len(state["tag"])
    keep = {k: np.ascontiguousarray(v) for k, v in state.items() if isinstance(v, np.ndarray)}
    keep["tag"] = keep["tag"].astype(np.uint32, copy=False)
    if "type" in keep:
        keep["type"] = keep["type"].astype(np.uint32, copy=False)
    v = StateView()
    v.n = n
    v.tag = _ptr(keep["tag"], C.c_uint32)
    v.type = _ptr(keep.get("type"), C.c_uint32)
    for f in ("pos", "vel", "mass", "cutoff_radius", "radius", "inv_inertia", "omega", "quat", "force", "torque"):
        if f in keep:
            setattr(v, f, _ptr(keep[f], C.c_double))
    if "image" in keep:
        keep["image"] = keep["image"].astype(np.int32)
        v.image = _ptr(keep["image"], C.c_int32)
    return v, keep


def _download_buffers(n, dem):
    out = {
        "tag": np.zeros(n, np.uint32), "type": np.zeros(n, np.uint32), "pos": np.zeros((n, 3)),
        "vel": np.zeros((n, 3)), "force": np.zeros((n, 3)), "mass": np.zeros(n),
        "cutoff_radius": np.zeros(n), "image": np.zeros((n, 3), np.int32),
    }
    if dem:
        out.update(radius=np.zeros(n), inv_inertia=np.zeros(n), omega=np.zeros((n, 3)),
                   torque=np.zeros((n, 3)), quat=np.zeros((n, 4)))
    v = StateView()
    v.n = n
    v.tag = _ptr(out["tag"], C.c_uint32)
    v.type = _ptr(out["type"], C.c_uint32)
    v.image = _ptr(out["image"], C.c_int32)
    for f in ("pos", "vel", "force", "mass", "cutoff_radius", "radius", "inv_inertia", "omega", "torque", "quat"):
        if f in out:
            setattr(v, f, _ptr(out[f], C.c_double))
    return v, out


def rsa_spheres(n, box_lo, box_hi, rmin, rmax, sep_factor=1.1, inset=True, seed=0, max_attempts=0):
    """mdg_rsa_spheres: seeded random sequential addition (host, native)."""
    lib = load()
    pos = np.zeros((n, 3))
    rad = np.zeros(n)
    lo = (C.c_double * 3)(*box_lo)
    hi = (C.c_double * 3)(*box_hi)
    placed = C.c_size_t()
    st = lib.mdg_rsa_spheres(n, lo, hi, rmin, rmax, sep_factor, int(inset), seed, max_attempts,
                             _ptr(pos, C.c_double), _ptr(rad, C.c_double), C.byref(placed))
    if st != MDG_OK:
        raise MdgError(st, f"mdg_rsa_spheres placed {placed.value}/{n}")
    return pos, rad


def counter_draw(seed, stream, index):
    """mdg_counter_draw: draw `index` of the generators' counter-based stream."""
    return int(load().mdg_counter_draw(int(seed), int(stream), int(index)))


class Server:
    """Continuous-batching server (mdg_server_*): typed slots, HBM-budget
    admission, one multi-step device launch per pump, retirement of finished
    jobs."""

    def __init__(self, slot_configs, slot_capacities, hbm_budget, groups=None):
        """``groups``: per-slot group ids (slots of one group, one kind,
        share a batch context and stream); default one group per kind."""
        self.lib = load()
        n = len(slot_configs)
        arr = (Config * n)()
        self._keep = []
        for k, c in enumerate(slot_configs):
            cc, mats = to_c_config(c)
            arr[k] = cc
            self._keep.append(mats)
        caps = (C.c_size_t * n)(*[int(x) for x in slot_capacities])
        h = C.c_void_p()
        if groups is None:
            _check(self.lib.mdg_server_create(arr, caps, n, int(hbm_budget), C.byref(h)), "mdg_server_create")
        else:
            g = (C.c_int * n)(*[int(x) for x in groups])
            _check(self.lib.mdg_server_create_grouped(arr, caps, g, n, int(hbm_budget), C.byref(h)),
                   "mdg_server_create_grouped")
        self.h = h
        self.nslots = n
        self.slot_configs = list(slot_configs)
        self.meta = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.mdg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, cfg, state, steps):
        cc, mats = to_c_config(cfg)
        v, keep = _upload_view(state)
        jid = C.c_int64()
        _check(self.lib.mdg_server_submit(self.h, C.byref(cc), C.byref(v), int(steps), C.byref(jid)),
               "mdg_server_submit")
        self.meta[jid.value] = (cfg.kind == "dem", len(state["tag"]))
        return jid.value

    def pump(self, max_steps):
        a, p = C.c_int(), C.c_int()
        _check(self.lib.mdg_server_pump(self.h, int(max_steps), C.byref(a), C.byref(p)), "mdg_server_pump")
        return a.value, p.value

    def poll(self):
        buf = (JobInfo * 256)()
        out = []
        while True:
            n = C.c_int()
            _check(self.lib.mdg_server_poll(self.h, buf, 256, C.byref(n)), "mdg_server_poll")
            out += [{f: getattr(buf[k], f) for f, _ in JobInfo._fields_} for k in range(n.value)]
            if n.value < 256:
                return out

    def _ctx_of(self, slot):
        ctx, sys_ = C.c_void_p(), C.c_int()
        _check(self.lib.mdg_server_slot_context(self.h, int(slot), C.byref(ctx), C.byref(sys_)),
               "mdg_server_slot_context")
        return ctx.value, sys_.value

    def _view(self, handle):
        """Non-owning Context over the server's context `handle`; particle
        counts are those of the jobs resident now."""
        slots = [k for k in range(self.nslots) if self._ctx_of(k)[0] == handle]
        c = Context.__new__(Context)
        c.lib, c.h, c.owner = self.lib, C.c_void_p(handle), False
        c.nsys = len(slots)
        c.configs, c._keep, c.n = [self.slot_configs[k] for k in slots], [], [0] * len(slots)
        for r in self.resident():
            if r["slot"] in slots:
                c.n[self._ctx_of(r["slot"])[1]] = int(r["n"])
        return c

    def slot_context(self, slot):
        """(non-owning Context holding `slot`, the slot's system index in it):
        diagnostics -- timed steps, pairs, history, a resident job's state."""
        h, q = self._ctx_of(slot)
        return self._view(h), q

    def contexts(self):
        """Every batch context of the server (one per particle kind), as
        non-owning Contexts."""
        hs = []
        for k in range(self.nslots):
            h = self._ctx_of(k)[0]
            if h not in hs:
                hs.append(h)
        return [self._view(h) for h in hs]

    def download_resident(self, slot):
        """State of the job resident in `slot` now (diagnostics)."""
        c, q = self.slot_context(slot)
        return c.download(q)

    def history_resident(self, slot):
        c, q = self.slot_context(slot)
        return c.history(q)

    def pairs_resident(self, slot):
        c, q = self.slot_context(slot)
        return c.pairs(q)

    def launches(self):
        return int(self.stats()["launches"])

    def resident(self):
        buf = (JobInfo * 1024)()
        n = C.c_int()
        _check(self.lib.mdg_server_resident(self.h, buf, 1024, C.byref(n)), "mdg_server_resident")
        return [{f: getattr(buf[k], f) for f, _ in JobInfo._fields_} for k in range(min(n.value, 1024))]

    def stats(self):
        v = ServerStats()
        _check(self.lib.mdg_server_stats(self.h, C.byref(v)), "mdg_server_stats")
        return {f: getattr(v, f) for f, _ in ServerStats._fields_}

    def stream(self):
        ctx = C.c_void_p()
        _check(self.lib.mdg_server_context(self.h, C.byref(ctx)), "mdg_server_context")
        v = C.c_void_p()
        _check(self.lib.mdg_get_stream(ctx, C.byref(v)), "mdg_get_stream")
        return v.value or 0

    def fetch(self, jid):
        dem, n = self.meta.pop(jid)
        v, out = _download_buffers(n, dem)
        _check(self.lib.mdg_server_fetch(self.h, int(jid), C.byref(v)), "mdg_server_fetch")
        return out


class Context:
    """One device context advancing one or more independent systems."""

    def __init__(self, configs, capacities):
        if isinstance(configs, SimConfig):
            configs, capacities = [configs], [capacities]
        self.lib = load()
        self.configs = list(configs)
        n = len(self.configs)
        arr = (Config * n)()
        self._keep = []
        for k, c in enumerate(self.configs):
            cc, mats = to_c_config(c)
            arr[k] = cc
            self._keep.append(mats)
        caps = (C.c_size_t * n)(*[int(x) for x in capacities])
        h = C.c_void_p()
        _check(self.lib.mdg_batch_create(arr, caps, n, C.byref(h)), "mdg_batch_create")
        self.h = h
        self.nsys = n
        self.n = [0] * n

    def close(self):
        if getattr(self, "h", None) and getattr(self, "owner", True):
            self.lib.mdg_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state -------------------------------------------------------------------
    def generate_fcc(self, density, temperature, mass=1.0, skin=1.25, seed=0, sys=0, type_fractions=None,
                     type_masses=None):
        """mdg_generate_fcc: the FCC lattice of fcc_insert made on the device
        in system `sys` (cells per axis from the config's box); returns N."""
        f = FccSpec(density=float(density), temperature=float(temperature), mass=float(mass), skin=float(skin),
                    seed=int(seed))
        fr = list(type_fractions or [])
        f.n_types = len(fr)
        for k, v in enumerate(fr):
            f.type_fractions[k] = float(v)
        for k, v in enumerate(type_masses or []):
            f.type_masses[k] = float(v)
        n = C.c_size_t()
        _check(self.lib.mdg_generate_fcc(self.h, sys, C.byref(f), C.byref(n)), "mdg_generate_fcc")
        self.n[sys] = n.value
        return n.value

    def generate_gas(self, n, radius, density=2500.0, sep_factor=1.1, inset=True, velocity="speed", speed=0.5,
                     material=0, seed=0, max_proposals=0, sys=0):
        """mdg_generate_gas: the granular gas of the grid-parallel RSA made on
        the device in system `sys`; ``radius`` r or (rmin, rmax); ``velocity``
        "speed", "maxwell_rms" or "gaussian".  Returns the spheres placed."""
        rmin, rmax = (radius, radius) if not isinstance(radius, (tuple, list)) else radius
        g = GasSpec(n=int(n), rmin=float(rmin), rmax=float(rmax), density=float(density),
                    sep_factor=float(sep_factor), inset=int(bool(inset)), velocity_mode=VEL_MODES[velocity],
                    speed=float(speed), material=int(material), seed=int(seed), max_proposals=int(max_proposals))
        placed = C.c_size_t()
        st = self.lib.mdg_generate_gas(self.h, sys, C.byref(g), C.byref(placed))
        if st != MDG_OK:
            raise MdgError(st, f"mdg_generate_gas placed {placed.value}/{n}")
        self.n[sys] = int(n)
        return placed.value

    def upload(self, state, sys=0):
        n = len(state["tag"])
        keep = {k: np.ascontiguousarray(v) for k, v in state.items() if isinstance(v, np.ndarray)}
        v = StateView()
        v.n = n
        v.tag = _ptr(keep["tag"].astype(np.uint32, copy=False), C.c_uint32)
        t = keep.get("type")
        v.type = _ptr(t.astype(np.uint32, copy=False), C.c_uint32) if t is not None else None
        v.pos = _ptr(keep["pos"], C.c_double)
        v.vel = _ptr(keep["vel"], C.c_double)
        v.mass = _ptr(keep["mass"], C.c_double)
        v.cutoff_radius = _ptr(keep["cutoff_radius"], C.c_double)
        if "image" in keep:
            keep["image"] = keep["image"].astype(np.int32)
            v.image = _ptr(keep["image"], C.c_int32)
        for f in ("radius", "inv_inertia", "omega", "quat", "force", "torque"):
            if f in keep:
                setattr(v, f, _ptr(keep[f], C.c_double))
        _check(self.lib.mdg_upload_state(self.h, sys, C.byref(v)), "mdg_upload_state")
        self.n[sys] = n

    def download(self, sys=0):
        n = self.n[sys]
        dem = self.configs[sys].kind == "dem"
        out = {
            "tag": np.zeros(n, np.uint32), "type": np.zeros(n, np.uint32), "pos": np.zeros((n, 3)),
            "vel": np.zeros((n, 3)), "force": np.zeros((n, 3)), "mass": np.zeros(n),
            "cutoff_radius": np.zeros(n), "image": np.zeros((n, 3), np.int32),
        }
        if dem:
            out.update(radius=np.zeros(n), inv_inertia=np.zeros(n), omega=np.zeros((n, 3)),
                       torque=np.zeros((n, 3)), quat=np.zeros((n, 4)))
        v = StateView()
        v.n = n
        v.tag = _ptr(out["tag"], C.c_uint32)
        v.type = _ptr(out["type"], C.c_uint32)
        v.image = _ptr(out["image"], C.c_int32)
        for f in ("pos", "vel", "force", "mass", "cutoff_radius", "radius", "inv_inertia", "omega", "torque", "quat"):
            if f in out:
                setattr(v, f, _ptr(out[f], C.c_double))
        _check(self.lib.mdg_download_state(self.h, sys, C.byref(v)), "mdg_download_state")
        return out

    def step(self, nsteps=1):
        _check(self.lib.mdg_step(self.h, int(nsteps)), "mdg_step")

    def force_only(self):
        _check(self.lib.mdg_force_only(self.h), "mdg_force_only")

    def pairs(self, sys=0):
        cnt = C.c_size_t()
        _check(self.lib.mdg_get_pairs(self.h, sys, None, 0, C.byref(cnt)), "mdg_get_pairs")
        buf = np.zeros((max(1, cnt.value), 2), np.uint32)
        _check(self.lib.mdg_get_pairs(self.h, sys, _ptr(buf, C.c_uint32), cnt.value, C.byref(cnt)),
               "mdg_get_pairs")
        return buf[: cnt.value]

    def history(self, sys=0):
        cnt = C.c_size_t()
        _check(self.lib.mdg_get_history(self.h, sys, None, None, 0, C.byref(cnt)), "mdg_get_history")
        keys = np.zeros((max(1, cnt.value), 2), np.uint32)
        vals = np.zeros((max(1, cnt.value), 7))
        _check(self.lib.mdg_get_history(self.h, sys, _ptr(keys, C.c_uint32), _ptr(vals, C.c_double), cnt.value,
                                        C.byref(cnt)), "mdg_get_history")
        return keys[: cnt.value], vals[: cnt.value]

    def set_history(self, keys, vals, sys=0):
        keys = np.ascontiguousarray(keys, np.uint32)
        vals = np.ascontiguousarray(vals, np.float64)
        _check(self.lib.mdg_set_history(self.h, sys, len(keys), _ptr(keys, C.c_uint32), _ptr(vals, C.c_double)),
               "mdg_set_history")

    def thermo(self, sys=0):
        t = Thermo()
        _check(self.lib.mdg_thermo(self.h, sys, C.byref(t)), "mdg_thermo")
        return {f: (list(getattr(t, f)) if f == "virial" else getattr(t, f)) for f, _ in Thermo._fields_}

    def synchronize(self):
        _check(self.lib.mdg_synchronize(self.h), "mdg_synchronize")

    def launches(self):
        return int(self.lib.mdg_kernel_launches(self.h))

    def timed_steps(self, nsteps, l2_flush_bytes=0):
        """Per-step device timings (ms): array (nsteps, 5) = step, initial,
        rebuild, force, final; plus kernels per step and rebuild flags."""
        buf = (StepTiming * max(1, nsteps))()
        _check(self.lib.mdg_timed_steps(self.h, int(nsteps), int(l2_flush_bytes), buf), "mdg_timed_steps")
        t = np.array([[b.step_ms, *b.phase_ms] for b in buf[:nsteps]])
        return t, np.array([b.kernels for b in buf[:nsteps]]), np.array([b.rebuilt for b in buf[:nsteps]])

    def configure(self, cfg, sys=0):
        cc, mats = to_c_config(cfg)
        self._keep.append(mats)
        _check(self.lib.mdg_configure_system(self.h, sys, C.byref(cc)), "mdg_configure_system")
        self.configs[sys] = cfg

    def status(self, sys=0):
        v = C.c_int32()
        _check(self.lib.mdg_get_status(self.h, sys, C.byref(v)), "mdg_get_status")
        return v.value

    def autotune(self, steps=40, tpp=True, skin=True, bins=True):
        """mdg_autotune: pick threads per particle, skin fraction and bin size
        by trial runs; call after upload, before the first step."""
        o = TuneOpts(steps, int(tpp), int(skin), int(bins))
        r = TuneResult()
        _check(self.lib.mdg_autotune(self.h, C.byref(o), C.byref(r)), "mdg_autotune")
        return {"tpp": r.tpp, "skin_fraction": list(r.skin_fraction), "bin_factor": list(r.bin_factor),
                "ms_before": r.ms_before, "ms_after": r.ms_after, "trials": r.trials}

    def rdf(self, sys=0, r_max=3.0, nbins=200):
        """mdg_rdf: (r_low, g, counts) with the reference's normalisation
        g_k = counts_k V / (N (N-1)/2 x shell_k) (md_measure/src/lib.rs:420-440)."""
        counts = np.zeros(nbins, np.uint64)
        _check(self.lib.mdg_rdf(self.h, sys, float(r_max), int(nbins), _ptr(counts, C.c_uint64)), "mdg_rdf")
        cfg = self.configs[sys]
        vol = float(np.prod(cfg.box))
        n = float(self.thermo(sys)["n"])
        dr = r_max / nbins
        k = np.arange(nbins, dtype=np.float64)
        shell = (4.0 / 3.0) * np.pi * (((k + 1) * dr) ** 3 - (k * dr) ** 3)
        npairs = n * (n - 1.0) / 2.0
        g = counts.astype(np.float64) * vol / (npairs * shell)
        return k * dr, g, counts

    def msd_reset(self, sys=0):
        _check(self.lib.mdg_msd_reset(self.h, sys), "mdg_msd_reset")

    def msd(self, sys=0):
        v = C.c_double()
        _check(self.lib.mdg_msd(self.h, sys, C.byref(v)), "mdg_msd")
        return v.value

    def stream_priority(self, priority):
        """mdg_set_stream_priority: run on a new stream of CUDA priority
        `priority` (lower first, clamped to the device's range)."""
        _check(self.lib.mdg_set_stream_priority(self.h, int(priority)), "mdg_set_stream_priority")

    def threads_per_particle(self, tpp=None):
        if tpp is not None:
            _check(self.lib.mdg_set_threads_per_particle(self.h, int(tpp)), "mdg_set_threads_per_particle")
        return int(self.lib.mdg_get_threads_per_particle(self.h))

    def build_mode(self, mode):
        """List-build work split of every system: 0 warp per bin, 1 warp per
        particle, 2 thread per particle, -1 automatic (same rows in all)."""
        _check(self.lib.mdg_set_build_mode(self.h, int(mode)), "mdg_set_build_mode")

    def stream(self):
        """The context's CUDA stream handle (as an int), for events and
        ordering with the caller's own work."""
        v = C.c_void_p()
        _check(self.lib.mdg_get_stream(self.h, C.byref(v)), "mdg_get_stream")
        return v.value or 0

    def progress(self):
        """(remaining, status, step) arrays over all systems, one device read."""
        n = self.nsys
        rem, sta, stp = np.zeros(n, np.int64), np.zeros(n, np.int32), np.zeros(n, np.int64)
        _check(self.lib.mdg_get_progress(self.h, _ptr(rem, C.c_int64), _ptr(sta, C.c_int32), _ptr(stp, C.c_int64)),
               "mdg_get_progress")
        return rem, sta, stp

    def set_remaining(self, steps, sys=0):
        _check(self.lib.mdg_set_remaining(self.h, sys, int(steps)), "mdg_set_remaining")

    def remaining(self, sys=0):
        v = C.c_int64()
        _check(self.lib.mdg_get_remaining(self.h, sys, C.byref(v)), "mdg_get_remaining")
        return v.value

    def set_graph_mode(self, on):
        _check(self.lib.mdg_set_graph_mode(self.h, int(on)), "mdg_set_graph_mode")
