"""ctypes wrapper of the CPU FP64 oracle (oracle/mdg_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  Never imported by the product
package.  Parity pin: see mdg_oracle.h (known-answer tests from the
reference's unit tests; the reference itself is Rust and cannot be built).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libmdg_oracle.so")


def build(verbose=False):
    src = os.path.join(HERE, "mdg_oracle.cpp")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(src),
                                                          os.path.getmtime(os.path.join(HERE, "mdg_oracle.h"))):
        return LIB
    r = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if verbose or r.returncode:
        print(r.stdout, r.stderr)
    if r.returncode:
        raise RuntimeError("oracle build failed")
    return LIB


class OrcMaterial(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "youngs_mod", "poisson_ratio", "restitution", "friction", "rolling_friction", "twisting_friction",
        "cohesion_energy", "surface_energy", "kn", "kt", "rolling_stiffness", "rolling_damping",
        "twisting_stiffness", "twisting_damping")]


class OrcWall(C.Structure):
    _fields_ = [("point", C.c_double * 3), ("normal", C.c_double * 3), ("bound_lo", C.c_double * 3),
                ("bound_hi", C.c_double * 3), ("velocity", C.c_double * 3), ("material", C.c_int)]


class OrcLJPair(C.Structure):
    _fields_ = [("epsilon", C.c_double), ("sigma", C.c_double), ("cutoff", C.c_double)]


class OrcConfig(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("lo", C.c_double * 3), ("hi", C.c_double * 3), ("dt", C.c_double),
        ("skin_fraction", C.c_double), ("bin_size", C.c_double),
        ("every", C.c_int), ("check", C.c_int), ("sort_every", C.c_int), ("newton", C.c_int),
        ("n_materials", C.c_int), ("materials", C.POINTER(OrcMaterial)),
        ("contact_model", C.c_int), ("adhesion_model", C.c_int), ("rolling_model", C.c_int),
        ("twisting_model", C.c_int),
        ("lj_epsilon", C.c_double), ("lj_sigma", C.c_double), ("lj_cutoff", C.c_double),
        ("nose_hoover", C.c_int), ("nh_temperature", C.c_double), ("nh_coupling", C.c_double),
        ("virial", C.c_int),
        ("fixed", C.c_int * 3), ("n_walls", C.c_int), ("walls", C.POINTER(OrcWall)),
        ("langevin", C.c_int), ("lv_temperature", C.c_double), ("lv_damping", C.c_double),
        ("lv_seed", C.c_uint64), ("n_lj_types", C.c_int), ("lj_pairs", C.POINTER(OrcLJPair)),
    ]


F_POS, F_VEL, F_FORCE, F_OMEGA, F_TORQUE, F_QUAT, F_MASS, F_RADIUS, F_LBP = range(9)
_lib = None


def _load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        P = C.POINTER
        lib.orc_create.restype = C.c_void_p
        lib.orc_create.argtypes = [P(OrcConfig)]
        lib.orc_destroy.argtypes = [C.c_void_p]
        lib.orc_load.argtypes = [C.c_void_p, C.c_size_t, P(C.c_uint32), P(C.c_uint32)] + [P(C.c_double)] * 9
        lib.orc_step.argtypes = [C.c_void_p, C.c_long]
        lib.orc_set_force.argtypes = [C.c_void_p, C.c_size_t, P(C.c_double), P(C.c_double)]
        lib.orc_force_only.argtypes = [C.c_void_p]
        lib.orc_nlocal.argtypes = [C.c_void_p]
        lib.orc_nlocal.restype = C.c_size_t
        lib.orc_get_field.argtypes = [C.c_void_p, C.c_int, P(C.c_double)]
        lib.orc_get_tags.argtypes = [C.c_void_p, P(C.c_uint32)]
        lib.orc_get_types.argtypes = [C.c_void_p, P(C.c_uint32)]
        lib.orc_get_scale.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
        lib.orc_rsa_spheres.argtypes = [C.c_size_t, P(C.c_double), P(C.c_double), C.c_double, C.c_double,
                                        C.c_double, C.c_int, C.c_uint64, C.c_uint64, P(C.c_double), P(C.c_double),
                                        P(C.c_size_t)]
        lib.orc_get_image.argtypes = [C.c_void_p, P(C.c_int32)]
        lib.orc_get_pairs.argtypes = [C.c_void_p, P(C.c_uint32), C.c_size_t]
        lib.orc_get_pairs.restype = C.c_size_t
        lib.orc_get_history.argtypes = [C.c_void_p, P(C.c_uint32), P(C.c_double), C.c_size_t]
        lib.orc_get_history.restype = C.c_size_t
        lib.orc_set_history.argtypes = [C.c_void_p, C.c_size_t, P(C.c_uint32), P(C.c_double)]
        lib.orc_thermo.argtypes = [C.c_void_p, P(C.c_double)]
        lib.orc_overlap_count.argtypes = [C.c_void_p]
        lib.orc_overlap_count.restype = C.c_long
        _lib = lib
    return _lib


def rsa_spheres(n, box_lo, box_hi, rmin, rmax, sep_factor=1.1, inset=True, seed=0, max_attempts=0):
    """Seeded random sequential addition of spheres by the oracle: the same
    spheres as the library's mdg_rsa_spheres for the same arguments, made
    without loading the library (inputs of the CPU arm)."""
    lib = _load()
    pos = np.zeros((n, 3))
    rad = np.zeros(n)
    lo = (C.c_double * 3)(*box_lo)
    hi = (C.c_double * 3)(*box_hi)
    placed = C.c_size_t()
    r = lib.orc_rsa_spheres(n, lo, hi, rmin, rmax, sep_factor, int(inset), seed, max_attempts,
                            pos.ctypes.data_as(C.POINTER(C.c_double)), rad.ctypes.data_as(C.POINTER(C.c_double)),
                            C.byref(placed))
    if r:
        raise RuntimeError(f"orc_rsa_spheres placed {placed.value}/{n}")
    return pos, rad


def _p(a, ct=C.c_double):
    return None if a is None else np.ascontiguousarray(a).ctypes.data_as(C.POINTER(ct))


class Oracle:
    """One CPU simulation following the reference's single-rank schedule."""

    def __init__(self, cfg):
        self.lib = _load()
        mats = (OrcMaterial * max(1, len(cfg.materials)))()
        for k, m in enumerate(cfg.materials):
            for f, _ in OrcMaterial._fields_:
                setattr(mats[k], f, float(getattr(m, f)))
        c = OrcConfig()
        c.kind = 0 if cfg.kind == "dem" else 1
        c.lo[:] = [float(x) for x in cfg.box_lo]
        c.hi[:] = [float(x) for x in cfg.box_hi]
        c.dt = float(cfg.dt)
        c.skin_fraction, c.bin_size = float(cfg.skin_fraction), float(cfg.bin_size)
        c.every, c.check, c.sort_every, c.newton = int(cfg.every), int(cfg.check), int(cfg.sort_every), int(cfg.newton)
        c.n_materials = len(cfg.materials) if cfg.kind == "dem" else 0
        c.materials = C.cast(mats, C.POINTER(OrcMaterial))
        c.contact_model = {"hertz": 0, "hooke": 1}[cfg.contact_model]
        c.adhesion_model = {"jkr": 0, "dmt": 1}[cfg.adhesion_model]
        c.rolling_model = {"constant": 0, "sds": 1}[cfg.rolling_model]
        c.twisting_model = {"constant": 0, "sds": 1}[cfg.twisting_model]
        c.lj_epsilon, c.lj_sigma, c.lj_cutoff = float(cfg.lj_epsilon), float(cfg.lj_sigma), float(cfg.lj_cutoff)
        c.nose_hoover = int(cfg.nose_hoover)
        c.nh_temperature, c.nh_coupling = float(cfg.nh_temperature), float(cfg.nh_coupling)
        c.virial = int(cfg.virial)
        c.fixed[:] = [int(x) for x in getattr(cfg, "fixed", (0, 0, 0))]
        wl = list(getattr(cfg, "walls", ()))
        walls = (OrcWall * max(1, len(wl)))()
        for k, w in enumerate(wl):
            for f in ("point", "normal", "bound_lo", "bound_hi", "velocity"):
                getattr(walls[k], f)[:] = [float(x) for x in getattr(w, f)]
            walls[k].material = int(w.material)
        c.n_walls = len(wl) if cfg.kind == "dem" else 0
        c.walls = C.cast(walls, C.POINTER(OrcWall))
        c.langevin = int(getattr(cfg, "langevin", False))
        c.lv_temperature = float(getattr(cfg, "lv_temperature", 0.85))
        c.lv_damping = float(getattr(cfg, "lv_damping", 1.0))
        c.lv_seed = int(getattr(cfg, "lv_seed", 12345))
        nt = int(getattr(cfg, "lj_types", 0)) if cfg.kind == "lj" else 0
        ljp = (OrcLJPair * max(1, nt * nt))()
        if nt > 1:
            for k, (e, s, rc) in enumerate(cfg.lj_pairs):
                ljp[k].epsilon, ljp[k].sigma, ljp[k].cutoff = float(e), float(s), float(rc)
        c.n_lj_types = nt
        c.lj_pairs = C.cast(ljp, C.POINTER(OrcLJPair))
        self._mats = mats
        self.h = self.lib.orc_create(C.byref(c))
        self.kind = cfg.kind

    def close(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, st):
        n = len(st["tag"])
        keep = {k: np.ascontiguousarray(v) for k, v in st.items() if isinstance(v, np.ndarray)}
        self._keep = keep
        dem = self.kind == "dem"
        r = self.lib.orc_load(
            self.h, n, _p(keep["tag"].astype(np.uint32), C.c_uint32), _p(keep["type"].astype(np.uint32), C.c_uint32),
            _p(keep["pos"]), _p(keep["vel"]), _p(keep["mass"]), _p(keep["cutoff_radius"]),
            _p(keep.get("radius")) if dem else None, _p(keep.get("density")) if dem else None,
            _p(keep.get("inv_inertia")) if dem else None, _p(keep.get("omega")) if dem else None,
            _p(keep.get("quat")) if dem else None)
        if r:
            raise RuntimeError(f"orc_load failed: {r}")
        for f in ("force", "torque"):
            if f in keep:
                for i in range(n):
                    row = np.ascontiguousarray(keep[f][i], np.float64)
                    args = (row, None) if f == "force" else (None, row)
                    self.lib.orc_set_force(self.h, i, _p(args[0]), _p(args[1]))

    def step(self, n=1):
        r = self.lib.orc_step(self.h, int(n))
        if r:
            raise RuntimeError(f"oracle step error {r}")

    def force_only(self):
        r = self.lib.orc_force_only(self.h)
        if r:
            raise RuntimeError(f"oracle force error {r}")

    @property
    def n(self):
        return int(self.lib.orc_nlocal(self.h))

    def field(self, f, width=3):
        out = np.zeros((self.n, width)) if width > 1 else np.zeros(self.n)
        self.lib.orc_get_field(self.h, f, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def state(self):
        n = self.n
        tags = np.zeros(n, np.uint32)
        self.lib.orc_get_tags(self.h, tags.ctypes.data_as(C.POINTER(C.c_uint32)))
        types = np.zeros(n, np.uint32)
        self.lib.orc_get_types(self.h, types.ctypes.data_as(C.POINTER(C.c_uint32)))
        img = np.zeros((n, 3), np.int32)
        self.lib.orc_get_image(self.h, img.ctypes.data_as(C.POINTER(C.c_int32)))
        st = {"tag": tags, "type": types, "pos": self.field(F_POS), "vel": self.field(F_VEL),
              "force": self.field(F_FORCE), "image": img, "mass": self.field(F_MASS, 1)}
        if self.kind == "dem":
            st.update(omega=self.field(F_OMEGA), torque=self.field(F_TORQUE), quat=self.field(F_QUAT, 4),
                      radius=self.field(F_RADIUS, 1))
        return st

    def pair_scale(self):
        """Per local atom (storage order, like state()): the sums over its
        pairs of |f_pair| and |tau_pair| at the last force evaluation."""
        fs, ts = np.zeros(self.n), np.zeros(self.n)
        self.lib.orc_get_scale(self.h, fs.ctypes.data_as(C.POINTER(C.c_double)),
                               ts.ctypes.data_as(C.POINTER(C.c_double)))
        return fs, ts

    def pairs(self):
        n = self.lib.orc_get_pairs(self.h, None, 0)
        buf = np.zeros((max(1, n), 2), np.uint32)
        self.lib.orc_get_pairs(self.h, buf.ctypes.data_as(C.POINTER(C.c_uint32)), n)
        return buf[:n]

    def history(self):
        n = self.lib.orc_get_history(self.h, None, None, 0)
        k = np.zeros((max(1, n), 2), np.uint32)
        v = np.zeros((max(1, n), 7))
        self.lib.orc_get_history(self.h, k.ctypes.data_as(C.POINTER(C.c_uint32)),
                                 v.ctypes.data_as(C.POINTER(C.c_double)), n)
        return k[:n], v[:n]

    def set_history(self, keys, vals):
        keys = np.ascontiguousarray(keys, np.uint32)
        vals = np.ascontiguousarray(vals, np.float64)
        r = self.lib.orc_set_history(self.h, len(keys), keys.ctypes.data_as(C.POINTER(C.c_uint32)),
                                     vals.ctypes.data_as(C.POINTER(C.c_double)))
        if r:
            raise RuntimeError("orc_set_history failed")

    def thermo(self):
        out = np.zeros(16)
        self.lib.orc_thermo(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        keys = ["ke", "pe", "temp", "p_xi", "granular_temp", "momentum"]
        d = {k: float(out[i]) for i, k in enumerate(keys)}
        d["virial"] = list(out[6:12])
        d["nbuilds"] = int(out[12])
        d["step"] = int(out[13])
        return d

    def lj_tails(self):
        e, p = C.c_double(), C.c_double()
        self.lib.orc_lj_tails(self.h, C.byref(e), C.byref(p))
        return e.value, p.value

    def overlaps(self):
        return int(self.lib.orc_overlap_count(self.h))
