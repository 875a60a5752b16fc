"""Restart files in the reference's format (the on-disk state either side of a run).

The reference writes `RestartData` (crates/mddem_print/src/lib.rs:297-376) per
rank as `restart_{step}_rank{rank}.bin` (bincode) or `.json` (serde_json)
(lib.rs:1050-1066).  Field order: natoms u64, total_cycle u64, dt f64, tag
[u32], atom_type [u32], pos_x/y/z, vel_x/y/z, force_x/y/z, mass,
cutoff_radius [f64], atom_data_buffers [[f64]] (one buffer per registered
per-atom extension, crates/mddem_core/src/atom.rs:255-284), then the legacy
omega/torque/ang_mom x/y/z [f64] and quaternion [[f64; 4]] (written empty).

bincode 1.3.3 (Cargo.lock) with its default options: little-endian,
fixed-width integers, every sequence prefixed by its length as u64, fixed-size
arrays without a prefix, usize as u64.

Extensions, in registration order for the granular plugins: DemAtom (the
AtomData derive packs fields in declaration order, crates/mddem_derive/src/
lib.rs:244-245: radius, density, inv_inertia, quaternion[4], omega[3],
ang_mom[3], torque[3], body_id = 17 doubles per atom, dem_atom/src/lib.rs:
530-557), then ContactHistoryStore (dem_granular/src/tangential.rs:98-132:
per atom its contact count, then partner tag and the 7 spring values of each
contact).  LJ systems carry no extension.

States are the dicts of ``inputs`` / ``capi.Context.download`` (positions,
velocities, ... indexed in the file's atom order); history is (keys, vals)
as ``capi.Context.history`` returns: (owner tag, partner tag) and the 7
doubles of the reference's canonical frame.
"""
from __future__ import annotations

import json
import math
import struct

import numpy as np

DEM_PACK = 17

_VEC3 = ("pos", "vel", "force")


def _density(st):
    if "density" in st:
        return np.asarray(st["density"], dtype=np.float64)
    r = np.asarray(st["radius"], dtype=np.float64)
    return np.asarray(st["mass"], dtype=np.float64) / (4.0 / 3.0 * math.pi * r ** 3)


def restart_fields(state, history=None, step=0, dt=0.0):
    """The RestartData fields (ordered dict) of one system's state."""
    n = len(state["tag"])
    f = {"natoms": n, "total_cycle": int(step), "dt": float(dt),
         "tag": np.asarray(state["tag"], dtype=np.uint32),
         "atom_type": np.asarray(state.get("type", np.zeros(n, np.uint32)), dtype=np.uint32)}
    for k in _VEC3:
        a = np.asarray(state.get(k, np.zeros((n, 3))), dtype=np.float64).reshape(n, 3)
        for c, ax in enumerate("xyz"):
            f[f"{k}_{ax}"] = np.ascontiguousarray(a[:, c])
    f["mass"] = np.asarray(state["mass"], dtype=np.float64)
    f["cutoff_radius"] = np.asarray(state["cutoff_radius"], dtype=np.float64)
    bufs = []
    if "radius" in state:
        dem = np.zeros((n, DEM_PACK))
        dem[:, 0] = state["radius"]
        dem[:, 1] = _density(state)
        dem[:, 2] = state["inv_inertia"]
        dem[:, 3:7] = state.get("quat", np.tile([1.0, 0.0, 0.0, 0.0], (n, 1)))
        dem[:, 7:10] = state.get("omega", np.zeros((n, 3)))
        dem[:, 10:13] = state.get("ang_mom", np.zeros((n, 3)))
        dem[:, 13:16] = state.get("torque", np.zeros((n, 3)))
        dem[:, 16] = state.get("body_id", np.zeros(n))
        bufs.append(dem.ravel())
        # contact history, grouped under each atom in the file's atom order
        per = {}
        if history is not None:
            keys, vals = history
            for (o, p), v in zip(np.asarray(keys).tolist(), np.asarray(vals)):
                per.setdefault(int(o), []).append((int(p), v))
        h = []
        for t in f["tag"].tolist():
            lst = per.get(int(t), [])
            h.append(float(len(lst)))
            for p, v in lst:
                h.append(float(p))
                h.extend(float(x) for x in v)
        bufs.append(np.asarray(h, dtype=np.float64))
    f["atom_data_buffers"] = bufs
    for k in ("omega", "torque", "ang_mom"):
        for ax in "xyz":
            f[f"{k}_{ax}"] = np.zeros(0)
    f["quaternion"] = np.zeros((0, 4))
    return f


def _bincode(f):
    out = [struct.pack("<QQd", f["natoms"], f["total_cycle"], f["dt"])]

    def seq(a, fmt):
        a = np.ascontiguousarray(a)
        out.append(struct.pack("<Q", len(a)))
        out.append(a.astype(fmt, copy=False).tobytes())

    seq(f["tag"], "<u4")
    seq(f["atom_type"], "<u4")
    for k in _VEC3:
        for ax in "xyz":
            seq(f[f"{k}_{ax}"], "<f8")
    seq(f["mass"], "<f8")
    seq(f["cutoff_radius"], "<f8")
    out.append(struct.pack("<Q", len(f["atom_data_buffers"])))
    for b in f["atom_data_buffers"]:
        seq(b, "<f8")
    for k in ("omega", "torque", "ang_mom"):
        for ax in "xyz":
            seq(f[f"{k}_{ax}"], "<f8")
    q = np.ascontiguousarray(f["quaternion"], dtype="<f8").reshape(-1, 4)
    out.append(struct.pack("<Q", len(q)))
    out.append(q.tobytes())
    return b"".join(out)


def _from_bincode(b):
    off = 0

    def take(fmt):
        nonlocal off
        v = struct.unpack_from(fmt, b, off)
        off += struct.calcsize(fmt)
        return v

    def seq(dtype, width=1):
        nonlocal off
        (m,) = take("<Q")
        nbytes = m * width * np.dtype(dtype).itemsize
        a = np.frombuffer(b, dtype=dtype, count=m * width, offset=off).copy()
        off += nbytes
        return a.reshape(m, width) if width > 1 else a

    natoms, cycle, dt = take("<QQd")
    f = {"natoms": natoms, "total_cycle": cycle, "dt": dt, "tag": seq("<u4"), "atom_type": seq("<u4")}
    for k in _VEC3:
        for ax in "xyz":
            f[f"{k}_{ax}"] = seq("<f8")
    f["mass"] = seq("<f8")
    f["cutoff_radius"] = seq("<f8")
    (nb,) = take("<Q")
    f["atom_data_buffers"] = [seq("<f8") for _ in range(nb)]
    for k in ("omega", "torque", "ang_mom"):
        for ax in "xyz":
            f[f"{k}_{ax}"] = seq("<f8")
    f["quaternion"] = seq("<f8", 4)
    if off != len(b):
        raise ValueError(f"restart: {len(b) - off} trailing bytes")
    return f


def _to_json(f):
    d = {}
    for k, v in f.items():
        if k == "atom_data_buffers":
            d[k] = [np.asarray(x).tolist() for x in v]
        elif isinstance(v, np.ndarray):
            d[k] = v.tolist()
        else:
            d[k] = v
    return json.dumps(d)


def _from_json(text):
    d = json.loads(text)
    f = {"natoms": int(d["natoms"]), "total_cycle": int(d["total_cycle"]), "dt": float(d["dt"]),
         "tag": np.asarray(d["tag"], dtype=np.uint32), "atom_type": np.asarray(d["atom_type"], dtype=np.uint32)}
    for k, v in d.items():
        if k in f:
            continue
        if k == "atom_data_buffers":
            f[k] = [np.asarray(x, dtype=np.float64) for x in v]
        elif k == "quaternion":
            f[k] = np.asarray(v, dtype=np.float64).reshape(-1, 4)
        else:
            f[k] = np.asarray(v, dtype=np.float64)
    for k in ("omega", "torque", "ang_mom"):
        for ax in "xyz":
            f.setdefault(f"{k}_{ax}", np.zeros(0))
    f.setdefault("quaternion", np.zeros((0, 4)))
    return f


def fields_to_state(f):
    """(state dict, history (keys, vals) or None, step, dt) from RestartData
    fields; reads the DemAtom and contact-history buffers, or the legacy
    rotational fields of old files."""
    n = len(f["tag"])
    st = {"tag": f["tag"], "type": f["atom_type"], "mass": f["mass"], "cutoff_radius": f["cutoff_radius"]}
    for k in _VEC3:
        st[k] = np.stack([f[f"{k}_{ax}"] for ax in "xyz"], axis=1) if n else np.zeros((0, 3))
    hist = None
    bufs = f["atom_data_buffers"]
    if bufs and len(bufs[0]) == DEM_PACK * n and n:
        dem = np.asarray(bufs[0]).reshape(n, DEM_PACK)
        st.update(radius=dem[:, 0].copy(), density=dem[:, 1].copy(), inv_inertia=dem[:, 2].copy(),
                  quat=dem[:, 3:7].copy(), omega=dem[:, 7:10].copy(), ang_mom=dem[:, 10:13].copy(),
                  torque=dem[:, 13:16].copy(), body_id=dem[:, 16].copy())
        if len(bufs) > 1:
            h = np.asarray(bufs[1])
            keys, vals, pos = [], [], 0
            for t in f["tag"].tolist():
                if pos >= len(h):
                    raise ValueError("restart: contact-history buffer too short")
                craw = float(h[pos])
                pos += 1
                # a whole number >= 0 whose entries (8 doubles each) fit in the buffer
                if not (math.isfinite(craw) and craw >= 0 and craw == math.floor(craw)
                        and craw <= (len(h) - pos) // 8):
                    raise ValueError("restart: contact-history count is not a whole number within the buffer")
                cnt = int(craw)
                for _ in range(cnt):
                    keys.append((t, int(h[pos])))
                    vals.append(h[pos + 1:pos + 8])
                    pos += 8
            if pos != len(h):
                raise ValueError("restart: contact-history buffer length does not match its counts")
            hist = (np.asarray(keys, dtype=np.uint32).reshape(-1, 2), np.asarray(vals).reshape(-1, 7))
    elif len(f.get("omega_x", [])) == n and n:
        st["omega"] = np.stack([f["omega_x"], f["omega_y"], f["omega_z"]], axis=1)
        if len(f.get("torque_x", [])) == n:
            st["torque"] = np.stack([f["torque_x"], f["torque_y"], f["torque_z"]], axis=1)
        if len(f.get("quaternion", [])) == n:
            st["quat"] = np.asarray(f["quaternion"])
    return st, hist, int(f["total_cycle"]), float(f["dt"])


def restart_filename(step, rank=0, fmt="bincode"):
    return f"restart_{step}_rank{rank}." + ("json" if fmt == "json" else "bin")


def write_restart(path, state, history=None, step=0, dt=0.0, fmt="bincode"):
    """Write one system's state in the reference's restart format."""
    f = restart_fields(state, history, step, dt)
    if fmt == "json":
        with open(path, "w") as fh:
            fh.write(_to_json(f))
    else:
        with open(path, "wb") as fh:
            fh.write(_bincode(f))


def read_restart(path):
    """(state, history or None, step, dt) from a restart file (format from
    the extension: .json, else bincode)."""
    if str(path).endswith(".json"):
        with open(path) as fh:
            return fields_to_state(_from_json(fh.read()))
    with open(path, "rb") as fh:
        return fields_to_state(_from_bincode(fh.read()))
