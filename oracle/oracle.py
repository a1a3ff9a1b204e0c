"""ctypes loader of the oracle -- TEST INFRASTRUCTURE, NOT THE PRODUCT.

The oracle (oracle/blobs_oracle.cpp) is a CPU restatement of the reference
blobs step (darthdeus/blobs 0.2.1, blobs/src/physics.rs) used only as the
checker by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
Parity of the step is unpinned by the reference (it ships no step test or
golden vector); the spatial hash and transform composition are pinned by the
reference's own tests (tests/test_oracle_kat.py).
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_P = ctypes.c_void_p


class OracleScene(ctypes.Structure):
    _fields_ = [
        ("gravity", ctypes.c_double * 2), ("substeps", ctypes.c_uint32), ("joint_iterations", ctypes.c_uint32),
        ("collisions_enabled", ctypes.c_uint32), ("maintain_spatial_hash", ctypes.c_uint32),
        ("record_events", ctypes.c_uint32), ("old_dt", ctypes.c_double),
        ("n_bodies", ctypes.c_uint32), ("pos", _P), ("pos_old", _P), ("acc", _P), ("vel", _P), ("vreq", _P),
        ("vreq_set", _P), ("body_type", _P), ("rotation", _P), ("angvel", _P), ("torque", _P),
        ("gravity_mod", _P), ("mass", _P), ("inertia", _P), ("bound_radius", _P),
        ("n_colliders", ctypes.c_uint32), ("col_parent", _P), ("col_offset", _P), ("col_radius", _P),
        ("col_mass_override", _P), ("col_sensor", _P), ("col_memb", _P), ("col_filt", _P), ("col_snap", _P),
        ("n_springs", ctypes.c_uint32), ("spr_a", _P), ("spr_b", _P), ("spr_rest", _P), ("spr_k", _P),
        ("spr_c", _P),
        ("n_joints", ctypes.c_uint32), ("jnt_a", _P), ("jnt_b", _P), ("jnt_anchor_a", _P), ("jnt_anchor_b", _P),
        ("jnt_distance", _P), ("jnt_target", _P), ("jnt_order", _P),
        ("n_circles", ctypes.c_uint32), ("circles", _P),
        ("box_enabled", ctypes.c_uint32), ("box_lo", ctypes.c_double * 2), ("box_hi", ctypes.c_double * 2),
    ]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _b
        _b.build()
    L = ctypes.CDLL(LIB_PATH)
    u32, u64, i32, f32, f64 = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_float, ctypes.c_double
    sigs = {
        "oracle_world_new": (_P, [ctypes.POINTER(OracleScene), i32]),
        "oracle_world_free": (None, [_P]),
        "oracle_world_step": (i32, [_P, f64, u32]),
        "oracle_world_time_steps": (f64, [_P, f64, u32, ctypes.POINTER(i32)]),
        "oracle_world_get_bodies": (None, [_P, _P, _P, _P, _P, _P]),
        "oracle_world_get_snapshots": (None, [_P, _P]),
        "oracle_world_get_mass": (None, [_P, _P, _P]),
        "oracle_world_contacts": (u64, [_P]),
        "oracle_world_last_substep_contacts": (u64, [_P]),
        "oracle_world_pushouts": (u64, [_P]),
        "oracle_world_time": (f64, [_P]),
        "oracle_world_events": (u64, [_P, _P, _P, _P, _P, u64]),
        "oracle_world_clear_events": (None, [_P]),
        "oracle_world_set_grid_pairs": (None, [_P, i32]),
        "oracle_world_trace": (None, [_P, i32]),
        "oracle_world_trace_states": (u64, [_P, _P, u64]),
        "oracle_world_trace_pairs": (u64, [_P, _P, u64]),
        "oracle_world_trace_counts": (u64, [_P, _P, u64]),
        "oracle_mass_inertia_f32": (None, [ctypes.POINTER(OracleScene), _P, _P]),
        "oracle_body_collider_transform": (None, [f32, f32, f32, f32, f32, _P]),
        "oracle_contact_pairs": (u64, [u32, _P, _P, _P, _P, _P, _P, _P, u64]),
        "oracle_sh_new": (_P, [f32]),
        "oracle_sh_free": (None, [_P]),
        "oracle_sh_insert": (u64, [_P, f32, f32, f32]),
        "oracle_sh_insert_with_id": (None, [_P, u64, f32, f32, f32]),
        "oracle_sh_remove": (i32, [_P, u64]),
        "oracle_sh_move_point": (i32, [_P, u64, f32, f32]),
        "oracle_sh_cell_coords": (None, [_P, f32, f32, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
        "oracle_sh_next_id": (u64, [_P]),
        "oracle_sh_point": (i32, [_P, u64, ctypes.POINTER(f32), ctypes.POINTER(f32)]),
        "oracle_sh_cell_len": (u64, [_P, ctypes.c_int32, ctypes.c_int32]),
        "oracle_sh_query": (u64, [_P, f32, f32, f32, _P, _P, u64]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _d(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    return a if shape is None else a.reshape(shape)


def _scene_struct(scene, keep, *, joint_order=None, record_events=False, maintain_spatial_hash=False,
                  old_dt=1.0, world: Optional[int] = None):
    """Fill an OracleScene from a blobs_gb300.scenes.Scene (one world)."""
    def p(a, dtype):
        if a is None:
            return None
        a = np.ascontiguousarray(np.asarray(a, dtype=dtype))
        keep.append(a)
        return a.ctypes.data

    st = OracleScene()
    st.gravity[0], st.gravity[1] = float(scene.gravity[0]), float(scene.gravity[1])
    st.substeps = int(scene.substeps)
    st.joint_iterations = int(scene.joint_iterations)
    st.collisions_enabled = 1 if scene.collisions_enabled else 0
    st.maintain_spatial_hash = 1 if maintain_spatial_hash else 0
    st.record_events = 1 if record_events else 0
    st.old_dt = float(old_dt)
    st.n_bodies = scene.n_bodies
    st.pos = p(scene.pos, np.float64)
    st.pos_old = p(scene.pos_old, np.float64)
    st.acc = p(scene.acc, np.float64)
    st.vel = p(scene.vel, np.float64)
    st.vreq = p(scene.vreq, np.float64)
    st.vreq_set = p(scene.vreq_set, np.uint8)
    st.body_type = p(scene.body_type, np.uint8)
    st.rotation = p(scene.rotation, np.float64)
    st.angvel = p(scene.angvel, np.float64)
    st.torque = p(scene.torque, np.float64)
    st.gravity_mod = p(scene.gravity_mod, np.float64)
    st.mass = p(scene.mass, np.float64)
    st.inertia = p(scene.inertia, np.float64)
    st.bound_radius = None
    st.n_colliders = scene.n_colliders
    st.col_parent = p(scene.col_parent, np.uint32)
    st.col_offset = p(scene.col_offset, np.float64)
    st.col_radius = p(scene.col_radius, np.float64)
    st.col_mass_override = p(scene.col_mass_override, np.float64)
    st.col_sensor = p(scene.col_sensor, np.uint8)
    st.col_memb = p(scene.col_memb, np.uint32)
    st.col_filt = p(scene.col_filt, np.uint32)
    st.col_snap = p(scene.col_snap, np.float64)
    st.n_springs = scene.n_springs
    st.spr_a = p(scene.spr_a, np.uint32)
    st.spr_b = p(scene.spr_b, np.uint32)
    st.spr_rest = p(scene.spr_rest, np.float64)
    st.spr_k = p(scene.spr_k, np.float64)
    st.spr_c = p(scene.spr_c, np.float64)
    st.n_joints = scene.n_joints
    st.jnt_a = p(scene.jnt_a, np.uint32)
    st.jnt_b = p(scene.jnt_b, np.uint32)
    st.jnt_anchor_a = p(scene.jnt_anchor_a, np.float64)
    st.jnt_anchor_b = p(scene.jnt_anchor_b, np.float64)
    st.jnt_distance = p(scene.jnt_distance, np.float64)
    st.jnt_target = p(scene.jnt_target, np.float64)
    st.jnt_order = p(joint_order, np.uint32)
    st.n_circles = int(scene.circles.shape[0])
    st.circles = p(scene.circles, np.float64)
    if scene.world_box is not None:
        b = scene.world_box[0 if world is None else world]
        st.box_enabled = 1
        st.box_lo[0], st.box_lo[1], st.box_hi[0], st.box_hi[1] = (float(b[0]), float(b[1]), float(b[2]),
                                                                  float(b[3]))
    return st


class OracleWorld:
    """One reference world stepped on the CPU (precision 32 = f32-faithful,
    64 = the same algorithm in f64).  Batched scenes are stepped world by
    world: see :func:`step_batched`."""

    def __init__(self, scene, precision: int = 32, *, joint_order=None, record_events: bool = False,
                 maintain_spatial_hash: bool = False, old_dt: float = 1.0, grid_pairs: bool = False):
        """grid_pairs: enumerate the contact loop's pairs through a uniform
        grid of the collider snapshots -- the same pairs in the same order as
        the reference's C^2/2 loop (physics.rs:248-249), for full-size checks.
        A push-out (coincident centres) in this mode ends the step with status
        GRID_PUSHOUT; scenes whose extent does not fit a grid fall back to the
        C^2/2 loop."""
        if scene.n_worlds != 1:
            raise ValueError("OracleWorld takes one world; unpack batched scenes first")
        self._keep = []
        st = _scene_struct(scene, self._keep, joint_order=joint_order, record_events=record_events,
                           maintain_spatial_hash=maintain_spatial_hash, old_dt=old_dt)
        self._h = lib().oracle_world_new(ctypes.byref(st), int(precision))
        self._keep = None
        if grid_pairs:
            lib().oracle_world_set_grid_pairs(self._h, 1)
        self.n_bodies = scene.n_bodies
        self.n_colliders = scene.n_colliders
        self.precision = precision

    def close(self):
        if self._h:
            lib().oracle_world_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dt: float, n_steps: int = 1) -> int:
        return int(lib().oracle_world_step(self._h, float(dt), int(n_steps)))

    def time_steps(self, dt: float, n_steps: int) -> float:
        st = ctypes.c_int()
        t = lib().oracle_world_time_steps(self._h, float(dt), int(n_steps), ctypes.byref(st))
        if st.value:
            raise RuntimeError("oracle step status %d" % st.value)
        return float(t)

    def bodies(self):
        n = self.n_bodies
        pos, po, vel = np.zeros((n, 2)), np.zeros((n, 2)), np.zeros((n, 2))
        rot, av = np.zeros(n), np.zeros(n)
        lib().oracle_world_get_bodies(self._h, pos.ctypes.data, po.ctypes.data, vel.ctypes.data, rot.ctypes.data,
                                      av.ctypes.data)
        return {"pos": pos, "pos_old": po, "vel": vel, "rotation": rot, "angvel": av}

    def snapshots(self):
        out = np.zeros((self.n_colliders, 2))
        lib().oracle_world_get_snapshots(self._h, out.ctypes.data)
        return out

    def mass(self):
        m, I = np.zeros(self.n_bodies), np.zeros(self.n_bodies)
        lib().oracle_world_get_mass(self._h, m.ctypes.data, I.ctypes.data)
        return m, I

    @property
    def contacts(self) -> int:
        return int(lib().oracle_world_contacts(self._h))

    @property
    def last_substep_contacts(self) -> int:
        return int(lib().oracle_world_last_substep_contacts(self._h))

    @property
    def pushouts(self) -> int:
        return int(lib().oracle_world_pushouts(self._h))

    @property
    def time(self) -> float:
        return float(lib().oracle_world_time(self._h))

    def trace(self, on: bool = True) -> None:
        """Start (and clear) or stop the substep trace."""
        lib().oracle_world_trace(self._h, 1 if on else 0)

    def traced(self):
        """The substep trace: a list of per-substep dicts with the state at the
        substep's start (pos, pos_old, snap, vel as float64 arrays) and the
        contacts it resolved (hi, lo collider ids; pushed flags)."""
        L = lib()
        n, c = self.n_bodies, self.n_colliders
        ns = int(L.oracle_world_trace_states(self._h, None, 0))
        st = np.zeros(ns)
        if ns:
            L.oracle_world_trace_states(self._h, st.ctypes.data, ns)
        npairs = int(L.oracle_world_trace_pairs(self._h, None, 0))
        pr = np.zeros((npairs, 2), np.uint32)
        if npairs:
            L.oracle_world_trace_pairs(self._h, pr.ctypes.data, npairs)
        nsub = int(L.oracle_world_trace_counts(self._h, None, 0))
        counts = np.zeros(nsub, np.uint64)
        if nsub:
            L.oracle_world_trace_counts(self._h, counts.ctypes.data, nsub)
        per = 6 * n + 2 * c
        assert ns == per * nsub, (ns, per, nsub)
        out, k = [], 0
        for t in range(nsub):
            x = st[per * t: per * (t + 1)]
            q = pr[k: k + int(counts[t])]
            k += int(counts[t])
            out.append({"pos": x[:2 * n].reshape(n, 2), "pos_old": x[2 * n:4 * n].reshape(n, 2),
                        "snap": x[4 * n:4 * n + 2 * c].reshape(c, 2), "vel": x[4 * n + 2 * c:].reshape(n, 2),
                        "hi": q[:, 0].astype(np.int64), "lo": (q[:, 1] & 0x7FFFFFFF).astype(np.int64),
                        "pushed": (q[:, 1] >> 31).astype(bool)})
        return out

    def events(self):
        n = int(lib().oracle_world_events(self._h, None, None, None, None, 0))
        a, b = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        va, vb = np.zeros((n, 2)), np.zeros((n, 2))
        if n:
            lib().oracle_world_events(self._h, a.ctypes.data, b.ctypes.data, va.ctypes.data, vb.ctypes.data, n)
        return a, b, va, vb


def mass_inertia_f32(scene):
    keep = []
    st = _scene_struct(scene, keep)
    m, I = np.zeros(scene.n_bodies, np.float32), np.zeros(scene.n_bodies, np.float32)
    lib().oracle_mass_inertia_f32(ctypes.byref(st), m.ctypes.data, I.ctypes.data)
    return m, I


def body_collider_transform(theta, px, py, ox, oy):
    out = np.zeros(6, np.float32)
    lib().oracle_body_collider_transform(theta, px, py, ox, oy, out.ctypes.data)
    return out


def contact_pairs(snap, radius, parent=None, memb=None, filt=None, cap=None):
    snap = np.ascontiguousarray(snap, np.float32)
    radius = np.ascontiguousarray(radius, np.float32)
    n = len(radius)
    keep = [np.ascontiguousarray(x, np.uint32) if x is not None else None for x in (parent, memb, filt)]
    ptrs = [None if x is None else x.ctypes.data for x in keep]
    k = int(lib().oracle_contact_pairs(n, snap.ctypes.data, radius.ctypes.data, *ptrs, None, None, 0))
    oi, oj = np.zeros(max(k, 1), np.uint32), np.zeros(max(k, 1), np.uint32)
    lib().oracle_contact_pairs(n, snap.ctypes.data, radius.ctypes.data, *ptrs, oi.ctypes.data, oj.ctypes.data, k)
    return oi[:k], oj[:k]


class SpatialHash:
    """The reference SpatialHash (spatial.rs:31-195), restated."""

    def __init__(self, cell_size: float):
        self._h = lib().oracle_sh_new(float(cell_size))

    def __del__(self):
        try:
            lib().oracle_sh_free(self._h)
        except Exception:
            pass

    def insert(self, x, y, r) -> int:
        return int(lib().oracle_sh_insert(self._h, x, y, r))

    def insert_with_id(self, id_, x, y, r):
        lib().oracle_sh_insert_with_id(self._h, id_, x, y, r)

    def remove(self, id_) -> bool:
        return bool(lib().oracle_sh_remove(self._h, id_))

    def move_point(self, id_, dx, dy) -> bool:
        return bool(lib().oracle_sh_move_point(self._h, id_, dx, dy))

    def cell_coords(self, x, y):
        cx, cy = ctypes.c_int32(), ctypes.c_int32()
        lib().oracle_sh_cell_coords(self._h, x, y, ctypes.byref(cx), ctypes.byref(cy))
        return cx.value, cy.value

    @property
    def next_id(self) -> int:
        return int(lib().oracle_sh_next_id(self._h))

    def point(self, id_):
        x, y = ctypes.c_float(), ctypes.c_float()
        if not lib().oracle_sh_point(self._h, id_, ctypes.byref(x), ctypes.byref(y)):
            return None
        return x.value, y.value

    def cell_len(self, cx, cy):
        n = int(lib().oracle_sh_cell_len(self._h, cx, cy))
        return None if n == 2 ** 64 - 1 else n

    def query(self, x, y, qr):
        n = int(lib().oracle_sh_query(self._h, x, y, qr, None, None, 0))
        ids, pos = np.zeros(max(n, 1), np.uint64), np.zeros((max(n, 1), 2), np.float32)
        lib().oracle_sh_query(self._h, x, y, qr, ids.ctypes.data, pos.ctypes.data, n)
        return ids[:n], pos[:n]
