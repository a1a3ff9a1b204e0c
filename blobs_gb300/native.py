"""ctypes binding of the C ABI in include/blobs_gpu.h.

This module loads ``libblobs_gb300.so`` (built in-tree by
``blobs_gb300.build``).  There is no fallback: if the library is missing the
import of :func:`lib` raises, and every call that needs a GPU returns
``BLOBS_ERR_NO_DEVICE`` when there is none.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import scenes

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libblobs_gb300.so")

OK = 0
ERR_INVALID_HANDLE = 1
ERR_INVALID_ARGUMENT = 2
ERR_OVERFLOW = 3
ERR_NAN = 4
ERR_CUDA = 5
ERR_TIMEOUT = 6
ERR_NO_DEVICE = 7
ERR_OUT_OF_MEMORY = 8
ERR_STATE = 9


class BlobsError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__("%s failed: %s (status %d)" % (what, status_string(status), status))


class Config(ctypes.Structure):
    _fields_ = [("gravity", ctypes.c_float * 2), ("substeps", ctypes.c_uint32),
                ("joint_iterations", ctypes.c_uint32), ("collisions_enabled", ctypes.c_uint32),
                ("cell_size", ctypes.c_float), ("device", ctypes.c_int32)]


_P = ctypes.c_void_p
_SCENE_FIELDS = [
    ("n_worlds", ctypes.c_uint32), ("world_body_offsets", _P), ("world_collider_offsets", _P),
    ("world_spring_offsets", _P), ("world_joint_offsets", _P), ("world_box", _P),
    ("n_bodies", ctypes.c_uint32), ("pos", _P), ("pos_old", _P), ("acc", _P), ("vel", _P), ("vreq", _P),
    ("vreq_set", _P), ("body_type", _P), ("rotation", _P), ("angvel", _P), ("torque", _P), ("gravity_mod", _P),
    ("mass", _P), ("inertia", _P),
    ("n_colliders", ctypes.c_uint32), ("col_parent", _P), ("col_offset", _P), ("col_radius", _P),
    ("col_sensor", _P), ("col_memb", _P), ("col_filt", _P), ("col_snap", _P),
    ("n_springs", ctypes.c_uint32), ("spr_a", _P), ("spr_b", _P), ("spr_rest", _P), ("spr_k", _P), ("spr_c", _P),
    ("n_joints", ctypes.c_uint32), ("jnt_a", _P), ("jnt_b", _P), ("jnt_anchor_a", _P), ("jnt_anchor_b", _P),
    ("jnt_distance", _P), ("jnt_target", _P),
    ("n_circles", ctypes.c_uint32), ("circles", _P),
]


class SceneStruct(ctypes.Structure):
    _fields_ = _SCENE_FIELDS


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libblobs_gb300.so is missing (%s): run `python -c 'import __graft_entry__ as g; "
                          "g.build()'` first; there is no CPU fallback" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    u32, i32, f32, f64, u64 = ctypes.c_uint32, ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_uint64
    pp = ctypes.POINTER(ctypes.c_void_p)
    sigs = {
        "blobs_abi_version": (i32, []),
        "blobs_config_default": (None, [ctypes.POINTER(Config)]),
        "blobs_status_string": (ctypes.c_char_p, [i32]),
        "blobs_world_create": (i32, [ctypes.POINTER(Config), pp]),
        "blobs_world_destroy": (i32, [_P]),
        "blobs_world_set_config": (i32, [_P, ctypes.POINTER(Config)]),
        "blobs_world_load": (i32, [_P, ctypes.POINTER(SceneStruct), f32]),
        "blobs_world_step": (i32, [_P, f64]),
        "blobs_world_rollout": (i32, [_P, f64, u32]),
        "blobs_world_fixed_step": (i32, [_P, f64]),
        "blobs_world_sync": (i32, [_P]),
        "blobs_world_read_bodies": (i32, [_P, _P, _P, _P, _P, _P]),
        "blobs_world_read_snapshots": (i32, [_P, _P]),
        "blobs_world_contact_count": (i32, [_P, ctypes.POINTER(u64), ctypes.POINTER(u64)]),
        "blobs_world_pushout_count": (i32, [_P, ctypes.POINTER(u64)]),
        "blobs_world_deferred_count": (i32, [_P, ctypes.POINTER(u64), ctypes.POINTER(u64)]),
        "blobs_world_time": (i32, [_P, ctypes.POINTER(f64), ctypes.POINTER(f64)]),
        "blobs_world_joint_order": (i32, [_P, _P, ctypes.POINTER(u32)]),
        "blobs_world_snapshot": (i32, [_P]),
        "blobs_world_restore": (i32, [_P]),
        "blobs_joint_schedule": (i32, [u32, u32, _P, _P, _P, _P, ctypes.POINTER(u32), _P, ctypes.POINTER(u32)]),
        "blobs_body_mass_inertia": (i32, [u32, u32, _P, _P, _P, _P, _P, _P, _P]),
        "blobs_world_set_stream": (i32, [_P, _P]),
        "blobs_world_write_bodies": (i32, [_P, _P, _P, _P, _P, _P]),
        "blobs_world_set_timing": (i32, [_P, i32]),
        "blobs_world_rollout_record": (i32, [_P, f64, u32, u32]),
        "blobs_world_backward": (i32, [_P, _P, _P, _P]),
        "blobs_world_emit_pairs": (i32, [_P, i32, _P, u64, ctypes.POINTER(u64)]),
        "blobs_world_grid": (i32, [_P, u32, ctypes.POINTER(f32), ctypes.POINTER(f32), _P, ctypes.POINTER(u32),
                                   ctypes.POINTER(u32)]),
        "blobs_world_kernel_launches": (i32, [_P, ctypes.POINTER(u64)]),
        "blobs_world_phase_times": (i32, [_P, ctypes.POINTER(f64), ctypes.POINTER(u64), u32]),
        "blobs_world_set_events": (i32, [_P, i32, u32]),
        "blobs_world_autotune": (i32, [_P, ctypes.POINTER(SceneStruct), f32, f64, u32, ctypes.POINTER(f32)]),
        "blobs_spatial_hash_create": (i32, [f32, i32, pp]),
        "blobs_spatial_hash_destroy": (i32, [_P]),
        "blobs_spatial_hash_set_points": (i32, [_P, u64, _P, _P, _P]),
        "blobs_spatial_hash_query": (i32, [_P, u64, _P, _P, _P, _P, u64, ctypes.POINTER(u64)]),
        "blobs_world_drain_events": (i32, [_P, _P, _P, _P, _P, u64, ctypes.POINTER(u64), ctypes.POINTER(u64)]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def status_string(status: int) -> str:
    try:
        return lib().blobs_status_string(status).decode()
    except ImportError:
        return "status %d" % status


def check(status: int, what: str) -> None:
    if status != OK:
        raise BlobsError(status, what)


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def mass_inertia(scene: scenes.Scene):
    """RigidBody::update_mass_and_inertia for every body of the scene, from the
    library's host helper (rigid_body.rs:96-128 with the doubled handles)."""
    n, c = scene.n_bodies, scene.n_colliders
    m = np.zeros(n, np.float32)
    I = np.zeros(n, np.float32)
    mo = np.ascontiguousarray(scene.col_mass_override, np.float32) if c else None
    check(lib().blobs_body_mass_inertia(n, c, _ptr(np.ascontiguousarray(scene.col_parent, np.uint32)),
                                        _ptr(np.ascontiguousarray(scene.col_offset, np.float32)),
                                        _ptr(np.ascontiguousarray(scene.col_radius, np.float32)), _ptr(mo),
                                        _ptr(np.ascontiguousarray(scene.col_sensor, np.uint8)),
                                        _ptr(m), _ptr(I)), "blobs_body_mass_inertia")
    return m, I


def joint_schedule(n_bodies: int, jnt_a, jnt_b):
    """The GPU's joint processing schedule for a joint list, computed on the
    host (blobs_joint_schedule): (order, block_joint_start, colour_start) --
    block k sweeps order[block_joint_start[k]:block_joint_start[k+1]], colour k
    is order[colour_start[k]:colour_start[k+1]]."""
    a = np.ascontiguousarray(np.asarray(jnt_a, np.uint32))
    b = np.ascontiguousarray(np.asarray(jnt_b, np.uint32))
    n = len(a)
    order = np.zeros(max(1, n), np.uint32)
    blocks = np.zeros(n + 1, np.uint32)
    colours = np.zeros(n + 1, np.uint32)
    nblk, ncol = ctypes.c_uint32(), ctypes.c_uint32()
    check(lib().blobs_joint_schedule(int(n_bodies), n, _ptr(a), _ptr(b), _ptr(order), _ptr(blocks),
                                     ctypes.byref(nblk), _ptr(colours), ctypes.byref(ncol)), "joint_schedule")
    return order[:n], blocks[:nblk.value + 1], colours[:ncol.value + 1]


def make_config(scene: Optional[scenes.Scene] = None, *, cell_size: float = 0.0, device: int = 0) -> Config:
    cfg = Config()
    lib().blobs_config_default(ctypes.byref(cfg))
    if scene is not None:
        cfg.gravity[0], cfg.gravity[1] = float(scene.gravity[0]), float(scene.gravity[1])
        cfg.substeps = int(scene.substeps)
        cfg.joint_iterations = int(scene.joint_iterations)
        cfg.collisions_enabled = 1 if scene.collisions_enabled else 0
    cfg.cell_size = float(cell_size)
    cfg.device = int(device)
    return cfg


class World:
    """One device world (a reference ``Physics``, or a batch of them)."""

    def __init__(self, scene: Optional[scenes.Scene] = None, *, cell_size: float = 0.0, device: int = 0,
                 old_dt: float = 1.0):
        self._h = ctypes.c_void_p()
        self.cfg = make_config(scene, cell_size=cell_size, device=device)
        check(lib().blobs_world_create(ctypes.byref(self.cfg), ctypes.byref(self._h)), "blobs_world_create")
        self.n_bodies = 0
        self.n_colliders = 0
        self.n_joints = 0
        if scene is not None:
            self.load(scene, old_dt=old_dt)

    def close(self) -> None:
        if self._h:
            lib().blobs_world_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def load(self, scene: scenes.Scene, old_dt: float = 1.0) -> None:
        st, keep = self._scene_struct(scene)
        check(lib().blobs_world_load(self._h, ctypes.byref(st), float(old_dt)), "blobs_world_load")
        self.n_bodies = scene.n_bodies
        self.n_colliders = scene.n_colliders
        self.n_joints = scene.n_joints

    def autotune(self, scene: scenes.Scene, dt: float, trial_steps: int = 5, old_dt: float = 1.0) -> float:
        """Time a few broadphase cell edges on `scene`, keep the fastest and
        reload the scene with it; returns the chosen scale."""
        st, keep = self._scene_struct(scene)
        scale = ctypes.c_float()
        check(lib().blobs_world_autotune(self._h, ctypes.byref(st), float(old_dt), float(dt), int(trial_steps),
                                         ctypes.byref(scale)), "blobs_world_autotune")
        self.n_bodies = scene.n_bodies
        self.n_colliders = scene.n_colliders
        self.n_joints = scene.n_joints
        return float(scale.value)

    def _scene_struct(self, scene: scenes.Scene):
        keep = []

        def arr(a, dtype):
            if a is None:
                return None
            a = np.ascontiguousarray(np.asarray(a, dtype=dtype))
            keep.append(a)
            return a.ctypes.data

        if scene.mass is None or scene.inertia is None:
            mass, inertia = mass_inertia(scene)
        else:
            mass, inertia = scene.mass, scene.inertia
        st = SceneStruct()
        st.n_worlds = scene.n_worlds
        st.world_body_offsets = arr(scene.world_body_offsets, np.uint32)
        st.world_collider_offsets = arr(scene.world_collider_offsets, np.uint32)
        st.world_spring_offsets = arr(scene.world_spring_offsets, np.uint32)
        st.world_joint_offsets = arr(scene.world_joint_offsets, np.uint32)
        st.world_box = arr(scene.world_box, np.float32)
        st.n_bodies = scene.n_bodies
        st.pos = arr(scene.pos, np.float32)
        st.pos_old = arr(scene.pos_old, np.float32)
        st.acc = arr(scene.acc, np.float32)
        st.vel = arr(scene.vel, np.float32)
        st.vreq = arr(scene.vreq, np.float32)
        st.vreq_set = arr(scene.vreq_set, np.uint8)
        st.body_type = arr(scene.body_type, np.uint8)
        st.rotation = arr(scene.rotation, np.float32)
        st.angvel = arr(scene.angvel, np.float32)
        st.torque = arr(scene.torque, np.float32)
        st.gravity_mod = arr(scene.gravity_mod, np.float32)
        st.mass = arr(mass, np.float32)
        st.inertia = arr(inertia, np.float32)
        st.n_colliders = scene.n_colliders
        st.col_parent = arr(scene.col_parent, np.uint32)
        st.col_offset = arr(scene.col_offset, np.float32)
        st.col_radius = arr(scene.col_radius, np.float32)
        st.col_sensor = arr(scene.col_sensor, np.uint8)
        st.col_memb = arr(scene.col_memb, np.uint32)
        st.col_filt = arr(scene.col_filt, np.uint32)
        st.col_snap = arr(scene.col_snap, np.float32)
        st.n_springs = scene.n_springs
        st.spr_a = arr(scene.spr_a, np.uint32)
        st.spr_b = arr(scene.spr_b, np.uint32)
        st.spr_rest = arr(scene.spr_rest, np.float32)
        st.spr_k = arr(scene.spr_k, np.float32)
        st.spr_c = arr(scene.spr_c, np.float32)
        st.n_joints = scene.n_joints
        st.jnt_a = arr(scene.jnt_a, np.uint32)
        st.jnt_b = arr(scene.jnt_b, np.uint32)
        st.jnt_anchor_a = arr(scene.jnt_anchor_a, np.float32)
        st.jnt_anchor_b = arr(scene.jnt_anchor_b, np.float32)
        st.jnt_distance = arr(scene.jnt_distance, np.float32)
        st.jnt_target = arr(scene.jnt_target, np.float32)
        st.n_circles = int(scene.circles.shape[0])
        st.circles = arr(scene.circles, np.float32)
        return st, keep

    def step(self, dt: float) -> None:
        check(lib().blobs_world_step(self._h, float(dt)), "blobs_world_step")

    def rollout(self, dt: float, n_steps: int) -> None:
        check(lib().blobs_world_rollout(self._h, float(dt), int(n_steps)), "blobs_world_rollout")

    def fixed_step(self, frame_time: float) -> None:
        check(lib().blobs_world_fixed_step(self._h, float(frame_time)), "blobs_world_fixed_step")

    def sync(self) -> None:
        check(lib().blobs_world_sync(self._h), "blobs_world_sync")

    def set_stream(self, stream_handle: int) -> None:
        """Run on the caller's cudaStream_t (an int handle, e.g. torch's
        ``torch.cuda.current_stream().cuda_stream``); 0 = the world's own."""
        check(lib().blobs_world_set_stream(self._h, ctypes.c_void_p(int(stream_handle) or None)), "set_stream")

    def write_bodies(self, pos=None, pos_old=None, vel=None, rotation=None, angvel=None) -> None:
        """Asynchronous host->device write; the arrays must stay alive (and,
        for an overlapped copy, be pinned) until the next synchronising call."""
        ptrs = []
        for a, width in ((pos, 2), (pos_old, 2), (vel, 2), (rotation, 1), (angvel, 1)):
            if a is None:
                ptrs.append(None)
                continue
            if a.dtype != np.float32 or not a.flags.c_contiguous or a.size != self.n_bodies * width:
                raise ValueError("write_bodies wants C-contiguous float32 arrays of the body count")
            ptrs.append(a.ctypes.data)
        check(lib().blobs_world_write_bodies(self._h, *ptrs), "write_bodies")

    def read_bodies_into(self, pos=None, pos_old=None, vel=None, rotation=None, angvel=None) -> None:
        check(lib().blobs_world_read_bodies(self._h, _ptr(pos), _ptr(pos_old), _ptr(vel), _ptr(rotation),
                                            _ptr(angvel)), "read_bodies")

    def set_timing(self, enabled, contact_only: bool = False) -> None:
        """Per-phase CUDA events in the step graphs (contact_only: around the
        contact phase alone)."""
        mode = (2 if contact_only else 1) if enabled else 0
        check(lib().blobs_world_set_timing(self._h, mode), "set_timing")

    def emit_pairs(self, contacts_only: bool, cap: Optional[int] = None):
        """(hi, lo) collider pairs of the broadphase (see blobs_world_emit_pairs),
        sorted; grows the buffer once on BLOBS_ERR_OVERFLOW."""
        n = ctypes.c_uint64()
        cap = 1024 if cap is None else cap
        buf = np.zeros((max(cap, 1), 2), np.uint32)
        st = lib().blobs_world_emit_pairs(self._h, 1 if contacts_only else 0, _ptr(buf), cap, ctypes.byref(n))
        if st == ERR_OVERFLOW:
            buf = np.zeros((max(int(n.value), 1), 2), np.uint32)
            st = lib().blobs_world_emit_pairs(self._h, 1 if contacts_only else 0, _ptr(buf), int(n.value),
                                              ctypes.byref(n))
        check(st, "emit_pairs")
        out = buf[:int(n.value)]
        return out[np.lexsort((out[:, 1], out[:, 0]))]

    def grid(self, world: int = 0):
        """(cell size, f32 reciprocal, origin (2,), log2 width, log2 height) of a world's grid."""
        cs, inv, lw, lh = ctypes.c_float(), ctypes.c_float(), ctypes.c_uint32(), ctypes.c_uint32()
        org = np.zeros(2, np.float32)
        check(lib().blobs_world_grid(self._h, world, ctypes.byref(cs), ctypes.byref(inv), _ptr(org),
                                     ctypes.byref(lw), ctypes.byref(lh)), "grid")
        return cs.value, inv.value, org, lw.value, lh.value

    def rollout_record(self, dt: float, n_steps: int, checkpoint_every: int = 16) -> None:
        """Differentiable rollout: n_steps steps with checkpoints for backward()."""
        check(lib().blobs_world_rollout_record(self._h, float(dt), int(n_steps), int(checkpoint_every)),
              "rollout_record")

    def backward(self, dl_dpos: np.ndarray, n_springs: int):
        """dL/d(velocity requests) (n, 2) and dL/d(spring stiffness) (n_springs,)
        of the last recorded rollout, given dL/d(final positions) (n, 2)."""
        g = np.ascontiguousarray(dl_dpos, np.float32).reshape(self.n_bodies, 2)
        gv = np.zeros((self.n_bodies, 2), np.float32)
        gk = np.zeros(max(n_springs, 1), np.float32)
        check(lib().blobs_world_backward(self._h, _ptr(g), _ptr(gv), _ptr(gk)), "backward")
        return gv, gk[:n_springs]

    def set_events(self, enabled: bool = True, capacity: int = 1 << 20) -> None:
        """Record CollisionEvents (physics.rs:304-311) into a device buffer of `capacity`."""
        check(lib().blobs_world_set_events(self._h, 1 if enabled else 0, int(capacity) if enabled else 0),
              "set_events")

    def drain_events(self, cap: Optional[int] = None):
        """collision_recv.try_iter(): (a, b, impact_vel_a, impact_vel_b) of the
        events since the last drain, in the reference's order."""
        n, left = ctypes.c_uint64(), ctypes.c_uint64()
        if cap is None:
            st = lib().blobs_world_drain_events(self._h, None, None, None, None, 0, ctypes.byref(n),
                                                ctypes.byref(left))
            check(st, "drain_events")
            cap = int(left.value)
        a, b = np.zeros(max(cap, 1), np.uint32), np.zeros(max(cap, 1), np.uint32)
        va, vb = np.zeros((max(cap, 1), 2), np.float32), np.zeros((max(cap, 1), 2), np.float32)
        check(lib().blobs_world_drain_events(self._h, _ptr(a), _ptr(b), _ptr(va), _ptr(vb), cap, ctypes.byref(n),
                                             ctypes.byref(left)), "drain_events")
        k = int(n.value)
        return a[:k], b[:k], va[:k], vb[:k]

    def kernel_launches(self) -> int:
        n = ctypes.c_uint64()
        check(lib().blobs_world_kernel_launches(self._h, ctypes.byref(n)), "kernel_launches")
        return int(n.value)

    PHASES = ("scan", "scatter_forces", "contact", "joints", "integrate")

    def phase_times(self):
        ms = (ctypes.c_double * 5)()
        n = (ctypes.c_uint64 * 5)()
        check(lib().blobs_world_phase_times(self._h, ms, n, 5), "phase_times")
        return {p: (ms[i], int(n[i])) for i, p in enumerate(self.PHASES)}

    def read_bodies(self):
        n = self.n_bodies
        pos = np.zeros((n, 2), np.float32)
        pos_old = np.zeros((n, 2), np.float32)
        vel = np.zeros((n, 2), np.float32)
        rot = np.zeros(n, np.float32)
        av = np.zeros(n, np.float32)
        check(lib().blobs_world_read_bodies(self._h, _ptr(pos), _ptr(pos_old), _ptr(vel), _ptr(rot), _ptr(av)),
              "blobs_world_read_bodies")
        return {"pos": pos, "pos_old": pos_old, "vel": vel, "rotation": rot, "angvel": av}

    def read_snapshots(self) -> np.ndarray:
        out = np.zeros((self.n_colliders, 2), np.float32)
        check(lib().blobs_world_read_snapshots(self._h, _ptr(out)), "blobs_world_read_snapshots")
        return out

    def contact_count(self):
        t, l = ctypes.c_uint64(), ctypes.c_uint64()
        check(lib().blobs_world_contact_count(self._h, ctypes.byref(t), ctypes.byref(l)), "contact_count")
        return int(t.value), int(l.value)

    def deferred_count(self):
        """(total, last substep) bodies whose contacts were resolved by a warp each."""
        t, l = ctypes.c_uint64(), ctypes.c_uint64()
        check(lib().blobs_world_deferred_count(self._h, ctypes.byref(t), ctypes.byref(l)), "deferred_count")
        return int(t.value), int(l.value)

    def pushout_count(self) -> int:
        t = ctypes.c_uint64()
        check(lib().blobs_world_pushout_count(self._h, ctypes.byref(t)), "pushout_count")
        return int(t.value)

    def time(self):
        t, a = ctypes.c_double(), ctypes.c_double()
        check(lib().blobs_world_time(self._h, ctypes.byref(t), ctypes.byref(a)), "time")
        return t.value, a.value

    def snapshot(self) -> None:
        """Keep the world's whole state (blobs_world_snapshot)."""
        check(lib().blobs_world_snapshot(self._h), "snapshot")

    def restore(self) -> None:
        """Back to the state of the last snapshot (blobs_world_restore)."""
        check(lib().blobs_world_restore(self._h), "restore")

    def joint_order(self):
        order = np.zeros(max(1, self.n_joints), np.uint32)
        nc = ctypes.c_uint32()
        check(lib().blobs_world_joint_order(self._h, _ptr(order), ctypes.byref(nc)), "joint_order")
        return order[:self.n_joints], int(nc.value)


class SpatialHash:
    """SpatialHash (spatial.rs) on the device: set_points replaces the point
    set; query runs SpatialHash::query for many query points."""

    def __init__(self, cell_size: float, device: int = 0):
        h = ctypes.c_void_p()
        check(lib().blobs_spatial_hash_create(float(cell_size), int(device), ctypes.byref(h)),
              "blobs_spatial_hash_create")
        self._h = h

    def close(self):
        if self._h:
            lib().blobs_spatial_hash_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_points(self, ids, xy, radius) -> None:
        ids = np.ascontiguousarray(ids, np.uint64)
        xy = np.ascontiguousarray(xy, np.float32).reshape(-1, 2)
        radius = np.ascontiguousarray(radius, np.float32)
        check(lib().blobs_spatial_hash_set_points(self._h, len(ids), _ptr(ids), _ptr(xy), _ptr(radius)),
              "blobs_spatial_hash_set_points")

    def query(self, qxy, qradius, cap: Optional[int] = None):
        """(offsets (nq + 1,), ids) with each query's ids ascending."""
        qxy = np.ascontiguousarray(qxy, np.float32).reshape(-1, 2)
        qradius = np.ascontiguousarray(qradius, np.float32)
        nq = len(qradius)
        offsets = np.zeros(nq + 1, np.uint64)
        total = ctypes.c_uint64()
        if cap is None:
            st = lib().blobs_spatial_hash_query(self._h, nq, _ptr(qxy), _ptr(qradius), _ptr(offsets), None, 0,
                                                ctypes.byref(total))
            if st not in (OK, ERR_OVERFLOW):
                check(st, "blobs_spatial_hash_query")
            cap = int(total.value)
        ids = np.zeros(max(cap, 1), np.uint64)
        check(lib().blobs_spatial_hash_query(self._h, nq, _ptr(qxy), _ptr(qradius), _ptr(offsets), _ptr(ids), cap,
                                             ctypes.byref(total)), "blobs_spatial_hash_query")
        return offsets, ids[:int(total.value)]
