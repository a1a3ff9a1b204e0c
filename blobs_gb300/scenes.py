"""Seeded synthetic scenes for the blobs step (no dataset exists for this path).

A :class:`Scene` is the structure-of-arrays form of a reference ``Physics``
world (blobs/src/physics.rs:3-34) in arena order: what
``RigidBodyBuilder`` / ``ColliderBuilder`` / ``Spring`` / ``create_fixed_joint``
would have inserted, one record per slot.  Several independent worlds can be
packed back to back (:func:`pack`), which is the batched mode.

The generators build the five workloads of the benchmark definition with
numpy PCG64 seeds; every float is float32 and computed with float32
operations where the reference computes it (joint distance, target angle).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence

import numpy as np

ALL_GROUPS = 0xFFFFFFFF
DYNAMIC, STATIC, KINEMATIC_POSITION, KINEMATIC_VELOCITY = 0, 1, 2, 3


def _f32(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if shape is not None:
        a = a.reshape(shape)
    return a


@dataclasses.dataclass
class Scene:
    # bodies (rigid_body.rs:42-74)
    pos: np.ndarray                      # (n, 2) position
    vreq: np.ndarray                     # (n, 2) velocity_request value
    vreq_set: np.ndarray                 # (n,)  velocity_request is Some
    body_type: np.ndarray                # (n,)  RigidBodyType
    gravity_mod: np.ndarray              # (n,)
    rotation: np.ndarray                 # (n,)
    angvel: np.ndarray                   # (n,)
    # colliders (collider.rs:3-20)
    col_parent: np.ndarray               # (c,) dense body index
    col_offset: np.ndarray               # (c, 2) offset.translation
    col_radius: np.ndarray               # (c,)
    col_mass_override: np.ndarray        # (c,) NaN = None
    col_sensor: np.ndarray               # (c,)
    col_memb: np.ndarray                 # (c,)
    col_filt: np.ndarray                 # (c,)
    # springs (springs.rs:16-22)
    spr_a: np.ndarray
    spr_b: np.ndarray
    spr_rest: np.ndarray
    spr_k: np.ndarray
    spr_c: np.ndarray
    # fixed joints (joints.rs:7-19)
    jnt_a: np.ndarray
    jnt_b: np.ndarray
    jnt_anchor_a: np.ndarray
    jnt_anchor_b: np.ndarray
    jnt_distance: np.ndarray
    jnt_target: np.ndarray
    # circle constraints (lib.rs:189-193), (k, 3)
    circles: np.ndarray
    # knobs (physics.rs:6-27)
    gravity: np.ndarray = dataclasses.field(default_factory=lambda: np.array([0.0, -9.81], np.float32))
    substeps: int = 8
    joint_iterations: int = 4
    collisions_enabled: bool = True
    # optional state
    pos_old: Optional[np.ndarray] = None
    acc: Optional[np.ndarray] = None
    vel: Optional[np.ndarray] = None
    torque: Optional[np.ndarray] = None
    col_snap: Optional[np.ndarray] = None
    mass: Optional[np.ndarray] = None
    inertia: Optional[np.ndarray] = None
    # batching: offsets (n_worlds + 1) per arena, walls per world (n_worlds, 4)
    world_body_offsets: Optional[np.ndarray] = None
    world_collider_offsets: Optional[np.ndarray] = None
    world_spring_offsets: Optional[np.ndarray] = None
    world_joint_offsets: Optional[np.ndarray] = None
    world_box: Optional[np.ndarray] = None
    # workload description
    dt: float = 1.0 / 60.0
    n_steps: int = 1
    name: str = "scene"
    seed: int = 0

    @property
    def n_bodies(self) -> int:
        return int(self.pos.shape[0])

    @property
    def n_colliders(self) -> int:
        return int(self.col_parent.shape[0])

    @property
    def n_springs(self) -> int:
        return int(self.spr_a.shape[0])

    @property
    def n_joints(self) -> int:
        return int(self.jnt_a.shape[0])

    @property
    def n_worlds(self) -> int:
        return 1 if self.world_body_offsets is None else int(len(self.world_body_offsets) - 1)

    def single_collider(self) -> bool:
        return (self.n_colliders == self.n_bodies
                and np.array_equal(self.col_parent, np.arange(self.n_bodies, dtype=np.uint32))
                and not np.any(self.col_offset))

    def copy(self) -> "Scene":
        return dataclasses.replace(self, **{
            f.name: (getattr(self, f.name).copy() if isinstance(getattr(self, f.name), np.ndarray)
                     else getattr(self, f.name))
            for f in dataclasses.fields(self)})


def empty_scene(n_bodies: int = 0) -> Scene:
    z2 = np.zeros((0, 2), np.float32)
    zu = np.zeros(0, np.uint32)
    zf = np.zeros(0, np.float32)
    return Scene(
        pos=np.zeros((n_bodies, 2), np.float32), vreq=np.zeros((n_bodies, 2), np.float32),
        vreq_set=np.zeros(n_bodies, np.uint8), body_type=np.zeros(n_bodies, np.uint8),
        gravity_mod=np.ones(n_bodies, np.float32), rotation=np.zeros(n_bodies, np.float32),
        angvel=np.zeros(n_bodies, np.float32),
        col_parent=zu.copy(), col_offset=z2.copy(), col_radius=zf.copy(), col_mass_override=zf.copy(),
        col_sensor=np.zeros(0, np.uint8), col_memb=zu.copy(), col_filt=zu.copy(),
        spr_a=zu.copy(), spr_b=zu.copy(), spr_rest=zf.copy(), spr_k=zf.copy(), spr_c=zf.copy(),
        jnt_a=zu.copy(), jnt_b=zu.copy(), jnt_anchor_a=z2.copy(), jnt_anchor_b=z2.copy(),
        jnt_distance=zf.copy(), jnt_target=zf.copy(), circles=np.zeros((0, 3), np.float32))


def spheres(pos, radius, vel=None, *, gravity=(0.0, -9.81), box=None, body_type=None) -> Scene:
    """One single-sphere body per row, the demo's spawn idiom
    (demo/src/simulation.rs:99-146): position, velocity_request, a collider at
    offset zero whose absolute transform starts at the body position."""
    pos = _f32(pos, (-1, 2))
    n = pos.shape[0]
    s = empty_scene(n)
    s.pos = pos
    if vel is not None:
        s.vreq = _f32(vel, (n, 2))
        s.vreq_set = np.ones(n, np.uint8)
    if body_type is not None:
        s.body_type = np.ascontiguousarray(np.asarray(body_type, np.uint8))
    s.col_parent = np.arange(n, dtype=np.uint32)
    s.col_offset = np.zeros((n, 2), np.float32)
    s.col_radius = _f32(radius, (n,))
    s.col_mass_override = np.full(n, np.nan, np.float32)
    s.col_sensor = np.zeros(n, np.uint8)
    s.col_memb = np.full(n, ALL_GROUPS, np.uint32)
    s.col_filt = np.full(n, ALL_GROUPS, np.uint32)
    s.gravity = _f32(gravity, (2,))
    if box is not None:
        s.world_box = _f32(box, (1, 4))
    return s


def fixed_joint_params(pos_a, pos_b, anchor_a, anchor_b, rot_a, rot_b):
    """Physics::create_fixed_joint (physics.rs:184-207, :230): distance =
    |pa + anchor_a - pb - anchor_b| in float32, target_angle = rot_b - rot_a."""
    pa, pb = _f32(pos_a, (-1, 2)), _f32(pos_b, (-1, 2))
    aa, ab = _f32(anchor_a, (-1, 2)), _f32(anchor_b, (-1, 2))
    d = ((pa + aa) - pb) - ab
    dist = np.sqrt((d[:, 0] * d[:, 0]) + (d[:, 1] * d[:, 1])).astype(np.float32)
    tgt = (_f32(rot_b) - _f32(rot_a)).astype(np.float32)
    return dist, tgt


def add_fixed_joints(s: Scene, a, b, anchor_a=None, anchor_b=None) -> None:
    a = np.asarray(a, np.uint32)
    b = np.asarray(b, np.uint32)
    k = len(a)
    anchor_a = np.zeros((k, 2), np.float32) if anchor_a is None else _f32(anchor_a, (k, 2))
    anchor_b = np.zeros((k, 2), np.float32) if anchor_b is None else _f32(anchor_b, (k, 2))
    dist, tgt = fixed_joint_params(s.pos[a], s.pos[b], anchor_a, anchor_b, s.rotation[a], s.rotation[b])
    s.jnt_a = np.concatenate([s.jnt_a, a])
    s.jnt_b = np.concatenate([s.jnt_b, b])
    s.jnt_anchor_a = np.concatenate([s.jnt_anchor_a, anchor_a])
    s.jnt_anchor_b = np.concatenate([s.jnt_anchor_b, anchor_b])
    s.jnt_distance = np.concatenate([s.jnt_distance, dist])
    s.jnt_target = np.concatenate([s.jnt_target, tgt])


def add_springs(s: Scene, a, b, k, c, rest=None) -> None:
    a = np.asarray(a, np.uint32)
    b = np.asarray(b, np.uint32)
    if rest is None:
        d = s.pos[b] - s.pos[a]
        rest = np.sqrt((d[:, 0] * d[:, 0]) + (d[:, 1] * d[:, 1])).astype(np.float32)
    s.spr_a = np.concatenate([s.spr_a, a])
    s.spr_b = np.concatenate([s.spr_b, b])
    s.spr_rest = np.concatenate([s.spr_rest, _f32(rest, (-1,))])
    s.spr_k = np.concatenate([s.spr_k, _f32(k, (-1,)) * np.ones(len(a), np.float32)])
    s.spr_c = np.concatenate([s.spr_c, _f32(c, (-1,)) * np.ones(len(a), np.float32)])


def _nonoverlapping(rng, n, rmin, rmax, lo, hi, max_tries=2000):
    """Rejection sampling of non-overlapping spheres inside walls [lo, hi]^2."""
    cell = 2.0 * rmax
    grid = {}
    pos = np.zeros((n, 2), np.float32)
    rad = rng.uniform(rmin, rmax, n).astype(np.float32)
    for i in range(n):
        r = float(rad[i])
        for _ in range(max_tries):
            p = rng.uniform(lo + r, hi - r, 2).astype(np.float32)
            cx, cy = int(math.floor(p[0] / cell)), int(math.floor(p[1] / cell))
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for j in grid.get((cx + dx, cy + dy), ()):
                        q = pos[j]
                        if (float(p[0]) - q[0]) ** 2 + (float(p[1]) - q[1]) ** 2 < (r + rad[j]) ** 2:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                pos[i] = p
                grid.setdefault((cx, cy), []).append(i)
                break
        else:
            raise RuntimeError("could not place sphere %d" % i)
    return pos, rad


def box_side(n: int, rmin: float, rmax: float, packing: float) -> float:
    """Side of the square box in which n spheres with r ~ U[rmin, rmax] cover
    `packing` of the area (E[r^2] = (rmax^3 - rmin^3) / (3 (rmax - rmin)))."""
    er2 = (rmax ** 3 - rmin ** 3) / (3.0 * (rmax - rmin))
    return math.sqrt(n * math.pi * er2 / packing)


def sparse_spheres(seed: int = 1, n: int = 1000, steps: int = 600) -> Scene:
    """1,000 single-sphere bodies, r ~ U[0.1, 0.3], non-overlapping in a 40x40
    walled box, v ~ N(0, 1) per axis, g = (0, -9.81), dt = 1/60, 600 steps."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos, rad = _nonoverlapping(rng, n, 0.1, 0.3, -20.0, 20.0)
    vel = rng.normal(0.0, 1.0, (n, 2)).astype(np.float32)
    s = spheres(pos, rad, vel, box=(-20.0, -20.0, 20.0, 20.0))
    s.dt, s.n_steps, s.name, s.seed = 1.0 / 60.0, steps, "sparse_spheres-1k-walled", seed
    return s


def dense_spheres(seed: int = 2, n: int = 1_000_000, steps: int = 1000, literal_box: bool = False,
                  packing: float = 0.40) -> Scene:
    """1M single-sphere bodies, r ~ U[0.05, 0.15], uniform with overlaps in a
    walled square box at 40% packing (side 291.7 for 1M; the literal 2000x2000
    box of the workload text is 0.85% packing and is kept as `literal_box`),
    v ~ N(0, 0.5), g = (0, -9.81), dt = 1/120, 1,000 steps, cell = 2 rmax.
    `packing` changes the box (the settled pile of the rollout's later steps
    is about twice as dense as the start)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    side = 2000.0 if literal_box else box_side(n, 0.05, 0.15, packing)
    h = side / 2.0
    rad = rng.uniform(0.05, 0.15, n).astype(np.float32)
    pos = rng.uniform(-h, h, (n, 2)).astype(np.float32)
    pos = np.clip(pos, -h + rad[:, None], h - rad[:, None]).astype(np.float32)
    vel = rng.normal(0.0, 0.5, (n, 2)).astype(np.float32)
    s = spheres(pos, rad, vel, box=(-h, -h, h, h))
    s.dt, s.n_steps, s.seed = 1.0 / 120.0, steps, seed
    s.name = "dense_spheres-%d-%s" % (n, "2000box" if literal_box else "40pct")
    return s


def _pairs_within(pos, radius_max, rng=None):
    """All body pairs (i < j) closer than radius_max, sorted."""
    from scipy.spatial import cKDTree
    pairs = cKDTree(pos.astype(np.float64)).query_pairs(radius_max, output_type="ndarray").astype(np.int64)
    if len(pairs) == 0:
        return pairs.reshape(0, 2)
    pairs.sort(axis=1)
    d = pos[pairs[:, 0]].astype(np.float64) - pos[pairs[:, 1]]
    pairs = pairs[(d * d).sum(1) < radius_max * radius_max]
    return pairs[np.lexsort((pairs[:, 1], pairs[:, 0]))]


def jointed_bodies(seed: int = 3, n: int = 200_000, n_joints: int = 50_000, n_springs: int = 100_000,
            side: float = 1500.0, steps: int = 500) -> Scene:
    """200k bodies with 1-4 sphere colliders at offsets uniform in a disc of
    radius 0.5, r ~ U[0.1, 0.25]; 50k fixed joints between random body pairs
    closer than 1.5 (sampled without replacement from all such pairs); 100k
    springs, rest = initial distance, k log-U[10, 1e4], c U[0, 2], between
    random pairs closer than 3.0 (1.5 does not hold enough pairs at this
    density); walled 1500x1500 box, dt = 1/120, 500 steps."""
    rng = np.random.Generator(np.random.PCG64(seed))
    h = side / 2.0
    pos = rng.uniform(-h + 1.0, h - 1.0, (n, 2)).astype(np.float32)
    ncol = rng.integers(1, 5, n)
    s = empty_scene(n)
    s.pos = pos
    vel = rng.normal(0.0, 0.5, (n, 2)).astype(np.float32)
    s.vreq = vel
    s.vreq_set = np.ones(n, np.uint8)
    c = int(ncol.sum())
    s.col_parent = np.repeat(np.arange(n, dtype=np.uint32), ncol)
    rr = np.sqrt(rng.uniform(0.0, 1.0, c)) * 0.5
    th = rng.uniform(0.0, 2.0 * np.pi, c)
    s.col_offset = np.stack([rr * np.cos(th), rr * np.sin(th)], 1).astype(np.float32)
    s.col_radius = rng.uniform(0.1, 0.25, c).astype(np.float32)
    s.col_mass_override = np.full(c, np.nan, np.float32)
    s.col_sensor = np.zeros(c, np.uint8)
    s.col_memb = np.full(c, ALL_GROUPS, np.uint32)
    s.col_filt = np.full(c, ALL_GROUPS, np.uint32)
    near = _pairs_within(pos, 1.5, rng)
    pick = rng.choice(len(near), size=min(n_joints, len(near)), replace=False)
    pick.sort()
    jp = near[pick]
    add_fixed_joints(s, jp[:, 0], jp[:, 1])
    far = _pairs_within(pos, 3.0, rng)
    pick = rng.choice(len(far), size=min(n_springs, len(far)), replace=False)
    pick.sort()
    sp = far[pick]
    k = np.exp(rng.uniform(np.log(10.0), np.log(1e4), len(sp))).astype(np.float32)
    cdamp = rng.uniform(0.0, 2.0, len(sp)).astype(np.float32)
    add_springs(s, sp[:, 0], sp[:, 1], k, cdamp)
    s.world_box = np.array([[-h, -h, h, h]], np.float32)
    s.dt, s.n_steps, s.name, s.seed = 1.0 / 120.0, steps, "jointed_bodies-%d-structured" % n, seed
    return s


def random_world(rng, n: int, rmin: float, rmax: float, packing: float, vel_sigma: float,
                 spring_frac: float = 0.0, k_range=(200.0, 200.0), c_range=(1.0, 1.0)) -> Scene:
    """Single-sphere bodies uniform (overlaps allowed) in a walled square box
    at the given packing; a fraction of bodies gets a spring to one of its
    nearest neighbours (rest = initial distance)."""
    side = box_side(n, rmin, rmax, packing)
    h = side / 2.0
    rad = rng.uniform(rmin, rmax, n).astype(np.float32)
    pos = rng.uniform(-h, h, (n, 2)).astype(np.float32)
    pos = np.clip(pos, -h + rad[:, None], h - rad[:, None]).astype(np.float32)
    vel = rng.normal(0.0, vel_sigma, (n, 2)).astype(np.float32)
    s = spheres(pos, rad, vel, box=(-h, -h, h, h))
    if spring_frac > 0.0:
        m = max(1, int(round(spring_frac * n)))
        src = rng.choice(n, size=m, replace=False)
        # a random one of the 4 nearest bodies
        from scipy.spatial import cKDTree
        kk = min(5, n)
        _, nn = cKDTree(pos.astype(np.float64)).query(pos[src].astype(np.float64), k=kk)
        nn = np.asarray(nn).reshape(m, kk)[:, 1:] if kk > 1 else np.asarray(nn).reshape(m, 1)
        dst = nn[np.arange(m), rng.integers(0, nn.shape[1], m)]
        dst = np.where(dst == src, (src + 1) % n, dst)
        a, b = np.minimum(src, dst), np.maximum(src, dst)
        k = np.exp(rng.uniform(np.log(k_range[0]), np.log(k_range[1]), m)).astype(np.float32)
        c = rng.uniform(c_range[0], c_range[1], m).astype(np.float32)
        add_springs(s, a, b, k, c)
    return s


def pack(worlds: Sequence[Scene]) -> Scene:
    """Pack independent worlds back to back (batched mode)."""
    def cat(name, dtype, width=None):
        arrs = [getattr(w, name) for w in worlds]
        return np.ascontiguousarray(np.concatenate(arrs).astype(dtype))

    out = empty_scene(0)
    body_off = np.zeros(len(worlds) + 1, np.uint32)
    col_off = np.zeros(len(worlds) + 1, np.uint32)
    spr_off = np.zeros(len(worlds) + 1, np.uint32)
    jnt_off = np.zeros(len(worlds) + 1, np.uint32)
    for i, w in enumerate(worlds):
        body_off[i + 1] = body_off[i] + w.n_bodies
        col_off[i + 1] = col_off[i] + w.n_colliders
        spr_off[i + 1] = spr_off[i] + w.n_springs
        jnt_off[i + 1] = jnt_off[i] + w.n_joints
    for name, dt in [("pos", np.float32), ("vreq", np.float32), ("vreq_set", np.uint8), ("body_type", np.uint8),
                     ("gravity_mod", np.float32), ("rotation", np.float32), ("angvel", np.float32),
                     ("col_offset", np.float32), ("col_radius", np.float32), ("col_mass_override", np.float32),
                     ("col_sensor", np.uint8), ("col_memb", np.uint32), ("col_filt", np.uint32),
                     ("spr_rest", np.float32), ("spr_k", np.float32), ("spr_c", np.float32),
                     ("jnt_anchor_a", np.float32), ("jnt_anchor_b", np.float32), ("jnt_distance", np.float32),
                     ("jnt_target", np.float32)]:
        setattr(out, name, cat(name, dt))
    out.col_parent = np.concatenate([w.col_parent + body_off[i] for i, w in enumerate(worlds)]).astype(np.uint32)
    out.spr_a = np.concatenate([w.spr_a + body_off[i] for i, w in enumerate(worlds)]).astype(np.uint32)
    out.spr_b = np.concatenate([w.spr_b + body_off[i] for i, w in enumerate(worlds)]).astype(np.uint32)
    out.jnt_a = np.concatenate([w.jnt_a + body_off[i] for i, w in enumerate(worlds)]).astype(np.uint32)
    out.jnt_b = np.concatenate([w.jnt_b + body_off[i] for i, w in enumerate(worlds)]).astype(np.uint32)
    out.circles = worlds[0].circles.copy()
    out.gravity = worlds[0].gravity.copy()
    out.substeps, out.joint_iterations = worlds[0].substeps, worlds[0].joint_iterations
    out.collisions_enabled = worlds[0].collisions_enabled
    out.world_body_offsets, out.world_collider_offsets = body_off, col_off
    out.world_spring_offsets, out.world_joint_offsets = spr_off, jnt_off
    if all(w.world_box is not None for w in worlds):
        out.world_box = np.concatenate([w.world_box for w in worlds]).astype(np.float32)
    out.dt, out.n_steps = worlds[0].dt, worlds[0].n_steps
    out.name = "batch-%d" % len(worlds)
    return out


def unpack_world(s: Scene, w: int) -> Scene:
    """World `w` of a packed scene as a standalone scene."""
    b0, b1 = int(s.world_body_offsets[w]), int(s.world_body_offsets[w + 1])
    c0, c1 = int(s.world_collider_offsets[w]), int(s.world_collider_offsets[w + 1])
    s0, s1 = int(s.world_spring_offsets[w]), int(s.world_spring_offsets[w + 1])
    j0, j1 = int(s.world_joint_offsets[w]), int(s.world_joint_offsets[w + 1])
    out = empty_scene(0)
    for name in ["pos", "vreq", "vreq_set", "body_type", "gravity_mod", "rotation", "angvel"]:
        setattr(out, name, np.ascontiguousarray(getattr(s, name)[b0:b1]))
    for name in ["col_offset", "col_radius", "col_mass_override", "col_sensor", "col_memb", "col_filt"]:
        setattr(out, name, np.ascontiguousarray(getattr(s, name)[c0:c1]))
    out.col_parent = (s.col_parent[c0:c1] - b0).astype(np.uint32)
    for name in ["spr_rest", "spr_k", "spr_c"]:
        setattr(out, name, np.ascontiguousarray(getattr(s, name)[s0:s1]))
    out.spr_a = (s.spr_a[s0:s1] - b0).astype(np.uint32)
    out.spr_b = (s.spr_b[s0:s1] - b0).astype(np.uint32)
    for name in ["jnt_anchor_a", "jnt_anchor_b", "jnt_distance", "jnt_target"]:
        setattr(out, name, np.ascontiguousarray(getattr(s, name)[j0:j1]))
    out.jnt_a = (s.jnt_a[j0:j1] - b0).astype(np.uint32)
    out.jnt_b = (s.jnt_b[j0:j1] - b0).astype(np.uint32)
    out.circles = s.circles.copy()
    out.gravity = s.gravity.copy()
    out.substeps, out.joint_iterations, out.collisions_enabled = s.substeps, s.joint_iterations, s.collisions_enabled
    if s.world_box is not None:
        out.world_box = s.world_box[w:w + 1].copy()
    out.dt, out.n_steps, out.name = s.dt, s.n_steps, "%s[%d]" % (s.name, w)
    return out


def uneven_batch(seed: int = 4, n_worlds: int = 4096, nmin: int = 64, nmax: int = 8192, steps: int = 100) -> Scene:
    """4,096 independent worlds, body counts log-uniform in [64, 8192],
    single spheres r ~ U[0.1, 0.3] at 35% packing in their own walled box,
    v ~ N(0, 1); 10% of each world's bodies get a spring (k = 200, c = 1,
    rest = initial distance) to one of their 4 nearest neighbours; dt = 1/60,
    100-step rollouts."""
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.exp(rng.uniform(np.log(nmin), np.log(nmax), n_worlds)).astype(np.int64)
    worlds = [random_world(rng, int(c), 0.1, 0.3, 0.35, 1.0, spring_frac=0.10) for c in counts]
    s = pack(worlds)
    s.dt, s.n_steps, s.seed = 1.0 / 60.0, steps, seed
    s.name = "uneven_batch-%dworlds-%dbodies" % (n_worlds, s.n_bodies)
    return s


def gradient_batch(seed: int = 5, n_worlds: int = 256, n_per: int = 2048, n_springs: int = 1024, steps: int = 120,
            n_marked: int = 64):
    """256 worlds x 2,048 spheres, r ~ U[0.1, 0.2] at 30% packing (walled box,
    side 22.4), 1,024 springs per world between random nearby pairs with
    k log-U[100, 5000] and c = 0, v ~ N(0, 1); dt = 1/60, 120 steps.  Returns
    (scene, marked body indices, targets): loss = mean over worlds and the 64
    marked bodies of |x_final - target|^2."""
    rng = np.random.Generator(np.random.PCG64(seed))
    worlds = []
    marked = []
    targets = []
    for w in range(n_worlds):
        s = random_world(rng, n_per, 0.1, 0.2, 0.30, 1.0)
        near = _pairs_within(s.pos, 1.0, rng)
        pick = np.sort(rng.choice(len(near), size=min(n_springs, len(near)), replace=False))
        k = np.exp(rng.uniform(np.log(100.0), np.log(5000.0), len(pick))).astype(np.float32)
        add_springs(s, near[pick, 0], near[pick, 1], k, np.zeros(len(pick), np.float32))
        worlds.append(s)
        m = np.sort(rng.choice(n_per, size=n_marked, replace=False))
        marked.append(m)
        targets.append(s.pos[m] + rng.normal(0.0, 1.0, (n_marked, 2)).astype(np.float32))
    s = pack(worlds)
    s.dt, s.n_steps, s.seed = 1.0 / 60.0, steps, seed
    s.name = "gradient_batch-%dx%d" % (n_worlds, n_per)
    return s, marked, targets
