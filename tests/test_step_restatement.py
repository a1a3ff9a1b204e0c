"""The oracle's step against a second, independent restatement of the
reference's substep loop, written here line by line in NumPy float32
scalars (every operation rounds to f32, none is fused, as in the Rust
source): Physics::step -> integrate (physics.rs:78-82, :397-422) with
apply_gravity (:369-375), brute_force_collisions (:241-317, push-out branch
and snapshot refresh included), Spring::apply_force (springs.rs:25-47, the
f32 - Vec2 broadcast included), update_objects (:323-367, the old_dt quirk
included) and apply_constraints (:377-395), plus the axis-aligned wall
extension after the constraints, and the CollisionEvent of every pair in
contact (:288-311), and solve_fixed_joints (:424-477, atan2 through the C
library's atan2f, which the oracle also calls).  Single-sphere bodies at
offset zero, with sensors and collision groups (groups.rs:52-57).

The oracle and this restatement share no code; agreeing bit for bit over
several steps of overlapping worlds (three-way and coincident contacts,
velocity requests, static bodies, damped springs, a circle constraint,
walls) pins the oracle's order of operations to the reference's.
"""
import ctypes
import ctypes.util

import numpy as np
import pytest

from blobs_gb300 import scenes
from oracle import oracle

F = np.float32

_libm = ctypes.CDLL(ctypes.util.find_library("m"))
_libm.atan2f.restype = ctypes.c_float
_libm.atan2f.argtypes = [ctypes.c_float, ctypes.c_float]
for _fn in (_libm.sinf, _libm.cosf):
    _fn.restype = ctypes.c_float
    _fn.argtypes = [ctypes.c_float]


def _atan2(y, x):
    """f32::atan2 (the C library's atan2f)."""
    return F(_libm.atan2f(float(y), float(x)))


def _sinf(x):
    return F(_libm.sinf(float(x)))


def _cosf(x):
    return F(_libm.cosf(float(x)))


def _len(x, y):
    # glam Vec2::length: (x*x + y*y).sqrt()
    return np.sqrt(F(x * x) + F(y * y))


class RefWorld:
    """The reference Physics in f32 scalars: bodies in arena order, each
    with its colliders (handles listed twice, physics.rs:144 and
    collider.rs:180), colliders in arena order."""

    def __init__(self, s):
        n, nc = s.n_bodies, len(s.col_parent)
        self.n, self.nc = n, nc
        self.pos = [[F(v) for v in row] for row in s.pos]
        self.pos_old = [list(r) for r in self.pos]
        self.vreq = [([F(v) for v in s.vreq[i]] if s.vreq_set[i] else None) for i in range(n)]
        self.static = [bool(s.body_type[i] == 1) for i in range(n)]
        self.gmod = [F(v) for v in s.gravity_mod]
        self.rot = [F(v) for v in s.rotation]
        self.vel = [[F(0.0), F(0.0)] for _ in range(n)]
        self.parent = [int(v) for v in s.col_parent]
        self.off = [[F(v) for v in o] for o in s.col_offset]
        self.r = [F(v) for v in s.col_radius]
        self.sensor = [bool(v) for v in s.col_sensor]
        self.memb = [int(v) for v in s.col_memb]
        self.filt = [int(v) for v in s.col_filt]
        self.mass_override = [None if np.isnan(v) else F(v) for v in s.col_mass_override]
        self.cols = [[] for _ in range(n)]
        for c in range(nc):
            self.cols[self.parent[c]] += [c, c]
        # rigid_body.rs:96-128 with collider.rs:40-42: mass_override or
        # radius * 2 per listed handle, sensors add nothing, a total of 0
        # becomes 1
        self.m = []
        for i in range(n):
            m = F(0.0)
            for c in self.cols[i]:
                if not self.sensor[c]:
                    mc = self.mass_override[c]
                    m = F(m + (F(self.r[c] * F(2.0)) if mc is None else mc))
            self.m.append(F(1.0) if m == F(0.0) else m)
        # the wall extension's bounding radius: max |offset| + radius
        self.bound = [F(0.0)] * n
        for c in range(nc):
            self.bound[self.parent[c]] = max(self.bound[self.parent[c]], F(_len(*self.off[c]) + self.r[c]))
        if s.col_snap is not None:
            self.snap = [[F(v) for v in row] for row in s.col_snap]
        else:
            self.snap = [self._xform(self.parent[c], c) for c in range(nc)]
        self.g = [F(v) for v in s.gravity]
        self.old_dt = F(1.0)  # Physics::new
        self.circles = [[F(v) for v in c] for c in s.circles]
        self.box = [F(v) for v in s.world_box[0]] if s.world_box is not None and len(s.world_box) else None
        self.springs = [(int(a), int(b), F(rest), F(k), F(c))
                        for a, b, rest, k, c in zip(s.spr_a, s.spr_b, s.spr_rest, s.spr_k, s.spr_c)]
        self.joints = [(int(a), int(b), [F(v) for v in aa], [F(v) for v in ab], F(d), F(t))
                       for a, b, aa, ab, d, t in zip(s.jnt_a, s.jnt_b, s.jnt_anchor_a, s.jnt_anchor_b,
                                                     s.jnt_distance, s.jnt_target)]
        self.contacts = 0
        self.events = []  # (a, b, impact velocity a, impact velocity b)
        self.group_skips = 0  # pairs in range that the groups keep apart

    def _xform(self, i, c):
        """(body.transform() * collider.offset).translation: Mat2::from_angle
        columns (cos, sin), (-sin, cos) times the offset, plus the position."""
        sn, cs = _sinf(self.rot[i]), _cosf(self.rot[i])
        ox, oy = self.off[c]
        p = self.pos[i]
        return [F(F(F(cs * ox) + F(F(-sn) * oy)) + p[0]), F(F(F(sn * ox) + F(cs * oy)) + p[1])]

    def step(self, delta):
        dt_total = F(delta)                      # delta as f32
        dt = F(dt_total / F(8.0))                # integrate: delta / substeps
        for _ in range(8):
            acc = [[F(0.0), F(0.0)] for _ in range(self.n)]
            for i in range(self.n):             # apply_gravity
                if not self.static[i]:
                    acc[i][0] = F(acc[i][0] + F(self.g[0] * self.gmod[i]))
                    acc[i][1] = F(acc[i][1] + F(self.g[1] * self.gmod[i]))
            for spring in self.springs:
                self._spring(spring, acc)
            self._collisions()
            self._joints(dt)
            self._update_objects(dt, acc)
            self._constraints()

    def _spring(self, spring, acc):
        a, b, rest, k, c = spring
        pa, pb = self.pos[a], self.pos[b]
        dx, dy = F(pb[0] - pa[0]), F(pb[1] - pa[1])
        dist = _len(dx, dy)
        ux, uy = F(dx / dist), F(dy / dist)
        rvx, rvy = F(self.vel[a][0] - self.vel[b][0]), F(self.vel[a][1] - self.vel[b][1])
        dot = F(F(rvx * ux) + F(rvy * uy))
        cd = F(c * dot)
        damp_x, damp_y = F(cd * ux), F(cd * uy)
        sk = F(k * F(dist - rest))
        mx, my = F(sk - damp_x), F(sk - damp_y)  # f32 - Vec2: the scalar minus each component
        fx, fy = F(ux * mx), F(uy * my)
        if not self.static[a]:  # RigidBody::apply_force: a = F / m
            acc[a][0] = F(acc[a][0] + F(fx / self.m[a]))
            acc[a][1] = F(acc[a][1] + F(fy / self.m[a]))
        if not self.static[b]:
            acc[b][0] = F(acc[b][0] + F(F(-fx) / self.m[b]))
            acc[b][1] = F(acc[b][1] + F(F(-fy) / self.m[b]))

    def _collisions(self):
        P, S = self.pos, self.snap
        for a in range(self.nc):                # idx_a, then idx_b among the earlier keys
            for b in range(a):
                # InteractionGroups::test, both ways
                if not (self.memb[a] & self.filt[b] and self.memb[b] & self.filt[a]):
                    if _len(F(S[a][0] - S[b][0]), F(S[a][1] - S[b][1])) < F(self.r[a] + self.r[b]):
                        self.group_skips += 1
                    continue
                ia, ib = self.parent[a], self.parent[b]
                if ia == ib:                    # colliders share a rigid body
                    continue
                ax, ay = F(S[a][0] - S[b][0]), F(S[a][1] - S[b][1])
                dist = _len(ax, ay)
                min_dist = F(self.r[a] + self.r[b])
                if not dist < min_dist:
                    continue
                if dist < F(1e-6):
                    P[ia][0] = F(P[ia][0] + F(0.01))
                    P[ia][1] = F(P[ia][1] + F(0.0))
                    P[ib][0] = F(P[ib][0] - F(0.01))
                    P[ib][1] = F(P[ib][1] - F(0.0))
                    # position + offset translation (not rotated)
                    S[a] = [F(P[ia][0] + self.off[a][0]), F(P[ia][1] + self.off[a][1])]
                    S[b] = [F(P[ib][0] + self.off[b][0]), F(P[ib][1] + self.off[b][1])]
                    ax, ay = F(S[a][0] - S[b][0]), F(S[a][1] - S[b][1])
                    dist = _len(ax, ay)
                impact = (list(self.vel[ia]), list(self.vel[ib]))
                if not self.sensor[a] and not self.sensor[b]:
                    nx, ny = F(ax / dist), F(ay / dist)
                    delta = F(min_dist - dist)
                    ratio = F(F(1.0) - F(self.m[ia] / F(self.m[ia] + self.m[ib])))
                    ka = F(ratio * delta)
                    P[ia][0] = F(P[ia][0] + F(ka * nx))
                    P[ia][1] = F(P[ia][1] + F(ka * ny))
                    kb = F(F(F(1.0) - ratio) * delta)
                    P[ib][0] = F(P[ib][0] - F(kb * nx))
                    P[ib][1] = F(P[ib][1] - F(kb * ny))
                self.contacts += 1
                self.events.append((a, b, impact[0], impact[1]))

    def _joints(self, dt):
        for _ in range(4):  # joint_iterations
            for a, b, anc_a, anc_b, jd, target in self.joints:
                pa, pb = self.pos[a], self.pos[b]
                wa = [F(pa[0] + anc_a[0]), F(pa[1] + anc_a[1])]
                wb = [F(pb[0] + anc_b[0]), F(pb[1] + anc_b[1])]
                dx, dy = F(wb[0] - wa[0]), F(wb[1] - wa[1])
                dist = _len(dx, dy)
                if dist < F(1e-6):
                    continue
                off = F(dist - jd)
                cx, cy = F(F(off * dx) / dist), F(F(off * dy) / dist)  # off_by * delta / distance
                ia, ib = F(F(1.0) / self.m[a]), F(F(1.0) / self.m[b])  # recip
                inv_sum = F(ia + ib)
                if self.static[a]:
                    pb[0], pb[1] = F(pb[0] - F(inv_sum * cx)), F(pb[1] - F(inv_sum * cy))
                elif self.static[b]:
                    pa[0], pa[1] = F(pa[0] + F(inv_sum * cx)), F(pa[1] + F(inv_sum * cy))
                else:
                    ratio = F(ia / inv_sum)
                    pa[0], pa[1] = F(pa[0] + F(ratio * cx)), F(pa[1] + F(ratio * cy))
                    q = F(F(1.0) - ratio)
                    pb[0], pb[1] = F(pb[0] - F(q * cx)), F(pb[1] - F(q * cy))
                ang_a = _atan2(dy, dx)
                ang_b = F(-_atan2(dy, F(-dx)))
                corr = F(F(F(ang_b - ang_a) - target) * F(0.5))
                self.rot[a] = F(self.rot[a] + F(corr * dt))
                self.rot[b] = F(self.rot[b] - F(corr * dt))

    def _update_objects(self, dt, acc):
        for i in range(self.n):
            p, po = self.pos[i], self.pos_old[i]
            if self.static[i]:
                self.pos_old[i] = list(p)
                self.vel[i] = [F(0.0), F(0.0)]
                continue
            if self.vreq[i] is not None:
                q = self.vreq[i]
                self.vreq[i] = None
                po = [F(p[0] - F(q[0] * dt)), F(p[1] - F(q[1] * dt))]
            k = F(dt / self.old_dt)
            dx, dy = F(F(p[0] - po[0]) * k), F(F(p[1] - po[1]) * k)
            self.old_dt = dt
            self.pos_old[i] = list(p)
            self.pos[i] = [F(p[0] + F(dx + F(F(acc[i][0] * dt) * dt))),
                           F(p[1] + F(dy + F(F(acc[i][1] * dt) * dt)))]
            # no torque: angular_velocity and rotation keep their values
            self.vel[i] = [F(dx / dt), F(dy / dt)]
        for i in range(self.n):
            for c in self.cols[i]:
                self.snap[c] = self._xform(i, c)

    def _constraints(self):
        for cx, cy, radius in self.circles:
            for i in range(self.n):
                tx, ty = F(self.pos[i][0] - cx), F(self.pos[i][1] - cy)
                dist = _len(tx, ty)
                if dist > radius:
                    self.pos[i] = [F(cx + F(F(tx / dist) * radius)), F(cy + F(F(ty / dist) * radius))]
        if self.box is not None:
            lo_x, lo_y, hi_x, hi_y = self.box
            for i in range(self.n):
                r = self.bound[i]
                self.pos[i][0] = min(max(self.pos[i][0], F(lo_x + r)), F(hi_x - r))
                self.pos[i][1] = min(max(self.pos[i][1], F(lo_y + r)), F(hi_y - r))

    def bodies(self):
        return {"pos": np.array(self.pos, np.float64), "pos_old": np.array(self.pos_old, np.float64),
                "vel": np.array(self.vel, np.float64), "rotation": np.array(self.rot, np.float64)}


def _world(seed, n, walls, circle, coincident, statics, springs=False, sensors_groups=False, joints=False):
    rng = np.random.Generator(np.random.PCG64(seed))
    h = 0.9
    pos = rng.uniform(-h, h, (n, 2)).astype(np.float32)
    rad = rng.uniform(0.05, 0.15, n).astype(np.float32)
    vel = rng.normal(0.0, 1.0, (n, 2)).astype(np.float32)
    if coincident:
        pos[7] = pos[3]  # the push-out branch (physics.rs:272-286)
    bt = np.zeros(n, np.uint8)
    if statics:
        bt[::9] = 1
    s = scenes.spheres(pos, rad, vel, box=(-1.0, -1.0, 1.0, 1.0) if walls else None, body_type=bt)
    if circle:
        s.circles = np.array([[0.1, -0.05, 0.8]], np.float32)
    if sensors_groups:
        s.col_sensor = (np.arange(n) % 5 == 2).astype(np.uint8)
        s.col_memb = rng.choice(np.array([1, 2, 3, 0xffffffff], np.uint32), n)
        s.col_filt = rng.choice(np.array([1, 2, 3, 0xffffffff], np.uint32), n)
    if joints:
        # chains of four and pairs, anchors off the centres, some to static bodies
        a = np.array([1, 2, 3, 10, 20, 27, 30, 40], np.uint32)
        b = np.array([2, 3, 4, 11, 21, 28, 31, 41], np.uint32)
        scenes.add_fixed_joints(s, a, b, rng.uniform(-0.05, 0.05, (8, 2)), rng.uniform(-0.05, 0.05, (8, 2)))
    if springs:
        a = rng.integers(0, n, 40)
        b = (a + rng.integers(1, n, 40)) % n
        s.spr_a, s.spr_b = a.astype(np.uint32), b.astype(np.uint32)
        s.spr_rest = rng.uniform(0.1, 0.6, 40).astype(np.float32)
        s.spr_k = rng.uniform(5.0, 80.0, 40).astype(np.float32)
        s.spr_c = rng.uniform(0.0, 2.0, 40).astype(np.float32)
    return s


@pytest.mark.parametrize("seed,walls,circle,coincident,statics,springs", [
    (1, True, False, False, False, False),
    (2, False, True, True, False, False),
    (3, True, True, False, True, False),
    (4, True, False, True, True, False),
    (6, True, False, False, False, True),
    (7, True, True, True, True, True),
])
def test_oracle_equals_the_line_by_line_restatement(seed, walls, circle, coincident, statics, springs):
    s = _world(seed, 48, walls, circle, coincident, statics, springs)
    dt, steps = 1.0 / 60.0, 3
    ref = RefWorld(s)
    for _ in range(steps):
        ref.step(dt)
    o = oracle.OracleWorld(s, 32)
    assert o.step(dt, steps) == 0
    got = o.bodies()
    want = ref.bodies()
    assert ref.contacts > 100  # overlapping worlds: many contacts each substep
    for k in ("pos", "pos_old", "vel"):
        assert np.array_equal(got[k], want[k]), (k, float(np.abs(got[k] - want[k]).max()))
    assert o.contacts == ref.contacts
    if coincident:
        assert o.pushouts >= 1
    if springs:
        # the springs move the result (both sides read them)
        s.spr_a, s.spr_b = s.spr_a[:0], s.spr_b[:0]
        s.spr_rest, s.spr_k, s.spr_c = s.spr_rest[:0], s.spr_k[:0], s.spr_c[:0]
        bare = RefWorld(s)
        for _ in range(steps):
            bare.step(dt)
        assert not np.array_equal(bare.bodies()["pos"], want["pos"])


def test_restatement_reacts_to_the_pair_order():
    """The restatement is sensitive to what it pins: resolving the pairs with
    the inner index first (a different sequence) changes the result."""
    s = _world(5, 32, True, False, False, False)
    a = RefWorld(s)
    a.step(1.0 / 60.0)
    b = RefWorld(s)
    orig = b._collisions

    def swapped():
        P, S = b.pos, b.snap
        # same pairs, each body's partners visited in descending order
        for a_ in range(b.n - 1, -1, -1):
            for c in range(a_ - 1, -1, -1):
                ax, ay = F(S[a_][0] - S[c][0]), F(S[a_][1] - S[c][1])
                dist = _len(ax, ay)
                md = F(b.r[a_] + b.r[c])
                if not dist < md:
                    continue
                nx, ny = F(ax / dist), F(ay / dist)
                d = F(md - dist)
                ratio = F(F(1.0) - F(b.m[a_] / F(b.m[a_] + b.m[c])))
                ka, kb = F(ratio * d), F(F(F(1.0) - ratio) * d)
                P[a_][0], P[a_][1] = F(P[a_][0] + F(ka * nx)), F(P[a_][1] + F(ka * ny))
                P[c][0], P[c][1] = F(P[c][0] - F(kb * nx)), F(P[c][1] - F(kb * ny))
    b._collisions = swapped
    b.step(1.0 / 60.0)
    b._collisions = orig
    assert not np.array_equal(a.bodies()["pos"], b.bodies()["pos"])


@pytest.mark.parametrize("seed,coincident", [(8, False), (9, True)])
def test_oracle_events_sensors_and_groups_equal_the_restatement(seed, coincident):
    """Sensors (counted and reported, never corrected, mass 1), collision
    groups, and the event stream in the reference's order with the parents'
    calculated_velocity as impact velocities."""
    s = _world(seed, 48, True, False, coincident, True, True, sensors_groups=True)
    dt, steps = 1.0 / 60.0, 3
    ref = RefWorld(s)
    for _ in range(steps):
        ref.step(dt)
    o = oracle.OracleWorld(s, 32, record_events=True)
    assert o.step(dt, steps) == 0
    got, want = o.bodies(), ref.bodies()
    for k in ("pos", "pos_old", "vel"):
        assert np.array_equal(got[k], want[k]), (k, float(np.abs(got[k] - want[k]).max()))
    a, b, va, vb = o.events()
    assert len(a) == len(ref.events) == ref.contacts == o.contacts and len(a) > 100
    assert np.array_equal(a, [e[0] for e in ref.events]) and np.array_equal(b, [e[1] for e in ref.events])
    assert np.array_equal(va, np.array([e[2] for e in ref.events], np.float64))
    assert np.array_equal(vb, np.array([e[3] for e in ref.events], np.float64))
    # sensors and groups both bite: some reported pairs are not corrected,
    # some pairs in range are not reported
    assert any(ref.sensor[e[0]] or ref.sensor[e[1]] for e in ref.events)
    assert ref.group_skips > 0


@pytest.mark.parametrize("seed,statics", [(10, False), (11, True)])
def test_oracle_fixed_joints_equal_the_restatement(seed, statics):
    """Fixed joints between single-sphere bodies (anchors not rotated, as in
    the reference), swept 4 times per substep in arena order; positions and
    rotations equal the oracle's bit for bit."""
    s = _world(seed, 48, True, False, False, statics, True, joints=True)
    dt, steps = 1.0 / 60.0, 3
    ref = RefWorld(s)
    for _ in range(steps):
        ref.step(dt)
    o = oracle.OracleWorld(s, 32)
    assert o.step(dt, steps) == 0
    got, want = o.bodies(), ref.bodies()
    for k in ("pos", "pos_old", "vel", "rotation"):
        assert np.array_equal(got[k], want[k]), (k, float(np.abs(got[k] - want[k]).max()))
    assert np.abs(want["rotation"]).max() > 1e-3  # the joints turned the bodies
    if statics:
        assert any(ref.static[j[0]] or ref.static[j[1]] for j in ref.joints)


def _multi_world(seed, n=28):
    """Bodies of one to three colliders at offsets, some sensors and group
    masks and mass overrides, static and kinematic bodies, per-body gravity
    scales, jointed in pairs and chains (so the bodies turn and the offsets
    rotate), springs, walls."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = scenes.empty_scene(n)
    s.pos = rng.uniform(-0.8, 0.8, (n, 2)).astype(np.float32)
    s.vreq = rng.normal(0.0, 1.0, (n, 2)).astype(np.float32)
    s.vreq_set = np.ones(n, np.uint8)
    # static bodies, and kinematic ones (RigidBodyType 2, 3: moved like
    # dynamic ones by this loop, which only tests is_static)
    s.body_type = np.where(np.arange(n) % 11 == 5, 1, np.where(np.arange(n) % 7 == 3, 2 + (np.arange(n) % 2), 0))
    s.body_type = s.body_type.astype(np.uint8)
    s.gravity_mod = rng.uniform(0.0, 2.0, n).astype(np.float32)
    k = rng.integers(1, 4, n)
    parent = np.repeat(np.arange(n), k).astype(np.uint32)
    nc = len(parent)
    s.col_parent = parent
    s.col_offset = rng.uniform(-0.12, 0.12, (nc, 2)).astype(np.float32)
    s.col_radius = rng.uniform(0.04, 0.1, nc).astype(np.float32)
    s.col_mass_override = np.where(rng.uniform(0, 1, nc) < 0.2, rng.uniform(0.05, 0.5, nc), np.nan).astype(np.float32)
    s.col_sensor = (rng.uniform(0, 1, nc) < 0.15).astype(np.uint8)
    s.col_memb = rng.choice(np.array([1, 2, 3, 0xffffffff], np.uint32), nc)
    s.col_filt = rng.choice(np.array([1, 3, 0xffffffff, 0xffffffff], np.uint32), nc)
    s.gravity = np.array([0.0, -9.81], np.float32)
    s.world_box = np.array([[-1.0, -1.0, 1.0, 1.0]], np.float32)
    a = np.array([0, 1, 2, 6, 9, 14, 15, 20, 24], np.uint32)
    b = np.array([1, 2, 3, 7, 10, 16, 5, 21, 25], np.uint32)
    scenes.add_fixed_joints(s, a, b, rng.uniform(-0.05, 0.05, (9, 2)), rng.uniform(-0.05, 0.05, (9, 2)))
    sa = rng.integers(0, n, 12)
    s.spr_a, s.spr_b = sa.astype(np.uint32), ((sa + rng.integers(1, n, 12)) % n).astype(np.uint32)
    s.spr_rest = rng.uniform(0.1, 0.5, 12).astype(np.float32)
    s.spr_k = rng.uniform(5.0, 50.0, 12).astype(np.float32)
    s.spr_c = rng.uniform(0.0, 1.0, 12).astype(np.float32)
    return s


@pytest.mark.parametrize("seed", [12, 13])
def test_oracle_multi_collider_bodies_equal_the_restatement(seed):
    """The general path's semantics: colliders at rotated offsets (sinf and
    cosf of the body's rotation), the same-body skip, mass summed over the
    doubled handle list with overrides and sensors, the wall extension's
    bounding radius; positions, rotations and events bit for bit."""
    s = _multi_world(seed)
    dt, steps = 1.0 / 60.0, 3
    ref = RefWorld(s)
    for _ in range(steps):
        ref.step(dt)
    o = oracle.OracleWorld(s, 32, record_events=True)
    assert o.step(dt, steps) == 0
    got, want = o.bodies(), ref.bodies()
    for k in ("pos", "pos_old", "vel", "rotation"):
        assert np.array_equal(got[k], want[k]), (k, float(np.abs(got[k] - want[k]).max()))
    a, b, va, vb = o.events()
    assert len(a) == len(ref.events) == o.contacts and len(a) > 50
    assert np.array_equal(a, [e[0] for e in ref.events]) and np.array_equal(b, [e[1] for e in ref.events])
    assert np.array_equal(va, np.array([e[2] for e in ref.events], np.float64))
    assert np.array_equal(vb, np.array([e[3] for e in ref.events], np.float64))
    assert np.abs(want["rotation"]).max() > 1e-3 and max(len(c) for c in ref.cols) == 6
    assert np.array_equal(o.snapshots(), np.array(ref.snap, np.float64))
