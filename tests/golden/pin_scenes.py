"""Scenes for pinning the oracle against the reference itself, and their
f32 oracle digests (tests/golden/reference_pin.json).

The reference is a Rust crate and no Rust toolchain exists here, so these
scenes are built for a maintainer who has one: every input comes from a
32-bit xorshift stream turned into f32 values by operations that are exact
or single IEEE f32 roundings, so a few lines of Rust generate the same bits
(the harness is in INTEGRATION.md).  The scenes use only the reference's own
features: no wall extension (a circle constraint keeps the bodies together
instead), springs, sensors, collision groups, velocity requests,
two-collider bodies (without joints, so no rotation reaches them), static
and kinematic bodies, per-body gravity scales, and fixed joints between
single-collider bodies (whose rotations, through the C library's atan2f,
do not reach the positions).

    xorshift32:  x ^= x << 13; x ^= x >> 17; x ^= x << 5   (mod 2^32)
    unit():      next x, then (x >> 8) as f32 * 2^-24       (exact)
    lerp(a, b):  a + ((b - a) * unit())                     (each operation an f32 rounding)
    index(n):    (unit() * n as f32) as u32                 (truncation)

Run from the repository root to regenerate the fixture:

    python tests/golden/pin_scenes.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from blobs_gb300 import scenes  # noqa: E402
from oracle import oracle  # noqa: E402

F = np.float32
ALL = 0xFFFFFFFF
FIXTURE = os.path.join(HERE, "reference_pin.json")


class XorShift32:
    def __init__(self, seed: int):
        assert seed != 0
        self.x = seed & 0xFFFFFFFF

    def next(self) -> int:
        x = self.x
        x ^= (x << 13) & 0xFFFFFFFF
        x ^= x >> 17
        x ^= (x << 5) & 0xFFFFFFFF
        self.x = x
        return x

    def unit(self):
        return F(self.next() >> 8) * F(2.0 ** -24)

    def lerp(self, a, b):
        a, b = F(a), F(b)
        return F(a + F(F(b - a) * self.unit()))

    def index(self, n: int) -> int:
        return int(F(self.unit() * F(n)))


def _bodies(g, n, h, rmin, rmax, vmax, ncol, spread=0.0):
    """Bodies in [-h, h]^2 with a velocity request each; `ncol` colliders per
    body, the first at the centre and the others at offsets of up to
    `spread`.  Returns the scene (collider snapshots = position + offset)."""
    s = scenes.empty_scene(n)
    pos = np.zeros((n, 2), np.float32)
    vel = np.zeros((n, 2), np.float32)
    par, off, rad = [], [], []
    for i in range(n):
        pos[i] = (g.lerp(-h, h), g.lerp(-h, h))
        vel[i] = (g.lerp(-vmax, vmax), g.lerp(-vmax, vmax))
        for c in range(ncol):
            par.append(i)
            off.append((F(0.0), F(0.0)) if c == 0 else (g.lerp(-spread, spread), g.lerp(-spread, spread)))
            rad.append(g.lerp(rmin, rmax))
    s.pos, s.vreq, s.vreq_set = pos, vel, np.ones(n, np.uint8)
    s.col_parent = np.array(par, np.uint32)
    s.col_offset = np.array(off, np.float32).reshape(-1, 2)
    s.col_radius = np.array(rad, np.float32)
    nc = len(par)
    s.col_mass_override = np.full(nc, np.nan, np.float32)
    s.col_sensor = np.zeros(nc, np.uint8)
    s.col_memb = np.full(nc, ALL, np.uint32)
    s.col_filt = np.full(nc, ALL, np.uint32)
    s.col_snap = (pos[s.col_parent] + s.col_offset).astype(np.float32)
    s.gravity = np.array([0.0, -9.81], np.float32)
    return s


def pin_scenes():
    """(name, scene, steps, dt) of the fixture, in this order."""
    out = []
    g = XorShift32(0x9E3779B9)
    s = _bodies(g, 400, 3.0, 0.05, 0.15, 1.0, 1)
    s.circles = np.array([[0.0, 0.0, 4.0]], np.float32)
    out.append(("pin_spheres_400", s, 10, 1.0 / 60.0))

    g = XorShift32(0x2545F491)
    s = _bodies(g, 300, 2.5, 0.05, 0.15, 1.0, 1)
    masks = np.array([1, 2, 3, ALL], np.uint32)
    s.col_sensor = np.array([1 if i % 7 == 3 else 0 for i in range(300)], np.uint8)
    s.col_memb = np.array([masks[g.index(4)] for _ in range(300)], np.uint32)
    s.col_filt = np.array([masks[g.index(4)] for _ in range(300)], np.uint32)
    a, b, rest, k, c = [], [], [], [], []
    for _ in range(60):
        ia = g.index(300)
        ib = (ia + 1 + g.index(299)) % 300
        a.append(ia), b.append(ib)
        rest.append(g.lerp(0.2, 0.6)), k.append(g.lerp(10.0, 100.0)), c.append(g.lerp(0.0, 1.0))
    s.spr_a, s.spr_b = np.array(a, np.uint32), np.array(b, np.uint32)
    s.spr_rest, s.spr_k, s.spr_c = (np.array(v, np.float32) for v in (rest, k, c))
    s.circles = np.array([[0.0, 0.0, 3.5]], np.float32)
    out.append(("pin_springs_groups_300", s, 8, 1.0 / 60.0))

    g = XorShift32(0x6A09E667)
    s = _bodies(g, 200, 2.5, 0.04, 0.1, 0.5, 2, spread=0.1)
    s.circles = np.array([[0.0, 0.0, 3.5]], np.float32)
    out.append(("pin_two_collider_200", s, 6, 1.0 / 60.0))

    # RigidBodyType: Dynamic 0, Static 1, KinematicPositionBased 2,
    # KinematicVelocityBased 3; gravity_mod drawn after all bodies
    g = XorShift32(0xBB67AE85)
    s = _bodies(g, 300, 2.5, 0.05, 0.15, 1.0, 1)
    s.body_type = np.array([1 if i % 9 == 4 else (2 + i % 2 if i % 13 == 6 else 0) for i in range(300)], np.uint8)
    s.gravity_mod = np.array([g.lerp(0.0, 2.0) for _ in range(300)], np.float32)
    s.circles = np.array([[0.0, 0.0, 3.5]], np.float32)
    out.append(("pin_body_types_300", s, 8, 1.0 / 60.0))

    # fixed joints (Physics::create_fixed_joint after all bodies, in this
    # order); single-collider bodies, so the rotations the joints drive do
    # not reach the positions
    g = XorShift32(0x3C6EF372)
    s = _bodies(g, 200, 2.5, 0.05, 0.15, 1.0, 1)
    ja, jb, aa, ab = [], [], [], []
    for _ in range(40):
        a = g.index(200)
        b = (a + 1 + g.index(199)) % 200
        ja.append(a), jb.append(b)
        aa.append((g.lerp(-0.05, 0.05), g.lerp(-0.05, 0.05)))
        ab.append((g.lerp(-0.05, 0.05), g.lerp(-0.05, 0.05)))
    scenes.add_fixed_joints(s, ja, jb, aa, ab)
    s.circles = np.array([[0.0, 0.0, 3.5]], np.float32)
    out.append(("pin_joints_200", s, 8, 1.0 / 60.0))
    return out


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def inputs_of(s):
    """Digests of the generated inputs (row-major f32, little-endian)."""
    return {"pos": digest(s.pos), "vreq": digest(s.vreq), "col_offset": digest(s.col_offset),
            "col_radius": digest(s.col_radius)}


def states():
    fixture = {}
    for name, s, steps, dt in pin_scenes():
        s.dt = dt
        o = oracle.OracleWorld(s, 32)
        assert o.step(dt, steps) == 0
        b = o.bodies()
        fixture[name] = {"steps": steps, "dt": "1/60", "bodies": s.n_bodies, "colliders": s.n_colliders,
                         "inputs": inputs_of(s), "pos": digest(b["pos"]), "pos_old": digest(b["pos_old"]),
                         "vel": digest(b["vel"]), "contacts": int(o.contacts)}
    return fixture


def main():
    with open(FIXTURE, "w") as f:
        json.dump(states(), f, indent=1, sort_keys=True)
        f.write("\n")
    print(FIXTURE)


if __name__ == "__main__":
    main()
