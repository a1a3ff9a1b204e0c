"""The oracle against the reference's own known-answer tests.

blobs/src/tests.rs:26-90 (SpatialHash) and blobs/src/collider.rs:340-389
(body / collider transforms) are the only golden vectors the reference holds
for this path; the step itself has none ("parity unpinned"), so the rest of
this file pins the oracle's step to hand-computed float32 values of the
reference formulas in physics.rs / springs.rs / rigid_body.rs.
"""
import math

import numpy as np
import pytest

from blobs_gb300 import scenes
from oracle import oracle

f32 = np.float32


# ---- blobs/src/tests.rs -----------------------------------------------------

def _create_spatial_hash():  # tests.rs:16-24
    h = oracle.SpatialHash(100.0)
    for p in [(50.0, 50.0), (150.0, 150.0), (250.0, 250.0), (350.0, 350.0), (450.0, 450.0)]:
        h.insert(p[0], p[1], 1.0)
    return h


def test_get_cell_coords():  # tests.rs:26-34
    h = _create_spatial_hash()
    for k in range(5):
        v = 50.0 + 100.0 * k
        assert h.cell_coords(v, v) == (k, k)


def test_insert():  # tests.rs:36-53
    h = oracle.SpatialHash(100.0)
    i = h.insert(50.5, -25.5, 1.0)
    assert i == 0
    assert h.next_id == 1
    cx, cy = h.cell_coords(50.5, -25.5)
    assert (cx, cy) == (0, -1)  # floor(-0.255) = -1
    assert h.cell_len(cx, cy) >= 1
    x, y = h.point(i)
    assert abs(x - 50.5) < 1e-6 and abs(y + 25.5) < 1e-6


def test_insert_and_query():  # tests.rs:55-65
    h = oracle.SpatialHash(1.0)
    p1 = h.insert(0.0, 0.0, 0.0)
    p2 = h.insert(2.0, 2.0, 0.0)
    ids, _ = h.query(1.0, 1.0, 1.5)
    assert len(ids) == 2
    assert set(ids.tolist()) == {p1, p2}


def test_move_point():  # tests.rs:67-79
    h = oracle.SpatialHash(1.0)
    p = h.insert(0.0, 0.0, 0.0)
    assert h.move_point(p, 2.0, 2.0)
    ids, pos = h.query(1.0, 1.0, 1.5)
    assert len(ids) == 1
    assert ids[0] == p and tuple(pos[0]) == (2.0, 2.0)


def test_remove():  # tests.rs:81-90
    h = oracle.SpatialHash(1.0)
    p = h.insert(0.0, 0.0, 0.0)
    h.remove(p)
    ids, _ = h.query(0.0, 0.0, 1.5)
    assert len(ids) == 0


# ---- blobs/src/collider.rs:340-389 -------------------------------------------

def test_simple_body_transform():  # collider.rs:340-351
    m = oracle.body_collider_transform(0.0, 2.0, 3.0, 0.0, 0.0)
    np.testing.assert_allclose(m, [1, 0, 0, 1, 2, 3], atol=1e-6)


def test_body_transform_rotated():  # collider.rs:353-365
    m = oracle.body_collider_transform(f32(math.pi / 2), 2.0, 3.0, 0.0, 0.0)
    np.testing.assert_allclose(m[:4], [0, 1, -1, 0], atol=1e-6)  # Mat2::from_angle(pi/2), column major


def test_collider_offset():  # collider.rs:367-389
    m = oracle.body_collider_transform(f32(math.pi / 2), 2.0, 3.0, 1.0, 1.0)
    # from_angle(pi/2) * (1, 1) + (2, 3) = (-1, 1) + (2, 3)
    np.testing.assert_allclose(m[4:], [1.0, 4.0], atol=1e-6)


# ---- hand-computed f32 values of the reference formulas ----------------------

def _one_substep(scene, dt=1.0 / 60.0):
    scene = scene.copy()
    scene.substeps = 1
    w = oracle.OracleWorld(scene, 32)
    assert w.step(dt, 1) == 0
    return w


def test_mass_is_doubled():
    """Each collider handle is pushed twice (collider.rs:180, physics.rs:144):
    a single sphere of radius r weighs 4r, inertia 2 * (0.5 * 2r * r^2)."""
    s = scenes.spheres([[0, 0], [5, 0]], [0.25, 0.5])
    m, I = oracle.mass_inertia_f32(s)
    assert m.tolist() == [1.0, 2.0]
    np.testing.assert_array_equal(I, f32(2) * (f32(0.5) * (f32(2) * s.col_radius) * (s.col_radius * s.col_radius)))


def test_first_dynamic_body_sees_old_dt():
    """physics.rs:338-339: old_dt starts at 1.0 and is overwritten by the first
    non-static body, so only that body's first displacement is scaled by dt."""
    s = scenes.spheres([[0, 0], [10, 0], [20, 0]], [0.1, 0.1, 0.1], gravity=(0, 0), body_type=[1, 0, 0])
    s.pos_old = s.pos - np.array([[0, 0], [1, 0], [1, 0]], np.float32)  # moving +1 per step
    dt = f32(1.0 / 60.0)
    w = _one_substep(s, float(dt))
    b = w.bodies()
    assert b["pos"][1, 0] == f32(10) + f32(f32(1) * (dt / f32(1.0)))  # first dynamic: scaled by dt / 1.0
    assert b["pos"][2, 0] == f32(20) + f32(1)                        # others: dt / dt = 1
    assert b["pos"][0, 0] == 0.0                                      # static untouched


def test_spring_broadcast_quirk():
    """springs.rs:41: `k * (dist - rest) - damping_force` is f32 - Vec2, i.e.
    the scalar is broadcast to both components before the component-wise
    product with the direction."""
    s = scenes.spheres([[0, 0], [3, 4]], [0.1, 0.1], gravity=(0, 0))
    s.vel = np.array([[1, 0], [0, 1]], np.float32)
    scenes.add_springs(s, [0], [1], k=[10.0], c=[0.5], rest=[4.0])
    s.collisions_enabled = False
    dt = f32(0.01)
    w = _one_substep(s, float(dt))
    d = np.array([3, 4], np.float32)
    dist = np.sqrt(f32(25))
    dirn = d / dist
    rv = np.array([1, -1], np.float32)
    dmp = (f32(0.5) * f32(dirn[0] * rv[0] + dirn[1] * rv[1])) * dirn
    fm = f32(10) * (dist - f32(4)) - dmp          # the broadcast
    f = dirn * fm
    m = f32(0.4)                                  # 4 r
    acc_a = f / m
    # pos_old = pos (no velocity request), ratio dt / old_dt(=1) for body 0
    disp0 = np.zeros(2, np.float32)
    want0 = np.array([0, 0], np.float32) + (disp0 + (acc_a * dt) * dt)
    np.testing.assert_array_equal(w.bodies()["pos"][0].astype(np.float32), want0)


def test_pushout_coincident_spheres():
    """physics.rs:272-286: two coincident spheres are pushed +-0.01 in x, then
    separated by the usual mass-ratio correction."""
    s = scenes.spheres([[1, 1], [1, 1]], [0.5, 0.5], gravity=(0, 0))
    dt = 1.0 / 60.0
    w = _one_substep(s, dt)
    assert w.pushouts == 1 and w.contacts == 1
    # update_objects stores the post-contact position in position_old
    b = w.bodies()["pos_old"].astype(np.float32)
    # collider 1 (outer index) is a: +0.01, collider 0 is b: -0.01; axis = 0.02
    pa, pb = f32(1) + f32(0.01), f32(1) - f32(0.01)
    dist = pa - pb
    delta = f32(1.0) - dist
    ratio = f32(1) - f32(2) / (f32(2) + f32(2))
    assert b[1, 0] == pa + (ratio * delta) * f32(1)
    assert b[0, 0] == pb - ((f32(1) - ratio) * delta) * f32(1)


def test_f32_close_to_f64_one_substep():
    s = scenes.sparse_spheres(seed=3, n=200)
    w32 = _one_substep(s)
    w64 = oracle.OracleWorld(s.copy(), 64)
    s64 = s.copy()
    s64.substeps = 1
    w64 = oracle.OracleWorld(s64, 64)
    w64.step(1.0 / 60.0, 1)
    np.testing.assert_allclose(w32.bodies()["pos"], w64.bodies()["pos"], rtol=1e-6, atol=1e-5)


def test_contact_pairs_bruteforce_matches_step_count():
    s = scenes.dense_spheres(seed=9, n=2000, steps=1)
    i, j = oracle.contact_pairs(s.pos, s.col_radius)
    s1 = s.copy()
    s1.substeps = 1
    w = oracle.OracleWorld(s1, 32)
    w.step(1.0 / 120.0, 1)
    assert w.contacts == len(i)
    assert np.all(i > j)
