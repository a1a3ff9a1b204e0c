"""The oracle's grid-enumerated contact loop against its C^2/2 loop.

`OracleWorld(..., grid_pairs=True)` finds the contact pairs of a substep
through a uniform grid of the collider snapshots and resolves them in the
reference's order (physics.rs:248-249: i ascending, j < i ascending), so that
full-size scenes (1M spheres, 3.5M batched bodies) can be checked against the
oracle in seconds.  This file pins that mode to the plain loop, bit for bit,
on every kind of scene the tests use (no GPU).
"""
import numpy as np
import pytest

from blobs_gb300 import scenes
from oracle import oracle

GRID_PUSHOUT = 8


def run(scene, steps, precision=32, grid=False, **kw):
    o = oracle.OracleWorld(scene, precision, grid_pairs=grid, **kw)
    st = o.step(scene.dt, steps)
    out = o.bodies()
    out["snap"] = o.snapshots()
    out["status"], out["contacts"], out["pushouts"] = st, o.contacts, o.pushouts
    if kw.get("record_events"):
        out["events"] = o.events()
    return out, o


def assert_same(a, b):
    assert a["status"] == b["status"] == 0
    assert a["contacts"] == b["contacts"] and a["contacts"] > 0
    for k in ("pos", "pos_old", "vel", "rotation", "snap"):
        assert np.array_equal(a[k], b[k]), k


def random_groups_scene(seed, n):
    rng = np.random.Generator(np.random.PCG64(seed))
    s = scenes.random_world(rng, n, 0.1, 0.3, 0.35, 1.0, spring_frac=0.2)
    s.col_sensor = (rng.random(s.n_colliders) < 0.1).astype(np.uint8)
    s.col_memb = rng.choice(np.array([1, 2, 0xFFFFFFFF], np.uint32), s.n_colliders)
    s.col_filt = rng.choice(np.array([1, 3, 0xFFFFFFFF], np.uint32), s.n_colliders)
    return s


@pytest.mark.parametrize("name,steps,precision", [
    ("sparse", 20, 32), ("dense", 3, 32), ("dense", 2, 64), ("jointed", 2, 32), ("jointed", 1, 64),
    ("groups", 3, 32), ("batch_world", 4, 32)])
def test_grid_pairs_equal_the_plain_loop(name, steps, precision):
    s = {"sparse": lambda: scenes.sparse_spheres(seed=1, n=1000),
         "dense": lambda: scenes.dense_spheres(seed=2, n=6000),
         "jointed": lambda: scenes.jointed_bodies(seed=3, n=2500, n_joints=400, n_springs=700, side=55.0),
         "groups": lambda: random_groups_scene(4, 2500),
         "batch_world": lambda: scenes.unpack_world(scenes.gradient_batch(seed=5, n_worlds=2, n_per=1500,
                                                                          n_springs=700)[0], 1)}[name]()
    a, _ = run(s, steps, precision)
    b, _ = run(s, steps, precision, grid=True)
    assert_same(a, b)


def test_grid_pairs_give_the_same_events_and_trace():
    s = random_groups_scene(7, 1500)
    a, oa = run(s, 2, record_events=True)
    b, ob = run(s, 0, grid=True, record_events=True)
    ob.trace(True)
    oa2 = oracle.OracleWorld(s, 32)
    oa2.trace(True)
    assert ob.step(s.dt, 2) == 0 and oa2.step(s.dt, 2) == 0
    for x, y in zip(a["events"], ob.events()):
        assert np.array_equal(x, y)
    ta, tb = oa2.traced(), ob.traced()
    assert len(ta) == len(tb) == 2 * s.substeps
    for u, v in zip(ta, tb):
        for k in ("hi", "lo", "pushed", "pos", "snap"):
            assert np.array_equal(u[k], v[k]), k


def test_scene_too_wide_for_a_grid_falls_back_to_the_plain_loop():
    """Two clusters 1e5 apart: the grid would need far more cells than
    colliders, so the mode uses the C^2/2 loop for the substep."""
    rng = np.random.Generator(np.random.PCG64(72))
    a = rng.uniform(-3, 3, (300, 2)).astype(np.float32)
    b = (rng.uniform(-3, 3, (300, 2)) + np.array([1e5, -7e4])).astype(np.float32)
    s = scenes.spheres(np.concatenate([a, b]), rng.uniform(0.1, 0.3, 600).astype(np.float32),
                       rng.normal(0, 1, (600, 2)).astype(np.float32))
    s.dt = 1.0 / 60.0
    assert_same(run(s, 10)[0], run(s, 10, grid=True)[0])


def test_pushout_stops_the_grid_mode():
    """Coincident centres: the push-out moves two snapshots mid-loop, which a
    grid built at the substep's start cannot follow; the mode says so."""
    s = scenes.spheres([[1, 1], [1, 1], [5, 5]], [0.5, 0.5, 0.2], gravity=(0, 0))
    assert run(s, 1)[0]["status"] == 0
    assert run(s, 1, grid=True)[0]["status"] == GRID_PUSHOUT


def test_trivial_worlds():
    for s in (scenes.empty_scene(0), scenes.spheres([[0.0, 0.0]], [0.2])):
        s.dt = 1.0 / 60.0
        a, b = run(s, 2), run(s, 2, grid=True)
        assert a[0]["status"] == b[0]["status"] == 0
        assert np.array_equal(a[0]["pos"], b[0]["pos"])
