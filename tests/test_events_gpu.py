"""Collision event stream: blobs_world_set_events / blobs_world_drain_events
against the oracle's CollisionEvent list (physics.rs:304-311, lib.rs:146-153).

Every event -- collider pair (a > b), impact velocities -- and their order
(substep by substep, outer collider ascending, inner ascending) must equal
the f32 oracle's, bit for bit.
"""
import numpy as np
import pytest

from blobs_gb300 import native, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu


def oracle_events(scene, steps, dt, clear_after=0):
    o = oracle.OracleWorld(scene, 32, record_events=True)
    if clear_after:
        assert o.step(dt, clear_after) == 0
        lib = oracle.lib()
        lib.oracle_world_clear_events(o._h)
    assert o.step(dt, steps) == 0
    a, b, va, vb = o.events()
    return a, b, va.astype(np.float32), vb.astype(np.float32)


def assert_same_events(got, want):
    ga, gb, gva, gvb = got
    wa, wb, wva, wvb = want
    assert len(ga) == len(wa), (len(ga), len(wa))
    assert len(wa) > 0
    assert np.array_equal(ga, wa) and np.array_equal(gb, wb)
    assert np.array_equal(gva, wva) and np.array_equal(gvb, wvb)


def gpu_events(scene, steps, dt, rollout=False, capacity=1 << 20):
    """Events of `steps` steps; also checks that recording them leaves the
    trajectory unchanged (bit for bit)."""
    def run(events):
        with native.World(scene) as w:
            if events:
                w.set_events(True, capacity)
            if rollout:
                w.step(dt)
                w.rollout(dt, steps - 1)
            else:
                for _ in range(steps):
                    w.step(dt)
            ev = w.drain_events() if events else None
            return ev, w.read_bodies()
    ev, bodies = run(True)
    _, plain = run(False)
    for k in ("pos", "pos_old", "vel"):
        assert np.array_equal(bodies[k], plain[k]), k
    return ev, bodies["pos"]


@pytest.mark.parametrize("rollout", [False, True])
def test_events_single_spheres(rollout):
    s = scenes.sparse_spheres(seed=41, n=400)
    got, pos = gpu_events(s, 6, s.dt, rollout=rollout)
    assert_same_events(got, oracle_events(s, 6, s.dt))


def test_events_with_springs_and_walls():
    rng = np.random.Generator(np.random.PCG64(42))
    s = scenes.random_world(rng, 600, 0.1, 0.3, 0.35, 1.0, spring_frac=0.2, k_range=(50.0, 500.0),
                            c_range=(0.0, 1.0))
    got, _ = gpu_events(s, 4, s.dt)
    assert_same_events(got, oracle_events(s, 4, s.dt))


def test_events_multi_collider_sensors_groups():
    s = scenes.jointed_bodies(seed=43, n=3000, n_joints=0, n_springs=500, side=60.0)
    rng = np.random.Generator(np.random.PCG64(43))
    s.col_sensor = (rng.random(s.n_colliders) < 0.1).astype(np.uint8)
    s.col_memb = rng.choice(np.array([1, 2, 0xFFFFFFFF], np.uint32), s.n_colliders)
    s.col_filt = rng.choice(np.array([1, 3, 0xFFFFFFFF], np.uint32), s.n_colliders)
    got, _ = gpu_events(s, 3, s.dt)
    assert_same_events(got, oracle_events(s, 3, s.dt))


def test_events_batched_worlds():
    rng = np.random.Generator(np.random.PCG64(44))
    worlds = [scenes.random_world(rng, int(n), 0.1, 0.3, 0.35, 1.0, spring_frac=0.1 * (i % 2))
              for i, n in enumerate([90, 300, 150, 500])]
    s = scenes.pack(worlds)
    s.dt = 1.0 / 60.0
    (a, b, va, vb), _ = gpu_events(s, 3, s.dt)
    co = s.world_collider_offsets
    world_of = np.searchsorted(co, a, side="right") - 1
    for w in range(s.n_worlds):
        sel = world_of == w
        got = (a[sel] - co[w], b[sel] - co[w], va[sel], vb[sel])
        assert_same_events(got, oracle_events(scenes.unpack_world(s, w), 3, s.dt))


def test_events_enabled_mid_run_and_partial_drains():
    s = scenes.sparse_spheres(seed=45, n=400)
    with native.World(s) as w:
        for _ in range(3):
            w.step(s.dt)  # velocities kept as displacements until events are on
        w.set_events(True, 1 << 16)
        for _ in range(3):
            w.step(s.dt)
        a1, b1, va1, vb1 = w.drain_events(cap=7)
        rest = w.drain_events()
    want = oracle_events(s, 3, s.dt, clear_after=3)
    got = tuple(np.concatenate([x, y]) for x, y in zip((a1, b1, va1, vb1), rest))
    assert len(a1) == 7
    assert_same_events(got, want)


def test_events_overflow_drops_the_batch_and_reports_the_count():
    s = scenes.random_world(np.random.Generator(np.random.PCG64(46)), 600, 0.1, 0.3, 0.35, 1.0)
    total = len(oracle_events(s, 2, s.dt)[0])
    assert total > 100
    with native.World(s) as w:
        w.set_events(True, 100)
        w.step(s.dt)
        w.step(s.dt)
        with pytest.raises(native.BlobsError) as ei:
            w.drain_events()
        assert ei.value.status == native.ERR_OVERFLOW
        # the next batch starts empty
        w.set_events(True, 1 << 16)
        assert len(w.drain_events()[0]) == 0


def test_drain_without_events_is_a_state_error():
    s = scenes.sparse_spheres(seed=47, n=50)
    with native.World(s) as w:
        with pytest.raises(native.BlobsError) as ei:
            w.drain_events()
        assert ei.value.status == native.ERR_STATE


def test_events_with_fixed_joints_in_gpu_order():
    """Single-collider bodies with fixed joints take the joint path's contact
    kernel; against the oracle run in the GPU's joint processing order the events
    (pairs, order, impact velocities) are bit-exact."""
    rng = np.random.Generator(np.random.PCG64(48))
    s = scenes.random_world(rng, 1500, 0.1, 0.25, 0.25, 0.5)
    near = scenes._pairs_within(s.pos, 1.0)
    pick = np.sort(rng.choice(len(near), 500, replace=False))
    scenes.add_fixed_joints(s, near[pick, 0], near[pick, 1])
    with native.World(s) as w:
        w.set_events(True, 1 << 20)
        for _ in range(3):
            w.step(s.dt)
        got = w.drain_events()
        order = w.joint_order()[0]
    o = oracle.OracleWorld(s, 32, record_events=True, joint_order=order)
    assert o.step(s.dt, 3) == 0
    a, b, va, vb = o.events()
    assert_same_events(got, (a, b, va.astype(np.float32), vb.astype(np.float32)))
