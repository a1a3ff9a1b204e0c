"""Crowded bodies: the step kernel leaves a body whose 3x3 cells hold more
than 64 candidates, or which has more than 32 near candidates (12 in the
event, recording and per-body-record variants), to a warp of its own
(k_step_deferred).  These worlds make both happen -- a dense
overlapping field plus a tight clump -- and check that the result is still
the reference's, bit for bit: positions and contact counts against the f32
oracle, the collision-event list against the oracle's, and the recorded
contacts of the differentiable rollout against the f64 replay of the
oracle's trace (physics.rs:241-367).
"""
import numpy as np
import pytest

from blobs_gb300 import native, scenes
from oracle import oracle

from adjoint_replay import replay_gradients

pytestmark = pytest.mark.gpu


def crowded_scene(seed=61, n=4000, clump=160, packing=1.2, walls=True):
    """n spheres r ~ U[0.05, 0.15] at `packing` with overlaps, plus `clump`
    spheres in a disc of radius 0.6 (hundreds of candidates each)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    side = scenes.box_side(n, 0.05, 0.15, packing)
    h = side / 2.0
    rad = rng.uniform(0.05, 0.15, n + clump)
    pos = rng.uniform(-h + 0.2, h - 0.2, (n + clump, 2))
    th, rr = rng.uniform(0, 2 * np.pi, clump), 0.6 * np.sqrt(rng.uniform(0, 1, clump))
    pos[n:] = np.stack([rr * np.cos(th), rr * np.sin(th)], 1)
    vel = rng.normal(0.0, 0.5, pos.shape)
    return scenes.spheres(pos.astype(np.float32), rad.astype(np.float32), vel.astype(np.float32),
                          box=(-h, -h, h, h) if walls else None)


def contacts_per_body(s):
    """Contacts of each body in the scene's initial state (f64 distances)."""
    pos, rad = s.pos.astype(np.float64), s.col_radius.astype(np.float64)
    d = np.sqrt(((pos[:, None, :] - pos[None, :, :]) ** 2).sum(-1))
    hit = d < rad[:, None] + rad[None, :]
    np.fill_diagonal(hit, False)
    return hit.sum(1)


def test_crowded_world_bit_exact_with_deferred_bodies():
    s = crowded_scene()
    dt, steps = 1.0 / 120.0, 3
    with native.World(s) as w:
        for _ in range(steps):
            w.step(dt)
        got = w.read_bodies()
        contacts = w.contact_count()[0]
        deferred = w.deferred_count()[0]
    assert deferred > 100, deferred
    o = oracle.OracleWorld(s, 32)
    assert o.step(dt, steps) == 0
    assert o.pushouts == 0
    want = o.bodies()
    for k in ("pos", "pos_old", "vel"):
        assert np.array_equal(got[k].astype(np.float64), want[k]), k
    assert contacts == o.contacts


def test_dense_field_shares_phase_2_over_the_warp():
    """150% packing, no clump: ~6 near candidates per body, up to ~19, so
    the plain step's warps hold ~200-300 near pairs (several rounds of the
    warp's 128 pair slots) and bodies past 12 near candidates stay in the
    warp-shared phase 2 rather than being deferred; bit-exact all the same."""
    s = crowded_scene(seed=65, n=4000, clump=0, packing=1.5)
    dt, steps = 1.0 / 120.0, 3
    with native.World(s) as w:
        for _ in range(steps):
            w.step(dt)
        got = w.read_bodies()
        contacts = w.contact_count()[0]
    o = oracle.OracleWorld(s, 32)
    assert o.step(dt, steps) == 0
    assert o.pushouts == 0
    want = o.bodies()
    for k in ("pos", "pos_old", "vel"):
        assert np.array_equal(got[k].astype(np.float64), want[k]), k
    assert contacts == o.contacts and contacts > 2 * 4000 * 8 * steps  # ~250k


def test_crowded_world_events_match_the_oracle():
    s = crowded_scene(seed=62, n=2500, clump=120)
    dt, steps = 1.0 / 120.0, 2
    with native.World(s) as w:
        w.set_events(True, 1 << 22)
        for _ in range(steps):
            w.step(dt)
        ga, gb, gva, gvb = w.drain_events()
        assert w.deferred_count()[0] > 50
    o = oracle.OracleWorld(s, 32, record_events=True)
    assert o.step(dt, steps) == 0
    wa, wb, wva, wvb = o.events()
    assert len(ga) == len(wa) and len(wa) > 1000
    assert np.array_equal(ga, wa) and np.array_equal(gb, wb)
    assert np.array_equal(gva, wva.astype(np.float32)) and np.array_equal(gvb, wvb.astype(np.float32))


def test_crowded_world_gradients_match_the_replay():
    """The recorded contacts of deferred bodies (appended by the deferred
    kernel's ordered lane) give the same gradients as the replay of the
    oracle's trace."""
    # no clump: the recording keeps at most 16 contacts per body and substep;
    # at 120% packing some bodies have 13-15, which the recording kernels
    # (backward's recomputation of the segment) defer
    s = crowded_scene(seed=64, n=3000, clump=0, packing=1.2)
    assert contacts_per_body(s).max() > 12 and (contacts_per_body(s) > 12).sum() >= 5
    rng = np.random.Generator(np.random.PCG64(63))
    # a loss gradient on every body, so that every recorded contact matters
    g = rng.normal(0.0, 1.0, (s.n_bodies, 2)).astype(np.float32).astype(np.float64)
    dt, steps = 1.0 / 120.0, 1
    with native.World(s) as w:
        w.rollout_record(dt, steps, 1)
        final = w.read_bodies()["pos"].astype(np.float64)
        gv, _ = w.backward(g.astype(np.float32), s.n_springs)
    o = oracle.OracleWorld(s, 32)
    o.trace(True)
    assert o.step(dt, steps) == 0
    fin = o.bodies()["pos"]
    assert np.array_equal(fin.astype(np.float32), final.astype(np.float32))
    rv, _, worst = replay_gradients(s, o.traced(), fin, g, dt)
    scale = np.abs(rv).max()
    err = np.abs(gv.astype(np.float64) - rv)
    assert not np.any(err > 1e-3 * np.abs(rv) + 1e-4 * scale), (float(err.max()), float(scale))
