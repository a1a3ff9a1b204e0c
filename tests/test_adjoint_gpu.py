"""Differentiable rollout: blobs_world_rollout_record + blobs_world_backward.

Gradients of L = mean over marked bodies of |x_final - target|^2 with
respect to the initial velocity requests and the spring stiffnesses, from
the f32 GPU adjoint, checked two ways:

* against the f64 replay of the f32 oracle's own traced trajectory
  (tests/adjoint_replay.py): the GPU follows that trajectory bit for bit, so
  the comparison is tight -- every gradient within 1e-3 relative plus 1e-4
  of the largest gradient of its kind (f32 accumulation over the substeps);
* against f64 central finite differences of the oracle (h = 1e-4 for
  velocities, 1e-4 relative for stiffnesses) over horizons of two and four
  steps, where the f32 and f64 trajectories still resolve the same contacts:
  within 2e-3 relative (or 2e-7 of the largest gradient of the kind); a
  sample whose contact count changes within +-h is discarded and replaced;
* on the full differentiable-rollout batch with a checkpoint every 16 steps
  over 17, 24 and 33 steps (one and two checkpoints restored): against the
  replay, and against f64 central differences chained along the traced
  trajectory (adjoint_replay.tangent_fd), which need neither autograd nor
  the f64 oracle's own, diverging, trajectory.

Over longer horizons the f32 and f64 trajectories drift apart by ~1e-4 and
resolve different contacts, and the derivative of the contact correction
jumps at first touch, so finite differences of the f64 oracle stop being a
reference for the f32 trajectory's derivative; the replay is.
"""
import numpy as np
import pytest

from blobs_gb300 import native, scenes
from oracle import oracle

from adjoint_replay import replay_gradients, tangent_fd

pytestmark = pytest.mark.gpu


def make_scene(seed, n_worlds=3, n=160, n_springs=64, damping=(0.0, 0.5), walls=True, n_static=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    worlds, marked, targets = [], [], []
    for _ in range(n_worlds):
        side = scenes.box_side(n, 0.1, 0.2, 0.30)
        h = side / 2.0
        pos, rad = scenes._nonoverlapping(rng, n, 0.1, 0.2, -h, h)
        vel = rng.normal(0.0, 1.0, (n, 2)).astype(np.float32)
        bt = np.zeros(n, np.uint8)
        if n_static:
            bt[rng.choice(n, size=n_static, replace=False)] = 1
        s = scenes.spheres(pos, rad, vel, box=(-h, -h, h, h) if walls else None, body_type=bt)
        near = scenes._pairs_within(s.pos, 1.0)
        pick = np.sort(rng.choice(len(near), size=min(n_springs, len(near)), replace=False))
        k = np.exp(rng.uniform(np.log(100.0), np.log(5000.0), len(pick))).astype(np.float32)
        c = rng.uniform(damping[0], damping[1], len(pick)).astype(np.float32)
        scenes.add_springs(s, near[pick, 0], near[pick, 1], k, c)
        worlds.append(s)
        m = np.sort(rng.choice(n, size=16, replace=False))
        marked.append(m)
        targets.append(s.pos[m].astype(np.float64) + rng.normal(0.0, 1.0, (16, 2)))
    return scenes.pack(worlds), marked, targets


def loss_grad(final, scene, marked, targets):
    """dL/dx (float64, n x 2) over all worlds."""
    M = sum(len(m) for m in marked)
    g = np.zeros((scene.n_bodies, 2))
    for w, (m, t) in enumerate(zip(marked, targets)):
        b0 = int(scene.world_body_offsets[w])
        g[b0 + m] = 2.0 * (final[b0 + m] - t) / M
    return g


def gpu_gradients(scene, marked, targets, steps, every, warm_steps=0):
    with native.World(scene) as w:
        for _ in range(warm_steps):
            w.step(scene.dt)
        w.rollout_record(scene.dt, steps, every)
        final = w.read_bodies()["pos"].astype(np.float64)
        g = loss_grad(final, scene, marked, targets)
        gv, gk = w.backward(g.astype(np.float32), scene.n_springs)
        after = w.read_bodies()["pos"].astype(np.float64)
    return final, g, after, gv.astype(np.float64), gk.astype(np.float64)


def _close(got, want, what, floor=1e-4):
    scale = np.abs(want).max()
    err = np.abs(got - want)
    bad = err > 1e-3 * np.abs(want) + floor * scale
    assert not bad.any(), (what, int(bad.sum()), float(err.max()), float(scale))


@pytest.mark.parametrize("steps,every,n_worlds,n_static,warm,walls", [
    (8, 3, 3, 0, 0, True),    # batched worlds, damped springs, walls
    (12, 4, 1, 0, 0, True),   # one world
    (6, 6, 2, 12, 0, True),   # static bodies, one segment
    (5, 2, 2, 0, 1, True),    # velocity requests already consumed, old_dt = dt
    (7, 3, 2, 0, 0, False),   # no walls
])
def test_gradients_match_replay_of_traced_oracle(steps, every, n_worlds, n_static, warm, walls):
    scene, marked, targets = make_scene(seed=steps + 10 * n_static, n_worlds=n_worlds, n_static=n_static,
                                        walls=walls)
    final, g, after, gv, gk = gpu_gradients(scene, marked, targets, steps, every, warm_steps=warm)
    # backward() leaves the world in the rollout's final state
    assert np.array_equal(final, after)
    assert np.any(gk) and (np.any(gv) if warm == 0 else not np.any(gv))
    for w in range(scene.n_worlds):
        sub = scenes.unpack_world(scene, w)
        b0, b1 = int(scene.world_body_offsets[w]), int(scene.world_body_offsets[w + 1])
        s0, s1 = int(scene.world_spring_offsets[w]), int(scene.world_spring_offsets[w + 1])
        o = oracle.OracleWorld(sub, 32)
        assert o.step(scene.dt, warm) == 0
        o.trace(True)
        assert o.step(scene.dt, steps) == 0
        assert o.pushouts == 0
        fin = o.bodies()["pos"]
        # the GPU rollout is the f32 oracle's, bit for bit
        assert np.array_equal(fin.astype(np.float32), final[b0:b1].astype(np.float32)), w
        rv, rk, worst = replay_gradients(sub, o.traced(), fin, g[b0:b1], scene.dt,
                                         old_dt=1.0 if warm == 0 else float(np.float32(scene.dt) / 8),
                                         vreq_pending=warm == 0)
        _check_replay(worst, fin)
        if warm == 0:
            _close(gv[b0:b1], rv, ("dL/dv0", w))
        _close(gk[s0:s1], rk, ("dL/dk", w))


def _check_replay(worst, fin):
    """The f64 replay reproduces each recorded f32 substep to a few f32 ulps
    of the positions (velocities carry the rounding times 1 / dt)."""
    scale = 1.0 + float(np.abs(fin).max())
    assert max(worst["pos"], worst["pos_old"], worst["snap"]) < 4e-7 * scale, worst
    assert worst["vel"] < 2e-4 * scale, worst


def test_gradient_batch_short_horizon_matches_replay():
    """The differentiable-rollout batch at full size -- 256 worlds x 2,048
    spheres (r ~ U[0.1, 0.2], 30% packing, overlaps allowed at t = 0), 1,024
    springs per world, 64 marked bodies per world -- over 10 steps with a
    checkpoint every 4, worlds 0 and 255 checked against the replay.  Over
    the full 120 steps the derivative of this contact dynamics grows by
    orders of magnitude every few steps (max |dL/dv0| of one world: 4e-2 at
    step 10, 1e1 at 15, 1e12 at 40, 1e84 at 120, in f64) and leaves the f32
    range, so the check is made where it is finite."""
    scene, marked, targets = scenes.gradient_batch()
    steps = 10
    final, g, after, gv, gk = gpu_gradients(scene, marked, targets, steps, 4)
    assert np.array_equal(final, after)
    assert np.all(np.isfinite(gv)) and np.all(np.isfinite(gk))
    for w in (0, scene.n_worlds - 1):
        sub = scenes.unpack_world(scene, w)
        b0, b1 = int(scene.world_body_offsets[w]), int(scene.world_body_offsets[w + 1])
        s0, s1 = int(scene.world_spring_offsets[w]), int(scene.world_spring_offsets[w + 1])
        o = oracle.OracleWorld(sub, 32)
        o.trace(True)
        assert o.step(scene.dt, steps) == 0
        assert o.pushouts == 0
        fin = o.bodies()["pos"]
        assert np.array_equal(fin.astype(np.float32), final[b0:b1].astype(np.float32)), w
        rv, rk, worst = replay_gradients(sub, o.traced(), fin, g[b0:b1], scene.dt)
        _check_replay(worst, fin)
        _close(gv[b0:b1], rv, ("dL/dv0", w))
        _close(gk[s0:s1], rk, ("dL/dk", w))


def _pick(rng, g):
    """An index into g: three times in four among its non-zero entries (the
    parameters that reach the loss), else uniform."""
    nz = np.flatnonzero(g)
    if len(nz) and rng.random() < 0.75:
        return int(rng.choice(nz))
    return int(rng.integers(0, g.size))


def world_loss_f64(sub, m, t, M, steps, dt):
    o = oracle.OracleWorld(sub, 64)
    assert o.step(dt, steps) == 0
    d = o.bodies()["pos"][m] - t
    return float((d * d).sum()) / M, o.contacts


@pytest.mark.parametrize("steps", [2, 4])
def test_gradients_match_f64_finite_differences(steps):
    scene, marked, targets = make_scene(seed=21, n_worlds=3)
    final, g, after, gv, gk = gpu_gradients(scene, marked, targets, steps, 1)
    M = sum(len(m) for m in marked)
    same = []
    for w in range(scene.n_worlds):
        sub = scenes.unpack_world(scene, w)
        o32, o64 = oracle.OracleWorld(sub, 32), oracle.OracleWorld(sub, 64)
        o32.step(scene.dt, steps)
        o64.step(scene.dt, steps)
        same.append(o32.contacts == o64.contacts)
    assert any(same)
    floor_v, floor_k = 1e-4 * np.abs(gv).max(), 1e-4 * np.abs(gk).max()
    rng = np.random.Generator(np.random.PCG64(99))
    checked, discarded, worst = 0, 0, 0.0
    for trial in range(256):
        if checked >= 32:
            break
        if trial % 2 == 0:
            b, ax = divmod(_pick(rng, gv.reshape(-1)), 2)
            w = int(np.searchsorted(scene.world_body_offsets, b, side="right") - 1)
            i = b - int(scene.world_body_offsets[w])
            h = 1e-4
            sub = scenes.unpack_world(scene, w)
            plus, minus = sub.copy(), sub.copy()
            plus.vreq = sub.vreq.astype(np.float64)
            minus.vreq = sub.vreq.astype(np.float64)
            plus.vreq[i, ax] += h
            minus.vreq[i, ax] -= h
            g_gpu, floor = gv[b, ax], floor_v
        else:
            e = _pick(rng, gk)
            w = int(np.searchsorted(scene.world_spring_offsets, e, side="right") - 1)
            sp = e - int(scene.world_spring_offsets[w])
            sub = scenes.unpack_world(scene, w)
            h = 1e-4 * float(sub.spr_k[sp])
            plus, minus = sub.copy(), sub.copy()
            plus.spr_k = sub.spr_k.astype(np.float64)
            minus.spr_k = sub.spr_k.astype(np.float64)
            plus.spr_k[sp] += h
            minus.spr_k[sp] -= h
            g_gpu, floor = gk[e], floor_k
        if not same[w]:
            discarded += 1
            continue
        Lp, cp = world_loss_f64(plus, marked[w], targets[w], M, steps, scene.dt)
        Lm, cm = world_loss_f64(minus, marked[w], targets[w], M, steps, scene.dt)
        if cp != cm:
            discarded += 1
            continue
        fd = (Lp - Lm) / (2.0 * h)
        # the f64 trajectory is not the f32 one the GPU differentiates: at two
        # and four steps they differ by ~1e-6, which moves small gradients by
        # up to ~1.5e-3 of themselves
        err = abs(g_gpu - fd) / (2e-3 * max(abs(fd), floor))
        worst = max(worst, err)
        assert err <= 1.0, (trial, g_gpu, fd, floor)
        checked += 1
    assert checked == 32, (checked, discarded)
    print("steps %d: 32 samples within %.3g of the bound, %d discarded" % (steps, worst, discarded))


def test_zero_loss_weight_gives_zero_gradients():
    scene, marked, targets = make_scene(seed=5, n_worlds=2)
    with native.World(scene) as w:
        w.rollout_record(scene.dt, 6, 2)
        gv, gk = w.backward(np.zeros((scene.n_bodies, 2), np.float32), scene.n_springs)
    assert not np.any(gv) and not np.any(gk)


def test_backward_without_record_is_a_state_error():
    scene, _, _ = make_scene(seed=6, n_worlds=1)
    with native.World(scene) as w:
        with pytest.raises(native.BlobsError) as ei:
            w.backward(np.zeros((scene.n_bodies, 2), np.float32), scene.n_springs)
        assert ei.value.status == native.ERR_STATE


def test_reload_or_substep_change_drops_the_recording():
    scene, _, _ = make_scene(seed=8, n_worlds=1)
    small, _, _ = make_scene(seed=9, n_worlds=1, n=40)
    g = np.zeros((scene.n_bodies, 2), np.float32)
    with native.World(scene) as w:
        w.rollout_record(scene.dt, 3, 2)
        w.load(small)  # checkpoints of the old scene must not be restored
        with pytest.raises(native.BlobsError) as ei:
            w.backward(np.zeros((small.n_bodies, 2), np.float32), small.n_springs)
        assert ei.value.status == native.ERR_STATE
        w.load(scene)
        w.rollout_record(scene.dt, 3, 2)
        cfg = native.make_config(scene)
        cfg.substeps = 4
        native.check(native.lib().blobs_world_set_config(w._h, native.ctypes.byref(cfg)), "set_config")
        with pytest.raises(native.BlobsError) as ei:
            w.backward(g, scene.n_springs)
        assert ei.value.status == native.ERR_STATE


@pytest.mark.parametrize("n_worlds", [1, 2])
def test_recorded_rollout_equals_plain_steps(n_worlds):
    """The checkpointed forward pass is the ordinary step, bit for bit, and a
    world stepped on after backward() continues exactly as one that never
    recorded."""
    scene, _, _ = make_scene(seed=7, n_worlds=n_worlds)
    with native.World(scene) as w:
        w.rollout_record(scene.dt, 9, 4)
        a = w.read_bodies()
        w.backward(np.ones((scene.n_bodies, 2), np.float32), scene.n_springs)
        for _ in range(5):
            w.step(scene.dt)
        a2 = w.read_bodies()
        ca = w.contact_count()
    with native.World(scene) as w:
        for _ in range(9):
            w.step(scene.dt)
        b = w.read_bodies()
        for _ in range(5):
            w.step(scene.dt)
        b2 = w.read_bodies()
        cb = w.contact_count()
    for k in ("pos", "pos_old", "vel"):
        assert np.array_equal(a[k], b[k])
        assert np.array_equal(a2[k], b2[k])
    assert ca == cb


def test_autograd_function_wrapper():
    """torch.autograd.Function around rollout_record / backward (test harness
    only): the gradients torch accumulates are the direct backward's."""
    torch = pytest.importorskip("torch")
    scene, marked, targets = make_scene(seed=31, n_worlds=2)
    steps, every = 4, 2

    class Rollout(torch.autograd.Function):
        @staticmethod
        def forward(ctx, v0, k):
            s = scene.copy()
            s.vreq = v0.detach().numpy().astype(np.float32)
            s.spr_k = k.detach().numpy().astype(np.float32)
            w = native.World(s)
            w.rollout_record(s.dt, steps, every)
            ctx.world = w
            return torch.from_numpy(w.read_bodies()["pos"].astype(np.float64))

        @staticmethod
        def backward(ctx, grad_pos):
            w = ctx.world
            gv, gk = w.backward(grad_pos.numpy().astype(np.float32), scene.n_springs)
            w.close()
            return torch.from_numpy(gv.astype(np.float64)), torch.from_numpy(gk.astype(np.float64))

    v0 = torch.tensor(scene.vreq.astype(np.float64), requires_grad=True)
    k = torch.tensor(scene.spr_k.astype(np.float64), requires_grad=True)
    pos = Rollout.apply(v0, k)
    M = sum(len(m) for m in marked)
    loss = 0.0
    for w, (m, t) in enumerate(zip(marked, targets)):
        b0 = int(scene.world_body_offsets[w])
        d = pos[torch.from_numpy(b0 + m)] - torch.from_numpy(t)
        loss = loss + (d * d).sum() / M
    loss.backward()
    final, g, after, gv, gk = gpu_gradients(scene, marked, targets, steps, every)
    assert np.array_equal(pos.detach().numpy(), final)
    # deterministic adjoint: the same gradients bit for bit
    assert np.array_equal(v0.grad.numpy(), gv) and np.array_equal(k.grad.numpy(), gk)


def test_backward_is_deterministic():
    """Two backward passes over the same recording, and a second recorded
    rollout, give the same gradients bit for bit."""
    scene, marked, targets = make_scene(seed=33, n_worlds=3)
    with native.World(scene) as w:
        w.rollout_record(scene.dt, 8, 3)
        g = loss_grad(w.read_bodies()["pos"].astype(np.float64), scene, marked, targets).astype(np.float32)
        a = w.backward(g, scene.n_springs)
        b = w.backward(g, scene.n_springs)
    _, _, _, gv, gk = gpu_gradients(scene, marked, targets, 8, 3)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(a[0].astype(np.float64), gv) and np.array_equal(a[1].astype(np.float64), gk)


@pytest.mark.parametrize("steps", [17, 24, 33])
def test_gradient_batch_across_checkpoints_matches_finite_differences(steps):
    """The differentiable-rollout batch at full size (256 worlds x 2,048
    spheres, 1,024 springs per world, 64 marked bodies) with a checkpoint
    every 16 steps, over 17, 24 and 33 steps: the backward pass restores one
    or two checkpoints and recomputes their segments.  Worlds 0 and 255 are
    checked (1) in full against the f64 replay of the traced f32 oracle, and
    (2) at 32 sampled parameters (velocities and stiffnesses alternating)
    against f64 central finite differences chained along the same traced
    trajectory (adjoint_replay.tangent_fd: fourth-order stencil per substep,
    state step 1e-3, recorded contact sets), within 1e-3 relative with a
    floor of 1e-4 of the largest gradient of the kind in that world; a
    sample whose wall clamp changes inside the stencil is discarded and
    reported.  Finite differences of the f64 oracle from the initial state
    are no reference here: on these overlapping starts the f32 and f64
    trajectories are 0.5 units apart after 17 steps."""
    scene, marked, targets = scenes.gradient_batch()
    final, g, after, gv, gk = gpu_gradients(scene, marked, targets, steps, 16)
    assert np.array_equal(final, after)
    assert np.all(np.isfinite(gv)) and np.all(np.isfinite(gk))
    rng = np.random.Generator(np.random.PCG64(1000 + steps))
    checked, discarded, worst = 0, 0, 0.0
    for w in (0, scene.n_worlds - 1):
        sub = scenes.unpack_world(scene, w)
        b0, b1 = int(scene.world_body_offsets[w]), int(scene.world_body_offsets[w + 1])
        s0, s1 = int(scene.world_spring_offsets[w]), int(scene.world_spring_offsets[w + 1])
        o = oracle.OracleWorld(sub, 32)
        o.trace(True)
        assert o.step(scene.dt, steps) == 0
        assert o.pushouts == 0
        fin = o.bodies()["pos"]
        assert np.array_equal(fin.astype(np.float32), final[b0:b1].astype(np.float32)), w
        tr = o.traced()
        rv, rk, rworst = replay_gradients(sub, tr, fin, g[b0:b1], scene.dt)
        _check_replay(rworst, fin)
        # the f32 adjoint's own rounding, amplified along the horizon: within
        # 1e-4 of the largest gradient up to 24 steps, 3e-4 at 33
        floor = 1e-4 if steps <= 24 else 3e-4
        _close(gv[b0:b1], rv, ("dL/dv0", w, steps), floor)
        _close(gk[s0:s1], rk, ("dL/dk", w, steps), floor)
        wv, wk = gv[b0:b1], gk[s0:s1]
        floor_v, floor_k = 1e-4 * np.abs(wv).max(), 1e-4 * np.abs(wk).max()
        n_here = 0
        while n_here < 16:
            if n_here % 2 == 0:
                b, ax = divmod(_pick(rng, wv.reshape(-1)), 2)
                param, g_gpu, floor = ("v", b, ax), wv[b, ax], floor_v
            else:
                e = _pick(rng, wk)
                param, g_gpu, floor = ("k", e), wk[e], floor_k
            fd, changed = tangent_fd(sub, tr, g[b0:b1], scene.dt, param)
            if changed:
                discarded += 1
                assert discarded <= 16, discarded
                continue
            err = abs(g_gpu - fd) / (1e-3 * max(abs(fd), floor))
            worst = max(worst, err)
            assert err <= 1.0, (w, param, g_gpu, fd, floor)
            n_here += 1
            checked += 1
    assert checked == 32
    print("steps %d: 32 samples within %.3g of the bound, %d discarded" % (steps, worst, discarded))
