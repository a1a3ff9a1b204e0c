"""GPU parity of the step through the C ABI against the oracle.

Bit-exact where the reference arithmetic is reproducible (every contact /
spring / Verlet / constraint op is a separately rounded f32 op in the same
order; no push-out, no sin/cos of a non-zero rotation, no atan2), otherwise
within the stated tolerance of the f32 and f64 oracles.
"""
import numpy as np
import pytest

from blobs_gb300 import native, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu


def run_gpu(scene, steps, dt=None, **kw):
    dt = scene.dt if dt is None else dt
    with native.World(scene, **kw) as w:
        for _ in range(steps):
            w.step(dt)
        out = w.read_bodies()
        out["snap"] = w.read_snapshots()
        out["contacts"], out["contacts_last"] = w.contact_count()
        out["pushouts"] = w.pushout_count()
        out["joint_order"] = w.joint_order()[0] if scene.n_joints else None
    return out


def run_oracle(scene, steps, dt=None, precision=32, joint_order=None):
    dt = scene.dt if dt is None else dt
    w = oracle.OracleWorld(scene, precision, joint_order=joint_order)
    assert w.step(dt, steps) == 0
    out = w.bodies()
    out["snap"] = w.snapshots()
    out["contacts"] = w.contacts
    out["pushouts"] = w.pushouts
    return out


def assert_exact(got, want, keys=("pos", "pos_old", "vel")):
    for k in keys:
        g = got[k].astype(np.float64)
        bad = np.argwhere(g != want[k])
        assert len(bad) == 0, "%s: %d entries differ, first %s: gpu %s oracle %s" % (
            k, len(bad), bad[:3].tolist(), g[tuple(bad[0])], want[k][tuple(bad[0])])


# ---- 1,000 spheres in a walled box ---------------------------------------------

def test_sparse_single_step_bit_exact():
    s = scenes.sparse_spheres()
    got, want = run_gpu(s, 1), run_oracle(s, 1)
    assert_exact(got, want, ("pos", "pos_old", "vel", "snap"))
    assert got["contacts"] == want["contacts"]


def test_sparse_full_600_step_rollout_bit_exact():
    """All 600 steps (4,800 substeps): a single differing bit anywhere would
    grow chaotically, so equality at the end pins every substep."""
    s = scenes.sparse_spheres()
    got, want = run_gpu(s, s.n_steps), run_oracle(s, s.n_steps)
    assert want["pushouts"] == 0
    assert_exact(got, want, ("pos", "pos_old", "vel", "snap"))
    assert got["contacts"] == want["contacts"]


def test_rollout_graph_equals_eager_steps():
    s = scenes.sparse_spheres(seed=11, n=500)
    a = run_gpu(s, 40)
    with native.World(s) as w:
        w.step(s.dt)
        w.rollout(s.dt, 39)
        b = w.read_bodies()
    assert_exact(b, {k: a[k].astype(np.float64) for k in ("pos", "pos_old", "vel")})


def test_determinism_two_runs_bitwise_equal():
    s = scenes.dense_spheres(seed=5, n=20000)
    a, b = run_gpu(s, 5), run_gpu(s, 5)
    for k in ("pos", "pos_old", "vel"):
        assert np.array_equal(a[k], b[k])


# ---- dense overlapping spheres (scaled down) --------------------------------

@pytest.mark.parametrize("n", [4096, 30000])
def test_dense_scaled_bit_exact(n):
    s = scenes.dense_spheres(seed=2, n=n)
    got, want = run_gpu(s, 3), run_oracle(s, 3)
    assert want["pushouts"] == 0
    assert_exact(got, want, ("pos", "pos_old", "vel", "snap"))
    assert got["contacts"] == want["contacts"]


def test_sparse_f64_tolerance():
    """Sparse non-overlapping world: one step within |dx| <= 1e-4 (1 + |x|) of
    the f64 re-run, every component."""
    s = scenes.sparse_spheres(seed=21)
    got, want = run_gpu(s, 1), run_oracle(s, 1, precision=64)
    err = np.abs(got["pos"].astype(np.float64) - want["pos"])
    assert np.all(err <= 1e-4 * (1.0 + np.abs(want["pos"]))), err.max()


def test_dense_f64_tolerance():
    """Dense overlapping start (40% packing): the reference algorithm itself
    amplifies f32 rounding at contact-threshold flips (its f32 run deviates
    from f64 by up to ~1e-2 after 8 substeps, median ~1e-6).  Stated
    tolerance: 99% of components within 1e-4 (1 + |x|) of f64, and the GPU's
    largest deviation no larger than the f32 reference's own."""
    s = scenes.dense_spheres(seed=21, n=4096)
    got, want = run_gpu(s, 1), run_oracle(s, 1, precision=64)
    ref32 = run_oracle(s, 1, precision=32)
    err = np.abs(got["pos"].astype(np.float64) - want["pos"])
    err_ref = np.abs(ref32["pos"] - want["pos"])
    assert np.mean(err <= 1e-4 * (1.0 + np.abs(want["pos"]))) >= 0.99
    assert err.max() <= err_ref.max() * (1.0 + 1e-6)


def test_literal_2000_box_bit_exact():
    s = scenes.dense_spheres(seed=8, n=20000, literal_box=True)
    got, want = run_gpu(s, 2), run_oracle(s, 2)
    assert_exact(got, want)


# ---- springs, static bodies, sensors, groups, multi-collider bodies ---------

def test_springs_bit_exact():
    rng = np.random.Generator(np.random.PCG64(44))
    s = scenes.random_world(rng, 3000, 0.1, 0.3, 0.35, 1.0, spring_frac=0.3, k_range=(10.0, 1e4),
                            c_range=(0.0, 2.0))
    got, want = run_gpu(s, 10), run_oracle(s, 10)
    assert_exact(got, want)


def test_static_kinematic_bodies_sensors_groups_bit_exact():
    s = scenes.dense_spheres(seed=31, n=5000)
    rng = np.random.Generator(np.random.PCG64(31))
    s.body_type[rng.random(s.n_bodies) < 0.1] = scenes.STATIC
    # kinematic bodies integrate like dynamic ones: the reference only ever
    # tests is_static (rigid_body.rs:221-242, physics.rs:327)
    kin = rng.random(s.n_bodies) < 0.05
    s.body_type[kin & (s.body_type != scenes.STATIC)] = 2
    s.body_type[(rng.random(s.n_bodies) < 0.05) & (s.body_type == 0)] = 3
    s.col_sensor[rng.random(s.n_colliders) < 0.05] = 1
    s.col_memb = rng.choice(np.array([1, 2, 3, 0xFFFFFFFF], np.uint32), s.n_colliders)
    s.col_filt = rng.choice(np.array([1, 2, 0xFFFFFFFF], np.uint32), s.n_colliders)
    s.gravity_mod = rng.uniform(0.0, 2.0, s.n_bodies).astype(np.float32)
    got, want = run_gpu(s, 4), run_oracle(s, 4)
    assert_exact(got, want)
    assert got["contacts"] == want["contacts"]


def test_multi_collider_bodies_bit_exact():
    """The jointed-world layout (1-4 colliders per body) without joints:
    rotation stays 0, so the snapshots (rot(0) * offset + p) are exact and
    the merged per-body contact order is the reference's (outer collider,
    inner collider) sequence."""
    s = scenes.jointed_bodies(seed=3, n=6000, n_joints=0, n_springs=2000, side=90.0)
    s.jnt_a = s.jnt_a[:0]
    got, want = run_gpu(s, 4), run_oracle(s, 4)
    assert_exact(got, want, ("pos", "pos_old", "vel", "snap"))
    assert got["contacts"] == want["contacts"]


def test_pushout_on_the_general_path():
    """Multi-collider bodies with two colliders at the same point: the push-out
    branch (physics.rs:272-286) on the general contact path, bit-exact (no
    earlier contact of either body in the substep)."""
    s = scenes.spheres([[0.0, 0.0], [0.0, 0.0], [5.0, 5.0], [-5.0, 3.0]], [0.1, 0.1, 0.2, 0.15], gravity=(0.0, 0.0))
    # a second collider on bodies 1 and 3, away from the coincident pair
    s.col_parent = np.concatenate([s.col_parent, np.array([1, 3], np.uint32)])
    s.col_offset = np.concatenate([s.col_offset, np.array([[0.6, 0.0], [0.0, 0.4]], np.float32)])
    s.col_radius = np.concatenate([s.col_radius, np.array([0.1, 0.12], np.float32)])
    s.col_mass_override = np.concatenate([s.col_mass_override, np.full(2, np.nan, np.float32)])
    s.col_sensor = np.concatenate([s.col_sensor, np.zeros(2, np.uint8)])
    s.col_memb = np.concatenate([s.col_memb, np.full(2, scenes.ALL_GROUPS, np.uint32)])
    s.col_filt = np.concatenate([s.col_filt, np.full(2, scenes.ALL_GROUPS, np.uint32)])
    assert not s.single_collider()
    got, want = run_gpu(s, 1), run_oracle(s, 1)
    assert want["pushouts"] == 1 and got["pushouts"] == 1
    assert_exact(got, want, ("pos", "pos_old", "vel", "snap"))


def test_circle_constraint_bit_exact():
    s = scenes.sparse_spheres(seed=12, n=400)
    s.world_box = None
    s.circles = np.array([[0.0, 0.0, 12.0]], np.float32)
    got, want = run_gpu(s, 30), run_oracle(s, 30)
    assert_exact(got, want)


def test_collisions_disabled_bit_exact():
    s = scenes.sparse_spheres(seed=13, n=300)
    s.collisions_enabled = False
    got, want = run_gpu(s, 10), run_oracle(s, 10)
    assert_exact(got, want)
    assert got["contacts"] == 0


# ---- joints: per component, or coloured for large components ------------------

def test_joints_single_collider_positions_exact_in_gpu_order():
    """Single-collider bodies: snapshots do not depend on rotation, so the
    positions are bit-exact against the oracle run in the GPU's processing order;
    rotations use CUDA atan2f (tolerance 1e-5 rad)."""
    rng = np.random.Generator(np.random.PCG64(6))
    s = scenes.random_world(rng, 4000, 0.1, 0.25, 0.2, 0.5)
    near = scenes._pairs_within(s.pos, 1.0)
    pick = np.sort(rng.choice(len(near), 1500, replace=False))
    scenes.add_fixed_joints(s, near[pick, 0], near[pick, 1])
    got = run_gpu(s, 3)
    want = run_oracle(s, 3, joint_order=got["joint_order"])
    assert_exact(got, want)
    np.testing.assert_allclose(got["rotation"], want["rotation"], atol=1e-5)


@pytest.mark.parametrize("iterations", [4, 0, 1, 7])
def test_joints_small_components_exact_in_reference_order(iterations):
    """Joint components of at most 64 joints are swept one by one, each in
    the reference's arena order, which gives every body the reference's own
    sequence of updates: positions are bit-exact against the oracle run in
    the reference's joint order (joints created in a shuffled order, so the
    arena order is not sorted by body).  Up to 4 iterations the sweep defers
    the rotations to a second pass; 7 takes the single-pass sweep."""
    rng = np.random.Generator(np.random.PCG64(6))
    s = scenes.random_world(rng, 4000, 0.1, 0.25, 0.2, 0.5)
    s.joint_iterations = iterations
    near = scenes._pairs_within(s.pos, 1.0)
    pick = rng.choice(len(near), 1500, replace=False)  # unsorted: shuffled arena order
    scenes.add_fixed_joints(s, near[pick, 0], near[pick, 1])
    got = run_gpu(s, 3)
    want = run_oracle(s, 3)
    assert_exact(got, want)
    np.testing.assert_allclose(got["rotation"], want["rotation"], atol=1e-5)


def test_joints_long_chain_beside_small_components():
    """A 300-body chain (one component of 299 joints: the coloured sweep)
    beside small components (swept one by one): positions bit-exact against
    the oracle run in the GPU's processing order."""
    rng = np.random.Generator(np.random.PCG64(16))
    s = scenes.random_world(rng, 3000, 0.1, 0.25, 0.2, 0.5)
    chain = rng.permutation(3000)[:300]
    rest = np.setdiff1d(np.arange(3000), chain)
    near = scenes._pairs_within(s.pos, 1.0)
    near = near[np.isin(near[:, 0], rest) & np.isin(near[:, 1], rest)]
    pick = rng.choice(len(near), 800, replace=False)
    a = np.concatenate([chain[:-1], near[pick, 0]])
    b = np.concatenate([chain[1:], near[pick, 1]])
    order = rng.permutation(len(a))
    scenes.add_fixed_joints(s, a[order], b[order])
    got = run_gpu(s, 3)
    assert native_colours(s) > 1
    want = run_oracle(s, 3, joint_order=got["joint_order"])
    assert_exact(got, want)
    np.testing.assert_allclose(got["rotation"], want["rotation"], atol=1e-5)


def native_colours(scene):
    with native.World(scene) as w:
        return int(w.joint_order()[1])


def test_jointed_scaled_tolerance():
    """Multi-collider bodies + joints + springs: rotation enters the snapshots
    through sin/cos and the joints through atan2 (CUDA's, not glibc's), so
    one step is compared with tolerances.  Against the oracle run in the GPU's
    joint order: every component within 1e-4 (1 + |x|).  Against the f64
    re-run: the reference algorithm amplifies rounding at contact flips on
    this overlapping start (its own f32 run deviates from f64 by up to ~0.5),
    so 97% of components within 1e-4 (1 + |x|) and the largest deviation
    within 1% of the f32 reference's own."""
    s = scenes.jointed_bodies(seed=3, n=6000, n_joints=1500, n_springs=3000, side=90.0)
    got = run_gpu(s, 1)
    ref32 = run_oracle(s, 1, precision=32, joint_order=got["joint_order"])
    err = np.abs(got["pos"].astype(np.float64) - ref32["pos"])
    assert np.all(err <= 1e-4 * (1.0 + np.abs(ref32["pos"]))), err.max()
    ref64 = run_oracle(s, 1, precision=64, joint_order=got["joint_order"])
    err = np.abs(got["pos"].astype(np.float64) - ref64["pos"])
    err_ref = np.abs(ref32["pos"] - ref64["pos"])
    assert np.mean(err <= 1e-4 * (1.0 + np.abs(ref64["pos"]))) >= 0.97
    assert err.max() <= 1.01 * err_ref.max() + 1e-3


# ---- batched worlds -----------------------------------------------------------

def test_batched_worlds_bit_exact_per_world():
    s = scenes.uneven_batch(seed=14, n_worlds=24, nmin=64, nmax=1024)
    got = run_gpu(s, 5)
    for w in range(s.n_worlds):
        sub = scenes.unpack_world(s, w)
        want = run_oracle(sub, 5)
        b0, b1 = int(s.world_body_offsets[w]), int(s.world_body_offsets[w + 1])
        assert_exact({k: got[k][b0:b1] for k in ("pos", "pos_old", "vel")}, want)


# ---- known answers of the reference quirks on the GPU -------------------------

def test_pushout_coincident_spheres_gpu():
    s = scenes.spheres([[1, 1], [1, 1], [5, 5]], [0.5, 0.5, 0.2], gravity=(0, 0))
    got, want = run_gpu(s, 1), run_oracle(s, 1)
    assert got["pushouts"] == 1 == want["pushouts"]
    assert_exact(got, want)


def test_old_dt_ratio_changes_with_dt():
    s = scenes.sparse_spheres(seed=15, n=200)
    with native.World(s) as w:
        w.step(1 / 60)
        w.step(1 / 60)
        w.step(1 / 120)   # first dynamic body sees (1/960) / (1/480)
        w.step(1 / 120)
        got = w.read_bodies()
    o = oracle.OracleWorld(s, 32)
    o.step(1 / 60, 2)
    o.step(1 / 120, 2)
    assert_exact(got, o.bodies())


def test_body_collider_transform_gpu():
    """collider.rs:367-389 on the device: body at (2, 3) rotated pi/2, collider
    offset (1, 1) -> absolute translation (1, 4)."""
    s = scenes.empty_scene(1)
    s.pos = np.array([[2.0, 3.0]], np.float32)
    s.rotation = np.array([np.pi / 2], np.float32)
    s.col_parent = np.zeros(1, np.uint32)
    s.col_offset = np.array([[1.0, 1.0]], np.float32)
    s.col_radius = np.array([0.5], np.float32)
    s.col_mass_override = np.full(1, np.nan, np.float32)
    s.col_sensor = np.zeros(1, np.uint8)
    s.col_memb = np.full(1, scenes.ALL_GROUPS, np.uint32)
    s.col_filt = np.full(1, scenes.ALL_GROUPS, np.uint32)
    s.gravity = np.zeros(2, np.float32)
    s.body_type = np.array([scenes.STATIC], np.uint8)
    got = run_gpu(s, 1)
    np.testing.assert_allclose(got["snap"][0], [1.0, 4.0], atol=1e-5)


def test_fixed_step_accumulator():
    s = scenes.sparse_spheres(seed=16, n=100)
    with native.World(s) as w:
        w.fixed_step(0.05)        # 3 steps of 1/60 (max 3), accumulator 0
        t, acc = w.time()
        got = w.read_bodies()
    assert abs(t - 3 / 60) < 1e-12 and abs(acc - (0.05 - 3 / 60)) < 1e-12
    want = run_oracle(s, 3, dt=1 / 60)
    assert_exact(got, want)


# ---- degenerate and extreme inputs ------------------------------------------
def check_against_oracle(scene, dt, steps):
    got = run_gpu(scene, steps, dt)
    want = run_oracle(scene, steps, dt)
    assert_exact(got, want)
    assert got["contacts"] == want["contacts"]


def test_empty_world_steps():
    s = scenes.spheres(np.zeros((0, 2), np.float32), np.zeros(0, np.float32))
    with native.World(s) as w:
        w.step(1.0 / 60.0)
        w.rollout(1.0 / 60.0, 3)
        b = w.read_bodies()
        assert b["pos"].shape == (0, 2)
        assert w.contact_count() == (0, 0)


def test_single_body_falls_like_the_oracle():
    s = scenes.spheres(np.array([[0.5, 3.0]], np.float32), np.array([0.2], np.float32),
                       np.array([[0.3, 0.0]], np.float32))
    check_against_oracle(s, 1.0 / 60.0, 30)


def test_batch_with_empty_and_single_body_worlds():
    rng = np.random.Generator(np.random.PCG64(71))
    empty = scenes.spheres(np.zeros((0, 2), np.float32), np.zeros(0, np.float32), box=(-5, -5, 5, 5))
    one = scenes.spheres(np.array([[0.0, 1.0]], np.float32), np.array([0.3], np.float32),
                         np.array([[1.0, 0.5]], np.float32), box=(-5, -5, 5, 5))
    worlds = [scenes.random_world(rng, 200, 0.1, 0.3, 0.35, 1.0), empty, one,
              scenes.random_world(rng, 90, 0.1, 0.3, 0.35, 1.0), empty]
    s = scenes.pack(worlds)
    s.dt = 1.0 / 60.0
    with native.World(s) as w:
        for _ in range(12):
            w.step(s.dt)
        got = w.read_bodies()
    for i in range(s.n_worlds):
        sub = scenes.unpack_world(s, i)
        b0 = int(s.world_body_offsets[i])
        o = oracle.OracleWorld(sub, 32)
        assert o.step(s.dt, 12) == 0
        want = o.bodies()
        for k in ("pos", "pos_old", "vel"):
            assert np.array_equal(got[k][b0:b0 + sub.n_bodies].astype(np.float64), want[k]), (i, k)


def test_far_apart_clusters_share_a_wrapped_grid():
    """Two clusters 1e5 apart: the grid extent is capped, so the torus wraps
    and far cells alias; the exact test keeps the result exact."""
    rng = np.random.Generator(np.random.PCG64(72))
    a = rng.uniform(-3, 3, (300, 2)).astype(np.float32)
    b = (rng.uniform(-3, 3, (300, 2)) + np.array([1e5, -7e4])).astype(np.float32)
    pos = np.concatenate([a, b])
    rad = rng.uniform(0.1, 0.3, 600).astype(np.float32)
    vel = rng.normal(0, 1, (600, 2)).astype(np.float32)
    s = scenes.spheres(pos, rad, vel)
    check_against_oracle(s, 1.0 / 60.0, 10)
