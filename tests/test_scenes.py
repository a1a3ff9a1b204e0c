"""The seeded workload generators against the workloads they stand for (no
dataset exists; these are synthetic scenes with the stated shapes, sizes and
distributions).  No GPU."""
import math

import numpy as np

from blobs_gb300 import scenes


def packing(s):
    area = float(np.sum(np.pi * s.col_radius.astype(np.float64) ** 2))
    return area / float(np.prod(s.world_box[0, 2:] - s.world_box[0, :2]))


def test_sparse_spheres_1000_in_a_40_box():
    s = scenes.sparse_spheres()
    assert s.n_bodies == 1000 and s.single_collider() and s.dt == 1.0 / 60.0 and s.n_steps == 600
    assert s.col_radius.min() >= 0.1 and s.col_radius.max() <= 0.3
    assert np.array_equal(s.world_box[0], np.array([-20, -20, 20, 20], np.float32))
    d = np.sqrt(((s.pos[:, None, :] - s.pos[None, :, :]) ** 2).sum(-1))
    r = s.col_radius[:, None] + s.col_radius[None, :]
    np.fill_diagonal(d, np.inf)
    assert np.all(d >= r)  # rejection-sampled: no overlap at t = 0
    assert abs(float(s.vreq.std()) - 1.0) < 0.1 and s.vreq_set.all()


def test_dense_spheres_at_40_percent_packing():
    s = scenes.dense_spheres(n=200_000)  # the same generator as the 1M-sphere world, smaller
    assert s.dt == 1.0 / 120.0 and s.single_collider()
    assert 0.05 <= s.col_radius.min() and s.col_radius.max() <= 0.15
    assert abs(packing(s) - 0.40) < 0.01
    assert abs(float(s.vreq.std()) - 0.5) < 0.01
    lit = scenes.dense_spheres(n=1000, literal_box=True)
    assert float(lit.world_box[0, 2] - lit.world_box[0, 0]) == 2000.0
    assert abs(scenes.box_side(1_000_000, 0.05, 0.15, 0.40) - 291.7) < 0.1


def test_jointed_bodies_colliders_joints_springs():
    s = scenes.jointed_bodies(n=20000, n_joints=5000, n_springs=10000, side=475.0)
    per_body = np.bincount(s.col_parent, minlength=s.n_bodies)
    assert per_body.min() == 1 and per_body.max() == 4
    assert np.all(np.hypot(s.col_offset[:, 0], s.col_offset[:, 1]) <= 0.5)
    assert 0.1 <= s.col_radius.min() and s.col_radius.max() <= 0.25
    assert s.n_joints == 5000
    d = np.hypot(*(s.pos[s.jnt_a] - s.pos[s.jnt_b]).T)
    assert np.all(d < 1.5)
    assert len(set(zip(s.jnt_a.tolist(), s.jnt_b.tolist()))) == s.n_joints  # without replacement
    assert s.n_springs == 10000
    rest = np.hypot(*(s.pos[s.spr_a] - s.pos[s.spr_b]).T)
    np.testing.assert_allclose(s.spr_rest, rest, rtol=1e-6)
    assert 10.0 <= s.spr_k.min() and s.spr_k.max() <= 1e4 and 0 <= s.spr_c.min() and s.spr_c.max() <= 2.0
    assert s.dt == 1.0 / 120.0


def test_uneven_batch_log_uniform_worlds():
    s = scenes.uneven_batch(n_worlds=256)
    counts = np.diff(s.world_body_offsets)
    assert s.n_worlds == 256 and counts.min() >= 64 and counts.max() <= 8192
    # log-uniform body counts: the median is near the geometric mean of the range
    assert abs(math.log(float(np.median(counts))) - 0.5 * (math.log(64) + math.log(8192))) < 0.5
    assert s.dt == 1.0 / 60.0 and s.n_steps == 100
    boxes = np.prod(s.world_box[:, 2:] - s.world_box[:, :2], axis=1).astype(np.float64)
    disc = np.pi * s.col_radius.astype(np.float64) ** 2
    assert abs(disc.sum() / boxes.sum() - 0.35) < 0.005  # ~35% packing (each box sized for it)
    for w in (0, 100, 255):
        sub = scenes.unpack_world(s, w)
        assert abs(packing(sub) - 0.35) < 0.05  # small worlds: the radii's sampling spread
        assert 0.1 <= sub.col_radius.min() and sub.col_radius.max() <= 0.3
        assert abs(sub.n_springs - 0.1 * sub.n_bodies) <= 1


def test_gradient_batch_256_worlds_of_2048():
    s, marked, targets = scenes.gradient_batch(n_worlds=4)
    assert s.n_worlds == 4 and s.n_bodies == 4 * 2048 and s.n_springs == 4 * 1024
    assert s.dt == 1.0 / 60.0 and s.n_steps == 120
    assert all(len(m) == 64 for m in marked) and all(t.shape == (64, 2) for t in targets)
    sub = scenes.unpack_world(s, 0)
    assert abs(packing(sub) - 0.30) < 0.02
    assert 0.1 <= sub.col_radius.min() and sub.col_radius.max() <= 0.2
    assert 100.0 <= sub.spr_k.min() and sub.spr_k.max() <= 5000.0


def test_generators_are_seeded():
    a, b = scenes.dense_spheres(seed=7, n=5000), scenes.dense_spheres(seed=7, n=5000)
    assert np.array_equal(a.pos, b.pos) and np.array_equal(a.col_radius, b.col_radius)
    c = scenes.dense_spheres(seed=8, n=5000)
    assert not np.array_equal(a.pos, c.pos)


def test_pack_and_unpack_round_trip():
    rng = np.random.Generator(np.random.PCG64(12))
    worlds = [scenes.random_world(rng, n, 0.1, 0.3, 0.35, 1.0, spring_frac=0.2) for n in (50, 300, 120)]
    packed = scenes.pack(worlds)
    assert packed.n_worlds == 3 and packed.n_bodies == 470
    for k, w in enumerate(worlds):
        u = scenes.unpack_world(packed, k)
        for name in ("pos", "vreq", "col_radius", "col_offset", "spr_rest", "spr_k", "spr_c"):
            assert np.array_equal(getattr(u, name), getattr(w, name)), (k, name)
        assert np.array_equal(u.col_parent, w.col_parent) and np.array_equal(u.spr_a, w.spr_a)
        assert np.array_equal(u.spr_b, w.spr_b)
        assert np.array_equal(u.world_box[0], w.world_box[0])
