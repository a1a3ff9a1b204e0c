"""blobs_world_snapshot / blobs_world_restore: stepping after a restore
repeats the steps taken after the snapshot bit for bit, on every path
(uniform sphere world, batched worlds with springs, the general path with
multi-collider bodies and joints, the fixed-step accumulator)."""
import numpy as np
import pytest

from blobs_gb300 import native, scenes

pytestmark = pytest.mark.gpu


def jointed():
    s = scenes.jointed_bodies(seed=3, n=3000, n_joints=600, n_springs=800, side=70.0)
    return s


@pytest.mark.parametrize("make", [lambda: scenes.dense_spheres(seed=2, n=20000),
                                  lambda: scenes.uneven_batch(seed=8, n_worlds=12, nmin=64, nmax=2000),
                                  jointed], ids=["spheres", "batched", "general"])
def test_restore_repeats_the_same_steps(make):
    s = make()
    with native.World(s) as w:
        for _ in range(2):
            w.step(s.dt)
        w.snapshot()
        for _ in range(3):
            w.step(s.dt)
        first = w.read_bodies()
        c1 = w.contact_count()
        w.restore()
        for _ in range(3):
            w.step(s.dt)
        second = w.read_bodies()
        assert w.contact_count() == c1
    for k in ("pos", "pos_old", "vel", "rotation", "angvel"):
        assert np.array_equal(first[k], second[k]), k


def test_restore_brings_back_time_and_old_dt():
    s = scenes.sparse_spheres(seed=4, n=500)
    with native.World(s) as w:
        w.snapshot()  # before the first step: pending velocity requests, old_dt = 1
        w.fixed_step(0.05)
        a = w.read_bodies()
        t1 = w.time()
        w.restore()
        assert w.time() == (0.0, 0.0)
        w.fixed_step(0.05)
        b = w.read_bodies()
        assert w.time() == t1
    for k in ("pos", "pos_old", "vel"):
        assert np.array_equal(a[k], b[k]), k


def test_restore_without_snapshot_is_a_state_error():
    s = scenes.sparse_spheres(seed=5, n=50)
    with native.World(s) as w:
        with pytest.raises(native.BlobsError) as ei:
            w.restore()
        assert ei.value.status == native.ERR_STATE
        w.snapshot()
        w.load(s)  # a new scene drops the snapshot
        with pytest.raises(native.BlobsError):
            w.restore()
