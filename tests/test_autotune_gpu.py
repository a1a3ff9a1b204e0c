"""The broadphase autotuner (blobs_world_autotune): it picks the cell edge
by timing, and the result of a step does not depend on that choice -- the
tuned world steps bit for bit like the f32 oracle and like an untuned world."""
import numpy as np
import pytest

from blobs_gb300 import native, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_autotuned_single_world_matches_oracle():
    s = scenes.sparse_spheres(seed=61, n=3000)
    with native.World(s) as w:
        cs0 = w.grid()[0]
        scale = w.autotune(s, s.dt, trial_steps=3)
        assert scale in (1.0, 1.125, 1.25, 1.5, 1.75)
        cs = w.grid()[0]
        assert cs == pytest.approx(cs0 * scale, rel=1e-6)
        # the world was reloaded: the scene's initial state
        assert np.array_equal(w.read_bodies()["pos"], s.pos)
        for _ in range(20):
            w.step(s.dt)
        got = w.read_bodies()
    o = oracle.OracleWorld(s, 32)
    assert o.step(s.dt, 20) == 0
    want = o.bodies()
    for k in ("pos", "pos_old", "vel"):
        assert np.array_equal(got[k].astype(np.float64), want[k]), k


@pytest.mark.parametrize("scale", [1.0, 1.125, 1.25, 1.5, 1.75])
def test_every_candidate_edge_gives_the_same_rollout(scale):
    """Each scale the autotuner may choose, forced through a requested cell
    edge, reproduces the default rollout of a batched spring world."""
    s = scenes.uneven_batch(seed=62, n_worlds=24, nmin=64, nmax=1500, steps=5)
    with native.World(s) as w:
        w.rollout(s.dt, 12)
        want = w.read_bodies()
        cs0 = w.grid()[0]
    with native.World(s, cell_size=cs0 * scale) as w:
        assert w.grid()[0] == pytest.approx(cs0 * scale, rel=1e-6)
        w.rollout(s.dt, 12)
        got = w.read_bodies()
    for k in ("pos", "pos_old", "vel"):
        assert np.array_equal(got[k], want[k]), k
