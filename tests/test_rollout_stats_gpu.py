"""Multi-step rollouts against the f64 oracle by their statistics.

Pair-order and rounding differences make any two trajectories of this
contact dynamics diverge after a few dozen steps, so long rollouts are
compared by what the divergence leaves intact: kinetic and potential energy,
the largest and the number of penetrations, and the cumulative contact
count, sampled along the run.  (Against the f32 oracle the GPU rollout is
bit-exact -- tests/test_parity_gpu.py; this is the f64 comparison.)

Tolerances, from the f32 oracle's own distance to the f64 oracle on the
same scenes (its statistics are the GPU's):
  sparse_spheres (1,000 spheres, 600 steps, every 50): potential energy within 1%,
    kinetic energy within 5% of the run's peak, cumulative contacts within
    5% + 200, penetrations: count within 30% + 20, largest within 0.02;
  dense (3,000 spheres at 40% packing with overlaps, 120 steps, every 10):
    potential energy within 12% (+2% of the run's largest), kinetic energy
    within 20%, cumulative contacts within 10%, largest penetration within
    0.05.
"""
import numpy as np
import pytest
from scipy.spatial import cKDTree

from blobs_gb300 import native, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu


def stats(pos, vel, mass, radius, gravity):
    pos = pos.astype(np.float64)
    vel = vel.astype(np.float64)
    ke = 0.5 * float((mass * (vel * vel).sum(1)).sum())
    pe = -float((mass * (pos @ gravity.astype(np.float64))).sum())
    r = radius.astype(np.float64)
    pairs = cKDTree(pos).query_pairs(2 * r.max(), output_type="ndarray")
    d = np.sqrt(((pos[pairs[:, 0]] - pos[pairs[:, 1]]) ** 2).sum(1))
    pen = r[pairs[:, 0]] + r[pairs[:, 1]] - d
    pen = pen[pen > 0]
    return ke, pe, (float(pen.max()) if len(pen) else 0.0), len(pen)


def series(scene, steps, every):
    o = oracle.OracleWorld(scene, 64)
    mass, _ = o.mass()
    gpu, ref = [], []
    with native.World(scene) as w:
        for _ in range(steps // every):
            w.rollout(scene.dt, every)
            b = w.read_bodies()
            gpu.append(stats(b["pos"], b["vel"], mass, scene.col_radius, scene.gravity) + (w.contact_count()[0],))
            assert o.step(scene.dt, every) == 0
            ob = o.bodies()
            ref.append(stats(ob["pos"], ob["vel"], mass, scene.col_radius, scene.gravity) + (o.contacts,))
    return np.array(gpu, float), np.array(ref, float)


def test_sparse_rollout_statistics_match_f64():
    s = scenes.sparse_spheres(seed=1, n=1000)
    g, r = series(s, 600, 50)
    ke_peak = np.abs(r[:, 0]).max()
    assert np.all(np.abs(g[:, 1] - r[:, 1]) <= 0.01 * np.abs(r[:, 1])), (g[:, 1], r[:, 1])
    assert np.all(np.abs(g[:, 0] - r[:, 0]) <= 0.05 * ke_peak), (g[:, 0], r[:, 0])
    assert np.all(np.abs(g[:, 4] - r[:, 4]) <= 0.05 * r[:, 4] + 200), (g[:, 4], r[:, 4])
    assert np.all(np.abs(g[:, 3] - r[:, 3]) <= 0.3 * r[:, 3] + 20), (g[:, 3], r[:, 3])
    assert np.all(np.abs(g[:, 2] - r[:, 2]) <= 0.02), (g[:, 2], r[:, 2])


def test_dense_rollout_statistics_match_f64():
    s = scenes.dense_spheres(seed=2, n=3000)
    g, r = series(s, 120, 10)
    pe_big = np.abs(r[:, 1]).max()
    assert np.all(np.abs(g[:, 1] - r[:, 1]) <= 0.12 * np.abs(r[:, 1]) + 0.02 * pe_big), (g[:, 1], r[:, 1])
    assert np.all(np.abs(g[:, 0] - r[:, 0]) <= 0.2 * np.abs(r[:, 0])), (g[:, 0], r[:, 0])
    assert np.all(np.abs(g[:, 4] - r[:, 4]) <= 0.1 * r[:, 4]), (g[:, 4], r[:, 4])
    assert np.all(np.abs(g[:, 2] - r[:, 2]) <= 0.05), (g[:, 2], r[:, 2])
