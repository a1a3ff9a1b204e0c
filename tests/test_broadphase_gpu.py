"""The GPU broadphase's output pair sets (the cell-key + counting-sort +
cell-range pipeline that replaces spatial.rs / the O(C^2) loop of
physics.rs:241-317), bit-exact against CPU enumerations."""
import numpy as np
import pytest

from blobs_gb300 import native, scenes
from oracle import oracle
from tests.gridkey import grid_coord

pytestmark = pytest.mark.gpu


def cpu_candidates(snap, inv_cs, origin, log2w, log2h):
    """All (hi, lo) pairs whose wrapped cells are 3x3 neighbours."""
    W, H = 1 << log2w, 1 << log2h
    ix = grid_coord(snap[:, 0].astype(np.float32), origin[0], inv_cs) % W
    iy = grid_coord(snap[:, 1].astype(np.float32), origin[1], inv_cs) % H
    key = iy * W + ix
    order = np.argsort(key, kind="stable")
    buckets = {}
    for i in order:
        buckets.setdefault(int(key[i]), []).append(int(i))
    out = []
    for i in range(len(snap)):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                k = int(((iy[i] + dy) % H) * W + (ix[i] + dx) % W)
                for j in buckets.get(k, ()):
                    if j < i:
                        out.append((i, j))
    out = np.array(sorted(set(out)), np.uint32).reshape(-1, 2)
    return out


@pytest.mark.parametrize("n,literal", [(5000, False), (20000, True)])
def test_candidate_pairs_bit_exact(n, literal):
    s = scenes.dense_spheres(seed=40 + n, n=n, literal_box=literal)
    with native.World(s) as w:
        w.step(s.dt)
        snap = w.read_snapshots()
        cs, inv_cs, origin, lw, lh = w.grid()
        assert inv_cs == np.float32(1.0) / np.float32(cs)
        got = w.emit_pairs(contacts_only=False)
    want = cpu_candidates(snap, inv_cs, origin, lw, lh)
    assert got.shape == want.shape and np.array_equal(got, want)


def test_contact_pairs_equal_bruteforce():
    """The contact subset equals the reference's O(C^2) brute-force contact set
    (groups, parents and dist < ra + rb) on the same snapshots."""
    s = scenes.jointed_bodies(seed=41, n=4000, n_joints=0, n_springs=0, side=70.0)
    s.jnt_a = s.jnt_a[:0]
    rng = np.random.Generator(np.random.PCG64(41))
    s.col_memb = rng.choice(np.array([1, 2, 0xFFFFFFFF], np.uint32), s.n_colliders)
    s.col_filt = rng.choice(np.array([1, 3, 0xFFFFFFFF], np.uint32), s.n_colliders)
    with native.World(s) as w:
        w.step(s.dt)
        snap = w.read_snapshots()
        got = w.emit_pairs(contacts_only=True)
    i, j = oracle.contact_pairs(snap, s.col_radius, s.col_parent, s.col_memb, s.col_filt)
    want = np.stack([i, j], 1).astype(np.uint32)
    want = want[np.lexsort((want[:, 1], want[:, 0]))]
    assert len(want) > 100
    assert np.array_equal(got, want)


def test_emit_pairs_overflow_then_retry():
    """An undersized buffer reports BLOBS_ERR_OVERFLOW with the full count; a
    retry with that capacity succeeds (host-side fault injection)."""
    import ctypes
    s = scenes.dense_spheres(seed=42, n=3000)
    with native.World(s) as w:
        n = ctypes.c_uint64()
        buf = np.zeros((4, 2), np.uint32)
        st = native.lib().blobs_world_emit_pairs(w._h, 0, buf.ctypes.data, 4, ctypes.byref(n))
        assert st == native.ERR_OVERFLOW and n.value > 4
        full = w.emit_pairs(contacts_only=False, cap=int(n.value))
        assert len(full) == n.value
        # the world still steps correctly afterwards
        w.step(s.dt)
        got = w.read_bodies()
    ref = oracle.OracleWorld(s, 32)
    ref.step(s.dt, 1)
    np.testing.assert_array_equal(got["pos"].astype(np.float64), ref.bodies()["pos"])
