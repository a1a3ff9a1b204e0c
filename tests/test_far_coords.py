"""Contacts far from the broadphase grid's origin.

The reference finds every pair with sqrt(d.d) < ra + rb wherever the bodies
are (physics.rs:264-269).  The grid's cell coordinate
floor((v - origin) / cs) must therefore put two such spheres in
3x3-neighbouring cells at any distance from the origin; in plain f32 the
rounding of v - origin and of the product grows to several cells at 1e7
cells out, which would drop contacts silently.  These tests build worlds
with touching pairs 1e5 and 1e6 units from a cluster at the origin
(rmax 0.05, so up to ~2e7 cells out) and check that the device finds
exactly the oracle's contact pairs -- single-sphere and general world paths
and the allocation-free entry point -- and that the steps stay bit-exact.
"""
import ctypes

import numpy as np
import pytest

from blobs_gb300 import native, scenes
from oracle import oracle
from tests import gridkey

CENTRES = [(1.0e5, 0.0), (1.0e6, 3.0e5), (-1.0e6, -2.0e5)]


def far_pairs_scene(seed=91, n_near=400, n_pairs=400):
    """Spheres of radius U[0.03, 0.05] near the origin plus, around each
    far centre, n_pairs touching pairs (centre distance 0.9-0.999 of the
    radius sum, random direction), all positions distinct in f32."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = [rng.uniform(-5, 5, (n_near, 2))]
    rad = [rng.uniform(0.03, 0.05, n_near)]
    for cx, cy in CENTRES:
        a = np.array([cx, cy]) + rng.uniform(-30, 30, (n_pairs, 2))
        ra, rb = rng.uniform(0.03, 0.05, n_pairs), rng.uniform(0.03, 0.05, n_pairs)
        th = rng.uniform(0, 2 * np.pi, n_pairs)
        d = (ra + rb) * rng.uniform(0.9, 0.999, n_pairs)
        b = a + np.stack([np.cos(th), np.sin(th)], 1) * d[:, None]
        pos += [a, b]
        rad += [ra, rb]
    pos = np.concatenate(pos).astype(np.float32)
    rad = np.concatenate(rad).astype(np.float32)
    _, first = np.unique(pos, axis=0, return_index=True)
    keep = np.sort(first)
    pos, rad = pos[keep], rad[keep]
    vel = rng.normal(0, 0.2, pos.shape).astype(np.float32)
    return scenes.spheres(pos, rad, vel, gravity=(0.0, -9.81))


def oracle_pairs(snap, radius, **kw):
    hi, lo = oracle.contact_pairs(snap, radius, **kw)
    out = np.stack([hi, lo], 1).astype(np.uint32)
    return out[np.lexsort((out[:, 1], out[:, 0]))]


def world_grid_params(s):
    """The world path's grid edge and origin for a single world (world.cu)."""
    rmax = np.float32(s.col_radius.max())
    cs = np.float32(np.float32(2.0) * rmax * np.float32(1.0 + 1.0 / 64.0))
    inv = np.float32(1.0) / cs
    return cs, inv, np.float32(s.pos[:, 0].min() - cs), np.float32(s.pos[:, 1].min() - cs)


def test_far_scene_defeats_the_plain_formula_and_not_the_exact_one():
    """On the CPU: the scene's contact pairs land in neighbouring cells
    under the exact grid function, while the plain f32 formula puts some of
    them two or more cells apart (the hazard the exact path removes)."""
    s = far_pairs_scene()
    want = oracle_pairs(s.pos, s.col_radius)
    assert len(want) > 600
    cs, inv, ox, oy = world_grid_params(s)
    hi, lo = want[:, 0], want[:, 1]
    worst_plain = worst_exact = 0
    for axis, o in ((0, ox), (1, oy)):
        v = s.pos[:, axis]
        ge = gridkey.grid_coord(v, o, inv)
        gp = gridkey.grid_coord_plain(v, o, inv)
        worst_exact = max(worst_exact, int(np.abs(ge[hi] - ge[lo]).max()))
        worst_plain = max(worst_plain, int(np.abs(gp[hi] - gp[lo]).max()))
    assert worst_exact <= 1
    assert worst_plain >= 2


def test_grid_coord_equals_the_real_floor():
    """The exact path equals floor((v - o) * inv) of the real numbers (here
    float64, exact for these operands) except within 1e-6 of a cell edge."""
    rng = np.random.Generator(np.random.PCG64(5))
    v = np.concatenate([rng.uniform(-3e6, 3e6, 200000), rng.uniform(-1e9, 1e9, 20000)]).astype(np.float32)
    for o, inv in ((np.float32(-1.0e6 - 0.1), np.float32(1.0) / np.float32(0.1015625)),
                   (np.float32(12.5), np.float32(1.0) / np.float32(0.30467))):
        got = gridkey.grid_coord(v, o, inv)
        x = (v.astype(np.float64) - np.float64(o)) * np.float64(inv)
        ref = np.clip(np.floor(x), -2147483648, 2147483647).astype(np.int64)
        edge = np.abs(x - np.round(x)) < 1e-6 * np.maximum(1.0, np.abs(x) * 1e-9)
        assert np.array_equal(got[~edge], ref[~edge])


@pytest.mark.gpu
def test_far_pairs_single_sphere_world_path():
    s = far_pairs_scene()
    want = oracle_pairs(s.pos, s.col_radius)
    with native.World(s) as w:
        got = w.emit_pairs(contacts_only=True)
    assert np.array_equal(got, want), (len(got), len(want))


@pytest.mark.gpu
def test_far_pairs_single_sphere_steps_bit_exact():
    s = far_pairs_scene()
    dt, steps = 1.0 / 60.0, 3
    with native.World(s) as w:
        for _ in range(steps):
            w.step(dt)
        got = w.read_bodies()
        contacts = w.contact_count()[0]
        pairs_after = w.emit_pairs(contacts_only=True)
        snap = w.read_snapshots()
    o = oracle.OracleWorld(s, 32)
    assert o.step(dt, steps) == 0
    want = o.bodies()
    for k in ("pos", "pos_old", "vel"):
        assert np.array_equal(got[k].astype(np.float64), want[k]), k
    assert contacts == o.contacts
    assert np.array_equal(pairs_after, oracle_pairs(snap, s.col_radius))


@pytest.mark.gpu
def test_far_pairs_general_world_path():
    """One non-default membership moves the world to the general
    (multi-collider) path, which has its own key and candidate kernels."""
    s = far_pairs_scene()
    s.col_memb[0] = 1
    want = oracle_pairs(s.pos, s.col_radius, parent=s.col_parent, memb=s.col_memb, filt=s.col_filt)
    dt = 1.0 / 60.0
    with native.World(s) as w:
        got = w.emit_pairs(contacts_only=True)
        w.step(dt)
        body = w.read_bodies()
    assert np.array_equal(got, want), (len(got), len(want))
    o = oracle.OracleWorld(s, 32)
    assert o.step(dt, 1) == 0
    ref = o.bodies()
    for k in ("pos", "pos_old", "vel"):
        assert np.array_equal(body[k].astype(np.float64), ref[k]), k


@pytest.mark.gpu
def test_far_pairs_noalloc_entry_point():
    torch = pytest.importorskip("torch")
    s = far_pairs_scene()
    want = oracle_pairs(s.pos, s.col_radius)
    fn = native.lib().blobs_contact_pairs_noalloc
    P = ctypes.c_void_p
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_uint32, P, P, P, P, P, P, ctypes.c_uint64, P, P]
    dev = torch.device("cuda", 0)
    snap_d = torch.from_numpy(np.ascontiguousarray(s.pos, np.float32)).to(dev)
    rad_d = torch.from_numpy(np.ascontiguousarray(s.col_radius, np.float32)).to(dev)
    cap = len(want) + 16
    pairs_d = torch.full((2 * cap,), -1, dtype=torch.int32, device=dev)
    count_d = torch.zeros(1, dtype=torch.int64, device=dev)
    st = fn(s.n_colliders, snap_d.data_ptr(), rad_d.data_ptr(), None, None, None, pairs_d.data_ptr(), cap,
            count_d.data_ptr(), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    assert st == native.OK, native.status_string(st)
    torch.cuda.synchronize(dev)
    k = int(count_d.item())
    got = pairs_d[: 2 * k].cpu().numpy().view(np.uint32).reshape(-1, 2)
    got = got[np.lexsort((got[:, 1], got[:, 0]))]
    assert np.array_equal(got, want), (k, len(want))
