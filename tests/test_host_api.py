"""The C++ host mirror of the reference Physics API (include/blobs_physics.hpp)
driven by tests/cpp/physics_host_test.cpp."""
import os
import subprocess

import numpy as np
import pytest

from blobs_gb300 import native, scenes
from oracle import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def host_test_bin(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("cpp") / "physics_host_test")
    libdir = os.path.dirname(native.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "physics_host_test.cpp"), "-L" + libdir, "-lblobs_gb300",
           "-Wl,-rpath," + libdir, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_host_mirror_cpu_semantics(host_test_bin):
    r = subprocess.run([host_test_bin, "cpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_host_mirror_steps_bit_exact(host_test_bin, tmp_path):
    """A world inserted body by body through Physics::insert_rbd /
    insert_collider_with_parent and stepped through Physics::step equals the
    oracle bit for bit."""
    s = scenes.sparse_spheres(seed=17, n=400)
    s.body_type[::37] = scenes.STATIC
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inp, "wb") as f:
        np.array([s.n_bodies], np.uint32).tofile(f)
        s.gravity.astype(np.float32).tofile(f)
        s.world_box[0].astype(np.float32).tofile(f)
        for i in range(s.n_bodies):
            np.array([s.pos[i, 0], s.pos[i, 1], s.vreq[i, 0], s.vreq[i, 1], s.col_radius[i]], np.float32).tofile(f)
            np.array([s.body_type[i]], np.uint8).tofile(f)
    steps = 25
    r = subprocess.run([host_test_bin, "scene", inp, outp, str(steps), repr(s.dt)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = open(outp, "rb").read()
    got = np.frombuffer(raw[:24 * s.n_bodies], np.float32).reshape(-1, 6)
    off = 24 * s.n_bodies
    contacts, n_events = (int(x) for x in np.frombuffer(raw[off:off + 16], np.uint64))
    ev = raw[off + 16:]
    assert len(ev) == 24 * n_events
    ev_ids = np.frombuffer(ev, np.uint32).reshape(-1, 6)[:, :2]
    ev_vel = np.frombuffer(ev, np.float32).reshape(-1, 6)[:, 2:]
    w = oracle.OracleWorld(s, 32, record_events=True)
    assert w.step(s.dt, steps) == 0
    want = w.bodies()
    np.testing.assert_array_equal(got[:, 0:2].astype(np.float64), want["pos"])
    np.testing.assert_array_equal(got[:, 2:4].astype(np.float64), want["pos_old"])
    np.testing.assert_array_equal(got[:, 4:6].astype(np.float64), want["vel"])
    assert contacts == w.contacts
    # Physics::collision_events() (the collision_recv channel) in the reference's order
    a, b, va, vb = w.events()
    assert n_events == len(a) > 0
    np.testing.assert_array_equal(ev_ids[:, 0], a)
    np.testing.assert_array_equal(ev_ids[:, 1], b)
    np.testing.assert_array_equal(ev_vel[:, 0:2].astype(np.float64), va)
    np.testing.assert_array_equal(ev_vel[:, 2:4].astype(np.float64), vb)


@pytest.mark.gpu
def test_host_mirror_remove_and_continue(host_test_bin, tmp_path):
    """Host mutation round trip through the C++ mirror: step, remove bodies
    (remove_rbd) and last colliders (remove_col, which takes the body with
    it), step again.  Both phases equal the oracle bit for bit; the second
    phase is the oracle restarted from the first phase's state without the
    removed bodies (arena iteration skips the freed slots)."""
    s = scenes.sparse_spheres(seed=19, n=600)
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inp, "wb") as f:
        np.array([s.n_bodies], np.uint32).tofile(f)
        s.gravity.astype(np.float32).tofile(f)
        s.world_box[0].astype(np.float32).tofile(f)
        for i in range(s.n_bodies):
            np.array([s.pos[i, 0], s.pos[i, 1], s.vreq[i, 0], s.vreq[i, 1], s.col_radius[i]], np.float32).tofile(f)
            np.array([s.body_type[i]], np.uint8).tofile(f)
    s1, s2, every = 10, 12, 7
    r = subprocess.run([host_test_bin, "mutate", inp, outp, str(s1), str(s2), repr(s.dt), str(every)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.frombuffer(open(outp, "rb").read(), np.float32).reshape(-1, 8)
    first, second = raw[:s.n_bodies], raw[s.n_bodies:]
    o = oracle.OracleWorld(s, 32)
    assert o.step(s.dt, s1) == 0
    b = o.bodies()
    snap = o.snapshots()
    np.testing.assert_array_equal(first[:, 0:2].astype(np.float64), b["pos"])
    np.testing.assert_array_equal(first[:, 2:4].astype(np.float64), b["pos_old"])
    np.testing.assert_array_equal(first[:, 4:6].astype(np.float64), b["vel"])
    np.testing.assert_array_equal(first[:, 6:8].astype(np.float64), snap)
    keep = np.ones(s.n_bodies, bool)
    for i in range(0, s.n_bodies, every):
        keep[i] = False
        if i + 1 < s.n_bodies:
            keep[i + 1] = False
    idx = np.flatnonzero(keep)
    rest = scenes.spheres(b["pos"][idx], s.col_radius[idx], box=tuple(s.world_box[0]),
                          body_type=s.body_type[idx])
    rest.pos_old = b["pos_old"][idx]
    rest.vel = b["vel"][idx]
    rest.col_snap = snap[idx]
    o2 = oracle.OracleWorld(rest, 32, old_dt=float(np.float32(np.float32(s.dt) / np.float32(8))))
    assert o2.step(s.dt, s2) == 0
    b2 = o2.bodies()
    assert second.shape[0] == len(idx)
    np.testing.assert_array_equal(second[:, 0:2].astype(np.float64), b2["pos"])
    np.testing.assert_array_equal(second[:, 2:4].astype(np.float64), b2["pos_old"])
    np.testing.assert_array_equal(second[:, 4:6].astype(np.float64), b2["vel"])
