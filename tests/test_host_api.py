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
    s = scenes.config1(seed=17, n=400)
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
