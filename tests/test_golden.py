"""Committed golden states (tests/golden/oracle_states.json, made by
tests/golden/make_golden.py): SHA-256 digests of the f32 oracle's final
positions, previous positions and velocities on seeded scenes whose
arithmetic is IEEE +, -, *, / and sqrt only (no rotation), plus contact
counts.  The oracle must keep reproducing them (a change to the restatement
shows here first), and the GPU must reproduce them bit for bit."""
import json
import os

import pytest

from blobs_gb300 import native
from golden.make_golden import golden_scenes, state_of
from oracle import oracle

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_states.json")
CASES = {name: (s, steps) for name, s, steps in golden_scenes()}


def fixture():
    with open(FIXTURE) as f:
        return json.load(f)


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_the_golden_states(name):
    s, steps = CASES[name]
    want = fixture()[name]
    assert want["steps"] == steps and want["bodies"] == s.n_bodies
    o = oracle.OracleWorld(s, 32)
    assert o.step(s.dt, steps) == 0
    got = state_of(o.bodies(), o.contacts)
    assert got == {k: want[k] for k in got}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_reproduces_the_golden_states(name):
    s, steps = CASES[name]
    want = fixture()[name]
    with native.World(s) as w:
        for _ in range(steps):
            w.step(s.dt)
        got = state_of(w.read_bodies(), w.contact_count()[0])
    assert got == {k: want[k] for k in got}
