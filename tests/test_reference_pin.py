"""The reference-pinning scenes (tests/golden/pin_scenes.py): the f32
oracle's final states are committed as digests
(tests/golden/reference_pin.json), the target a Rust harness running the
reference itself on the same generated inputs must hit.
Here the oracle must keep reproducing them, the independent NumPy
restatement of the substep loop must reach the same digests, the
generator's inputs must stay what the fixture records, and the GPU step
must reproduce them bit for bit."""
import json
import os

import numpy as np
import pytest

from golden.pin_scenes import FIXTURE, XorShift32, digest, inputs_of, pin_scenes
from oracle import oracle
from test_step_restatement import RefWorld

CASES = {name: (s, steps, dt) for name, s, steps, dt in pin_scenes()}


def fixture():
    with open(FIXTURE) as f:
        return json.load(f)


def test_generator_stream():
    """The first values of the stream from seed 1 (Marsaglia's xorshift32,
    shifts 13, 17, 5), for a port of the generator to check against."""
    g = XorShift32(1)
    assert [g.next() for _ in range(4)] == [270369, 67634689, 2647435461, 307599695]
    g = XorShift32(1)
    assert g.unit() == np.float32(270369 >> 8) * np.float32(2.0 ** -24)


@pytest.mark.parametrize("name", sorted(CASES))
def test_inputs_are_the_recorded_ones(name):
    s, steps, dt = CASES[name]
    want = fixture()[name]
    assert inputs_of(s) == want["inputs"]
    assert (s.n_bodies, s.n_colliders, steps) == (want["bodies"], want["colliders"], want["steps"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_the_pin_states(name):
    s, steps, dt = CASES[name]
    want = fixture()[name]
    o = oracle.OracleWorld(s, 32)
    assert o.step(dt, steps) == 0
    b = o.bodies()
    assert {k: digest(b[k]) for k in ("pos", "pos_old", "vel")} == {k: want[k] for k in ("pos", "pos_old", "vel")}
    assert o.contacts == want["contacts"] > 1000


@pytest.mark.parametrize("name", sorted(CASES))
def test_restatement_reaches_the_pin_states(name):
    s, steps, dt = CASES[name]
    want = fixture()[name]
    ref = RefWorld(s)
    for _ in range(steps):
        ref.step(dt)
    b = ref.bodies()
    assert {k: digest(b[k]) for k in ("pos", "pos_old", "vel")} == {k: want[k] for k in ("pos", "pos_old", "vel")}
    assert ref.contacts == want["contacts"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_reproduces_the_pin_states(name):
    from blobs_gb300 import native
    s, steps, dt = CASES[name]
    want = fixture()[name]
    with native.World(s) as w:
        for _ in range(steps):
            w.step(dt)
        b = w.read_bodies()
        contacts = w.contact_count()[0]
    assert {k: digest(b[k]) for k in ("pos", "pos_old", "vel")} == {k: want[k] for k in ("pos", "pos_old", "vel")}
    assert contacts == want["contacts"]
