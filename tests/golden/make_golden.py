"""Regenerates tests/golden/oracle_states.json: the f32 oracle's final state
of seeded scenes, as SHA-256 digests of the float32 arrays plus contact
counts.  The scenes avoid rotation (no joints, no multi-collider offsets
under rotation), so their arithmetic is IEEE +, -, *, / and sqrt only and
the digests are the same on every host.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from blobs_gb300 import scenes  # noqa: E402
from oracle import oracle  # noqa: E402


def golden_scenes():
    """(name, scene, steps) -- the cases the fixture holds."""
    out = [("sparse_1000_60", scenes.sparse_spheres(seed=1, n=1000), 60),
           ("dense_4096_3", scenes.dense_spheres(seed=2, n=4096), 3)]
    rng = np.random.Generator(np.random.PCG64(4))
    s = scenes.random_world(rng, 1500, 0.1, 0.3, 0.35, 1.0, spring_frac=0.2, k_range=(50.0, 500.0),
                            c_range=(0.0, 1.0))
    s.col_sensor = (rng.random(s.n_colliders) < 0.1).astype(np.uint8)
    s.col_memb = rng.choice(np.array([1, 2, 0xFFFFFFFF], np.uint32), s.n_colliders)
    s.col_filt = rng.choice(np.array([1, 3, 0xFFFFFFFF], np.uint32), s.n_colliders)
    out.append(("springs_groups_1500_4", s, 4))
    g = scenes.gradient_batch(seed=5, n_worlds=1, n_per=1200, n_springs=500)[0]
    out.append(("gradient_world_1200_6", scenes.unpack_world(g, 0), 6))
    return out


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def state_of(bodies, contacts):
    return {"pos": digest(bodies["pos"]), "pos_old": digest(bodies["pos_old"]), "vel": digest(bodies["vel"]),
            "contacts": int(contacts)}


def main():
    fixture = {}
    for name, s, steps in golden_scenes():
        o = oracle.OracleWorld(s, 32)
        assert o.step(s.dt, steps) == 0
        fixture[name] = dict(state_of(o.bodies(), o.contacts), steps=steps, bodies=s.n_bodies)
    path = os.path.join(HERE, "oracle_states.json")
    with open(path, "w") as f:
        json.dump(fixture, f, indent=1, sort_keys=True)
        f.write("\n")
    print(path)


if __name__ == "__main__":
    main()
