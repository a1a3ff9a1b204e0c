"""The joint schedule of the general path (blobs_joint_schedule, host only).

solve_fixed_joints (physics.rs:424-477) sweeps every joint in arena order,
joint_iterations times.  Joints of different components (bodies linked by
chains of joints) touch disjoint bodies, so the GPU sweeps each small
component alone in arena order -- which gives every body the reference's own
sequence of updates -- and colours the joints of large components.  These
checks need no device: the processing order is a permutation, each small
component is one contiguous run in arena order inside one block, blocks fit
their shared-memory staging, and no two joints of a colour share a body.
"""
import numpy as np
import pytest

from blobs_gb300 import native, scenes

JB_MAX_JOINTS, JB_THREADS, JB_JOINTS, JB_BODIES = 64, 128, 512, 640


def components(n_bodies, a, b):
    parent = np.arange(n_bodies)

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x
    for x, y in zip(a, b):
        rx, ry = find(int(x)), find(int(y))
        if rx != ry:
            parent[max(rx, ry)] = min(rx, ry)
    return np.array([find(int(x)) for x in a])


def check_schedule(n_bodies, a, b):
    a, b = np.asarray(a, np.uint32), np.asarray(b, np.uint32)
    order, blocks, colours = native.joint_schedule(n_bodies, a, b)
    nj = len(a)
    assert sorted(order.tolist()) == list(range(nj))
    comp = components(n_bodies, a, b)
    sizes = {c: int((comp == c).sum()) for c in np.unique(comp)} if nj else {}
    n_small = int(blocks[-1]) if len(blocks) else 0
    assert blocks[0] == 0 and np.all(np.diff(blocks) > 0)
    small = order[:n_small]
    assert all(sizes[comp[j]] <= JB_MAX_JOINTS for j in small)
    assert all(sizes[comp[j]] > JB_MAX_JOINTS for j in order[n_small:])
    for k in range(len(blocks) - 1):
        blk = order[blocks[k]:blocks[k + 1]]
        assert len(blk) <= JB_JOINTS
        assert len(np.unique(np.concatenate([a[blk], b[blk]]))) <= JB_BODIES
        assert len(np.unique(comp[blk])) <= JB_THREADS
        # each component: one contiguous run, ascending (arena) order, inside this block
        runs = np.flatnonzero(np.diff(comp[blk])) + 1
        for run in np.split(blk, runs):
            assert np.all(np.diff(run) > 0)
            assert len(run) == sizes[comp[run[0]]]
    if len(colours) > 1:
        assert colours[0] == n_small and colours[-1] == nj
        for k in range(len(colours) - 1):
            col = order[colours[k]:colours[k + 1]]
            ends = np.concatenate([a[col], b[col]])
            assert len(np.unique(ends)) == len(ends)
    else:
        assert n_small == nj
    return order, blocks, colours


def test_jointed_world_joints():
    s = scenes.jointed_bodies(seed=3, n=20000, n_joints=5000, n_springs=0, side=475.0)
    order, blocks, colours = check_schedule(s.n_bodies, s.jnt_a, s.jnt_b)
    assert len(colours) <= 1  # all components small


def test_chain_and_hub_take_the_coloured_sweep():
    rng = np.random.Generator(np.random.PCG64(3))
    chain = rng.permutation(2000)[:300]
    a = list(chain[:-1])
    b = list(chain[1:])
    rest = np.setdiff1d(np.arange(2000), chain)
    hub = int(rest[0])
    a += [hub] * 70                       # a static-anchor-like hub: one component of 70 joints
    b += list(rest[1:71])
    pairs = rest[71:71 + 400].reshape(-1, 2)
    a += list(pairs[:, 0])
    b += list(pairs[:, 1])
    perm = rng.permutation(len(a))
    order, blocks, colours = check_schedule(2000, np.array(a)[perm], np.array(b)[perm])
    assert len(colours) > 2
    assert int(colours[-1] - colours[0]) == 299 + 70


@pytest.mark.parametrize("n", [0, 1, 7])
def test_small_cases(n):
    rng = np.random.Generator(np.random.PCG64(n))
    a = rng.integers(0, 20, n)
    b = (a + 1 + rng.integers(0, 18, n)) % 20
    check_schedule(20, a, b)


def test_many_components_fill_many_blocks():
    rng = np.random.Generator(np.random.PCG64(11))
    n = 60000
    a = np.arange(0, n, 2)
    b = a + 1
    order, blocks, colours = check_schedule(n, a, b)
    assert len(blocks) - 1 >= (n // 2) // JB_THREADS


def test_invalid_joints_are_rejected():
    with pytest.raises(native.BlobsError) as ei:
        native.joint_schedule(5, [0, 1], [1, 1])
    assert ei.value.status == native.ERR_INVALID_ARGUMENT
    with pytest.raises(native.BlobsError):
        native.joint_schedule(5, [0], [9])
