"""The allocation-free contact-pair entry point, blobs_contact_pairs_noalloc.

It serves hosts that must not allocate device memory while they run -- a
frame loop that cannot absorb the device-wide synchronisation of
cudaMalloc / cudaFree, or a host whose device memory belongs to its own
budgeted allocator.  It keeps all its scratch in one static device array of
the library, so this test checks, through the C ABI, that two calls in a row
on the same colliders both return exactly the contact pair set of the
allocating entry point blobs_world_emit_pairs(contacts_only = 1), and that a
collider count beyond the array's limit is refused.

This file is named to be collected last: the static array is shared by every
call in the process, and the test must pass alone and after all others.
"""
import ctypes

import numpy as np
import pytest

from blobs_gb300 import native, scenes

pytestmark = pytest.mark.gpu


def _bind():
    L = native.lib()
    fn = L.blobs_contact_pairs_noalloc
    P = ctypes.c_void_p
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_uint32, P, P, P, P, P, P, ctypes.c_uint64, P, P]
    L.blobs_noalloc_max_colliders.restype = ctypes.c_uint32
    L.blobs_noalloc_max_colliders.argtypes = []
    return fn, int(L.blobs_noalloc_max_colliders())


def test_noalloc_contact_pairs_match_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    fn, max_n = _bind()
    # multi-collider bodies with offsets and mixed groups exercise every filter
    s = scenes.jointed_bodies(seed=81, n=6000, n_joints=0, n_springs=0, side=70.0)
    rng = np.random.Generator(np.random.PCG64(81))
    s.col_memb = rng.choice(np.array([1, 2, 0xFFFFFFFF], np.uint32), s.n_colliders)
    s.col_filt = rng.choice(np.array([1, 3, 0xFFFFFFFF], np.uint32), s.n_colliders)
    assert s.n_colliders <= max_n
    with native.World(s) as w:
        w.step(s.dt)
        snap = w.read_snapshots()
        want = w.emit_pairs(contacts_only=True)
    assert len(want) > 100

    dev = torch.device("cuda", 0)
    snap_d = torch.from_numpy(np.ascontiguousarray(snap, np.float32)).to(dev)
    rad_d = torch.from_numpy(np.ascontiguousarray(s.col_radius, np.float32)).to(dev)
    parent_d = torch.from_numpy(np.ascontiguousarray(s.col_parent, np.uint32).view(np.int32)).to(dev)
    memb_d = torch.from_numpy(np.ascontiguousarray(s.col_memb, np.uint32).view(np.int32)).to(dev)
    filt_d = torch.from_numpy(np.ascontiguousarray(s.col_filt, np.uint32).view(np.int32)).to(dev)
    cap = len(want) + 64
    pairs_d = torch.zeros(2 * cap, dtype=torch.int32, device=dev)
    count_d = torch.zeros(1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream

    for call in range(2):
        pairs_d.fill_(-1)
        st = fn(s.n_colliders, snap_d.data_ptr(), rad_d.data_ptr(), parent_d.data_ptr(), memb_d.data_ptr(),
                filt_d.data_ptr(), pairs_d.data_ptr(), cap, count_d.data_ptr(), ctypes.c_void_p(stream))
        assert st == native.OK, (call, native.status_string(st))
        torch.cuda.synchronize(dev)
        k = int(count_d.item())
        assert k == len(want), (call, k, len(want))
        got = pairs_d[: 2 * k].cpu().numpy().view(np.uint32).reshape(-1, 2)
        got = got[np.lexsort((got[:, 1], got[:, 0]))]
        assert np.array_equal(got, want), call


def test_noalloc_rejects_more_colliders_than_its_scratch_holds():
    torch = pytest.importorskip("torch")
    fn, max_n = _bind()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float32, device=dev)
    count_d = torch.zeros(1, dtype=torch.int64, device=dev)
    st = fn(max_n + 1, buf.data_ptr(), buf.data_ptr(), None, None, None, buf.data_ptr(), 1, count_d.data_ptr(),
            None)
    assert st == native.ERR_INVALID_ARGUMENT
