"""The allocation-free contact-pair entry point, blobs_contact_pairs_noalloc.

It serves hosts that must not allocate device memory while they run -- a
frame loop that cannot absorb the device-wide synchronisation of
cudaMalloc / cudaFree, or a host whose device memory belongs to its own
budgeted allocator.  It keeps all its scratch in one static device array of
the library.  These tests call it through the C ABI and check its pair sets
against the oracle's all-pairs enumeration (oracle.contact_pairs) and against
the allocating entry point blobs_world_emit_pairs(contacts_only = 1): two
calls in a row, no colliders, more pairs than the output holds, the largest
collider count, a spread wide enough that the capped grid wraps, non-finite
snapshots and radii; that a collider count beyond the array's limit is
refused; and that a call leaves device free memory and the torch allocator's
counters unchanged.

This file is named to be collected last: the static array is shared by every
call in the process, and the tests must pass alone and after all others.
"""
import ctypes

import numpy as np
import pytest

from blobs_gb300 import native, scenes
from oracle import oracle

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


class Caller:
    """Device copies of one collider set and a call of the entry point."""

    def __init__(self, torch, snap, radius, parent=None, memb=None, filt=None, cap=None):
        self.torch = torch
        self.dev = torch.device("cuda", 0)
        self.fn, self.max_n = _bind()
        self.n = len(radius)

        def up(a, dt):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dt)
            if dt == np.uint32:
                a = a.view(np.int32)
            return torch.from_numpy(a.copy()).to(self.dev)

        self.snap = up(np.asarray(snap, np.float32).reshape(-1), np.float32)
        self.rad = up(radius, np.float32)
        self.parent, self.memb, self.filt = up(parent, np.uint32), up(memb, np.uint32), up(filt, np.uint32)
        self.cap = cap
        self.pairs = torch.zeros(2 * max(cap, 1), dtype=torch.int32, device=self.dev)
        self.count = torch.zeros(1, dtype=torch.int64, device=self.dev)
        self.stream = torch.cuda.current_stream(self.dev).cuda_stream

    @staticmethod
    def _p(t):
        return None if t is None else t.data_ptr()

    def call(self):
        self.pairs.fill_(-1)
        st = self.fn(self.n, self._p(self.snap), self._p(self.rad), self._p(self.parent), self._p(self.memb),
                     self._p(self.filt), self.pairs.data_ptr(), self.cap, self.count.data_ptr(),
                     ctypes.c_void_p(self.stream))
        return st

    def result(self):
        self.torch.cuda.synchronize(self.dev)
        k = int(self.count.item())
        got = self.pairs[: 2 * min(k, self.cap)].cpu().numpy().view(np.uint32).reshape(-1, 2)
        return k, got[np.lexsort((got[:, 1], got[:, 0]))]


def oracle_pairs(snap, radius, parent=None, memb=None, filt=None):
    hi, lo = oracle.contact_pairs(np.asarray(snap, np.float32).reshape(-1, 2), radius, parent, memb, filt)
    out = np.stack([hi, lo], 1).astype(np.uint32)
    return out[np.lexsort((out[:, 1], out[:, 0]))]


def check_against_oracle(torch, snap, radius, parent=None, memb=None, filt=None, calls=1):
    want = oracle_pairs(snap, radius, parent, memb, filt)
    c = Caller(torch, snap, radius, parent, memb, filt, cap=len(want) + 64)
    for call in range(calls):
        st = c.call()
        assert st == native.OK, (call, native.status_string(st))
        k, got = c.result()
        assert k == len(want), (call, k, len(want))
        assert np.array_equal(got, want), call
    return want


def test_noalloc_contact_pairs_match_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    _, max_n = _bind()
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
    got = check_against_oracle(torch, snap, s.col_radius, s.col_parent, s.col_memb, s.col_filt, calls=2)
    assert np.array_equal(got, want)


def test_noalloc_no_colliders():
    torch = pytest.importorskip("torch")
    c = Caller(torch, np.zeros((0, 2), np.float32), np.zeros(0, np.float32), cap=4)
    c.count.fill_(12345)
    assert c.call() == native.OK
    k, got = c.result()
    assert k == 0 and len(got) == 0


def test_noalloc_counts_pairs_beyond_cap():
    torch = pytest.importorskip("torch")
    rng = np.random.Generator(np.random.PCG64(3))
    snap = rng.uniform(0, 15, (3000, 2)).astype(np.float32)
    rad = rng.uniform(0.1, 0.3, 3000).astype(np.float32)
    want = oracle_pairs(snap, rad)
    assert len(want) > 100
    c = Caller(torch, snap, rad, cap=50)
    assert c.call() == native.OK
    k, got = c.result()
    assert k == len(want)  # the full count, although only `cap` pairs were written
    assert len(got) == 50
    wset = set(map(tuple, want.tolist()))
    assert all(tuple(p) in wset for p in got.tolist())


def test_noalloc_largest_collider_count():
    torch = pytest.importorskip("torch")
    _, max_n = _bind()
    rng = np.random.Generator(np.random.PCG64(4))
    snap = rng.uniform(0, 120, (max_n, 2)).astype(np.float32)
    rad = rng.uniform(0.1, 0.3, max_n).astype(np.float32)
    want = check_against_oracle(torch, snap, rad)
    assert len(want) > 10000


def test_noalloc_wide_spread_wraps_the_capped_grid():
    """~1e4 x 1e4 cells of extent against a cap of 2^17 cells: far cells
    alias on the torus; the exact test keeps the pair set exact."""
    torch = pytest.importorskip("torch")
    rng = np.random.Generator(np.random.PCG64(6))
    n = 4000
    centres = rng.uniform(-500, 500, (n // 2, 2))
    th = rng.uniform(0, 2 * np.pi, n // 2)
    ra, rb = rng.uniform(0.02, 0.05, n // 2), rng.uniform(0.02, 0.05, n // 2)
    other = centres + np.stack([np.cos(th), np.sin(th)], 1) * ((ra + rb) * rng.uniform(0.8, 1.1, n // 2))[:, None]
    snap = np.concatenate([centres, other]).astype(np.float32)
    rad = np.concatenate([ra, rb]).astype(np.float32)
    want = check_against_oracle(torch, snap, rad)
    assert len(want) > 500


def test_noalloc_non_finite_snapshots_and_radii():
    """NaN / inf snapshots and NaN radii touch nothing; a +inf radius
    touches every collider -- the reference test sqrt(d.d) < ra + rb."""
    torch = pytest.importorskip("torch")
    rng = np.random.Generator(np.random.PCG64(7))
    n = 2000
    snap = rng.uniform(0, 20, (n, 2)).astype(np.float32)
    rad = rng.uniform(0.1, 0.3, n).astype(np.float32)
    snap[5] = (np.nan, 1.0)
    snap[17] = (np.inf, 2.0)
    snap[29] = (3.0, -np.inf)
    rad[40] = np.nan
    check_against_oracle(torch, snap, rad)
    rad[77] = np.inf
    want = check_against_oracle(torch, snap, rad)
    assert np.count_nonzero((want[:, 0] == 77) | (want[:, 1] == 77)) > n - 10


def test_noalloc_allocates_no_device_memory():
    """After the first call (which loads the library's device module and so
    its static scratch array), calls leave the device's free memory and the
    torch allocator's counters unchanged."""
    torch = pytest.importorskip("torch")
    rng = np.random.Generator(np.random.PCG64(8))
    snap = rng.uniform(0, 30, (20000, 2)).astype(np.float32)
    rad = rng.uniform(0.05, 0.15, 20000).astype(np.float32)
    c = Caller(torch, snap, rad, cap=1 << 16)
    assert c.call() == native.OK
    c.result()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    stats0 = torch.cuda.memory_stats(0)
    for _ in range(3):
        assert c.call() == native.OK
    k, _ = c.result()
    assert k > 0
    free1, _ = torch.cuda.mem_get_info(0)
    stats1 = torch.cuda.memory_stats(0)
    assert free1 == free0
    for key in ("allocation.all.allocated", "reserved_bytes.all.current", "allocated_bytes.all.current"):
        assert stats1.get(key, 0) == stats0.get(key, 0), key


def test_noalloc_rejects_more_colliders_than_its_scratch_holds():
    torch = pytest.importorskip("torch")
    fn, max_n = _bind()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float32, device=dev)
    count_d = torch.zeros(1, dtype=torch.int64, device=dev)
    st = fn(max_n + 1, buf.data_ptr(), buf.data_ptr(), None, None, None, buf.data_ptr(), 1, count_d.data_ptr(),
            None)
    assert st == native.ERR_INVALID_ARGUMENT
