"""SpatialHash on the device (blobs_spatial_hash_*) against the oracle's
restatement of blobs/src/spatial.rs: the reference's own test cases
(tests.rs:27-90) and seeded random point sets, compared query by query as id
sets (the reference returns them in HashMap order, unspecified)."""
import numpy as np
import pytest

from blobs_gb300 import native
from oracle import oracle

pytestmark = pytest.mark.gpu


def per_query(offsets, ids):
    return [ids[int(offsets[q]):int(offsets[q + 1])].tolist() for q in range(len(offsets) - 1)]


def oracle_hash(cs, ids, xy, radius):
    sh = oracle.SpatialHash(cs)
    for i, p, r in zip(ids, xy, radius):
        sh.insert_with_id(int(i), float(p[0]), float(p[1]), float(r))
    return sh


def oracle_results(sh, qxy, qr):
    out = []
    for p, r in zip(qxy, qr):
        got = sh.query(float(p[0]), float(p[1]), float(r))
        out.append(sorted(int(i) for i in got[0]))
    return out


def test_reference_cases():
    # tests.rs:15-24 create_spatial_hash, queried around each point
    xy = np.array([[50, 50], [150, 150], [250, 250], [350, 350], [450, 450]], np.float32)
    with native.SpatialHash(100.0) as h:
        h.set_points(np.arange(5), xy, np.ones(5))
        off, ids = h.query(np.array([[150, 150], [50, 50], [450, 450]], np.float32), np.array([200, 1, 500]))
        assert per_query(off, ids) == [[0, 1, 2], [0], [3, 4]]
    # tests.rs:57-68 insert_and_query
    with native.SpatialHash(1.0) as h:
        h.set_points([0, 1], np.array([[0, 0], [2, 2]], np.float32), [0, 0])
        off, ids = h.query(np.array([[1, 1]], np.float32), [1.5])
        assert per_query(off, ids) == [[0, 1]]
        # tests.rs:70-80 move_point: (0, 0) + (2, 2), then the same query
        h.set_points([0], np.array([[0 + 2, 0 + 2]], np.float32), [0])
        off, ids = h.query(np.array([[1, 1]], np.float32), [1.5])
        assert per_query(off, ids) == [[0]]
        # tests.rs:82-90 remove
        h.set_points([], np.zeros((0, 2), np.float32), [])
        off, ids = h.query(np.array([[0, 0]], np.float32), [1.5])
        assert per_query(off, ids) == [[]]


@pytest.mark.parametrize("seed,n,nq,cs", [(1, 20000, 3000, 1.0), (2, 5000, 2000, 0.37), (3, 30000, 1000, 4.0)])
def test_random_sets_match_oracle(seed, n, nq, cs):
    rng = np.random.Generator(np.random.PCG64(seed))
    ids = rng.permutation(10 * n)[:n].astype(np.uint64)
    xy = rng.uniform(-60.0, 60.0, (n, 2)).astype(np.float32)
    radius = rng.uniform(0.0, 0.6, n).astype(np.float32)
    # points on cell borders
    xy[: n // 20] = (np.round(xy[: n // 20] / cs) * cs).astype(np.float32)
    qxy = rng.uniform(-65.0, 65.0, (nq, 2)).astype(np.float32)
    qr = rng.uniform(0.0, 3.0 * cs, nq).astype(np.float32)  # radii beyond one cell: the 3x3 limit shows
    with native.SpatialHash(cs) as h:
        h.set_points(ids, xy, radius)
        off, got = h.query(qxy, qr)
    want = oracle_results(oracle_hash(cs, ids, xy, radius), qxy, qr)
    assert per_query(off, got) == want
    assert sum(len(w) for w in want) > nq // 4


def test_edge_coordinates_match_oracle():
    """NaN (cell 0), huge values (saturated cells, wrapping neighbours),
    negative zero and values just below cell borders."""
    cs = 1.0
    pts = np.array([[np.nan, 0.5], [0.5, np.nan], [3e38, 3e38], [-3e38, -3e38], [3e38, -3e38],
                    [-0.0, -0.0], [np.nextafter(np.float32(1), np.float32(0)), 0.0], [1.0, 1.0], [-1e-30, 0.2],
                    [2147483520.0, 5.0], [-2147483648.0, 5.0]], np.float32)
    ids = np.arange(len(pts), dtype=np.uint64) * 7 + 3
    radius = np.full(len(pts), 0.5, np.float32)
    qxy = np.concatenate([pts, np.array([[0.0, 0.0], [0.9, 0.9], [-0.5, 0.5], [3e38, -3e38]], np.float32)])
    qr = np.full(len(qxy), np.inf, np.float32)  # every point of the nine cells passes the distance test
    qr[-4:] = 1.0
    with native.SpatialHash(cs) as h:
        h.set_points(ids, pts, radius)
        off, got = h.query(qxy, qr)
    want = oracle_results(oracle_hash(cs, ids, pts, radius), qxy, qr)
    assert per_query(off, got) == want


def test_capacity_too_small_reports_total():
    rng = np.random.Generator(np.random.PCG64(9))
    xy = rng.uniform(-5, 5, (500, 2)).astype(np.float32)
    with native.SpatialHash(1.0) as h:
        h.set_points(np.arange(500), xy, np.full(500, 0.5, np.float32))
        off, ids = h.query(xy[:50], np.full(50, 1.0, np.float32))
        with pytest.raises(native.BlobsError) as ei:
            h.query(xy[:50], np.full(50, 1.0, np.float32), cap=len(ids) - 1)
        assert ei.value.status == native.ERR_OVERFLOW
