"""The oracle's SpatialHash against an independent restatement of the
reference's (spatial.rs:31-195, the HashMap build: feature use-grid off),
written here line by line with NumPy float32 scalars: cell coordinates
`(v / cell_size).floor() as i32` (f32 division, saturating conversion, NaN
to 0), insert / insert_with_id, remove by the stored position's cell,
move_point re-binning only when the cell changes, and query over the 3x3
cells with `|p - q|^2 <= (qr + r)^2`.  The reference iterates HashSets, so
a query's result order is unspecified: results are compared as sorted
(id, x, y) rows.  Random sequences of a few thousand operations, including
points far from the origin and at cell boundaries.
"""
import numpy as np
import pytest

from oracle import oracle

F = np.float32


def _as_i32(q):
    """Rust `f32 as i32`: saturating, NaN -> 0."""
    if q != q:
        return 0
    if q >= F(2147483648.0):
        return 2147483647
    if q <= F(-2147483648.0):
        return -2147483648
    return int(q)


class RefHash:
    def __init__(self, cell_size):
        self.cs = F(cell_size)
        self.next_id = 0
        self.points = {}   # id -> (x, y, radius)
        self.grid = {}     # (cx, cy) -> set of ids

    def cell(self, x, y):
        with np.errstate(over="ignore", invalid="ignore"):  # f32 overflow to inf is the semantics
            return _as_i32(np.floor(F(x) / self.cs)), _as_i32(np.floor(F(y) / self.cs))

    def insert(self, x, y, r):
        i = self.next_id
        self.next_id += 1
        self.insert_with_id(i, x, y, r)
        return i

    def insert_with_id(self, i, x, y, r):
        self.grid.setdefault(self.cell(x, y), set()).add(i)
        self.points[i] = (F(x), F(y), F(r))

    def remove(self, i):
        p = self.points.pop(i, None)
        if p is None:
            return False
        c = self.cell(p[0], p[1])
        if c in self.grid:
            self.grid[c].discard(i)
        return True

    def move_point(self, i, dx, dy):
        p = self.points.get(i)
        if p is None:
            return False
        nx, ny = F(p[0] + F(dx)), F(p[1] + F(dy))
        old, new = self.cell(p[0], p[1]), self.cell(nx, ny)
        if old != new:
            if old in self.grid:
                self.grid[old].discard(i)
            self.grid.setdefault(new, set()).add(i)
        self.points[i] = (nx, ny, p[2])
        return True

    def query(self, x, y, qr):
        x, y, qr = F(x), F(y), F(qr)
        cx, cy = self.cell(x, y)
        out = []
        for ox in (-1, 0, 1):
            for oy in (-1, 0, 1):
                for i in self.grid.get((cx + ox, cy + oy), ()):
                    px, py, r = self.points[i]
                    d = F(qr + r)
                    ex, ey = F(px - x), F(py - y)
                    if F(F(ex * ex) + F(ey * ey)) <= F(d * d):
                        out.append((i, float(px), float(py)))
        return sorted(out)


def _rows(ids, pos):
    return sorted((int(i), float(p[0]), float(p[1])) for i, p in zip(ids, pos))


@pytest.mark.parametrize("seed,cell,spread", [(1, 2.0, 20.0), (2, 0.37, 5.0), (3, 1.0, 3.0e6)])
def test_oracle_spatial_hash_equals_the_restatement(seed, cell, spread):
    rng = np.random.Generator(np.random.PCG64(seed))
    ref, orc = RefHash(cell), oracle.SpatialHash(cell)
    live = []
    queries = 0
    for step in range(3000):
        op = rng.uniform()
        if op < 0.35 or not live:
            x, y = (F(v) for v in rng.uniform(-spread, spread, 2))
            if rng.uniform() < 0.1:  # on a cell boundary
                x = F(np.floor(x / F(cell)) * F(cell))
            r = F(rng.uniform(0.0, 2.0 * cell))
            a, b = ref.insert(x, y, r), orc.insert(x, y, r)
            assert a == b
            live.append(a)
        elif op < 0.6:
            i = live[rng.integers(len(live))]
            dx, dy = (F(v) for v in rng.normal(0.0, cell, 2))
            assert ref.move_point(i, dx, dy) == orc.move_point(i, dx, dy)
        elif op < 0.7:
            i = live.pop(rng.integers(len(live)))
            assert ref.remove(i) == orc.remove(i)
            assert ref.remove(i) == orc.remove(i) is False
        else:
            i = live[rng.integers(len(live))]
            px, py, _ = ref.points[i]
            x, y = F(px + F(rng.normal(0.0, cell))), F(py + F(rng.normal(0.0, cell)))
            qr = F(rng.uniform(0.0, 1.5 * cell))
            got = _rows(*orc.query(x, y, qr))
            assert got == ref.query(x, y, qr), step
            queries += 1
    assert queries > 500
    for i in live:
        p = ref.points[i]
        assert orc.point(i) == (float(p[0]), float(p[1]))
        assert orc.cell_coords(float(p[0]), float(p[1])) == ref.cell(p[0], p[1])


def test_cell_coordinates_of_extreme_values():
    ref, orc = RefHash(0.5), oracle.SpatialHash(0.5)
    for v in (0.0, -0.0, 0.49999997, 0.5, -0.5, -1e-45, 1e9, -1e9, 3.0e38, -3.0e38, np.inf, -np.inf, np.nan):
        assert orc.cell_coords(float(v), float(v)) == ref.cell(F(v), F(v)), v
