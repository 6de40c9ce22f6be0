"""The population layout's address arithmetic (mf-lbm-cuda_gb300/csrc/common.cuh,
Bricks): 2x2x2 bricks grouped into tiles of 2^lx x 2^ly x 2^lz bricks, each
tile storing its 19 directions one after the other.  Restated here in
Python: for every tile shape the library accepts, every (node of
[0, n+1]^3, direction) gets a distinct pair index below 19 * S, a brick's 8
nodes of one direction are 8 consecutive pairs starting on a multiple of 8
(one 64-byte burst in FP32), and a tile's slice of one direction is
contiguous."""
import itertools

import pytest

EX = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
EY = [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1]
EZ = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1]


class Bricks:
    def __init__(self, nx, ny, nz, lx, ly, lz):
        self.nbx, self.nby, self.nbz = (nx + 3) // 2, (ny + 3) // 2, (nz + 3) // 2
        self.lx, self.ly, self.lz = lx, ly, lz
        self.ntx = (self.nbx + (1 << lx) - 1) >> lx
        self.nty = (self.nby + (1 << ly) - 1) >> ly
        self.ntz = (self.nbz + (1 << lz) - 1) >> lz
        self.tile = 8 << (lx + ly + lz)
        self.S = self.tile * self.ntx * self.nty * self.ntz

    def ax(self, x):
        b = x >> 1
        return (b >> self.lx) * 19 * self.tile + ((b & ((1 << self.lx) - 1)) << 3) + (x & 1)

    def ay(self, y):
        b = y >> 1
        return ((b >> self.ly) * 19 * self.tile * self.ntx + ((b & ((1 << self.ly) - 1)) << (3 + self.lx))
                + ((y & 1) << 1))

    def az(self, z):
        b = z >> 1
        return ((b >> self.lz) * 19 * self.tile * self.ntx * self.nty
                + ((b & ((1 << self.lz) - 1)) << (3 + self.lx + self.ly)) + ((z & 1) << 2))

    def pair(self, x, y, z, q):
        return self.ax(x) + self.ay(y) + self.az(z) + q * self.tile


SHAPES = [(3, 2, 1), (0, 0, 0), (1, 1, 1), (4, 1, 1), (2, 3, 0), (5, 5, 1)]
SIZES = [(20, 20, 28), (21, 19, 30), (16, 17, 9)]


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(str(1 << v) for v in s))
@pytest.mark.parametrize("n", SIZES, ids=lambda n: "x".join(map(str, n)))
def test_pairs_are_distinct_and_in_range(n, shape):
    nx, ny, nz = n
    B = Bricks(nx, ny, nz, *shape)
    seen = set()
    for x, y, z in itertools.product(range(nx + 2), range(ny + 2), range(nz + 2)):
        for q in range(19):
            seen.add(B.pair(x, y, z, q))
    assert len(seen) == (nx + 2) * (ny + 2) * (nz + 2) * 19
    assert min(seen) >= 0 and max(seen) < 19 * B.S


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(str(1 << v) for v in s))
def test_bricks_and_tiles_are_contiguous(shape):
    nx, ny, nz = 21, 19, 30
    B = Bricks(nx, ny, nz, *shape)
    for bx, by, bz in itertools.product(range(B.nbx), range(B.nby), range(B.nbz)):
        for q in (0, 7, 18):
            ps = sorted(B.pair(2 * bx + (e & 1), 2 * by + ((e >> 1) & 1), 2 * bz + (e >> 2), q) for e in range(8))
            assert ps == list(range(ps[0], ps[0] + 8)) and ps[0] % 8 == 0
    # one direction of one tile: tile consecutive pairs
    tx, ty, tz = 1 << shape[0], 1 << shape[1], 1 << shape[2]
    for q in (0, 11):
        ps = sorted(B.pair(2 * bx + (e & 1), 2 * by + ((e >> 1) & 1), 2 * bz + (e >> 2), q)
                    for bx in range(tx) for by in range(ty) for bz in range(tz) for e in range(8))
        assert ps == list(range(q * B.tile, (q + 1) * B.tile))


def test_neighbour_pairs_are_sums_of_axis_terms():
    """The collision forms x +- e_q as ax(x +- 1) + ay(y +- 1) + az(z +- 1):
    the per-axis terms add up to the full pair index of the neighbour."""
    B = Bricks(20, 20, 28, 3, 2, 1)
    for x, y, z in itertools.product(range(1, 21), range(1, 21), range(1, 29, 3)):
        X = {d: B.ax(x + d) for d in (-1, 0, 1)}
        Y = {d: B.ay(y + d) for d in (-1, 0, 1)}
        Z = {d: B.az(z + d) for d in (-1, 0, 1)}
        for q in range(19):
            assert X[EX[q]] + Y[EY[q]] + Z[EZ[q]] == B.pair(x + EX[q], y + EY[q], z + EZ[q], 0)
