"""The brick layout's address arithmetic (mf-lbm-cuda_gb300/csrc/common.cuh,
Bricks::elem, and the parity deltas of collide_stream_kernel): every node of
[0, n+1]^3 gets a distinct element, and for every interior node and
direction the neighbours x + e_q and x - e_q sit at e0 + delta(q) and
e0 + delta(opp(q)) respectively."""
import pytest

EX = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
EY = [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1]
EZ = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1]
OPP = [0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15]


def make(nx, ny, nz):
    nbx, nby, nbz = (nx + 3) // 2, (ny + 3) // 2, (nz + 3) // 2

    def elem(x, y, z):
        return (((x >> 1) + nbx * ((y >> 1) + nby * (z >> 1))) << 3) | (x & 1) | ((y & 1) << 1) | ((z & 1) << 2)

    def deltas(x, y, z):
        bx8, bxy8 = 8 * nbx, 8 * nbx * nby
        dxp, dxm = (7, -1) if x & 1 else (1, -7)
        dyp, dym = (bx8 - 2, -2) if y & 1 else (2, 2 - bx8)
        dzp, dzm = (bxy8 - 4, -4) if z & 1 else (4, 4 - bxy8)
        pick = lambda c, p, m: p if c > 0 else (m if c < 0 else 0)
        return [pick(EX[q], dxp, dxm) + pick(EY[q], dyp, dym) + pick(EZ[q], dzp, dzm) for q in range(19)]

    return elem, deltas, nbx * nby * nbz * 8


@pytest.mark.parametrize("n", [(20, 20, 28), (21, 19, 30), (16, 17, 9)])
def test_elements_are_distinct_and_in_range(n):
    nx, ny, nz = n
    elem, _, S = make(nx, ny, nz)
    es = {elem(x, y, z) for x in range(nx + 2) for y in range(ny + 2) for z in range(nz + 2)}
    assert len(es) == (nx + 2) * (ny + 2) * (nz + 2)
    assert max(es) < S


@pytest.mark.parametrize("n", [(20, 20, 28), (21, 19, 30), (16, 17, 9)])
def test_neighbour_offsets(n):
    nx, ny, nz = n
    elem, deltas, _ = make(nx, ny, nz)
    for x in range(1, nx + 1):
        for y in range(1, ny + 1):
            for z in range(1, nz + 1):
                e0, d = elem(x, y, z), deltas(x, y, z)
                for q in range(19):
                    assert elem(x + EX[q], y + EY[q], z + EZ[q]) == e0 + d[q]
                    assert elem(x - EX[q], y - EY[q], z - EZ[q]) == e0 + d[OPP[q]]
