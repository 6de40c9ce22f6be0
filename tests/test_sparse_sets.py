"""Index arithmetic of the sparse colour-gradient passes
(mf-lbm-cuda_gb300/csrc/gradient.cuh: phi_brick_kernel, active_nodes_kernel),
restated in numpy.

The passes skip every node whose ISO4 stencil (the node and its 18 D3Q19
neighbours, s4-local i+2 .. i+4 on each axis) lies in eight 2x2x2 phi bricks
of one common code (all exactly +1 or all exactly -1): there every difference
of the ISO4 sums is +0 and the normal record is the zero record.  These tests
check, on random phase fields with sharp and diffuse interfaces and on odd and
even extents, that

  * every node of [-1, n+2]^3 belongs to exactly one node block c
    (nodes 2c-2 .. 2c-1 per axis), and the blocks range over
    [0, (n+4)/2] per axis;
  * the eight bricks c .. c+1 of a block lie inside the brick grid
    ((n+9)/2 bricks per axis of the s4 lattice) and cover the stencils of all
    of the block's nodes;
  * every node outside the active blocks has a stencil of one value (so its
    gradient is exactly zero), i.e. nothing with a non-zero gradient is
    skipped.
"""
import numpy as np
import pytest

EX = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
EY = [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1]
EZ = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1]


def brick_codes(phi4):
    """Per 2x2x2 brick of the s4 array (x fastest axis last in numpy order:
    phi4[z, y, x]); positions past the array end are ignored."""
    NZ, NY, NX = phi4.shape
    BZ, BY, BX = (NZ + 1) // 2, (NY + 1) // 2, (NX + 1) // 2
    pad = np.full((2 * BZ, 2 * BY, 2 * BX), np.nan)
    pad[:NZ, :NY, :NX] = phi4
    b = pad.reshape(BZ, 2, BY, 2, BX, 2)
    present = ~np.isnan(b)
    plus = np.all(np.where(present, b == 1.0, True), axis=(1, 3, 5))
    minus = np.all(np.where(present, b == -1.0, True), axis=(1, 3, 5))
    return np.where(plus, 1, np.where(minus, 2, 0)).astype(np.int8)


def active_blocks(codes, n):
    nx, ny, nz = n
    CX, CY, CZ = (nx + 4) // 2 + 1, (ny + 4) // 2 + 1, (nz + 4) // 2 + 1
    BZ, BY, BX = codes.shape
    assert CX + 1 <= BX and CY + 1 <= BY and CZ + 1 <= BZ
    c0 = codes[:CZ, :CY, :CX]
    same = np.ones_like(c0, dtype=bool)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                same &= codes[dz:dz + CZ, dy:dy + CY, dx:dx + CX] == c0
    quiet = (c0 != 0) & same
    return ~quiet


def random_phase(n, seed, sharp):
    """phi on the s4 lattice (4 ghost layers): +-1 regions from random balls,
    with a diffuse band unless `sharp`."""
    nx, ny, nz = n
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(nz + 8) - 3, np.arange(ny + 8) - 3, np.arange(nx + 8) - 3, indexing="ij")
    d = np.full(x.shape, 1e9)
    for _ in range(4):
        c = rng.uniform(0, [nx, ny, nz])
        r = rng.uniform(2, 0.4 * min(n))
        d = np.minimum(d, np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) - r)
    if sharp:
        return np.where(d < 0, 1.0, -1.0)
    phi = np.tanh(-d)
    phi[d < -2.5] = 1.0      # exactly +-1 away from the band
    phi[d > 2.5] = -1.0
    return phi


@pytest.mark.parametrize("n", [(20, 20, 28), (21, 19, 23), (16, 17, 9), (32, 24, 12)])
@pytest.mark.parametrize("sharp", [False, True], ids=["diffuse", "sharp"])
def test_skipped_nodes_have_uniform_stencils(n, sharp):
    nx, ny, nz = n
    phi4 = random_phase(n, seed=nx * 1000 + ny * 10 + nz, sharp=sharp)
    codes = brick_codes(phi4)
    assert codes.shape == ((nz + 9) // 2, (ny + 9) // 2, (nx + 9) // 2)
    act = active_blocks(codes, n)
    seen = np.zeros((nz + 4, ny + 4, nx + 4), dtype=np.int32)   # nodes -1 .. n+2
    skipped_nonzero = 0
    for cz in range(act.shape[0]):
        for cy in range(act.shape[1]):
            for cx in range(act.shape[2]):
                for e in range(8):
                    i, j, k = 2 * cx - 2 + (e & 1), 2 * cy - 2 + ((e >> 1) & 1), 2 * cz - 2 + (e >> 2)
                    if not (-1 <= i <= nx + 2 and -1 <= j <= ny + 2 and -1 <= k <= nz + 2):
                        continue
                    seen[k + 1, j + 1, i + 1] += 1
                    # the block's bricks cover the node's stencil
                    for q in range(19):
                        si, sj, sk = i + EX[q] + 3, j + EY[q] + 3, k + EZ[q] + 3    # s4-local
                        assert cx <= si // 2 <= cx + 1 and cy <= sj // 2 <= cy + 1 and cz <= sk // 2 <= cz + 1
                    if not act[cz, cy, cx]:
                        c = phi4[k + 3, j + 3, i + 3]
                        vals = [phi4[k + 3 + EZ[q], j + 3 + EY[q], i + 3 + EX[q]] for q in range(19)]
                        skipped_nonzero += any(v != c for v in vals)
    assert np.all(seen == 1), "every node of [-1, n+2]^3 in exactly one block"
    assert skipped_nonzero == 0
    # the fields are not trivial: both kinds of blocks occur
    assert act.any() and not act.all()


# ---------------------------------------------------------------------------
# Super-blocks (gradient.cuh: phi_brick_kernel, sb_active_kernel,
# sb_live_kernel): 4 x 4 x 4 phi bricks.  A super-block's fluid code is 1 (2)
# when every fluid node in it holds +1 (-1), 3 when it has no fluid node, 0
# otherwise; it is flagged when its code is 0 or it holds fluid of one sign
# next to a super-block with fluid of the other.  A pass processes the
# super-blocks within one super-block of those flagged by the previous pass.
#
# Restated here: between two passes the phi of a fluid node may change only
# where the node or one of its fluid D3Q19 neighbours holds another value
# (populations arrive from fluid neighbours or bounce back); a solid node's
# phi only where it is extrapolated from fluid nodes that changed (within two
# nodes); ghost nodes of walled faces never.  Then every changed node, every
# brick whose code can change and every node block whose activity can change
# lies in a processed super-block, while static non-uniform phi in solid and
# ghost nodes flags nothing.
# ---------------------------------------------------------------------------
def brick_fluid_codes(phi4, fluid4):
    """Per 2x2x2 brick: 1 / 2 when its fluid nodes are all +1 / -1, 3 without
    fluid nodes, 0 otherwise (phi_brick_code)."""
    NZ, NY, NX = phi4.shape
    BZ, BY, BX = (NZ + 1) // 2, (NY + 1) // 2, (NX + 1) // 2
    pv = np.zeros((2 * BZ, 2 * BY, 2 * BX))
    pf = np.zeros((2 * BZ, 2 * BY, 2 * BX), dtype=bool)
    pv[:NZ, :NY, :NX] = phi4
    pf[:NZ, :NY, :NX] = fluid4
    v = pv.reshape(BZ, 2, BY, 2, BX, 2)
    f = pf.reshape(BZ, 2, BY, 2, BX, 2)
    anyf = f.any(axis=(1, 3, 5))
    plus = np.all(~f | (v == 1.0), axis=(1, 3, 5))
    minus = np.all(~f | (v == -1.0), axis=(1, 3, 5))
    return np.where(~anyf, 3, np.where(plus, 1, np.where(minus, 2, 0))).astype(np.int8)


def super_codes(fcodes):
    BZ, BY, BX = fcodes.shape
    SZ, SY, SX = (BZ + 3) // 4, (BY + 3) // 4, (BX + 3) // 4
    pad = np.full((4 * SZ, 4 * SY, 4 * SX), 3, dtype=np.int8)   # bricks past the grid: no fluid
    pad[:BZ, :BY, :BX] = fcodes
    b = pad.reshape(SZ, 4, SY, 4, SX, 4)
    any0, any1, any2 = ((b == c).any(axis=(1, 3, 5)) for c in (0, 1, 2))
    return np.where(any0 | (any1 & any2), 0, np.where(any1, 1, np.where(any2, 2, 3))).astype(np.int8)


def neighbourhood(mask):
    """OR of mask over the 3 x 3 x 3 super-blocks around each (no wrap)."""
    out = mask.copy()
    SZ, SY, SX = mask.shape
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                src = mask[max(0, -dz):SZ - max(0, dz), max(0, -dy):SY - max(0, dy), max(0, -dx):SX - max(0, dx)]
                out[max(0, dz):SZ - max(0, -dz), max(0, dy):SY - max(0, -dy), max(0, dx):SX - max(0, -dx)] |= src
    return out


def flagged(sc):
    both = neighbourhood(sc == 1) & neighbourhood(sc == 2)
    return (sc == 0) | ((sc != 3) & both)


def shifted(a, q):
    """a at x + e_q, edge values repeated past the array (no wrap)."""
    p = np.pad(a, 1, mode="edge")
    return p[1 + EZ[q]:1 + EZ[q] + a.shape[0], 1 + EY[q]:1 + EY[q] + a.shape[1], 1 + EX[q]:1 + EX[q] + a.shape[2]]


def near(mask, hops):
    out = mask.copy()
    for _ in range(hops):
        m = out.copy()
        for q in range(1, 19):
            m |= shifted(out, q)
        out = m
    return out


def porous_fluid(n, seed):
    """Fluid nodes of [1, n]^3 on the s4 lattice, solid balls removed."""
    nx, ny, nz = n
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(nz + 8) - 3, np.arange(ny + 8) - 3, np.arange(nx + 8) - 3, indexing="ij")
    inside = (x >= 1) & (x <= nx) & (y >= 1) & (y <= ny) & (z >= 1) & (z <= nz)
    solid = np.zeros(x.shape, dtype=bool)
    for _ in range(6):
        c = rng.uniform(0, [nx, ny, nz])
        solid |= (x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 < rng.uniform(2, 6) ** 2
    return inside & ~solid


@pytest.mark.parametrize("n", [(40, 40, 56), (33, 29, 47), (64, 48, 40)])
@pytest.mark.parametrize("sharp", [False, True], ids=["diffuse", "sharp"])
def test_super_blocks_cover_every_change(n, sharp):
    nx, ny, nz = n
    rng = np.random.default_rng(nx)
    fluid = porous_fluid(n, seed=3 * nx + ny)
    phi = random_phase(n, seed=7 * nx + nz, sharp=sharp)
    # solid nodes: values extrapolated from fluid (arbitrary here); ghost
    # layers of walled faces: 0
    solid = ~fluid
    inside = np.zeros_like(fluid)
    inside[4:4 + nz, 4:4 + ny, 4:4 + nx] = True
    phi[solid & inside] = rng.uniform(-1, 1, size=int((solid & inside).sum()))
    phi[~inside] = 0.0

    # fluid nodes that may change: the node or a fluid neighbour holds another value
    may = fluid & ~np.isin(phi, (1.0, -1.0))
    for q in range(1, 19):
        may |= fluid & shifted(fluid, q) & (shifted(phi, q) != phi)
    new = phi.copy()
    pick = may & (rng.random(phi.shape) < 0.5)
    new[pick] = rng.uniform(-1, 1, size=int(pick.sum()))
    # solid nodes extrapolating from changed fluid nodes
    ext = solid & inside & near(new != phi, 2) & (rng.random(phi.shape) < 0.5)
    new[ext] = rng.uniform(-1, 1, size=int(ext.sum()))

    sc = super_codes(brick_fluid_codes(phi, fluid))
    flag = flagged(sc)
    live = neighbourhood(flag)
    # changed fluid nodes lie in flagged super-blocks or one node from one
    NZ, NY, NX = phi.shape
    fnode = np.repeat(np.repeat(np.repeat(flag, 8, 0), 8, 1), 8, 2)[:NZ, :NY, :NX]
    for k, j, i in np.argwhere((new != phi) & fluid & ~near(fnode, 1)):
        raise AssertionError(("fluid node", k, j, i))
    # every changed node, brick code and block activity in a processed super-block
    for k, j, i in np.argwhere(new != phi):
        assert live[(k // 2) // 4, (j // 2) // 4, (i // 2) // 4], ("node", k, j, i)
    codes_old, codes_new = brick_codes(phi), brick_codes(new)
    changed = np.argwhere(codes_old != codes_new)
    for bz, by, bx in changed:
        assert live[bz // 4, by // 4, bx // 4], ("brick", bz, by, bx)
    act_old, act_new = active_blocks(codes_old, n), active_blocks(codes_new, n)
    for cz, cy, cx in np.argwhere(act_old != act_new):
        assert live[cz // 4, cy // 4, cx // 4], ("block", cz, cy, cx)
    assert len(changed) > 0
    # the static non-uniform solid and ghost phi does not keep every
    # super-block live (it would, counted over all nodes)
    all_nodes = super_codes(np.where(codes_old == 0, 0, codes_old))
    assert neighbourhood(flagged(all_nodes)).sum() > live.sum()
