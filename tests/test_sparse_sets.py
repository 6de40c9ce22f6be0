"""Index arithmetic of the sparse colour-gradient passes
(mf-lbm-cuda_gb300/csrc/gradient.cuh: phi_mask_kernel, active_nodes_kernel,
sb_active_kernel, sb_live_kernel), restated in numpy.

The normal pass skips every node whose ISO4 stencil (the node and its 18
D3Q19 neighbours) is all exactly +1 or all exactly -1: there every
difference of the ISO4 sums is +0 and the normal record is the zero record.
The node listing decides this bit-parallel from per-row masks of the s4
lattice (8 nodes per byte); these tests check, on random phase fields with
sharp and diffuse interfaces and on odd and even extents, that the bitwise
rule lists exactly the candidate nodes with a non-uniform stencil, and (the
super-blocks) that every node, row mask and listing decision that can change
between two passes lies in a super-block the pass processes.  The 2x2x2
brick codes restated first are the super-blocks' fluid codes.
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


NEAR = 3 * 2.0 ** -22   # kNearOne of gradient.cuh


def near_value(phi, val):
    return (phi >= val - NEAR) & (phi <= val + NEAR)


def row_masks(phi4, SX):
    """pmask of phi_mask_kernel: per row (z, y) and byte b, bit x & 7 where phi
    is within NEAR of +1 (P) and of -1 (M); x = 8b + bit, zero past the row end."""
    NZ, NY, NX = phi4.shape
    pad = np.zeros((NZ, NY, 8 * SX))
    pad[:, :, :NX] = phi4
    valid = np.zeros(8 * SX, bool)
    valid[:NX] = True
    bits = (1 << np.arange(8)).astype(np.uint32)
    P = (near_value(pad, 1.0) & valid).reshape(NZ, NY, SX, 8) @ bits
    M = (near_value(pad, -1.0) & valid).reshape(NZ, NY, SX, 8) @ bits
    return P.astype(np.uint32), M.astype(np.uint32)


def listed_rows(P, M, C):
    """active_nodes_kernel's bitwise rule: candidates (C) whose 19-node stencil
    is not all +1 and not all -1, per row byte (rows 1 .. N-2 only)."""
    NZ, NY, SX = P.shape

    def window(A):   # bytes b-1, b, b+1 at bits 0, 8, 16
        lo = np.zeros_like(A)
        hi = np.zeros_like(A)
        lo[:, :, 1:] = A[:, :, :-1]
        hi[:, :, :-1] = A[:, :, 1:]
        return lo | (A << 8) | (hi << 16)

    out = np.zeros_like(P)
    zs, ys = slice(1, NZ - 1), slice(1, NY - 1)
    for A, acc in ((P, "up"), (M, "um")):
        w = window(A)
        u = np.full((NZ - 2, NY - 2, SX), 0xFFFFFFFF, np.uint32)
        for dz, dy in ((0, 0), (0, -1), (0, 1), (-1, 0), (1, 0)):
            ww = w[1 + dz:NZ - 1 + dz, 1 + dy:NY - 1 + dy]
            u &= (ww >> 7) & (ww >> 8) & (ww >> 9)
        for dz, dy in ((-1, -1), (-1, 1), (1, -1), (1, 1)):
            u &= A[1 + dz:NZ - 1 + dz, 1 + dy:NY - 1 + dy]
        if acc == "up":
            up = u
        else:
            um = u
    out[zs, ys] = C[zs, ys] & ~(up | um) & 0xFF
    return out


def iso4_norm(F, dt, fma):
    """|grad phi| of normal_at in the arithmetic of iso4_d* (operation order of
    gradient.cuh) for stencils F[..., 3, 3, 3] (z, y, x) in dtype dt; with fma,
    a * (face) + b * (edges) is one fused multiply-add (the fast flavour)."""
    F = F.astype(dt)
    a, b = dt(1) / dt(6), dt(1) / dt(12)

    def at(dx, dy, dz):
        return F[..., 1 + dz, 1 + dy, 1 + dx]

    def comb(face, edges):
        s = edges[0]
        for k, e in enumerate(edges[1:]):
            s = (s - e) if k % 2 == 0 else (s + e)   # e1 - e2 + e3 - e4 + ...
        if fma:   # round(a * face + (b * s)) with one rounding of the sum
            return (a.astype(np.float64) * face.astype(np.float64) + (b * s).astype(np.float64)).astype(dt)
        return a * face + b * s

    x = comb(at(1, 0, 0) - at(-1, 0, 0), [at(1, 1, 0), at(-1, -1, 0), at(1, -1, 0), at(-1, 1, 0),
                                          at(1, 0, 1), at(-1, 0, -1), at(1, 0, -1), at(-1, 0, 1)])
    y = comb(at(0, 1, 0) - at(0, -1, 0), [at(1, 1, 0), at(-1, -1, 0), at(-1, 1, 0), at(1, -1, 0),
                                          at(0, 1, 1), at(0, -1, -1), at(0, 1, -1), at(0, -1, 1)])
    z = comb(at(0, 0, 1) - at(0, 0, -1), [at(1, 0, 1), at(-1, 0, -1), at(-1, 0, 1), at(1, 0, -1),
                                          at(0, 1, 1), at(0, -1, -1), at(0, -1, 1), at(0, 1, -1)])
    return np.sqrt(x * x + y * y + z * z)


@pytest.mark.parametrize("dt", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("fma", [False, True], ids=["strict", "fast"])
def test_near_one_stencils_have_gradient_below_the_cut_off(dt, fma):
    """The bound behind the listing's tolerance: every stencil within NEAR of
    +1 (or -1) gives |grad phi| < 1e-6, the normal pass's zero-record cut-off,
    in the arithmetic the kernels use.  Worst cases: deviations of +-NEAR with
    the sign of each neighbour's projection on the extreme direction
    (1, 2/3, 1/3) and its permutations and reflections, and random
    deviations; the values as stored (NEAR and the nearest representable
    values inside it)."""
    rng = np.random.default_rng(3)
    E = np.array([(x, y, z) for z in (-1, 0, 1) for y in (-1, 0, 1) for x in (-1, 0, 1)], float).reshape(3, 3, 3, 3)
    dirs = []
    for perm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        for sg in np.array(np.meshgrid([1, -1], [1, -1], [1, -1])).T.reshape(-1, 3):
            v = np.array([1, 2 / 3, 1 / 3])[list(perm)] * sg
            dirs.append(v)
    dirs = np.array(dirs)
    d = dt(NEAR)
    worst = []
    for val in (1.0, -1.0):
        one = dt(val)
        lo, hi = one - d, one + d
        for v in dirs:
            proj = E @ v
            worst.append(np.where(proj > 0, hi, np.where(proj < 0, lo, one)))
    worst = np.array(worst, dt)
    rand = rng.uniform(-1, 1, size=(20000, 3, 3, 3)) * NEAR
    rand = np.concatenate([1 + rand, -1 + rand]).astype(dt)
    rand = np.clip(rand, np.where(rand > 0, dt(1) - d, dt(-1) - d), np.where(rand > 0, dt(1) + d, dt(-1) + d))
    for F in (worst, rand):
        nrm = iso4_norm(F, dt, fma)
        assert nrm.max() < 1e-6, nrm.max()
    # the bound is close to tight: the worst case reaches 1.2472 NEAR
    assert iso4_norm(worst, dt, fma).max() > 1.2 * NEAR


@pytest.mark.parametrize("n", [(20, 20, 28), (21, 19, 23), (16, 17, 9), (33, 24, 12)])
@pytest.mark.parametrize("sharp", [False, True], ids=["diffuse", "sharp"])
def test_row_masks_list_exactly_the_non_uniform_stencils(n, sharp):
    nx, ny, nz = n
    phi4 = random_phase(n, seed=nx * 1000 + ny * 10 + nz, sharp=sharp)
    rng = np.random.default_rng(nx + ny)
    # values a few ulps off +-1 in part of the bulk (within and beyond NEAR)
    bulk = np.isin(phi4, (1.0, -1.0)) & (rng.random(phi4.shape) < 0.3)
    phi4 = np.where(bulk, phi4 * (1 - rng.choice([1e-7, -5e-7, 7e-7, 9e-7, 2e-6], size=phi4.shape)), phi4)
    SX = ((nx + 9) // 2 + 3) // 4
    assert 8 * SX >= nx + 8
    # candidates: a random subset of [-1, n+2]^3 (walls_type <= 0), s4 x 2 .. n+5
    cand = np.zeros(phi4.shape, bool)
    cand[2:nz + 6, 2:ny + 6, 2:nx + 6] = rng.random((nz + 4, ny + 4, nx + 4)) < 0.8
    padc = np.zeros(phi4.shape[:2] + (8 * SX,), bool)
    padc[:, :, :nx + 8] = cand
    C = (padc.reshape(nz + 8, ny + 8, SX, 8) @ (1 << np.arange(8))).astype(np.uint32)
    P, M = row_masks(phi4, SX)
    L = listed_rows(P, M, C)
    listed = ((L[..., None] >> np.arange(8)) & 1).astype(bool).reshape(nz + 8, ny + 8, 8 * SX)[:, :, :nx + 8]
    # the direct rule
    uni = np.zeros(phi4.shape, bool)
    core = (slice(1, nz + 7), slice(1, ny + 7), slice(1, nx + 7))
    for val in (1.0, -1.0):
        u = np.ones((nz + 6, ny + 6, nx + 6), bool)
        for q in range(19):
            u &= near_value(phi4[1 + EZ[q]:nz + 7 + EZ[q], 1 + EY[q]:ny + 7 + EY[q], 1 + EX[q]:nx + 7 + EX[q]], val)
        uni[core] |= u
    assert np.array_equal(listed, cand & ~uni)
    assert listed.any() and (cand & uni).any()


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
    # listing decisions of the node pass (row masks, every node a candidate)
    SX = ((nx + 9) // 2 + 3) // 4
    C = np.full((nz + 8, ny + 8, SX), 0xFF, np.uint32)
    L_old = listed_rows(*row_masks(phi, SX), C)
    L_new = listed_rows(*row_masks(new, SX), C)
    for z, y, b in np.argwhere(L_old != L_new):
        assert live[(z // 2) // 4, (y // 2) // 4, b], ("listing", z, y, b)
    assert len(changed) > 0
    # the static non-uniform solid and ghost phi does not keep every
    # super-block live (it would, counted over all nodes)
    all_nodes = super_codes(np.where(codes_old == 0, 0, codes_old))
    assert neighbourhood(flagged(all_nodes)).sum() > live.sum()
