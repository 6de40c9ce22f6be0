"""Seeded synthetic porous media in the MF-LBM geometry ``.dat`` format.

The reference solver reads its solid/fluid voxel map from a binary file
(``src/Misc.cpp:139-192``, ``read_walls``): three ``int32`` dimensions
(``geometry_dims_type_size 4``) followed by one byte per voxel, 1 = solid,
0 = fluid.  The byte of voxel ``(i, j, k)`` (1-based) sits at
``(i-1) + ny*((j-1) + nx*(k-1))`` (``src/Misc.cpp:171``); the x and y strides
are swapped, which is only unambiguous when ``nx == ny``.  Every generator
here therefore produces ``nx == ny`` samples and the writer refuses others.

The reference ships no generator; these packs stand in for the micro-CT
images its inputs name.  Arrays are indexed ``[k, j, i]`` (z, y, x; x
fastest), matching the order of the file body when ``nx == ny``.
"""
from __future__ import annotations

import numpy as np

__all__ = ["sphere_pack", "write_dat", "read_dat", "porosity", "SplitMix64"]


class SplitMix64:
    """SplitMix64 generator: a fixed, platform-independent stream, so a seed
    produces the same pack under every numpy version and on every host."""

    MASK = (1 << 64) - 1

    def __init__(self, seed):
        self.s = int(seed) & self.MASK

    def next_u64(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & self.MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))


def _paint(solid, c, r, periodic_y):
    """Set every voxel within distance ``r`` of centre ``c`` (z, y, x) solid.

    Returns the number of voxels that changed from fluid to solid."""
    nz, ny, nx = solid.shape
    cz, cy, cx = c
    rr = int(np.ceil(r))
    z0, z1 = max(int(np.floor(cz)) - rr, 0), min(int(np.floor(cz)) + rr + 2, nz)
    x0, x1 = max(int(np.floor(cx)) - rr, 0), min(int(np.floor(cx)) + rr + 2, nx)
    if z0 >= z1 or x0 >= x1:
        return 0
    zz = np.arange(z0, z1)[:, None, None]
    xx = np.arange(x0, x1)[None, None, :]
    if periodic_y:
        ys = np.arange(int(np.floor(cy)) - rr, int(np.floor(cy)) + rr + 2)
        dy = ys - cy
        yidx = ys % ny
    else:
        y0, y1 = max(int(np.floor(cy)) - rr, 0), min(int(np.floor(cy)) + rr + 2, ny)
        if y0 >= y1:
            return 0
        yidx = np.arange(y0, y1)
        dy = yidx - cy
    inside = (zz - cz) ** 2 + dy[None, :, None] ** 2 + (xx - cx) ** 2 <= r * r
    sub = solid[z0:z1][:, yidx][:, :, x0:x1]
    new = inside & ~sub
    n_new = int(new.sum())
    if n_new:
        sub |= inside
        block = solid[z0:z1]
        block[:, yidx, x0:x1] = sub
    return n_new


def sphere_pack(shape, radius, porosity_target, *, seed, overlap=True,
                buffer_layers=2, periodic_y=False, max_attempts=200_000, tolerance=0.01,
                interpenetration=0.0):
    """Random sphere pack with a target porosity.

    shape            (nx, ny, nz) lattice size, flow along z, nx == ny.
    radius           a number (fixed radius) or a (rmin, rmax) pair drawn
                     uniformly per sphere.
    porosity_target  spheres are added until the porosity of the core region
                     (z outside the inlet/outlet buffers) drops to this value.
    overlap          False rejects a sphere whose centre is closer than the
                     sum of radii to an earlier one (non-overlapping pack);
                     centres may then lie up to one radius outside the x/y
                     faces, so cut spheres fill the gaps next to the walls.
    interpenetration with overlap=False, centres must be at least
                     r1 + r2 - interpenetration apart.
    buffer_layers    empty (fluid) slabs kept at the inlet and the outlet.
    periodic_y       spheres wrap around the y faces.
    max_attempts     a non-overlapping pack that jams before the target is
                     accepted when within `tolerance` of it.

    Returns a uint8 array [nz, ny, nx] with 1 = solid.
    """
    nx, ny, nz = (int(s) for s in shape)
    if nx != ny:
        raise ValueError("MF-LBM geometry files are only unambiguous for nx == ny")
    rng = SplitMix64(seed)
    solid = np.zeros((nz, ny, nx), dtype=bool)
    zc0, zc1 = buffer_layers, nz - buffer_layers
    core = solid[zc0:zc1]
    n_core = core.size
    n_solid = 0
    target_solid = (1.0 - porosity_target) * n_core
    centres, radii = [], []
    attempts = 0
    while n_solid < target_solid:
        attempts += 1
        if attempts > max_attempts:
            reached = 1 - n_solid / n_core
            if reached - porosity_target <= tolerance:
                break
            raise RuntimeError(f"pack did not reach porosity {porosity_target} (reached {reached:.4f})")
        r = float(radius) if np.isscalar(radius) else rng.uniform(radius[0], radius[1])
        ext = 0.0 if overlap else r
        c = (rng.uniform(0, zc1 - zc0), rng.uniform(0, ny) if periodic_y else rng.uniform(-ext, ny + ext),
             rng.uniform(-ext, nx + ext))
        if not overlap and centres:
            d = np.asarray(centres) - np.asarray(c)
            if periodic_y:
                d[:, 1] -= ny * np.round(d[:, 1] / ny)
            if np.any((d ** 2).sum(axis=1) < (np.asarray(radii) + r - interpenetration) ** 2):
                continue
        n_solid += _paint(core, c, r, periodic_y)
        centres.append(c)
        radii.append(r)
    return solid.astype(np.uint8)


def porosity(solid, buffer_layers=0):
    core = solid[buffer_layers:solid.shape[0] - buffer_layers]
    return 1.0 - float(core.sum()) / core.size


def write_dat(path, solid):
    """Write a [nz, ny, nx] 0/1 array in the reference ``.dat`` layout."""
    nz, ny, nx = solid.shape
    if nx != ny:
        raise ValueError("MF-LBM geometry files are only unambiguous for nx == ny")
    with open(path, "wb") as f:
        f.write(np.asarray([nx, ny, nz], dtype="<i4").tobytes())
        f.write(np.ascontiguousarray(solid, dtype=np.uint8).tobytes())


def read_dat(path, dims_type_size=4):
    """Read a reference ``.dat`` file into a [nz, ny, nx] uint8 array."""
    with open(path, "rb") as f:
        hdr = np.frombuffer(f.read(3 * dims_type_size), dtype="<i4" if dims_type_size == 4 else "<i8")
        nx, ny, nz = (int(v) for v in hdr)
        body = np.frombuffer(f.read(nx * ny * nz), dtype=np.uint8)
    if body.size != nx * ny * nz:
        raise ValueError(f"{path}: truncated geometry body")
    if nx != ny:
        raise ValueError("MF-LBM geometry files are only unambiguous for nx == ny")
    return body.reshape(nz, ny, nx).copy()
