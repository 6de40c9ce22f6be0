"""Learned warm start: the 3-D U-Net of the library (``mflbm_unet_*``) and the
glue between it and the lattice.

The network maps a pore geometry (solid mask and signed distance to the
nearest solid, both per lattice node) to a normalised flow field (u, v, w, p).
A warm start evaluates it, turns the prediction into physical fields and
fills the populations with their equilibrium (``mflbm_init_flow_mrt``: the
equilibrium fill of the reference's initialization_new_multi_pdf,
src/Init_multiphase.cpp:389-496, with the energy-square moment on the MRT
collision's own equilibrium); the plain lattice Boltzmann run then converges
from there.  Normalisation: velocities are stored as u nu / g and
pressure as (rho - <rho>) / (3 g), each divided by its training-set scale, so
that a single network serves any body force g and viscosity nu of the Stokes
regime.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import abi, lib
from .abi import ptr

N_IN, N_OUT = 2, 4

# D3Q19 directions (includes/Module.h:98-101 of the reference)
EX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
EY = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
EZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])


class UNet:
    """One network on the current device, sized for D x H x W inputs."""

    def __init__(self, D, H, W, seed=0):
        self.lib = lib.load()
        self.shape = (int(D), int(H), int(W))
        h = C.c_void_p()
        lib.check(self.lib.mflbm_unet_create(int(D), int(H), int(W), int(seed), C.byref(h)), "mflbm_unet_create")
        self.h = h
        n = C.c_longlong()
        lib.check(self.lib.mflbm_unet_param_count(self.h, C.byref(n)), "mflbm_unet_param_count")
        self.n_params = int(n.value)

    def close(self):
        if self.h:
            self.lib.mflbm_unet_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check_x(self, x, k):
        x = np.ascontiguousarray(x, dtype=np.float32)
        if x.shape != self.shape + (k,):
            raise ValueError(f"expected shape {self.shape + (k,)}, got {x.shape}")
        return x

    def forward(self, x):
        x = self._check_x(x, N_IN)
        y = np.empty(self.shape + (N_OUT,), np.float32)
        lib.check(self.lib.mflbm_unet_forward(self.h, ptr(x), ptr(y)), "mflbm_unet_forward")
        return y

    def train_step(self, x, target, mask, lr):
        x = self._check_x(x, N_IN)
        t = self._check_x(target, N_OUT)
        m = np.ascontiguousarray(mask, dtype=np.float32)
        loss = C.c_float()
        lib.check(self.lib.mflbm_unet_train_step(self.h, ptr(x), ptr(t), ptr(m), C.c_float(lr), C.byref(loss)),
                  "mflbm_unet_train_step")
        return float(loss.value)

    def gradients(self, x, target, mask):
        x = self._check_x(x, N_IN)
        t = self._check_x(target, N_OUT)
        m = np.ascontiguousarray(mask, dtype=np.float32)
        g = np.empty(self.n_params, np.float32)
        loss = C.c_float()
        lib.check(self.lib.mflbm_unet_gradients(self.h, ptr(x), ptr(t), ptr(m), ptr(g), C.byref(loss)),
                  "mflbm_unet_gradients")
        return float(loss.value), g

    def get_params(self):
        p = np.empty(self.n_params, np.float32)
        lib.check(self.lib.mflbm_unet_get_params(self.h, ptr(p)), "mflbm_unet_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {p.size}")
        lib.check(self.lib.mflbm_unet_set_params(self.h, ptr(p)), "mflbm_unet_set_params")


def conv_check(x, w, b, gy=None, relu=False):
    """One convolution layer and its gradients through mflbm_unet_conv_check:
    returns y (FP32 before rounding) and, with gy, (gx, gw, gb)."""
    D, H, W, cin = x.shape
    cout = w.shape[0]
    f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32)
    x, w, b, gy = f(x), f(w), f(b), f(gy)
    y = np.empty((D, H, W, cout), np.float32)
    gx = np.empty_like(x) if gy is not None else None
    gw = np.empty_like(w) if gy is not None else None
    gb = np.empty(cout, np.float32) if gy is not None else None
    lib.check(lib.load().mflbm_unet_conv_check(D, H, W, cin, cout, ptr(x), ptr(w), ptr(b), int(relu), ptr(gy),
                                               ptr(y), ptr(gx), ptr(gw), ptr(gb)), "mflbm_unet_conv_check")
    return (y, gx, gw, gb) if gy is not None else y


# ---------------------------------------------------------------------------
# geometry -> network inputs
# ---------------------------------------------------------------------------
def features(walls_global, shape, periodic=(False, True, True), sdf_scale=0.125):
    """Inputs of the network for a wall array (the s0 layout of
    ``lib.set_walls``: nz x ny x nx, non-zero = solid), computed on the
    device by ``mflbm_unet_features``: channel 0 the solid mask, channel 1
    the signed Euclidean distance to the nearest voxel of the other kind
    (positive in the fluid), times sdf_scale.  periodic: per axis (x, y, z)
    whether distances wrap around (minimum image)."""
    nx, ny, nz = shape
    w = np.ascontiguousarray(np.asarray(walls_global).reshape(nz, ny, nx), dtype=np.int32)
    x = np.empty((nz, ny, nx, N_IN), np.float32)
    bits = int(bool(periodic[0])) | int(bool(periodic[1])) << 1 | int(bool(periodic[2])) << 2
    lib.check(lib.load().mflbm_unet_features(ptr(w), nx, ny, nz, bits, C.c_float(sdf_scale), ptr(x)),
              "mflbm_unet_features")
    return x


# ---------------------------------------------------------------------------
# lattice <-> flow fields
# ---------------------------------------------------------------------------
def macro_fields(ctx):
    """rho and velocity (j / rho, j the first moment of both components) on
    the interior nodes, arrays [nz, ny, nx]."""
    L = ctx.L
    nx, ny, nz = L.nx, L.ny, L.nz
    pdf = ctx.download(("pdf",))["pdf"].reshape(2, 19, nz + 2, ny + 2, nx + 2)
    f = (pdf[0] + pdf[1])[:, 1:nz + 1, 1:ny + 1, 1:nx + 1].astype(np.float64)
    rho = f.sum(0)
    jx = np.tensordot(EX, f, 1)
    jy = np.tensordot(EY, f, 1)
    jz = np.tensordot(EZ, f, 1)
    r = np.where(rho > 0, rho, 1.0)
    return rho, jx / r, jy / r, jz / r


def flow_target(ctx, walls_global, nu, g):
    """Physical flow of a converged single-phase lattice as the network's raw
    targets (u nu / g, v nu / g, w nu / g, (rho - <rho>) / (3 g)) and the fluid
    mask; zero in solids."""
    L = ctx.L
    rho, u, v, w = macro_fields(ctx)
    fluid = (np.asarray(walls_global).reshape(L.nz, L.ny, L.nx) == 0)
    t = np.zeros(rho.shape + (N_OUT,), np.float32)
    s = nu / g
    t[..., 0] = u * s
    t[..., 1] = v * s
    t[..., 2] = w * s
    t[..., 3] = (rho - rho[fluid].mean()) / (3.0 * g)
    t[~fluid] = 0
    return t, fluid.astype(np.float32)


def fill_from_prediction(ctx, y, walls_global, nu, g, scales, mrt=True):
    """Equilibrium populations from a normalised prediction y [nz, ny, nx, 4]:
    velocity zero in solids, halos periodic along the context's periodic
    axes, formed on the device (mflbm_init_flow_predicted).  mrt: the
    collision's own equilibrium (as mflbm_init_flow_mrt), else the
    reference's a17 formula with the lattice weights (as mflbm_init_flow).
    walls_global is not needed (the context holds the walls); it is kept
    for the callers' symmetry with features()."""
    ctx.init_flow_predicted(y, nu, g, scales, mrt=mrt)


def predicted_permeability(y, scales, nx, ny, nz, walls_global):
    """k of the predicted field: the sum of u_z nu / g over the fluid voxels
    (walls_global == 0; the network's outputs at solid voxels are not
    trained and the fill sets them to rest) divided by (nx - 2) ny nz."""
    fluid = np.asarray(walls_global).reshape(nz, ny, nx) == 0
    return float(y[..., 2].astype(np.float64)[fluid].sum() * scales[2] / ((nx - 2) * ny * nz))


# ---------------------------------------------------------------------------
# training
# ---------------------------------------------------------------------------
def augment(x, t, m, flip_x, flip_y):
    """Mirror images of a sample (walls in x and periodic y are symmetric
    under x and y reflections; the flow direction z is kept)."""
    if flip_x:
        x, t, m = x[:, :, ::-1], t[:, :, ::-1].copy(), m[:, :, ::-1]
        t[..., 0] *= -1
    if flip_y:
        x, t, m = x[:, ::-1], t[:, ::-1].copy(), m[:, ::-1]
        t[..., 1] *= -1
    return np.ascontiguousarray(x), np.ascontiguousarray(t), np.ascontiguousarray(m)


def train(net, data, epochs, lr=2e-3, lr_end=1e-4, seed=0, log=None):
    """Adam over the samples (x, t_normalised, mask) for `epochs` passes with
    random mirror images and a cosine learning-rate decay.  Returns the mean
    loss of each epoch and the seconds spent."""
    rng = np.random.default_rng(seed)
    steps = epochs * len(data)
    losses = []
    t0 = time.perf_counter()
    it = 0
    for e in range(epochs):
        tot = 0.0
        for i in rng.permutation(len(data)):
            x, t, m = augment(*data[i], bool(rng.integers(2)), bool(rng.integers(2)))
            a = lr_end + 0.5 * (lr - lr_end) * (1 + np.cos(np.pi * it / max(steps - 1, 1)))
            tot += net.train_step(x, t, m, a)
            it += 1
        losses.append(tot / len(data))
        if log:
            log(f"epoch {e}: loss {losses[-1]:.4g}")
    return losses, time.perf_counter() - t0


def save(path, params, scales, meta=None):
    np.savez(path, params=params, scales=np.asarray(scales, np.float32), **(meta or {}))


def load_model(path):
    z = np.load(path)
    return z["params"], z["scales"]


def main():
    """Timing of the network on random inputs:
    python -m mflbm.unet --size 64 --steps 5"""
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=64)
    ap.add_argument("--steps", type=int, default=5)
    a = ap.parse_args()
    n = a.size
    rng = np.random.default_rng(0)
    net = UNet(n, n, n, seed=1)
    x = np.zeros((n, n, n, N_IN), np.float32)
    x[..., 0] = rng.random((n, n, n)) < 0.4
    x[..., 1] = rng.normal(size=(n, n, n))
    t = rng.normal(size=(n, n, n, N_OUT)).astype(np.float32)
    m = np.ones((n, n, n), np.float32)
    net.train_step(x, t, m, 1e-3)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        net.train_step(x, t, m, 1e-3)
    train_ms = 1e3 * (time.perf_counter() - t0) / a.steps
    t0 = time.perf_counter()
    for _ in range(a.steps):
        net.forward(x)
    fwd_ms = 1e3 * (time.perf_counter() - t0) / a.steps
    net.close()
    print(json.dumps({"size": n, "params": net.n_params, "train_step_ms": train_ms, "forward_ms": fwd_ms}))


if __name__ == "__main__":
    main()
