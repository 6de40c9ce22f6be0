"""ctypes binding of libmflbm.so (the C ABI of include/mflbm.h).

The library is the only compute path: if it is missing or cannot be loaded,
``load()`` raises; there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import abi
from .abi import Layout, ptr

PKG = Path(__file__).resolve().parent.parent
DEFAULT_LIB = PKG / "lib" / "libmflbm.so"

VP, I, LL, D = C.c_void_p, C.c_int, C.c_longlong, C.c_double

# name -> (restype, argtypes); every entry point of include/mflbm.h
SIGNATURES = {
    "mflbm_abi_version": (I, []),
    "mflbm_last_error": (C.c_char_p, []),
    "mflbm_kernel_launch_count": (C.c_ulonglong, []),
    "mflbm_params_from_control": (I, [VP, I, I, VP, VP]),
    "mflbm_set_walls": (I, [VP, VP, VP]),
    "mflbm_inlet_profile": (I, [VP, I, VP]),
    "mflbm_create": (I, [VP, C.POINTER(VP)]),
    "mflbm_destroy": (I, [VP]),
    "mflbm_set_params": (I, [VP, VP]),
    "mflbm_get_params": (I, [VP, VP]),
    "mflbm_preprocess_geometry": (I, [VP, VP, VP, VP, VP, VP, VP, VP]),
    "mflbm_upload_geometry": (I, [VP, VP, VP, VP, VP, VP]),
    "mflbm_init_fields": (I, [VP, I, D, VP]),
    "mflbm_upload_fields": (I, [VP] * 12),
    "mflbm_download_fields": (I, [VP] * 11),
    "mflbm_step": (I, [VP, I]),
    "mflbm_run": (I, [VP, I, I]),
    "mflbm_synchronize": (I, [VP]),
    "mflbm_interface_stats": (I, [VP, VP, VP, VP]),
    "mflbm_super_block_stats": (I, [VP, VP, VP, VP]),
    "mflbm_monitor_reduce": (I, [VP, I, I, VP]),
    "mflbm_monitor_reduce_noalloc": (I, [VP, I, I, VP]),
    "mflbm_monitor_profile": (I, [VP, VP, VP, I]),
    "mflbm_autotune": (I, [VP, I, VP]),
    "mflbm_set_tuning": (I, [VP, VP]),
    "mflbm_get_tuning": (I, [VP, VP]),
    "mflbm_batch_create": (I, [C.POINTER(VP), I, C.POINTER(VP)]),
    "mflbm_batch_run": (I, [VP, I, I]),
    "mflbm_batch_destroy": (I, [VP]),
    "mflbm_batch_set_options": (I, [VP, VP]),
    "mflbm_batch_get_options": (I, [VP, VP]),
    "mflbm_batch_autotune": (I, [VP, I, VP]),
    "mflbm_write_vtk": (I, [VP, I, I, C.c_char_p]),
    "mflbm_write_walls_vtk": (I, [VP, C.c_char_p]),
    "mflbm_write_checkpoint": (I, [VP, I, C.c_char_p]),
    "mflbm_read_checkpoint": (I, [VP, C.c_char_p, VP, C.POINTER(I)]),
    "mflbm_init_flow": (I, [VP, VP, VP, VP, VP]),
    "mflbm_init_flow_mrt": (I, [VP, VP, VP, VP, VP]),
    "mflbm_init_flow_predicted": (I, [VP, VP, C.c_double, C.c_double, VP, I]),
    "mflbm_unet_create": (I, [I, I, I, C.c_ulonglong, C.POINTER(VP)]),
    "mflbm_unet_destroy": (I, [VP]),
    "mflbm_unet_param_count": (I, [VP, C.POINTER(LL)]),
    "mflbm_unet_forward": (I, [VP, VP, VP]),
    "mflbm_unet_train_step": (I, [VP, VP, VP, VP, C.c_float, C.POINTER(C.c_float)]),
    "mflbm_unet_gradients": (I, [VP, VP, VP, VP, VP, C.POINTER(C.c_float)]),
    "mflbm_unet_get_params": (I, [VP, VP]),
    "mflbm_unet_set_params": (I, [VP, VP]),
    "mflbm_unet_conv_check": (I, [I, I, I, I, I, VP, VP, VP, I, VP, VP, VP, VP, VP]),
    "mflbm_unet_set_wait_limit": (I, [C.c_uint]),
    "mflbm_unet_features": (I, [VP, I, I, I, I, C.c_float, VP]),
    "mflbm_node_counts": (I, [VP, C.POINTER(LL)]),
    "mflbm_stream": (VP, [VP]),
    "mflbm_set_kernel_timing": (I, [VP, I]),
    "mflbm_kernel_times": (I, [VP, C.POINTER(D), C.POINTER(D), C.POINTER(I), C.POINTER(I)]),
}

_LIB = None


class MflbmError(RuntimeError):
    pass


def lib_path() -> Path:
    return Path(os.environ.get("MFLBM_LIB", str(DEFAULT_LIB)))


def load(path=None):
    """Load libmflbm.so (raises if it is absent: there is no fallback path)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else lib_path()
    if not p.exists():
        raise MflbmError(f"{p} not found: build it with mf-lbm-cuda_gb300/build.py (there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def check(rc, what=""):
    if rc < 0:
        msg = load().mflbm_last_error().decode(errors="replace")
        raise MflbmError(f"{what}: error {rc}: {msg}")
    return rc


def params_from_control(control, precision, fp_mode):
    p, d = abi.Params(), abi.Derived()
    check(load().mflbm_params_from_control(C.byref(control), precision, fp_mode, C.byref(p), C.byref(d)),
          "mflbm_params_from_control")
    return p, d


def set_walls(control, geometry):
    L = Layout(control.nxGlobal, control.nyGlobal, control.nzGlobal)
    wg = L.empty("s0", np.int32)
    g = None if geometry is None else np.ascontiguousarray(geometry, dtype=np.uint8)
    check(load().mflbm_set_walls(C.byref(control), ptr(g), ptr(wg)), "mflbm_set_walls")
    return wg


def inlet_profile(control, precision):
    L = Layout(control.nxGlobal, control.nyGlobal, control.nzGlobal)
    w = L.empty("plane1", np.float32 if precision == abi.MFLBM_FP32 else np.float64)
    check(load().mflbm_inlet_profile(C.byref(control), precision, ptr(w)), "mflbm_inlet_profile")
    return w


class Context:
    """One lattice on the current CUDA device."""

    def __init__(self, params: abi.Params):
        self.lib = load()
        self.params = params
        self.L = Layout(params.nx, params.ny, params.nz)
        self.T = np.float32 if params.precision == abi.MFLBM_FP32 else np.float64
        h = VP()
        check(self.lib.mflbm_create(C.byref(params), C.byref(h)), "mflbm_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.mflbm_destroy(self.h)
            self.h = VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def preprocess_geometry(self, walls_global, want_host=True):
        L = self.L
        out = {}
        if want_host:
            out = {"walls": L.empty("s2", np.int32), "walls_type": L.empty("s4", np.int32),
                   "s_nx": L.empty("s4", self.T), "s_ny": L.empty("s4", self.T), "s_nz": L.empty("s4", self.T)}
        cnt = abi.GeometryCounts()
        check(self.lib.mflbm_preprocess_geometry(self.h, ptr(np.ascontiguousarray(walls_global, np.int32)),
                                                 ptr(out.get("walls")), ptr(out.get("walls_type")),
                                                 ptr(out.get("s_nx")), ptr(out.get("s_ny")), ptr(out.get("s_nz")),
                                                 C.byref(cnt)), "mflbm_preprocess_geometry")
        out["counts"] = abi.struct_dict(cnt)
        return out

    def upload_geometry(self, walls, walls_type, s_nx, s_ny, s_nz):
        check(self.lib.mflbm_upload_geometry(self.h, ptr(walls), ptr(walls_type), ptr(s_nx), ptr(s_ny), ptr(s_nz)),
              "mflbm_upload_geometry")

    def init_fields(self, option, interface_z0, W_in=None):
        check(self.lib.mflbm_init_fields(self.h, int(option), float(interface_z0), ptr(W_in)), "mflbm_init_fields")

    def upload_fields(self, **a):
        names = ["pdf", "phi", "cn_x", "cn_y", "cn_z", "c_norm", "curv", "W_in", "f_convec_bc", "g_convec_bc",
                 "phi_convec_bc"]
        check(self.lib.mflbm_upload_fields(self.h, *[ptr(a.get(n)) for n in names]), "mflbm_upload_fields")

    def download(self, names=("pdf", "phi", "cn_x", "cn_y", "cn_z", "c_norm", "curv", "f_convec_bc",
                              "g_convec_bc", "phi_convec_bc"), out=None):
        """mflbm_download_fields into new arrays, or into the caller's arrays
        `out` (name -> C-contiguous array of the field's size and the context's
        dtype, e.g. pinned host buffers)."""
        order = ["pdf", "phi", "cn_x", "cn_y", "cn_z", "c_norm", "curv", "f_convec_bc", "g_convec_bc",
                 "phi_convec_bc"]
        if out is None:
            out = {n: self.L.empty(abi.FIELD_KINDS[n], self.T) for n in names}
        else:
            out = {n: out[n] for n in names}
            for n, a in out.items():
                want = int(np.prod(self.L.shape(abi.FIELD_KINDS[n])))
                if a.dtype != self.T or a.size != want or not a.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"download: out[{n!r}] must be a C-contiguous {np.dtype(self.T).name} "
                                     f"array of {want} values")
        check(self.lib.mflbm_download_fields(self.h, *[ptr(out.get(n)) for n in order]), "mflbm_download_fields")
        return out

    def init_flow(self, rho=None, u=None, v=None, w=None, mrt=False):
        """mflbm_init_flow (mrt: mflbm_init_flow_mrt): equilibrium populations
        from macroscopic fields (arrays of shape (nz+2, ny+2, nx+2) or flat,
        any of them None)."""
        a = [None if f is None else np.ascontiguousarray(f, dtype=self.T).ravel() for f in (rho, u, v, w)]
        n = (self.params.nx + 2) * (self.params.ny + 2) * (self.params.nz + 2)
        for f in a:
            if f is not None and f.size != n:
                raise ValueError(f"init_flow: expected {n} values per field, got {f.size}")
        fn = self.lib.mflbm_init_flow_mrt if mrt else self.lib.mflbm_init_flow
        check(fn(self.h, *[ptr(f) for f in a]), "mflbm_init_flow")

    def init_flow_predicted(self, y, nu, g, scales, mrt=True):
        """mflbm_init_flow_predicted: the equilibrium fill from a normalised
        prediction y [nz, ny, nx, 4] (float32), formed on the device."""
        L = self.L
        y = np.ascontiguousarray(y, dtype=np.float32)
        if y.shape != (L.nz, L.ny, L.nx, 4):
            raise ValueError(f"init_flow_predicted: expected shape {(L.nz, L.ny, L.nx, 4)}, got {y.shape}")
        sc = np.ascontiguousarray(scales, dtype=np.float32)
        check(self.lib.mflbm_init_flow_predicted(self.h, ptr(y), float(nu), float(g), ptr(sc), int(bool(mrt))),
              "mflbm_init_flow_predicted")

    def step(self, ntime):
        check(self.lib.mflbm_step(self.h, int(ntime)), "mflbm_step")

    def run(self, ntime_begin, nsteps):
        check(self.lib.mflbm_run(self.h, int(ntime_begin), int(nsteps)), "mflbm_run")

    def sync(self):
        check(self.lib.mflbm_synchronize(self.h), "mflbm_synchronize")

    def interface_stats(self):
        """mflbm_interface_stats: sizes of the last gradient pass's sparse sets."""
        v = [C.c_longlong(0) for _ in range(3)]
        check(self.lib.mflbm_interface_stats(self.h, *[C.byref(x) for x in v]), "mflbm_interface_stats")
        return {"interface_nodes": v[0].value, "solid_normals": v[1].value, "active_nodes": v[2].value}

    def super_block_stats(self):
        """mflbm_super_block_stats: super-blocks the last gradient pass processed
        and flagged, and their total."""
        v = [C.c_longlong(0) for _ in range(3)]
        check(self.lib.mflbm_super_block_stats(self.h, *[C.byref(x) for x in v]), "mflbm_super_block_stats")
        return {"processed": v[0].value, "flagged": v[1].value, "total": v[2].value}

    def monitor(self, n_exclude_inlet, n_exclude_outlet):
        m = abi.Monitor()
        check(self.lib.mflbm_monitor_reduce(self.h, int(n_exclude_inlet), int(n_exclude_outlet), C.byref(m)),
              "mflbm_monitor_reduce")
        return m.as_dict()

    def monitor_noalloc(self, n_exclude_inlet, n_exclude_outlet):
        """mflbm_monitor_reduce_noalloc: the same reductions with their
        partials in the library's static device array (no allocation)."""
        m = abi.Monitor()
        check(self.lib.mflbm_monitor_reduce_noalloc(self.h, int(n_exclude_inlet), int(n_exclude_outlet),
                                                    C.byref(m)), "mflbm_monitor_reduce_noalloc")
        return m.as_dict()

    def monitor_profile(self, track_phi=False):
        """Per-slice sums {row: array(nz)} (rows of abi.PROFILE_ROWS) and the
        extra monitor scalars (mflbm_monitor_profile)."""
        nz = self.L.nz
        sl = np.zeros((len(abi.PROFILE_ROWS), nz), dtype=np.float64)
        e = abi.MonitorExt()
        check(self.lib.mflbm_monitor_profile(self.h, ptr(sl), C.byref(e), int(bool(track_phi))),
              "mflbm_monitor_profile")
        return {n: sl[m] for m, n in enumerate(abi.PROFILE_ROWS)}, e.as_dict()

    def autotune(self, reps=5):
        """mflbm_autotune: population tile shape and block sizes of the step
        kernels; the state is unchanged."""
        t = abi.Tuning()
        check(self.lib.mflbm_autotune(self.h, int(reps), C.byref(t)), "mflbm_autotune")
        return t.as_dict()

    def set_tuning(self, collide=0, normals=0, curvature=0, extrapolate=0, tile=(0, 0, 0)):
        """mflbm_set_tuning: block sizes (0 keeps one) and, when `tile` is
        given, the population tile extent in bricks (x, y, z)."""
        t = abi.Tuning(collide, normals, curvature, extrapolate, 0.0, 0.0, *tile)
        check(self.lib.mflbm_set_tuning(self.h, C.byref(t)), "mflbm_set_tuning")

    def get_tuning(self):
        t = abi.Tuning()
        check(self.lib.mflbm_get_tuning(self.h, C.byref(t)), "mflbm_get_tuning")
        return t.as_dict()

    def write_vtk(self, vtk_type, path, precision_cmd=0):
        check(self.lib.mflbm_write_vtk(self.h, int(vtk_type), int(precision_cmd), str(path).encode()), "mflbm_write_vtk")

    def write_walls_vtk(self, path):
        check(self.lib.mflbm_write_walls_vtk(self.h, str(path).encode()), "mflbm_write_walls_vtk")

    def write_checkpoint(self, ntime, path):
        check(self.lib.mflbm_write_checkpoint(self.h, int(ntime), str(path).encode()), "mflbm_write_checkpoint")

    def read_checkpoint(self, path, W_in=None):
        """Returns the reference's ntime0 (stored step - 1)."""
        nt = I()
        check(self.lib.mflbm_read_checkpoint(self.h, str(path).encode(), ptr(W_in), C.byref(nt)),
              "mflbm_read_checkpoint")
        return nt.value

    def node_counts(self):
        c = (LL * 2)()
        check(self.lib.mflbm_node_counts(self.h, c), "mflbm_node_counts")
        return int(c[0]), int(c[1])

    def stream(self):
        return self.lib.mflbm_stream(self.h)

    def set_timing(self, enable):
        check(self.lib.mflbm_set_kernel_timing(self.h, int(bool(enable))), "mflbm_set_kernel_timing")

    def kernel_times(self):
        tc, tg, nc, ng = D(), D(), I(), I()
        check(self.lib.mflbm_kernel_times(self.h, C.byref(tc), C.byref(tg), C.byref(nc), C.byref(ng)),
              "mflbm_kernel_times")
        return tc.value, tg.value, nc.value


class Batch:
    """mflbm_batch: contexts advanced together, as one persistent launch
    (single-phase samples) or one CUDA graph launch per step pair."""

    def __init__(self, contexts):
        self.lib = load()
        self.contexts = list(contexts)           # kept alive while the batch exists
        arr = (VP * len(self.contexts))(*[c.h for c in self.contexts])
        h = VP()
        check(self.lib.mflbm_batch_create(arr, len(self.contexts), C.byref(h)), "mflbm_batch_create")
        self.h = h

    def run(self, ntime_begin, nsteps):
        check(self.lib.mflbm_batch_run(self.h, int(ntime_begin), int(nsteps)), "mflbm_batch_run")

    def options(self):
        o = abi.BatchOptions()
        check(self.lib.mflbm_batch_get_options(self.h, C.byref(o)), "mflbm_batch_get_options")
        return o.as_dict()

    def set_options(self, mode=None, block=None, wait_limit_s=None):
        o = abi.BatchOptions()
        check(self.lib.mflbm_batch_get_options(self.h, C.byref(o)), "mflbm_batch_get_options")
        if mode is not None:
            o.mode = mode
        if block is not None:
            o.block = block
        if wait_limit_s is not None:
            o.wait_limit_s = wait_limit_s
        check(self.lib.mflbm_batch_set_options(self.h, C.byref(o)), "mflbm_batch_set_options")

    def autotune(self, reps=3):
        """mflbm_batch_autotune: block size of the persistent launch and the
        population tile shape of every sample; states unchanged."""
        t = abi.Tuning()
        check(self.lib.mflbm_batch_autotune(self.h, int(reps), C.byref(t)), "mflbm_batch_autotune")
        return t.as_dict()

    def close(self):
        if self.h:
            self.lib.mflbm_batch_destroy(self.h)
            self.h = VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def setup_case(case, precision=abi.MFLBM_FP32, fp_mode=abi.MFLBM_FAST, geometry=None, want_host_geometry=False,
               storage=abi.MFLBM_STORE_NATIVE):
    """Build a ready-to-step Context for `case`: walls, device geometry
    preprocessing, start-up fields and colour gradient (the reference's
    start-up, src/main.cpp:71-99).  `storage` selects the population storage
    (abi.MFLBM_STORE_*).  Returns (context, info)."""
    control = case.control(precision)
    params, derived = params_from_control(control, precision, fp_mode)
    params.storage = storage
    geo = case.geometry_bytes() if geometry is None else geometry
    wg = set_walls(control, geo)
    W_in = inlet_profile(control, precision)
    ctx = Context(params)
    g = ctx.preprocess_geometry(wg, want_host=want_host_geometry)
    ctx.init_fields(control.initial_fluid_distribution_option, derived.interface_z0, W_in)
    info = {"params": params, "derived": derived, "control": control, "geometry": g, "W_in": W_in,
            "walls_global": wg}
    return ctx, info
