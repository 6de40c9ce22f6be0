"""Bindings of the CPU oracle (oracle/_build) and of the reference compiled as
host code (oracle/_ref), and helpers that run a case through either.  Test
infrastructure: used by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg only."""
from __future__ import annotations

import ctypes as C
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO / "mf-lbm-cuda_gb300"))
sys.path.insert(0, str(REPO))

from mflbm import abi  # noqa: E402
from mflbm.abi import Layout, ptr  # noqa: E402
from mflbm.cases import write_case_dir  # noqa: E402
from oracle import build as obuild  # noqa: E402

VP = C.c_void_p
FLOAT_FIELDS = ["pdf", "phi", "cn_x", "cn_y", "cn_z", "c_norm", "curv", "W_in",
                "f_convec_bc", "g_convec_bc", "phi_convec_bc", "s_nx", "s_ny", "s_nz"]
STATE_FIELDS = ["pdf", "phi", "cn_x", "cn_y", "cn_z", "c_norm", "curv",
                "f_convec_bc", "g_convec_bc", "phi_convec_bc"]


def force_relevant_pairs(d, ref):
    """(name, device, oracle) float64 arrays of the quantities the collision
    consumes: populations, phase field, the colour gradient c_norm * n and the
    surface-force factor c_norm * curv.  The unit normal alone is not compared
    because its direction is rounding noise where |grad phi| is near the 1e-6
    cut-off (those nodes carry no force)."""
    f = lambda a: a.astype(np.float64)
    out = [("pdf", f(d["pdf"]), f(ref["pdf"])), ("phi", f(d["phi"]), f(ref["phi"]))]
    for c in ("cn_x", "cn_y", "cn_z"):
        out.append((f"c_norm*{c}", f(d["c_norm"]) * f(d[c]), f(ref["c_norm"]) * f(ref[c])))
    interior_s2 = (slice(2, -2),) * 3   # nodes [1, n] of an s2 array
    interior_s1 = (slice(1, -1),) * 3   # nodes [1, n] of an s1 array
    out.append(("c_norm*curv", f(d["c_norm"][interior_s2]) * f(d["curv"][interior_s1]),
                f(ref["c_norm"][interior_s2]) * f(ref["curv"][interior_s1])))
    return out


# D3Q19 lattice vectors in the reference's direction order (includes/Module.h:98-100)
EX = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
EY = [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1]
EZ = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1]


def live_mass(pdf, walls, shape, jper=0, kper=0):
    """Total mass of both components held by the populations after an even
    step (and its boundary update), solid-node slots included, in FP64.

    The reference has no explicit wall bounce-back (src/main_iteration_GPU.cu:
    73-113, 348-384, 414-452): a population that a fluid node pushes towards a
    solid neighbour waits in a slot until the same node reads it back, and
    periodic faces are exchanged by copying slots into ghost layers, which
    leaves stale duplicates behind.  The live populations after an even step
    are therefore exactly
      * those the next odd step pulls: slot q of x - e_q for every fluid node
        x (a solid node's slot, a ghost copy or a fluid node's slot), and
      * those parked for the even step after it: slot q of a fluid node y
        whose neighbour y + e_q (periodic image on a periodic axis) is solid,
        which that node reads back as its bounced-back population.
    Each live population is counted once; in a closed domain (walls, periodic
    axes, no inlet or outlet) their sum is the conserved mass.
    `pdf` and `walls` are the reference-layout arrays (f1 and s2)."""
    nx, ny, nz = shape
    f = pdf.astype(np.float64).reshape(2, 19, nz + 2, ny + 2, nx + 2).sum(axis=0)
    fluid = walls.reshape(nz + 4, ny + 4, nx + 4)[2:-2, 2:-2, 2:-2] == 0   # nodes [1, n]^3
    total = 0.0
    for q in range(19):
        ex, ey, ez = EX[q], EY[q], EZ[q]
        pulled = f[q][1 - ez:nz + 1 - ez, 1 - ey:ny + 1 - ey, 1 - ex:nx + 1 - ex]
        total += float((pulled * fluid).sum())
        tz, ty, tx = np.arange(1, nz + 1) + ez, np.arange(1, ny + 1) + ey, np.arange(1, nx + 1) + ex
        if kper:
            tz = (tz - 1) % nz + 1
        if jper:
            ty = (ty - 1) % ny + 1
        solid_target = np.zeros((nz, ny, nx), bool)
        iz, iy, ix = (np.where((t >= 1) & (t <= m))[0] for t, m in ((tz, nz), (ty, ny), (tx, nx)))
        zz, yy, xx = np.ix_(iz, iy, ix)
        solid_target[zz, yy, xx] = ~fluid[tz[zz] - 1, ty[yy] - 1, tx[xx] - 1]
        total += float((f[q][1:-1, 1:-1, 1:-1] * (fluid & solid_target)).sum())
    return total


def dtype_of(precision):
    return np.float32 if precision == abi.MFLBM_FP32 else np.float64


def suffix(precision):
    return "f32" if precision == abi.MFLBM_FP32 else "f64"


_ORACLE = None


def oracle_lib():
    global _ORACLE
    if _ORACLE is None:
        lib = C.CDLL(str(obuild.build_oracle()))
        for s in ("f32", "f64"):
            getattr(lib, f"orc_geometry_preprocess_{s}").argtypes = [VP] * 8
            getattr(lib, f"orc_params_from_control_{s}").argtypes = [VP, C.c_int, VP, VP]
            getattr(lib, f"orc_inlet_profile_{s}").argtypes = [VP, VP]
            getattr(lib, f"orc_init_fields_{s}").argtypes = [VP, C.c_int, C.c_double] + [VP] * 5
            getattr(lib, f"orc_color_gradient_{s}").argtypes = [VP] * 12
            getattr(lib, f"orc_step_{s}").argtypes = [VP, C.c_int] + [VP] * 16
            getattr(lib, f"orc_run_{s}").argtypes = [VP, C.c_int, C.c_int] + [VP] * 16
            getattr(lib, f"orc_collide_{s}").argtypes = [VP, C.c_int] + [VP] * 8
            getattr(lib, f"orc_macro_vars_{s}").argtypes = [VP] * 13
            getattr(lib, f"orc_monitor_{s}").argtypes = [VP] * 9 + [C.c_int, C.c_int, VP]
            getattr(lib, f"orc_write_vtk_{s}").argtypes = [VP] * 9 + [C.c_int, C.c_int, C.c_char_p]
            getattr(lib, f"orc_write_checkpoint_{s}").argtypes = [VP, C.c_int] + [VP] * 5 + [C.c_char_p]
        lib.orc_write_walls_vtk.argtypes = [C.c_longlong] * 3 + [VP, C.c_char_p]
        lib.orc_set_walls.argtypes = [VP, VP, VP]
        lib.orc_max_threads.restype = C.c_int
        _ORACLE = lib
    return _ORACLE


class OracleState:
    """A complete host state of one case in the reference layouts."""

    def __init__(self, case, precision, fp_mode=abi.MFLBM_STRICT, geometry=None):
        self.case = case
        self.precision = precision
        self.T = dtype_of(precision)
        self.s = suffix(precision)
        self.lib = oracle_lib()
        self.control = case.control(precision)
        nx, ny, nz = case.shape
        self.L = L = Layout(nx, ny, nz)
        self.geometry = case.geometry_bytes() if geometry is None else geometry
        self.a = {}
        for n in FLOAT_FIELDS:
            self.a[n] = L.empty(abi.FIELD_KINDS[n], self.T)
        for n in ("walls", "walls_type", "walls_global"):
            self.a[n] = L.empty(abi.FIELD_KINDS[n], np.int32)
        self.params = abi.Params()
        self.derived = abi.Derived()
        self.counts = abi.GeometryCounts()
        f = lambda name: getattr(self.lib, f"orc_{name}_{self.s}")
        self.lib.orc_set_walls(C.byref(self.control), ptr(np.ascontiguousarray(self.geometry)),
                               ptr(self.a["walls_global"]))
        f("geometry_preprocess")(C.byref(self.control), ptr(self.a["walls_global"]), ptr(self.a["walls"]),
                                 ptr(self.a["walls_type"]), ptr(self.a["s_nx"]), ptr(self.a["s_ny"]),
                                 ptr(self.a["s_nz"]), C.byref(self.counts))
        f("params_from_control")(C.byref(self.control), fp_mode, C.byref(self.params), C.byref(self.derived))
        f("inlet_profile")(C.byref(self.control), ptr(self.a["W_in"]))
        f("init_fields")(C.byref(self.params), self.control.initial_fluid_distribution_option,
                         self.derived.interface_z0, ptr(self.a["pdf"]), ptr(self.a["phi"]),
                         ptr(self.a["f_convec_bc"]), ptr(self.a["g_convec_bc"]), ptr(self.a["phi_convec_bc"]))
        self.color_gradient()
        self.ntime = 1

    def _f(self, name):
        return getattr(self.lib, f"orc_{name}_{self.s}")

    def color_gradient(self):
        a = self.a
        self._f("color_gradient")(C.byref(self.params), ptr(a["walls"]), ptr(a["walls_type"]), ptr(a["s_nx"]),
                                  ptr(a["s_ny"]), ptr(a["s_nz"]), ptr(a["phi"]), ptr(a["cn_x"]), ptr(a["cn_y"]),
                                  ptr(a["cn_z"]), ptr(a["c_norm"]), ptr(a["curv"]))

    def run(self, nsteps):
        a = self.a
        self._f("run")(C.byref(self.params), self.ntime, nsteps, ptr(a["walls"]), ptr(a["walls_type"]),
                       ptr(a["s_nx"]), ptr(a["s_ny"]), ptr(a["s_nz"]), ptr(a["pdf"]), ptr(a["phi"]),
                       ptr(a["cn_x"]), ptr(a["cn_y"]), ptr(a["cn_z"]), ptr(a["c_norm"]), ptr(a["curv"]),
                       ptr(a["W_in"]), ptr(a["f_convec_bc"]), ptr(a["g_convec_bc"]), ptr(a["phi_convec_bc"]))
        self.ntime += nsteps

    def macro(self):
        """compute_macro_vars on a copy (rho, u, v, w and phi with solids zeroed)."""
        a = self.a
        out = {n: self.L.empty("s1", self.T) for n in ("rho", "u", "v", "w")}
        phi = a["phi"].copy()
        self._f("macro_vars")(C.byref(self.params), ptr(a["walls"]), ptr(a["pdf"]), ptr(phi), ptr(a["cn_x"]),
                              ptr(a["cn_y"]), ptr(a["cn_z"]), ptr(a["c_norm"]), ptr(a["curv"]), ptr(out["rho"]),
                              ptr(out["u"]), ptr(out["v"]), ptr(out["w"]))
        out["phi"] = phi
        return out

    def write_outputs(self, folder, ntime):
        """The output files of OUTPUT_FILES for the current state (oracle writers)."""
        a, folder = self.a, Path(folder)
        for name, (vtk_type, cmd) in VTK_FILES.items():
            rc = self._f("write_vtk")(C.byref(self.params), ptr(a["walls"]), ptr(a["pdf"]), ptr(a["phi"]),
                                      ptr(a["cn_x"]), ptr(a["cn_y"]), ptr(a["cn_z"]), ptr(a["c_norm"]),
                                      ptr(a["curv"]), vtk_type, cmd, str(folder / name).encode())
            assert rc == 0, name
        nx, ny, nz = self.case.shape
        assert self.lib.orc_write_walls_vtk(nx, ny, nz, ptr(a["walls"]), str(folder / "walls_bin.vtk").encode()) == 0
        assert self._f("write_checkpoint")(C.byref(self.params), ntime, ptr(a["pdf"]), ptr(a["phi"]),
                                           ptr(a["f_convec_bc"]), ptr(a["g_convec_bc"]), ptr(a["phi_convec_bc"]),
                                           str(folder / "checkpoint").encode()) == 0

    def monitor(self, nex_in=None, nex_out=None):
        k = self.case.control_keys()
        nex_in = int(k["n_exclude_inlet"]) if nex_in is None else nex_in
        nex_out = int(k["n_exclude_outlet"]) if nex_out is None else nex_out
        a = self.a
        m = abi.Monitor()
        self._f("monitor")(C.byref(self.params), ptr(a["walls"]), ptr(a["pdf"]), ptr(a["phi"]), ptr(a["cn_x"]),
                           ptr(a["cn_y"]), ptr(a["cn_z"]), ptr(a["c_norm"]), ptr(a["curv"]), nex_in, nex_out,
                           C.byref(m))
        return m.as_dict()


# Output files compared with the reference's own writers: name -> (vtk_type,
# output_fieldData_precision_cmd), plus walls_bin.vtk and the checkpoint.
VTK_FILES = {"vtk1_cmd0.vtk": (1, 0), "vtk1_cmd1.vtk": (1, 1), "vtk2.vtk": (2, 0), "vtk3_cmd0.vtk": (3, 0),
             "vtk3_cmd1.vtk": (3, 1)}
OUTPUT_FILES = list(VTK_FILES) + ["walls_bin.vtk", "checkpoint"]


def file_digest(path):
    import hashlib
    return hashlib.sha256(Path(path).read_bytes()).hexdigest()


def reference_outputs(lib, workdir, ntime):
    """Run the reference's writers (ref_write_outputs) in `workdir` and return
    {name: sha256} keyed like OUTPUT_FILES."""
    lib.ref_write_outputs.argtypes = [C.c_char_p, C.c_int]
    devnull = os.open(os.devnull, os.O_WRONLY)
    saved = os.dup(1)
    os.dup2(devnull, 1)
    try:
        rc = lib.ref_write_outputs(str(workdir).encode(), ntime)
    finally:
        os.dup2(saved, 1)
        os.close(devnull)
        os.close(saved)
    if rc != 0:
        raise RuntimeError(f"ref_write_outputs failed ({rc})")
    w = Path(workdir)
    ff = w / "results" / "out3.field_data"
    nt = f"{ntime:010d}"
    files = {"vtk1_cmd0.vtk": w / "vtk1_cmd0.tmp", "vtk1_cmd1.vtk": ff / "full_flow_field" / f"full_flow_field_{nt}.vtk",
             "vtk2.vtk": ff / "phase_distribution" / f"small_{nt}.vtk", "vtk3_cmd0.vtk": w / "vtk3_cmd0.tmp",
             "vtk3_cmd1.vtk": ff / "full_flow_field" / f"force_vector_{nt}.vtk", "walls_bin.vtk": ff / "walls_bin.vtk",
             "checkpoint": w / "results" / "out2.checkpoint" / "id0000"}
    return {n: file_digest(f) for n, f in files.items()}


# ---------------------------------------------------------------------------
# The reference compiled as host code.  Its state is global, so each case runs
# in a fresh process (see run_reference_case).
# ---------------------------------------------------------------------------
def ref_lib(precision):
    paths = obuild.build_ref()
    if not paths:
        return None
    lib = C.CDLL(str(paths[suffix(precision)]))
    lib.ref_init.argtypes = [C.c_char_p]
    lib.ref_init.restype = C.c_int
    lib.ref_step.argtypes = [C.c_int]
    lib.ref_ptr.argtypes = [C.c_char_p]
    lib.ref_ptr.restype = VP
    lib.ref_scalar.argtypes = [C.c_char_p]
    lib.ref_scalar.restype = C.c_double
    return lib


def ref_array(lib, L, name, T):
    kind = abi.FIELD_KINDS[name]
    dt = np.int32 if name in abi.INT_FIELDS else T
    n = int(np.prod(L.shape(kind)))
    p = lib.ref_ptr(name.encode())
    if not p:
        return None
    buf = (C.c_char * (n * np.dtype(dt).itemsize)).from_address(p)
    return np.frombuffer(buf, dtype=dt).reshape(L.shape(kind)).copy()


def run_reference_case(case, precision, checkpoints, fields=STATE_FIELDS, workdir=None, geometry=None,
                       outputs=False):
    """Run `case` through oracle/_ref; returns {step: {field: array}} at each
    checkpoint step (0 = after start-up) plus '_scalars', and with `outputs`
    the digests of the reference's output files after the last step
    ('_outputs')."""
    lib = ref_lib(precision)
    if lib is None:
        raise RuntimeError("reference sources unavailable")
    T = dtype_of(precision)
    L = Layout(*case.shape)
    tmp = workdir or tempfile.mkdtemp(prefix="mflbm_ref_")
    write_case_dir(case, tmp, geometry=geometry)
    devnull = os.open(os.devnull, os.O_WRONLY)
    saved = os.dup(1)
    os.dup2(devnull, 1)
    try:
        rc = lib.ref_init(tmp.encode())
    finally:
        os.dup2(saved, 1)
        os.close(devnull)
        os.close(saved)
    if rc != 0:
        raise RuntimeError(f"ref_init failed ({rc})")
    out = {}
    grab = lambda: {n: ref_array(lib, L, n, T) for n in fields}
    scal = ["lbm_gamma", "force_z", "la_nui1", "la_nui2", "lbm_beta", "phi_inlet", "sa_inject", "uin_avg",
            "relaxation", "cos_theta", "rho_in", "rho_out", "num_solid_boundary_global",
            "num_fluid_boundary_global", "num_solid_boundary", "num_fluid_boundary", "pore_sum",
            "interface_z0", "A_xy", "uin_avg_0", "flowrate"]
    out["_scalars"] = {n: lib.ref_scalar(n.encode()) for n in scal}
    out["_geometry"] = {n: ref_array(lib, L, n, T) for n in ("walls", "walls_type", "s_nx", "s_ny", "s_nz", "W_in")}
    if 0 in checkpoints:
        out[0] = grab()
    nt = 1
    for cp in sorted(c for c in checkpoints if c > 0):
        while nt <= cp:
            lib.ref_step(nt)
            nt += 1
        out[cp] = grab()
    if outputs:
        out["_outputs"] = reference_outputs(lib, tmp, max(checkpoints))
    return out
