"""ctypes mirror of include/mflbm.h (structures, enums, array layouts)."""
from __future__ import annotations

import ctypes as C

import numpy as np

MFLBM_OK = 0
MFLBM_FP32, MFLBM_FP64 = 1, 2
MFLBM_FAST, MFLBM_STRICT = 0, 1
MFLBM_STORE_NATIVE, MFLBM_STORE_F16, MFLBM_STORE_BF16 = 0, 1, 2


class Params(C.Structure):
    _fields_ = [
        ("nx", C.c_longlong), ("ny", C.c_longlong), ("nz", C.c_longlong),
        ("precision", C.c_int), ("fp_mode", C.c_int),
        ("jper", C.c_int), ("kper", C.c_int),
        ("domain_wall_status_z_min", C.c_int), ("domain_wall_status_z_max", C.c_int),
        ("inlet_BC", C.c_int), ("outlet_BC", C.c_int),
        ("porous_plate_cmd", C.c_int), ("Z_porous_plate", C.c_int),
        ("lbm_gamma", C.c_double), ("force_z", C.c_double),
        ("la_nui1", C.c_double), ("la_nui2", C.c_double),
        ("lbm_beta", C.c_double), ("phi_inlet", C.c_double),
        ("sa_inject", C.c_double), ("uin_avg", C.c_double),
        ("relaxation", C.c_double), ("cos_theta", C.c_double),
        ("rho_in", C.c_double), ("rho_out", C.c_double),
        ("storage", C.c_int), ("reserved", C.c_int),
    ]


class Control(C.Structure):
    _fields_ = [
        ("nxGlobal", C.c_longlong), ("nyGlobal", C.c_longlong), ("nzGlobal", C.c_longlong),
        ("iper", C.c_int), ("jper", C.c_int), ("kper", C.c_int),
        ("domain_wall_status_x_min", C.c_int), ("domain_wall_status_x_max", C.c_int),
        ("domain_wall_status_y_min", C.c_int), ("domain_wall_status_y_max", C.c_int),
        ("domain_wall_status_z_min", C.c_int), ("domain_wall_status_z_max", C.c_int),
        ("inlet_BC", C.c_int), ("outlet_BC", C.c_int),
        ("porous_plate_cmd", C.c_int), ("Z_porous_plate", C.c_int),
        ("initial_fluid_distribution_option", C.c_int),
        ("rho_out_BC", C.c_int),
        ("fluid1_viscosity", C.c_double), ("fluid2_viscosity", C.c_double),
        ("surface_tension", C.c_double), ("theta", C.c_double), ("RK_beta", C.c_double),
        ("capillary_number", C.c_double), ("saturation_injection", C.c_double),
        ("initial_interface_position", C.c_double), ("body_force_0", C.c_double),
    ]


class Derived(C.Structure):
    _fields_ = [("A_xy", C.c_double), ("uin_avg_0", C.c_double),
                ("flowrate", C.c_double), ("interface_z0", C.c_double)]


class GeometryCounts(C.Structure):
    _fields_ = [("num_solid_boundary_global", C.c_longlong),
                ("num_fluid_boundary_global", C.c_longlong),
                ("num_solid_boundary", C.c_longlong),
                ("num_fluid_boundary", C.c_longlong),
                ("pore_sum", C.c_longlong)]


class Monitor(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "vol1_sum", "vol2_sum", "mass1_sum", "mass2_sum", "saturation",
        "flux1_sum", "flux2_sum", "total_mass", "umax", "vol1_full", "vol2_full")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class MonitorExt(C.Structure):
    _fields_ = [("umax2", C.c_double), ("usq1", C.c_double), ("usq2", C.c_double), ("pre_w", C.c_double),
                ("pre_nw", C.c_double), ("n_w", C.c_longlong), ("n_nw", C.c_longlong),
                ("breakthrough", C.c_longlong), ("dphi_max", C.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [("collide_block", C.c_int), ("normals_block", C.c_int), ("curvature_block", C.c_int),
                ("extrapolate_block", C.c_int), ("step_ms_before", C.c_double), ("step_ms_after", C.c_double),
                ("tile_x", C.c_int), ("tile_y", C.c_int), ("tile_z", C.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


MFLBM_BATCH_AUTO, MFLBM_BATCH_GRAPH, MFLBM_BATCH_PERSISTENT = 0, 1, 2
MFLBM_E_TIMEOUT = -6


class BatchOptions(C.Structure):
    _fields_ = [("mode", C.c_int), ("block", C.c_int), ("wait_limit_s", C.c_double), ("used_mode", C.c_int),
                ("grid", C.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


# rows of the per-slice monitor sums (mflbm_monitor_profile)
PROFILE_ROWS = ["fl1", "fl2", "vol1", "vol2", "mass1", "mass2", "pre"]


def struct_dict(s):
    return {n: getattr(s, n) for n, _ in s._fields_}


class Layout:
    """Sizes of the reference's padded arrays (includes/Idx_gpu.cuh:54-70)."""

    def __init__(self, nx, ny, nz):
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)

    @property
    def s0(self):
        return self.nx * self.ny * self.nz

    @property
    def s1(self):
        return (self.nx + 2) * (self.ny + 2) * (self.nz + 2)

    @property
    def s2(self):
        return (self.nx + 4) * (self.ny + 4) * (self.nz + 4)

    @property
    def s4(self):
        return (self.nx + 8) * (self.ny + 8) * (self.nz + 8)

    @property
    def f1(self):
        return self.s1 * 38

    @property
    def cnv(self):
        return (self.nx + 2) * (self.ny + 2) * 19

    @property
    def plane1(self):
        return (self.nx + 2) * (self.ny + 2)

    def shape(self, kind):
        nx, ny, nz = self.nx, self.ny, self.nz
        g = {"s0": 0, "s1": 1, "s2": 2, "s4": 4}
        if kind in g:
            h = g[kind]
            return (nz + 2 * h, ny + 2 * h, nx + 2 * h)
        if kind == "f1":
            return (2, 19, nz + 2, ny + 2, nx + 2)
        if kind == "cnv":
            return (19, ny + 2, nx + 2)
        if kind == "plane1":
            return (ny + 2, nx + 2)
        raise KeyError(kind)

    def empty(self, kind, dtype):
        return np.zeros(self.shape(kind), dtype=dtype)


# name -> layout kind of every reference array the hot path reads or writes
FIELD_KINDS = {
    "pdf": "f1", "phi": "s4", "cn_x": "s2", "cn_y": "s2", "cn_z": "s2", "c_norm": "s2",
    "curv": "s1", "W_in": "plane1", "f_convec_bc": "cnv", "g_convec_bc": "cnv",
    "phi_convec_bc": "plane1", "walls": "s2", "walls_type": "s4", "s_nx": "s4", "s_ny": "s4",
    "s_nz": "s4", "walls_global": "s0", "rho": "s1", "u": "s1", "v": "s1", "w": "s1",
}
INT_FIELDS = {"walls", "walls_type", "walls_global"}


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)
