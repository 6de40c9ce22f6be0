"""Simulation cases: control-file keys, the benchmark workloads, input folders.

A case is a ``simulation_control.txt`` key set (every key the reference's
``read_parameter_multi`` requires, ``src/IO_multiphase.cpp:47-187``) plus a
seeded synthetic geometry.  ``write_case_dir`` lays a case out exactly as the
reference expects its working directory (``input/simulation_control.txt``,
``input/job_status.txt``, ``input/Geometry_File_Path.txt``, the ``.dat``).

Flow is along z (the reference's only open axis); x is always walled.  The
workload names say what they are: ``drainage_<nx>x<ny>x<nz>``.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .geometry import sphere_pack, write_dat

# Every key read_parameter_multi requires, with a neutral default.
DEFAULT_KEYS = {
    "initial_fluid_distribution_option": 1,
    "breakthrough_check": 0,
    "steady_state_option": 0,
    "convergence_criteria": "1e-4",
    "benchmark_cmd": 1,
    "output_fieldData_precision_cmd": 0,
    "extreme_large_sim_cmd": 0,
    "modify_geometry_cmd": 0,
    "external_geometry_read_cmd": 1,
    "geometry_dims_type_size": 4,
    "geometry_preprocess_cmd": 0,
    "porous_plate_cmd": 0,
    "change_inlet_fluid_phase_cmd": 0,
    "nxGlobal": 32, "nyGlobal": 32, "nzGlobal": 32,
    "n_exclude_inlet": 2, "n_exclude_outlet": 2,
    "domain_wall_status_x_min": 1, "domain_wall_status_x_max": 1,
    "domain_wall_status_y_min": 1, "domain_wall_status_y_max": 1,
    "domain_wall_status_z_min": 0, "domain_wall_status_z_max": 0,
    "iper": 0, "jper": 0, "kper": 0,
    "fluid1_viscosity": "0.16666666666666666", "fluid2_viscosity": "0.16666666666666666",
    "surface_tension": "0.01", "theta": "45", "RK_beta": "0.95",
    "inlet_BC": 1, "outlet_BC": 1,
    "target_inject_pore_volume": "-1.0",
    "capillary_number": "1e-3",
    "saturation_injection": "1.0",
    "initial_interface_position": "2.0",
    "body_force_0": "0.0",
    "target_fluid1_saturation": "0.5",
    "Z_porous_plate": 0,
    "max_time_step": 1000, "max_time_step_benchmark": 100,
    "ntime_visual": 1000000, "ntime_animation": 1000000, "monitor_timer": 1000000,
    "monitor_profile_timer_ratio": 1, "computation_time_timer": 1000000,
    "display_steps_timer": 1000000,
    "checkpoint_save_timer": "1000.0", "checkpoint_2rd_save_timer": "1000.0",
    "simulation_duration_timer": "1000.0",
    "d_vol_animation": "-1.0", "d_vol_detail": "-1.0", "d_vol_monitor": "-1.0",
    "rho_in_new": 0, "rho_out_BC": 0,
    "block_Threads_X": 128, "block_Threads_Y": 1, "block_Threads_Z": 1,
}

_INT_CONTROL = ["nxGlobal", "nyGlobal", "nzGlobal", "iper", "jper", "kper",
                "domain_wall_status_x_min", "domain_wall_status_x_max",
                "domain_wall_status_y_min", "domain_wall_status_y_max",
                "domain_wall_status_z_min", "domain_wall_status_z_max",
                "inlet_BC", "outlet_BC", "porous_plate_cmd", "Z_porous_plate",
                "initial_fluid_distribution_option", "rho_out_BC"]
_FLOAT_CONTROL = ["fluid1_viscosity", "fluid2_viscosity", "surface_tension", "theta", "RK_beta",
                  "capillary_number", "saturation_injection", "initial_interface_position",
                  "body_force_0"]


@dataclass
class Geometry:
    radius: object = 6.0            # number or (rmin, rmax)
    porosity: float = 0.6
    overlap: bool = False
    buffer_layers: int = 2
    seed: int = 0
    empty: bool = False             # True: no spheres (open duct)
    interpenetration: float = 0.0   # non-overlapping packs: allowed centre-distance deficit


@dataclass
class Case:
    name: str
    keys: dict = field(default_factory=dict)
    geometry: Geometry = field(default_factory=Geometry)

    def control_keys(self):
        k = dict(DEFAULT_KEYS)
        k.update(self.keys)
        return k

    @property
    def shape(self):
        k = self.control_keys()
        return int(k["nxGlobal"]), int(k["nyGlobal"]), int(k["nzGlobal"])

    def geometry_bytes(self):
        """The .dat body as a uint8 [nz, ny, nx] array (1 = solid)."""
        nx, ny, nz = self.shape
        g = self.geometry
        if g.empty:
            return np.zeros((nz, ny, nx), np.uint8)
        return sphere_pack((nx, ny, nz), g.radius, g.porosity, seed=g.seed, overlap=g.overlap,
                           buffer_layers=g.buffer_layers, interpenetration=g.interpenetration,
                           periodic_y=bool(int(self.control_keys()["jper"])))

    def control(self, precision):
        """mflbm_control with values parsed as the reference's T_P parser would
        (stof / stod of the decimal string, src/utils.cpp:113,141)."""
        k = self.control_keys()
        c = abi.Control()
        for n in _INT_CONTROL:
            setattr(c, n, int(k[n]))
        for n in _FLOAT_CONTROL:
            s = str(k[n])
            v = float(np.float32(s)) if precision == abi.MFLBM_FP32 else float(s)
            setattr(c, n, v)
        return c

    def control_text(self):
        return "".join(f"{n} {v}\n" for n, v in self.control_keys().items())


def write_case_dir(case: Case, root: str, geometry=None, job_status="new_simulation"):
    """Write the reference's input folder for `case` under `root`."""
    os.makedirs(os.path.join(root, "input", "geometry"), exist_ok=True)
    with open(os.path.join(root, "input", "simulation_control.txt"), "w") as f:
        f.write(case.control_text())
    with open(os.path.join(root, "input", "job_status.txt"), "w") as f:
        f.write(job_status)
    geo_stem = "input/geometry/sample_0"
    with open(os.path.join(root, "input", "Geometry_File_Path.txt"), "w") as f:
        f.write(f"geo_file_path_\t{geo_stem}\n\ngeo_boundary_file_path_\t{geo_stem}\n")
    if geometry is None:
        geometry = case.geometry_bytes()
    write_dat(os.path.join(root, geo_stem + ".dat"), geometry)
    return geometry


# ---------------------------------------------------------------------------
# Workloads.  Viscosity nu = (tau - 1/2)/3; Ca = u_in nu1 / gamma.
# ---------------------------------------------------------------------------
def drainage_48x48x64(seed=1100):
    """Two-phase drainage, 48 x 48 x 64, y periodic, velocity inlet u = 1e-4,
    convective outlet, tau 1.0 / 1.0, gamma 0.01, contact angle 45 deg,
    r = 6 spheres with centres at least 11 lu apart (non-overlapping up to a
    1 lu lens, which lets the pack reach porosity ~0.6 before jamming), with
    2-layer buffers."""
    return Case("drainage_48x48x64", {
        "nxGlobal": 48, "nyGlobal": 48, "nzGlobal": 64,
        "jper": 1, "domain_wall_status_y_min": 0, "domain_wall_status_y_max": 0,
        "inlet_BC": 1, "outlet_BC": 1,
        "fluid1_viscosity": "0.16666666666666666", "fluid2_viscosity": "0.16666666666666666",
        "surface_tension": "0.01", "theta": "45", "RK_beta": "0.95",
        "capillary_number": "1.6666666666666666e-3", "saturation_injection": "1.0",
        "initial_fluid_distribution_option": 1, "initial_interface_position": "2.0",
        "n_exclude_inlet": 2, "n_exclude_outlet": 2,
    }, Geometry(radius=6.0, porosity=0.6, overlap=False, buffer_layers=2, seed=seed, interpenetration=1.0))


def drainage_256x256x256(seed=1200):
    """Two-phase drainage, 256^3, walls on x and y, velocity inlet u = 5e-5,
    convective outlet, tau 0.8 / 0.8, gamma 0.005, contact angle 30 deg,
    overlapping spheres r ~ U[4, 10] at porosity 0.45 with 2-layer buffers."""
    return Case("drainage_256x256x256", {
        "nxGlobal": 256, "nyGlobal": 256, "nzGlobal": 256,
        "inlet_BC": 1, "outlet_BC": 1,
        "fluid1_viscosity": "0.1", "fluid2_viscosity": "0.1",
        "surface_tension": "0.005", "theta": "30", "RK_beta": "0.95",
        "capillary_number": "1e-3", "saturation_injection": "1.0",
        "initial_fluid_distribution_option": 1, "initial_interface_position": "2.0",
        "n_exclude_inlet": 2, "n_exclude_outlet": 2,
    }, Geometry(radius=(4.0, 10.0), porosity=0.45, overlap=True, buffer_layers=2, seed=seed))


def precision_case(n=(384, 384, 512), seed=1300):
    """Two-phase drainage for the precision study, default 384 x 384 x 512:
    walls on x and y, overlapping spheres r ~ U[4, 10] at porosity 0.40 with
    2-layer buffers, nu1 = 1/6, nu2 = 1/60 (tau 1.0 / 0.55), contact angle
    60 deg, gamma 0.01, velocity inlet at Ca = 1e-2 (u_in = 6e-4, chosen so
    that the front advances ~12 lu in 20 000 steps), convective outlet."""
    nx, ny, nz = n
    return Case(f"precision_{nx}x{ny}x{nz}", {
        "nxGlobal": nx, "nyGlobal": ny, "nzGlobal": nz,
        "inlet_BC": 1, "outlet_BC": 1,
        "fluid1_viscosity": "0.16666666666666666", "fluid2_viscosity": "0.016666666666666666",
        "surface_tension": "0.01", "theta": "60", "RK_beta": "0.95",
        "capillary_number": "1e-2", "saturation_injection": "1.0",
        "initial_fluid_distribution_option": 1, "initial_interface_position": "2.0",
        "n_exclude_inlet": 2, "n_exclude_outlet": 2,
    }, Geometry(radius=(4.0, 10.0), porosity=0.40, overlap=True, buffer_layers=2, seed=seed))


def small_case(kind: str, n=(20, 20, 28), seed=7):
    """Small cases covering every boundary kernel, for parity tests."""
    nx, ny, nz = n
    base = {"nxGlobal": nx, "nyGlobal": ny, "nzGlobal": nz}
    geo = Geometry(radius=(2.5, 4.0), porosity=0.6, overlap=True, buffer_layers=3, seed=seed)
    if kind == "velocity_convective":      # drainage, y periodic
        base.update({"jper": 1, "domain_wall_status_y_min": 0, "domain_wall_status_y_max": 0,
                     "inlet_BC": 1, "outlet_BC": 1, "capillary_number": "5e-2", "theta": "40",
                     "initial_interface_position": "5.0"})
    elif kind == "pressure_pressure":      # Zou-He inlet and outlet, imbibition
        base.update({"inlet_BC": 2, "outlet_BC": 2, "body_force_0": "2e-4", "theta": "60",
                     "saturation_injection": "0.0", "initial_fluid_distribution_option": 2,
                     "initial_interface_position": "6.0", "fluid2_viscosity": "0.05"})
    elif kind == "velocity_pressure":      # velocity inlet, Zou-He outlet
        base.update({"inlet_BC": 1, "outlet_BC": 2, "capillary_number": "5e-2",
                     "initial_interface_position": "4.0", "rho_out_BC": 1})
    elif kind == "periodic_drop":          # fully periodic y/z, static drop, body force
        base.update({"jper": 1, "kper": 1, "domain_wall_status_y_min": 0, "domain_wall_status_y_max": 0,
                     "initial_fluid_distribution_option": 5, "initial_interface_position": "5.0",
                     "body_force_0": "1e-5", "surface_tension": "0.02"})
        geo = Geometry(radius=3.0, porosity=0.85, overlap=False, buffer_layers=0, seed=seed)
    elif kind == "closed_contact":         # walls everywhere, sessile drop on the x wall
        base.update({"domain_wall_status_z_min": 1, "domain_wall_status_z_max": 1,
                     "initial_fluid_distribution_option": 3, "initial_interface_position": "7.0",
                     "theta": "70"})
        geo = Geometry(empty=True)
    elif kind == "plate_drainage":         # porous plate blocking fluid 1 near the outlet
        base.update({"inlet_BC": 1, "outlet_BC": 1, "capillary_number": "5e-2",
                     "porous_plate_cmd": 1, "Z_porous_plate": nz - 3,
                     "initial_interface_position": "5.0"})
    else:
        raise KeyError(kind)
    return Case(f"{kind}_{nx}x{ny}x{nz}", base, geo)


def permeability_sample(n, porosity, seed, body_force=1e-6, radius=(3.0, 6.0)):
    """Single-phase permeability sample (the multiphase path with phi = 1
    everywhere): an n^3 grain pack of the given porosity, periodic in y and z,
    walled in x, tau = 1 (nu = 1/6), driven by the body force along z.  The
    reference has no single-phase kernel; phi = 1 (initial interface beyond
    the domain) makes the second component vanish, and a neutral contact
    angle (90 degrees) makes the wetting extrapolation give phi = 1 on the
    solid nodes as well, so the phase gradient, recolouring and surface force
    are zero everywhere (any other angle puts a phase gradient, hence a
    surface force, on every wall-adjacent fluid node)."""
    keys = {"nxGlobal": n, "nyGlobal": n, "nzGlobal": n, "theta": "90",
            "jper": 1, "kper": 1, "domain_wall_status_y_min": 0, "domain_wall_status_y_max": 0,
            "domain_wall_status_z_min": 0, "domain_wall_status_z_max": 0,
            "initial_fluid_distribution_option": 1, "initial_interface_position": str(float(n + 10)),
            "fluid1_viscosity": "0.16666666666666666", "fluid2_viscosity": "0.16666666666666666",
            "body_force_0": repr(float(body_force)), "inlet_BC": 0, "outlet_BC": 0,
            "n_exclude_inlet": 0, "n_exclude_outlet": 0}
    geo = Geometry(radius=radius, porosity=porosity, overlap=True, buffer_layers=0, seed=seed)
    return Case(f"permeability_{n}x{n}x{n}_s{seed}", keys, geo)


SMALL_KINDS = ["velocity_convective", "pressure_pressure", "velocity_pressure",
               "periodic_drop", "closed_contact", "plate_drainage"]
