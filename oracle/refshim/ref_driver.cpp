/*
 * Host driver for the reference compiled as CPU code (oracle/_ref) — test
 * infrastructure only.
 *
 * It restates the launch sequence of main_iteration_kernel_GPU
 * (src/main_iteration_GPU.cu:1890-2056) as loops over the launch grid: each
 * "thread" runs the reference's own kernel function with blockDim = 1 and
 * blockIdx set to the node offset.  Kernels are race-free per launch (every
 * slot / cell is written by one thread and the extrapolations only read
 * nodes they never write), so the 3-D launches are parallelised with OpenMP
 * over (z, y).  Ranges follow the reference's grids except that the
 * normal-direction launch stops at x = n+2: its grid also covers x = n+3,
 * whose writes alias solid x-ghost cells of the next row and, at the very
 * last row, one element past the end of the array.
 *
 * Set-up runs the reference's own initialization_basic_multi /
 * initialization_new_multi / color_gradient in a working directory that holds
 * the reference's input files.
 */
#include <sys/stat.h>
#include <unistd.h>
#include <cstdio>
#include <cstring>
#include <string>

#include "externLib.h"
#include "solver_precision.h"
#include "preprocessor.h"
#include "Module_extern.h"
#include "Fluid_singlephase_extern.h"
#include "Fluid_multiphase_extern.h"
#include "Init_multiphase.h"
#include "Phase_gradient.h"
#include "Monitor.h"
#include "Misc.h"
#include "main_iteration_GPU.h"
#include "IO_multiphase.h"

thread_local shim_index3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0}, blockDim = {1, 1, 1};

extern "C" const char* cudaGetErrorString(cudaError_t) { return "host shim"; }

/* kernels defined in the reference's src/main_iteration_GPU.cu */
void kernel_odd_color_GPU(int, int, int, int, int, int, int*, T_P*, T_P*, T_P*, T_P*, T_P*, T_P*, T_P*);
void kernel_even_color_GPU(int, int, int, int, int, int, int*, T_P*, T_P*, T_P*, T_P*, T_P*, T_P*, T_P*);
void extrapolate_phi_toSolid(int*, T_P*);
void normalDirectionsOfInterfaces(int*, T_P*, T_P*, T_P*, T_P*, T_P*);
void alter_color_gradient_solid_surface_GPU(int*, T_P*, T_P*, T_P*, T_P*, T_P*, T_P*, T_P*);
void extrapolateNormalToSolid(int*, T_P*, T_P*, T_P*, T_P*);
void CSF_Forces(T_P*, T_P*, T_P*, T_P*);
void inlet_bounce_back_velocity_BC_before_odd_GPU(int*, T_P*, T_P*, T_P*);
void inlet_bounce_back_velocity_BC_after_odd_GPU(int*, T_P*, T_P*, T_P*);
void inlet_Zou_He_pressure_BC_before_odd_GPU(T_P, int*, T_P*, T_P*);
void inlet_Zou_He_pressure_BC_after_odd_GPU(T_P, int*, T_P*, T_P*);
void outlet_convective_BC_before_odd_GPU(int*, T_P*, T_P*, T_P*, T_P*, T_P*);
void outlet_convective_BC_after_odd_GPU(int*, T_P*, T_P*, T_P*, T_P*, T_P*);
void outlet_Zou_He_pressure_BC_before_odd_GPU(T_P, int*, T_P*, T_P*);
void outlet_Zou_He_pressure_BC_after_odd_GPU(T_P, int*, T_P*, T_P*);
void perioidc_BC_Z_even(T_P*);
void perioidc_BC_Y_even(T_P*);
void perioidc_BC_ZY_even(T_P*);
void perioidc_BC_Z_odd(T_P*);
void perioidc_BC_Y_odd(T_P*);
void perioidc_BC_ZY_odd(T_P*);
void periodic_phi_Z(int, T_P*);
void periodic_phi_Y(int, T_P*);
void periodic_phi_ZY(int, T_P*);
void porous_plate_BC_before_odd(T_P*);
void porous_plate_BC_after_odd(T_P*);

namespace {

/* Run `f` for blockIdx in [0,bx) x [0,by) x [0,bz) (blockDim = 1). */
template <class F>
void launch3(int bx, int by, int bz, F f) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < bz; ++z)
        for (int y = 0; y < by; ++y) {
            blockDim = {1, 1, 1};
            threadIdx = {0, 0, 0};
            for (int x = 0; x < bx; ++x) {
                blockIdx = {x, y, z};
                f();
            }
        }
}

template <class F>
void launch_serial(int bx, int by, int bz, F f) {
    blockDim = {1, 1, 1};
    threadIdx = {0, 0, 0};
    for (int z = 0; z < bz; ++z)
        for (int y = 0; y < by; ++y)
            for (int x = 0; x < bx; ++x) {
                blockIdx = {x, y, z};
                f();
            }
}

} // namespace

extern "C" void ref_bind(void);

extern "C" {

int ref_precision_bytes(void) { return (int)sizeof(T_P); }

/* Reference start-up (src/main.cpp:71-99) in `workdir`. */
int ref_init(const char* workdir) {
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return -1;
    if (chdir(workdir) != 0) return -2;
    relaxation = prc(1.);
    initialization_basic_multi();
    if (job_status == "new_simulation") initialization_new_multi();
    else initialization_old_multi();
    if (change_inlet_fluid_phase_cmd != 0) change_inlet_fluid_phase();
    ntime = ntime0;
    color_gradient();
    cal_saturation();
    ref_bind();
    copyConstantData();
    if (chdir(cwd) != 0) return -3;
    return 0;
}

/* One time step: main_iteration_kernel_GPU without its host copies. */
void ref_step(int nt) {
    ntime = nt;
    const int nx = (int)nxGlobal, ny = (int)nyGlobal, nz = (int)nzGlobal;
    const bool odd = (nt % 2) != 0;
    if (odd)
        launch3(nx, ny, nz, [&] { kernel_odd_color_GPU(1, nx, 1, ny, 1, nz, walls_d, pdf_d, phi_d, cn_x_d, cn_y_d, cn_z_d, curv_d, c_norm_d); });
    else
        launch3(nx, ny, nz, [&] { kernel_even_color_GPU(1, nx, 1, ny, 1, nz, walls_d, pdf_d, phi_d, cn_x_d, cn_y_d, cn_z_d, curv_d, c_norm_d); });
    if (kper) {
        launch_serial(nx, ny, 1, [&] { odd ? perioidc_BC_Z_odd(pdf_d) : perioidc_BC_Z_even(pdf_d); });
        launch_serial(nx, ny, 1, [&] { periodic_phi_Z(4, phi_d); });
    }
    if (jper) {
        launch_serial(nx, 1, nz, [&] { odd ? perioidc_BC_Y_odd(pdf_d) : perioidc_BC_Y_even(pdf_d); });
        launch_serial(nx, 1, nz, [&] { periodic_phi_Y(4, phi_d); });
    }
    if (jper && kper) {
        launch_serial(nx, 1, 1, [&] { odd ? perioidc_BC_ZY_odd(pdf_d) : perioidc_BC_ZY_even(pdf_d); });
        launch_serial(nx, 1, 1, [&] { periodic_phi_ZY(4, phi_d); });
    }
    if (kper == 0 && domain_wall_status_z_min == 0 && domain_wall_status_z_max == 0) {
        if (inlet_BC == 1)
            launch_serial(nx, ny, 1, [&] { odd ? inlet_bounce_back_velocity_BC_after_odd_GPU(walls_d, phi_d, pdf_d, W_in_d)
                                               : inlet_bounce_back_velocity_BC_before_odd_GPU(walls_d, phi_d, pdf_d, W_in_d); });
        else if (inlet_BC == 2)
            launch_serial(nx, ny, 1, [&] { odd ? inlet_Zou_He_pressure_BC_after_odd_GPU(rho_in, walls_d, phi_d, pdf_d)
                                               : inlet_Zou_He_pressure_BC_before_odd_GPU(rho_in, walls_d, phi_d, pdf_d); });
        if (outlet_BC == 1)
            launch_serial(nx, ny, 1, [&] { odd ? outlet_convective_BC_after_odd_GPU(walls_d, phi_d, phi_convec_bc_d, pdf_d, f_convec_bc_d, g_convec_bc_d)
                                               : outlet_convective_BC_before_odd_GPU(walls_d, phi_d, phi_convec_bc_d, pdf_d, f_convec_bc_d, g_convec_bc_d); });
        else if (outlet_BC == 2)
            launch_serial(nx, ny, 1, [&] { odd ? outlet_Zou_He_pressure_BC_after_odd_GPU(rho_out, walls_d, phi_d, pdf_d)
                                               : outlet_Zou_He_pressure_BC_before_odd_GPU(rho_out, walls_d, phi_d, pdf_d); });
    }
    if (porous_plate_cmd != 0)
        launch_serial(nx, ny, 1, [&] { odd ? porous_plate_BC_after_odd(pdf_d) : porous_plate_BC_before_odd(pdf_d); });
    launch3(nx + 6, ny + 6, nz + 6, [&] { extrapolate_phi_toSolid(walls_type_d, phi_d); });
    launch3(nx + 4, ny + 4, nz + 4, [&] { normalDirectionsOfInterfaces(walls_d, phi_d, cn_x_d, cn_y_d, cn_z_d, c_norm_d); });
    launch3(nx + 4, ny + 4, nz + 4, [&] { alter_color_gradient_solid_surface_GPU(walls_type_d, cn_x_d, cn_y_d, cn_z_d, c_norm_d, s_nx_d, s_ny_d, s_nz_d); });
    launch3(nx + 2, ny + 2, nz + 2, [&] { extrapolateNormalToSolid(walls_type_d, cn_x_d, cn_y_d, cn_z_d, phi_d); });
    launch3(nx, ny, nz, [&] { CSF_Forces(cn_x_d, cn_y_d, cn_z_d, curv_d); });
}

/* The reference's own output writers on the current state, in `workdir`
 * (src/IO_multiphase.cpp:252-305 save_checkpoint, :500-714
 * VTK_legacy_writer_3D, :800-841 VTK_walls_bin).  Order: the checkpoint and
 * the type-3 files first, because the type-1 and type-2 writers set phi to
 * zero on solid nodes of the host array they share with the state. */
int ref_write_outputs(const char* workdir, int nt) {
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return -1;
    if (chdir(workdir) != 0) return -2;
    const char* dirs[] = {"results", "results/out2.checkpoint", "results/out3.field_data",
                          "results/out3.field_data/full_flow_field", "results/out3.field_data/phase_distribution"};
    for (const char* d : dirs) mkdir(d, 0755);
    ntime = nt;
    save_checkpoint(0);
    output_fieldData_precision_cmd = 0;
    VTK_legacy_writer_3D(nt, 3);
    char name[256];
    snprintf(name, sizeof name, "results/out3.field_data/full_flow_field/force_vector_%010d.vtk", nt);
    rename(name, "vtk3_cmd0.tmp");
    output_fieldData_precision_cmd = 1;
    VTK_legacy_writer_3D(nt, 3);
    VTK_walls_bin();
    output_fieldData_precision_cmd = 0;
    VTK_legacy_writer_3D(nt, 1);
    snprintf(name, sizeof name, "results/out3.field_data/full_flow_field/full_flow_field_%010d.vtk", nt);
    rename(name, "vtk1_cmd0.tmp");
    output_fieldData_precision_cmd = 1;
    VTK_legacy_writer_3D(nt, 1);
    VTK_legacy_writer_3D(nt, 2);
    if (chdir(cwd) != 0) return -3;
    return 0;
}

/* Bind the "device" pointers of the kernels to the reference's host arrays
 * (the role of MemAllocate_*_GPU). */
void ref_bind(void) {
    walls_d = walls; walls_type_d = walls_type;
    s_nx_d = s_nx; s_ny_d = s_ny; s_nz_d = s_nz;
    pdf_d = pdf; phi_d = phi; cn_x_d = cn_x; cn_y_d = cn_y; cn_z_d = cn_z; c_norm_d = c_norm; curv_d = curv;
    W_in_d = W_in; rho_d = rho;
    f_convec_bc_d = f_convec_bc; g_convec_bc_d = g_convec_bc; phi_convec_bc_d = phi_convec_bc;
}

void ref_compute_macro_vars(void) { compute_macro_vars(); }

void* ref_ptr(const char* name) {
    const std::string n(name);
    if (n == "pdf") return pdf;
    if (n == "phi") return phi;
    if (n == "cn_x") return cn_x;
    if (n == "cn_y") return cn_y;
    if (n == "cn_z") return cn_z;
    if (n == "c_norm") return c_norm;
    if (n == "curv") return curv;
    if (n == "walls") return walls;
    if (n == "walls_type") return walls_type;
    if (n == "walls_global") return walls_global;
    if (n == "s_nx") return s_nx;
    if (n == "s_ny") return s_ny;
    if (n == "s_nz") return s_nz;
    if (n == "W_in") return W_in;
    if (n == "f_convec_bc") return f_convec_bc;
    if (n == "g_convec_bc") return g_convec_bc;
    if (n == "phi_convec_bc") return phi_convec_bc;
    if (n == "rho") return rho;
    if (n == "u") return u;
    if (n == "v") return v;
    if (n == "w") return w;
    return nullptr;
}

double ref_scalar(const char* name) {
    const std::string n(name);
    if (n == "nxGlobal") return (double)nxGlobal;
    if (n == "nyGlobal") return (double)nyGlobal;
    if (n == "nzGlobal") return (double)nzGlobal;
    if (n == "jper") return jper;
    if (n == "kper") return kper;
    if (n == "domain_wall_status_z_min") return domain_wall_status_z_min;
    if (n == "domain_wall_status_z_max") return domain_wall_status_z_max;
    if (n == "inlet_BC") return inlet_BC;
    if (n == "outlet_BC") return outlet_BC;
    if (n == "porous_plate_cmd") return porous_plate_cmd;
    if (n == "Z_porous_plate") return Z_porous_plate;
    if (n == "lbm_gamma") return lbm_gamma;
    if (n == "force_z") return force_z;
    if (n == "la_nui1") return la_nui1;
    if (n == "la_nui2") return la_nui2;
    if (n == "lbm_beta") return lbm_beta;
    if (n == "phi_inlet") return phi_inlet;
    if (n == "sa_inject") return sa_inject;
    if (n == "uin_avg") return uin_avg;
    if (n == "relaxation") return relaxation;
    if (n == "cos_theta") return cos_theta;
    if (n == "rho_in") return rho_in;
    if (n == "rho_out") return rho_out;
    if (n == "interface_z0") return interface_z0;
    if (n == "A_xy") return A_xy;
    if (n == "flowrate") return flowrate;
    if (n == "uin_avg_0") return uin_avg_0;
    if (n == "num_solid_boundary_global") return (double)num_solid_boundary_global;
    if (n == "num_fluid_boundary_global") return (double)num_fluid_boundary_global;
    if (n == "num_solid_boundary") return (double)num_solid_boundary;
    if (n == "num_fluid_boundary") return (double)num_fluid_boundary;
    if (n == "pore_sum") return (double)pore_sum;
    if (n == "saturation_full_domain") return saturation_full_domain;
    if (n == "ntime0") return ntime0;
    return -1e300;
}

} // extern "C"
