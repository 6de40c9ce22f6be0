// The reference's GPU entry points (include/mflbm_refshim.h) on top of the C
// ABI.  The globals below are declared with the names and types of the
// reference's extern headers (includes/Module_extern.h,
// Fluid_singlephase_extern.h, Fluid_multiphase_extern.h); the reference's
// main.cpp translation unit (or any host program playing its role) defines
// them.  Build with MFLBM_REF_DOUBLE for the reference's DOUBLE_PRECISION.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "../../include/mflbm.h"
#include "../../include/mflbm_refshim.h"

#ifdef MFLBM_REF_DOUBLE
typedef double T_P;
static const int kPrecision = MFLBM_FP64;
#else
typedef float T_P;
static const int kPrecision = MFLBM_FP32;
#endif

// ---- reference globals read by the hot path ----
extern long long nxGlobal, nyGlobal, nzGlobal;
extern int iper, jper, kper;
extern int domain_wall_status_x_min, domain_wall_status_x_max;
extern int domain_wall_status_y_min, domain_wall_status_y_max;
extern int domain_wall_status_z_min, domain_wall_status_z_max;
extern int inlet_BC, outlet_BC, porous_plate_cmd, Z_porous_plate;
extern int ntime, ntime_monitor, ntime_animation, ntime_visual, ntime_clock_sum;
extern double memory_gpu;
extern int *walls, *walls_type;
extern T_P *s_nx, *s_ny, *s_nz;
extern T_P *pdf, *W_in, *phi, *cn_x, *cn_y, *cn_z, *c_norm, *curv;
extern T_P *f_convec_bc, *g_convec_bc, *phi_convec_bc;
extern T_P lbm_gamma, lbm_beta, cos_theta, phi_inlet, sa_inject, la_nui2;
extern T_P force_z, uin_avg, rho_in, rho_out, relaxation, la_nui1;

namespace {

mflbm_context* g_ctx = nullptr;
mflbm_params g_params;

void check(int rc) {
    if (rc != MFLBM_OK) {
        std::fprintf(stderr, "CUDA Assert: %s %s %d\n", mflbm_last_error(), __FILE__, __LINE__);
        std::exit(rc < 0 ? -rc : rc);
    }
}

// mflbm_params from the reference's globals (the values copyConstantData and
// the launch arguments of main_iteration_kernel_GPU carry).
mflbm_params params_from_globals() {
    mflbm_params p;
    std::memset(&p, 0, sizeof p);
    p.nx = nxGlobal; p.ny = nyGlobal; p.nz = nzGlobal;
    p.precision = kPrecision;
    const char* mode = std::getenv("MFLBM_FP_MODE");
    p.fp_mode = (mode && std::strcmp(mode, "strict") == 0) ? MFLBM_STRICT : MFLBM_FAST;
    p.jper = jper; p.kper = kper;
    p.domain_wall_status_z_min = domain_wall_status_z_min;
    p.domain_wall_status_z_max = domain_wall_status_z_max;
    p.inlet_BC = inlet_BC; p.outlet_BC = outlet_BC;
    p.porous_plate_cmd = porous_plate_cmd; p.Z_porous_plate = Z_porous_plate;
    p.lbm_gamma = lbm_gamma; p.force_z = force_z;
    p.la_nui1 = la_nui1; p.la_nui2 = la_nui2; p.lbm_beta = lbm_beta;
    p.phi_inlet = phi_inlet; p.sa_inject = sa_inject; p.uin_avg = uin_avg;
    p.relaxation = relaxation; p.cos_theta = cos_theta;
    p.rho_in = rho_in; p.rho_out = rho_out;
    return p;
}

void ensure_context() {
    if (!g_ctx) {
        g_params = params_from_globals();
        check(mflbm_create(&g_params, &g_ctx));
        const double T = sizeof(T_P);
        const double n1 = double(nxGlobal + 2) * (nyGlobal + 2) * (nzGlobal + 2);
        const double n2 = double(nxGlobal + 4) * (nyGlobal + 4) * (nzGlobal + 4);
        const double n4 = double(nxGlobal + 8) * (nyGlobal + 8) * (nzGlobal + 8);
        memory_gpu += n1 * 38 * T + n4 * T + 4 * n2 * T + n1 * T + n2 * 4 + n4 * 4 * (1 + 3 * T / 4);
    }
}

void refresh_params() {
    mflbm_params p = params_from_globals();
    if (std::memcmp(&p, &g_params, sizeof p) != 0) {
        g_params = p;
        check(mflbm_set_params(g_ctx, &g_params));
    }
}

}  // namespace

void initialization_GPU() {
    std::cout << "***************************** GPU (sm_103a, libmflbm) **********************************" << std::endl;
    MemAllocate_geometry_GPU(1);
    MemAllocate_multi_GPU(1);
    std::cout << "Total amount of global memory needed on GPU (GB) = " << (memory_gpu / double(1024 * 1024 * 1024))
              << std::endl;
}

void MemAllocate_geometry_GPU(int flag) {
    if (flag == 1) {
        ensure_context();
        check(mflbm_upload_geometry(g_ctx, walls, walls_type, s_nx, s_ny, s_nz));
    } else if (g_ctx) {
        check(mflbm_destroy(g_ctx));
        g_ctx = nullptr;
    }
}

void MemAllocate_multi_GPU(int flag) {
    if (flag == 1) {
        ensure_context();
        const bool cv = outlet_BC == 1;
        check(mflbm_upload_fields(g_ctx, pdf, phi, cn_x, cn_y, cn_z, c_norm, curv, W_in, cv ? f_convec_bc : nullptr,
                                  cv ? g_convec_bc : nullptr, cv ? phi_convec_bc : nullptr));
    } else if (g_ctx) {
        check(mflbm_destroy(g_ctx));
        g_ctx = nullptr;
    }
}

void copyConstantData() {
    ensure_context();
    refresh_params();
}

void main_iteration_kernel_GPU() {
    ensure_context();
    refresh_params();  // rho_in / rho_out are launch arguments in the reference: always current
    check(mflbm_step(g_ctx, ntime));
    if (ntime % ntime_monitor == 0 || ntime % ntime_animation == 0 || ntime % ntime_visual == 0 ||
        ntime % ntime_clock_sum == 0) {
        std::cout << "Copying results back to the host side .... ";
        // the reference refreshes exactly these arrays (src/main_iteration_GPU.cu:2065-2072)
        check(mflbm_download_fields(g_ctx, pdf, phi, cn_x, cn_y, cn_z, c_norm, curv, nullptr, nullptr, nullptr));
        std::cout << " Complete " << std::endl;
    }
}
