// Definitions of the reference globals that the drop-in shim reads — the role
// the reference's src/main.cpp translation unit plays — for the drop-in test.
#ifdef MFLBM_REF_DOUBLE
typedef double T_P;
#else
typedef float T_P;
#endif
long long nxGlobal, nyGlobal, nzGlobal;
int iper, jper, kper;
int domain_wall_status_x_min, domain_wall_status_x_max;
int domain_wall_status_y_min, domain_wall_status_y_max;
int domain_wall_status_z_min, domain_wall_status_z_max;
int inlet_BC, outlet_BC, porous_plate_cmd, Z_porous_plate;
int ntime, ntime_monitor, ntime_animation, ntime_visual, ntime_clock_sum;
double memory_gpu;
int *walls, *walls_type;
T_P *s_nx, *s_ny, *s_nz;
T_P *pdf, *W_in, *phi, *cn_x, *cn_y, *cn_z, *c_norm, *curv;
T_P *f_convec_bc, *g_convec_bc, *phi_convec_bc;
T_P lbm_gamma, lbm_beta, cos_theta, phi_inlet, sa_inject, la_nui2;
T_P force_z, uin_avg, rho_in, rho_out, relaxation, la_nui1;
