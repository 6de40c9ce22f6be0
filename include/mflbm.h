/*
 * mflbm.h — C ABI of the GB300 (sm_103a) implementation of the MF-LBM
 * per-timestep hot path (D3Q19 colour-gradient two-phase lattice Boltzmann,
 * AA-pattern odd/even streaming).
 *
 * Every function returns MFLBM_OK (0) or a negative MFLBM_E* code; the text of
 * the last error on the calling thread is returned by mflbm_last_error().
 * No torch or C++ types appear in any signature: pointers are plain host
 * pointers unless a name ends in _dev.
 *
 * Array arguments use the reference's padded, 1-based layouts
 * (includes/Idx_gpu.cuh:54-70 of MF-LBM-CUDA):
 *   s0  (nx)(ny)(nz)                 no ghost layer
 *   s1  (nx+2)(ny+2)(nz+2)           one ghost layer   (curv, rho, u, v, w)
 *   s2  (nx+4)(ny+4)(nz+4)           two ghost layers  (walls, cn_x/y/z, c_norm)
 *   s4  (nx+8)(ny+8)(nz+8)           four ghost layers (phi, walls_type, s_nx/y/z)
 *   f1  (nx+2)(ny+2)(nz+2)*19*2      pdf[i_f1(x,y,z,e,g)], x fastest, then y, z,
 *                                    direction e (0..18), component g (0,1)
 *   cnv (nx+2)(ny+2)*19              f_convec_bc / g_convec_bc (icnv_f1)
 * Floating-point arrays hold `float` when precision == MFLBM_FP32 and
 * `double` when precision == MFLBM_FP64 (the reference's compile-time T_P,
 * includes/solver_precision.h:8-20).
 */
#ifndef MFLBM_H
#define MFLBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MFLBM_ABI_VERSION 1

enum {
    MFLBM_OK = 0,
    MFLBM_E_ARG = -1,      /* invalid argument or inconsistent parameters */
    MFLBM_E_CUDA = -2,     /* a CUDA runtime call failed */
    MFLBM_E_STATE = -3,    /* call out of order (e.g. step before upload) */
    MFLBM_E_NOMEM = -4,    /* device or host allocation failed */
    MFLBM_E_IO = -5        /* file could not be read or written */
};

enum { MFLBM_FP32 = 1, MFLBM_FP64 = 2 };         /* = reference SINGLE/DOUBLE_PRECISION */
enum { MFLBM_FAST = 0, MFLBM_STRICT = 1 };       /* strict: IEEE ops in reference order, no FMA contraction */

/*
 * Simulation parameters in the final form the reference host code hands to
 * its kernels (src/main_iteration_GPU.cu:14-47 copyConstantData and the
 * globals read by main_iteration_kernel_GPU, :1890-2056).  Floating-point
 * fields are given as double; with MFLBM_FP32 they must hold values exactly
 * representable as float (the reference's float globals widened), and the
 * library narrows them back without rounding.
 */
typedef struct mflbm_params {
    long long nx, ny, nz;              /* nxGlobal, nyGlobal, nzGlobal */
    int precision;                     /* MFLBM_FP32 or MFLBM_FP64 */
    int fp_mode;                       /* MFLBM_FAST or MFLBM_STRICT */
    int jper, kper;                    /* periodic y / z (x is always walled) */
    int domain_wall_status_z_min;      /* 1: solid wall at z = 1 */
    int domain_wall_status_z_max;      /* 1: solid wall at z = nz */
    int inlet_BC;                      /* 1 velocity (bounce-back), 2 Zou-He pressure */
    int outlet_BC;                     /* 1 convective, 2 Zou-He pressure */
    int porous_plate_cmd;              /* 0 none, 1 block fluid 1, 2 block fluid 2 */
    int Z_porous_plate;                /* plate plane */
    double lbm_gamma;                  /* surface tension */
    double force_z;                    /* body force along z */
    double la_nui1, la_nui2;           /* inverse kinematic viscosities */
    double lbm_beta;                   /* recolouring parameter beta */
    double phi_inlet;                  /* order parameter imposed at the inlet */
    double sa_inject;                  /* fluid-1 fraction of the injected fluid */
    double uin_avg;                    /* mean inlet velocity (convective outlet speed) */
    double relaxation;                 /* inlet relaxation factor (1 in the reference) */
    double cos_theta;                  /* cos(180 deg - contact angle) */
    double rho_in, rho_out;            /* Zou-He inlet / outlet densities */
} mflbm_params;

/*
 * Keys of input/simulation_control.txt that the hot path and its set-up read
 * (src/IO_multiphase.cpp:47-187).  mflbm_params_from_control() applies the
 * reference's derivations (src/IO_multiphase.cpp:198-206,
 * src/Init_multiphase.cpp:168-205,258-297) to produce mflbm_params.
 */
typedef struct mflbm_control {
    long long nxGlobal, nyGlobal, nzGlobal;
    int iper, jper, kper;
    int domain_wall_status_x_min, domain_wall_status_x_max;
    int domain_wall_status_y_min, domain_wall_status_y_max;
    int domain_wall_status_z_min, domain_wall_status_z_max;
    int inlet_BC, outlet_BC;
    int porous_plate_cmd, Z_porous_plate;
    int initial_fluid_distribution_option;
    int rho_out_BC;
    double fluid1_viscosity, fluid2_viscosity;
    double surface_tension, theta, RK_beta;
    double capillary_number, saturation_injection;
    double initial_interface_position, body_force_0;
} mflbm_control;

/* Derived quantities that set-up produces besides mflbm_params. */
typedef struct mflbm_derived {
    double A_xy;                       /* open inlet cross-section la_x * la_y */
    double uin_avg_0;                  /* Ca * gamma / nu1 */
    double flowrate;                   /* uin_avg_0 * A_xy */
    double interface_z0;               /* initial interface position */
} mflbm_derived;

/* Geometry counts (src/Geometry_preprocessing.cpp:208-222,389-401). */
typedef struct mflbm_geometry_counts {
    long long num_solid_boundary_global;   /* walls_type == 2 on [-3, n+4]^3 */
    long long num_fluid_boundary_global;   /* walls_type == -1 on [-3, n+4]^3 */
    long long num_solid_boundary;          /* walls_type == 2 on [-2, n+3]^3 */
    long long num_fluid_boundary;          /* walls_type == -1 on [-2, n+3]^3 */
    long long pore_sum;                    /* fluid nodes in [1, n]^3 */
} mflbm_geometry_counts;

/* FP64 monitor reductions over fluid nodes of [1,n]^3
 * (src/Monitor.cpp:17-140 monitor, :472-495 cal_saturation). */
typedef struct mflbm_monitor {
    double vol1_sum, vol2_sum;         /* sum of (1 +/- phi)/2 over the saturation window */
    double mass1_sum, mass2_sum;       /* sum of rho (1 +/- phi)/2 over the saturation window */
    double saturation;                 /* vol1 / (vol1 + vol2) */
    double flux1_sum, flux2_sum;       /* sum over all z of w (1 +/- phi)/2 */
    double total_mass;                 /* sum of every population of both components in [0,n+1]^3 */
    double umax;                       /* max |u| over fluid nodes */
    double vol1_full, vol2_full;       /* cal_saturation sums over [1,n]^3 */
} mflbm_monitor;

typedef struct mflbm_context mflbm_context;

/* ---- library ---------------------------------------------------------- */
int mflbm_abi_version(void);
const char* mflbm_last_error(void);
/* Number of kernels this library has launched in this process. */
unsigned long long mflbm_kernel_launch_count(void);

/* ---- set-up (host) ---------------------------------------------------- */
/* Reference: read_parameter_multi + initialization_basic_multi derivations
 * (src/IO_multiphase.cpp:198-242, src/Init_multiphase.cpp:168-205,258-269). */
int mflbm_params_from_control(const mflbm_control* ctl, int precision, int fp_mode,
                              mflbm_params* out, mflbm_derived* derived);

/* Reference: set_walls (src/Misc.cpp:17-118, 139-192): turns a .dat body
 * (bytes, index (i-1)+ny*((j-1)+nx*(k-1)), nx == ny) into walls_global (s0,
 * 1 solid / 0 fluid) with the domain walls of `ctl` added. */
int mflbm_set_walls(const mflbm_control* ctl, const uint8_t* geometry_bytes,
                    int32_t* walls_global);

/* Reference: inlet_vel_profile_rectangular (src/Misc.cpp:387-419) with the
 * uniform default of initialization_open_velocity_inlet_BC
 * (src/Init_multiphase.cpp:258-284).  W_in has (nx+2)(ny+2) entries. */
int mflbm_inlet_profile(const mflbm_control* ctl, int precision, void* W_in);

/* ---- context ---------------------------------------------------------- */
/* Reference: initialization_GPU + MemAllocate_*_GPU(1)
 * (src/Init_multiphase_GPU.cu:13-116).  Allocates every device buffer. */
int mflbm_create(const mflbm_params* params, mflbm_context** out);
/* Reference: MemAllocate_geometry_GPU(2) / MemAllocate_multi_GPU(2). */
int mflbm_destroy(mflbm_context* ctx);
/* Reference: copyConstantData (src/main_iteration_GPU.cu:14-47): replace the
 * physical parameters (same lattice size and precision). */
int mflbm_set_params(mflbm_context* ctx, const mflbm_params* params);

/* Device geometry preprocessing, bit-exact with geometry_preprocessing_new
 * (src/Geometry_preprocessing.cpp:29-403).  walls_global: s0 int32 (host).
 * Fills the context's walls / walls_type / solid normals and boundary lists;
 * the optional host outputs (may be NULL) receive copies in the reference
 * layouts (walls s2, walls_type s4, s_n* s4). */
int mflbm_preprocess_geometry(mflbm_context* ctx, const int32_t* walls_global,
                              int32_t* walls, int32_t* walls_type,
                              void* s_nx, void* s_ny, void* s_nz,
                              mflbm_geometry_counts* counts);

/* Upload a host-side geometry that was preprocessed elsewhere (the reference's
 * MemAllocate_geometry_GPU(1), src/Init_multiphase_GPU.cu:43-70). */
int mflbm_upload_geometry(mflbm_context* ctx, const int32_t* walls,
                          const int32_t* walls_type, const void* s_nx,
                          const void* s_ny, const void* s_nz);

/* Device version of initialization_new_multi + initialization_new_multi_pdf
 * (src/Init_multiphase.cpp:299-496) for options 1-5 (u = v = w = 0,
 * rho = 1), followed by the start-up colour gradient
 * (src/Phase_gradient.cpp:15-216).  W_in: (nx+2)(ny+2) host array or NULL. */
int mflbm_init_fields(mflbm_context* ctx, int initial_fluid_distribution_option,
                      double interface_z0, const void* W_in);

/* Reference: MemAllocate_multi_GPU(1) (src/Init_multiphase_GPU.cu:73-104):
 * upload a full host state.  Any pointer except pdf and phi may be NULL
 * (cn/c_norm/curv are then recomputed from phi; convective buffers are taken
 * from the pdf at z = nz). */
int mflbm_upload_fields(mflbm_context* ctx, const void* pdf, const void* phi,
                        const void* cn_x, const void* cn_y, const void* cn_z,
                        const void* c_norm, const void* curv, const void* W_in,
                        const void* f_convec_bc, const void* g_convec_bc,
                        const void* phi_convec_bc);

/* Reference: the device->host copies of main_iteration_kernel_GPU at output
 * steps (src/main_iteration_GPU.cu:2058-2076).  Any pointer may be NULL.
 * Blocks until the copies are complete. */
int mflbm_download_fields(mflbm_context* ctx, void* pdf, void* phi,
                          void* cn_x, void* cn_y, void* cn_z, void* c_norm,
                          void* curv, void* f_convec_bc, void* g_convec_bc,
                          void* phi_convec_bc);

/* ---- the hot path ----------------------------------------------------- */
/* One time step `ntime` (odd ntime: odd AA step) — the work of
 * main_iteration_kernel_GPU (src/main_iteration_GPU.cu:1890-2056) without its
 * host copies.  Asynchronous on the context's stream. */
int mflbm_step(mflbm_context* ctx, int ntime);
/* Steps ntime_begin .. ntime_begin + nsteps - 1, replayed from a captured
 * CUDA graph of one odd+even pair where possible.  Asynchronous. */
int mflbm_run(mflbm_context* ctx, int ntime_begin, int nsteps);
int mflbm_synchronize(mflbm_context* ctx);

/* FP64 device reductions (Monitor quantities) on the current state; the
 * state must be after an even step (src/Misc.cpp:222-274 semantics).
 * Blocks until the result is on the host. */
int mflbm_monitor_reduce(mflbm_context* ctx, int n_exclude_inlet,
                         int n_exclude_outlet, mflbm_monitor* out);

/* The same reductions without allocating device memory (no counterpart in
 * the reference).  mflbm_monitor_reduce allocates its per-block partials on
 * its first call; a caller whose lattice fills the GPU's memory, or that must
 * not let cudaMalloc / cudaFree synchronise the device while other work runs
 * on it, uses this entry point instead.  Its partials live in one fixed
 * device array of the library (10,250 doubles: 4 partial blocks per SM, up to
 * 256 SMs); a device with more SMs is rejected with MFLBM_E_ARG.
 *   - The first call on each device looks up that array's address (which may
 *     load the library's device code); make it before any stream capture.
 *   - All contexts on one device share the array: calls that overlap in time
 *     on the same device (two host threads, or contexts whose streams run
 *     concurrently) race on it and must be serialised by the caller.  Calls
 *     from one thread are serial, since each blocks until its result is on
 *     the host.
 *   - Nothing in the array needs clearing: each call writes every element it
 *     reads.
 * Same arguments, result and error behaviour as mflbm_monitor_reduce. */
int mflbm_monitor_reduce_noalloc(mflbm_context* ctx, int n_exclude_inlet,
                                 int n_exclude_outlet, mflbm_monitor* out);

/* ---- introspection ---------------------------------------------------- */
/* Counts of lattice nodes: [0] fluid nodes in [1,n]^3, [1] all nodes n^3. */
int mflbm_node_counts(mflbm_context* ctx, long long counts[2]);
/* CUDA stream (cudaStream_t) the context launches on. */
void* mflbm_stream(mflbm_context* ctx);
/* Per-launch device time (ms) of the collision kernel over the last
 * mflbm_run/mflbm_step calls made while timing was enabled; returns the
 * number of timed launches. */
int mflbm_set_kernel_timing(mflbm_context* ctx, int enable);
int mflbm_kernel_times(mflbm_context* ctx, double* collide_ms_total,
                       double* gradient_ms_total, int* n_collide, int* n_gradient);

#ifdef __cplusplus
}
#endif
#endif /* MFLBM_H */
