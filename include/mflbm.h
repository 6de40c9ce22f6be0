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

#define MFLBM_ABI_VERSION 3

enum {
    MFLBM_OK = 0,
    MFLBM_E_ARG = -1,      /* invalid argument or inconsistent parameters */
    MFLBM_E_CUDA = -2,     /* a CUDA runtime call failed */
    MFLBM_E_STATE = -3,    /* call out of order (e.g. step before upload) */
    MFLBM_E_NOMEM = -4,    /* device or host allocation failed */
    MFLBM_E_IO = -5,       /* file could not be read or written */
    MFLBM_E_TIMEOUT = -6   /* a bounded device-side wait ran out (the state is undefined) */
};

enum { MFLBM_FP32 = 1, MFLBM_FP64 = 2 };         /* = reference SINGLE/DOUBLE_PRECISION */
enum { MFLBM_FAST = 0, MFLBM_STRICT = 1 };       /* strict: IEEE ops in reference order, no FMA contraction */
/* Storage of the populations (no counterpart in the reference): the solver
 * precision itself, or, with MFLBM_FP32 only, 16-bit shifted deviations
 * s = g / w_q - 1 from the lattice weight w_q of the direction (FP16 or BF16;
 * the collision computes in FP32).  s is exact where a component is absent
 * (g = 0, s = -1) and of order 1e-3 where it fills the node. */
enum { MFLBM_STORE_NATIVE = 0, MFLBM_STORE_F16 = 1, MFLBM_STORE_BF16 = 2 };

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
    int storage;                       /* MFLBM_STORE_NATIVE (0, the reference's), _F16 or _BF16 */
    int reserved;
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

/* Scalars of the monitors that need more than the sums above
 * (src/Monitor.cpp:17-56 kinetic energy, :277-351 phase-field steady state,
 * :355-441 capillary-pressure steady state, :447-466 breakthrough), FP64. */
typedef struct mflbm_monitor_ext {
    double umax2;                      /* max |u|^2 over fluid nodes */
    double usq1, usq2;                 /* sum |u|^2 over fluid nodes with phi > 0.999 / phi < -0.999 */
    double pre_w, pre_nw;              /* sum rho over fluid nodes with phi < -0.99 / phi > 0.99 */
    long long n_w, n_nw;               /* their counts */
    long long breakthrough;            /* fluid nodes of slice z = nz-1 with phi > 0 */
    double dphi_max;                   /* max |phi - phi at the previous tracking call| over fluid nodes */
} mflbm_monitor_ext;

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
/* The context's current parameters (after mflbm_read_checkpoint they hold the
 * checkpoint's force_z and rho_in). */
int mflbm_get_params(mflbm_context* ctx, mflbm_params* out);

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

/* Warm-start entry: the equilibrium fill of initialization_new_multi_pdf
 * (src/Init_multiphase.cpp:389-496) with given macroscopic fields over the
 * phi already set, f_q = r w_q (1 + 3 c.u + 4.5 (c.u)^2 - 1.5 u.u), r = rho
 * (1 +- phi) / 2.  rho, u, v, w: host arrays of (nx+2)(ny+2)(nz+2) values in
 * the context's precision, index i + (nx+2)(j + (ny+2) k), each may be NULL
 * (rho = 1, velocity 0).  Call after mflbm_init_fields / mflbm_upload_fields. */
int mflbm_init_flow(mflbm_context* ctx, const void* rho, const void* u,
                    const void* v, const void* w);
/* No counterpart in the reference: the same fill with the energy-square
 * moment of the total populations set to the equilibrium of the collision
 * itself (the reference's MRT has 0 there at rest, the lattice weights give
 * 3 rho), so that the state starts on the collision's equilibrium instead of
 * relaxing that moment in the first steps -- the warm start's fill. */
int mflbm_init_flow_mrt(mflbm_context* ctx, const void* rho, const void* u,
                        const void* v, const void* w);
/* No counterpart in the reference: the warm start's fill from a prediction
 * in the U-Net's output format, formed on the device.  y: host array of
 * nx*ny*nz*4 floats (x fastest, 4 values per node): u nu/g, v nu/g, w nu/g
 * and (rho - <rho>)/(3 g), each divided by scales[c].  Fluid nodes get
 * u = y scale g/nu and rho = 1 + 3 g y scale, solid nodes rest; the halo
 * layers repeat the opposite interior layer along periodic y (jper) and z
 * (kper) and rest elsewhere; FP32 arithmetic (g/nu and 3 g rounded to
 * FP32).  Then the equilibrium fill of mflbm_init_flow (mrt = 0) or
 * mflbm_init_flow_mrt (mrt = 1). */
int mflbm_init_flow_predicted(mflbm_context* ctx, const float* y, double nu, double g,
                              const float* scales, int mrt);

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
/* Sizes of the last gradient pass's sparse sets (no reference counterpart;
 * diagnostics of the sparse colour-gradient passes): nodes of [-1, n+2]^3
 * with a non-zero interface normal, solid boundary nodes given a non-zero
 * extrapolated normal by that pass (the solid nodes of the super-blocks it
 * processed; elsewhere the solid normals are unchanged), and fluid nodes
 * whose normals were recomputed.
 * Synchronises the context's stream.  Any pointer may be NULL. */
int mflbm_interface_stats(mflbm_context* ctx, long long* interface_nodes, long long* solid_normals,
                          long long* active_nodes);
/* Super-blocks (4 x 4 x 4 bricks of 2 x 2 x 2 phi nodes) of the last
 * gradient pass: how many it processed, how many it flagged for the next
 * pass (phi may change within them), and the total.  Synchronises the
 * context's stream.  No counterpart in the reference. */
int mflbm_super_block_stats(mflbm_context* ctx, long long* processed, long long* flagged, long long* total);

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
 *   - Every call looks up that array's address on the current device; the
 *     first lookup on a device may load the library's device code, so make
 *     the first call before any stream capture.
 *   - All contexts on one device share the array: calls that overlap in time
 *     on the same device (two host threads, or contexts whose streams run
 *     concurrently) race on it and must be serialised by the caller.  Calls
 *     from one thread are serial, since each blocks until its result is on
 *     the host.
 *   - Nothing in the array needs clearing: each call writes every element it
 *     reads.
 * Same arguments and error behaviour as mflbm_monitor_reduce, and the same
 * result bit for bit (both use 4 partial blocks per SM of the device). */
int mflbm_monitor_reduce_noalloc(mflbm_context* ctx, int n_exclude_inlet,
                                 int n_exclude_outlet, mflbm_monitor* out);

/* Per-slice monitor sums (the profiles of src/Monitor.cpp:58-104) in FP64
 * on the current state (after an even step), deterministic: for slice
 * k = 1..nz, slices[m * nz + k - 1] holds, over the fluid nodes of the slice,
 * with a1 = (1 + phi)/2, a2 = (1 - phi)/2 and u, v, w the post-even velocity
 * of compute_macro_vars:
 *   m = 0: sum w a1   1: sum w a2   2: sum a1   3: sum a2
 *       4: sum rho a1 5: sum rho a2 6: sum rho
 * `ext` (may be NULL) receives the other monitor scalars; with track_phi != 0
 * dphi_max is measured against the phi of the previous tracking call (zero
 * before the first) and the current phi becomes the new reference.
 * Blocks until the results are on the host. */
int mflbm_monitor_profile(mflbm_context* ctx, double* slices, mflbm_monitor_ext* ext, int track_phi);

/* ---- output files in the reference's formats -------------------------- */

/* Reference: VTK_legacy_writer_3D (src/IO_multiphase.cpp:500-714) for the
 * current state (after an even step).  vtk_type 1: phi (0 on solids),
 * density and velocity (compute_macro_vars, src/Misc.cpp:222-274); 2: phi as
 * float (0 on solids); 3: phi, c_norm and the interface normal, under the
 * labels of type 1.  Types 1 and 3 name the data "float" when
 * output_fieldData_precision_cmd is 0 and "double" otherwise, and hold values
 * of the context's precision, as the reference does.  The body is assembled
 * on the device; `path` is the file to create (the reference names them
 * results/out3.field_data/{full_flow_field/full_flow_field_,
 * phase_distribution/small_,full_flow_field/force_vector_}%010d.vtk).
 * The device state is not modified. */
int mflbm_write_vtk(mflbm_context* ctx, int vtk_type,
                    int output_fieldData_precision_cmd, const char* path);
/* Reference: VTK_walls_bin (src/IO_multiphase.cpp:800-841), the solid
 * geometry as big-endian int (reference name: results/out3.field_data/
 * walls_bin.vtk). */
int mflbm_write_walls_vtk(mflbm_context* ctx, const char* path);
/* Reference: save_checkpoint (src/IO_multiphase.cpp:252-305), file part:
 * int ntime+1, force_z, rho_in, pdf (i_f1), phi (i_s4) and, with the
 * convective outlet, the three convective buffers, in the context's
 * precision and the host's byte order (reference name:
 * results/out2.checkpoint/id0000).  job_status.txt is the caller's. */
int mflbm_write_checkpoint(mflbm_context* ctx, int ntime, const char* path);
/* Reference: initialization_old_multi (src/Init_multiphase.cpp:501-537) +
 * the start-up colour gradient: loads a checkpoint written by the reference
 * or by mflbm_write_checkpoint for the same lattice, precision and outlet_BC
 * (anything else is rejected with MFLBM_E_ARG), sets force_z and rho_in from
 * it, uploads the fields (and W_in, the inlet profile of
 * mflbm_inlet_profile, unless NULL) and runs the gradient pass.  *ntime0
 * receives the stored step - 1 (the reference's ntime0). */
int mflbm_read_checkpoint(mflbm_context* ctx, const char* path, const void* W_in, int* ntime0);

/* ---- tuning and batches (no counterpart in the reference) -------------- */

typedef struct mflbm_tuning {
    int collide_block;                 /* threads per block of the collision */
    int normals_block;                 /* ... of the interface-normal kernel */
    int curvature_block;               /* ... of the curvature kernel */
    int extrapolate_block;             /* ... of the two solid-boundary extrapolations */
    double step_ms_before;             /* mean step time with the tuning found on entry */
    double step_ms_after;              /* ... with the chosen tuning */
    int tile_x, tile_y, tile_z;        /* population tile extent in 2x2x2 bricks (powers of
                                          two; x, y 1-32, z 1 or 2); default 8 x 4 x 2 */
} mflbm_tuning;

/* Times the step with several population tile shapes (the layout of the
 * populations in HBM: tiles of 2x2x2 bricks, each tile storing its 19
 * directions contiguously), then with 64, 128 and 256 threads per block for
 * each kernel family, keeps the fastest combination and reports it.  reps:
 * odd + even step pairs timed per candidate (>= 1).  The state is copied
 * aside first (temporary device memory of one state) and restored
 * afterwards; a change of tile shape moves every population exactly, so the
 * simulation's results are unchanged.  Not allowed while kernel timing is
 * on. */
int mflbm_autotune(mflbm_context* ctx, int reps, mflbm_tuning* out);
/* Sets block sizes (64, 128 or 256; 0 keeps the current value) and, when
 * tile_x/y/z are non-zero, the population tile shape (the populations are
 * moved to the new layout, results unchanged), e.g. to reuse a tuning found
 * on another context of the same size. */
int mflbm_set_tuning(mflbm_context* ctx, const mflbm_tuning* t);
/* The current block sizes and tile shape (step_ms_* are 0). */
int mflbm_get_tuning(mflbm_context* ctx, mflbm_tuning* out);

/* A batch of independent contexts on the current device, advanced together:
 * the odd + even step pairs of all of them are captured into one CUDA graph,
 * one branch per context, so one graph launch steps every sample and small
 * lattices run concurrently.  The contexts stay owned by the caller and must
 * outlive the batch; a context whose parameters, geometry or tuning change
 * is re-captured at the next run. */
typedef struct mflbm_batch mflbm_batch;
int mflbm_batch_create(mflbm_context* const* ctxs, int n, mflbm_batch** out);
/* Steps ntime_begin .. ntime_begin + nsteps - 1 of every context of the
 * batch; ntime_begin must be odd and nsteps even.  Blocks until done.
 * A batch of single-phase samples (every component-2 population exactly 0,
 * no interface, no inlet, outlet or plate; same precision, storage and
 * arithmetic flavour: the single-phase permeability workload) runs as one
 * persistent cooperative launch per up to 100 steps, every sample's work of
 * a phase spread over all blocks and the phases (collision, periodic z, y,
 * z-y) separated by grid barriers with bounded waits; the results are
 * bit-identical to stepping each context alone.  Other batches run as one
 * CUDA graph per step pair (a branch per context).  A barrier wait that runs
 * out returns MFLBM_E_TIMEOUT with the contexts' states undefined. */
int mflbm_batch_run(mflbm_batch* b, int ntime_begin, int nsteps);
int mflbm_batch_destroy(mflbm_batch* b);

enum { MFLBM_BATCH_AUTO = 0, MFLBM_BATCH_GRAPH = 1, MFLBM_BATCH_PERSISTENT = 2 };
typedef struct mflbm_batch_options {
    int mode;              /* MFLBM_BATCH_AUTO (persistent when the batch allows it), _GRAPH or
                              _PERSISTENT (an error if the batch does not allow it) */
    int block;             /* threads per block of the persistent launch: 64, 128 or 256 */
    double wait_limit_s;   /* bound of every grid-barrier wait, seconds (> 0, <= 60) */
    int used_mode;         /* out (get): mode of the last run */
    int grid;              /* out (get): blocks of the last persistent launch */
} mflbm_batch_options;
/* Defaults: MFLBM_BATCH_AUTO, 128 threads, 2 s. */
int mflbm_batch_set_options(mflbm_batch* b, const mflbm_batch_options* o);
int mflbm_batch_get_options(mflbm_batch* b, mflbm_batch_options* o);
/* Times the persistent launch with 64, 128 and 256 threads per block and
 * the population tile shapes 8x4x2, 2x2x2 and 8x8x2 bricks (applied to every
 * sample), `reps` step pairs each, keeps the fastest and reports it (tile
 * extents in out->tile_*, the block size in out->collide_block).  Every
 * context's state is copied aside first and restored; a tile change moves
 * the populations exactly, so results are unchanged.  Needs a batch that
 * runs persistent. */
int mflbm_batch_autotune(mflbm_batch* b, int reps, mflbm_tuning* out);

/* ---- learned warm start: 3-D U-Net --------------------------------------
 * (no counterpart in the reference)  4 levels of 16/32/64/128 channels, two
 * 3x3x3 convolutions + ReLU per level, 2x2x2 average pooling, nearest
 * up-sampling with concatenated skips, a final 3x3x3 convolution to 4
 * outputs.  BF16 weights and activations, FP32 accumulation on the tensor
 * cores, FP32 master weights, Adam.  Inputs per voxel: 2 channels (solid
 * mask, signed distance); outputs: 4 (u, v, w, p).  Host arrays are FP32,
 * D x H x W x channels with the channel fastest; D, H, W multiples of 8. */
typedef struct mflbm_unet mflbm_unet;
int mflbm_unet_create(int D, int H, int W, unsigned long long seed, mflbm_unet** out);
int mflbm_unet_destroy(mflbm_unet* net);
int mflbm_unet_param_count(mflbm_unet* net, long long* count);
/* x: D*H*W*2 inputs; y: D*H*W*4 outputs. */
int mflbm_unet_forward(mflbm_unet* net, const float* x, float* y);
/* One Adam step on the masked MSE of the 4 outputs against target
 * (D*H*W*4) over the voxels where mask (D*H*W) is non-zero; loss: the MSE
 * before the step (may be NULL). */
int mflbm_unet_train_step(mflbm_unet* net, const float* x, const float* target,
                          const float* mask, float lr, float* loss);
/* The loss and its gradient with respect to every weight and bias (same
 * layout as mflbm_unet_get_params), without an update. */
int mflbm_unet_gradients(mflbm_unet* net, const float* x, const float* target,
                         const float* mask, float* grads, float* loss);
/* Weights and biases as one FP32 vector of mflbm_unet_param_count values
 * (layer by layer: weights [cout][27][cin], then biases). */
int mflbm_unet_get_params(mflbm_unet* net, float* params);
int mflbm_unet_set_params(mflbm_unet* net, const float* params);
/* One convolution layer and its gradients, for checks against a CPU
 * restatement: x D*H*W*cin, w cout*27*cin (tap = 9 (dz+1) + 3 (dy+1) + dx+1),
 * b cout, gy D*H*W*cout or NULL; cin, cout multiples of 16.  Inputs are
 * rounded to BF16 on the device; y is the FP32 output before rounding, gx
 * the BF16 data gradient widened to FP32, gw and gb FP32. */
int mflbm_unet_conv_check(int D, int H, int W, int cin, int cout, const float* x,
                          const float* w, const float* b, int relu, const float* gy,
                          float* y, float* gx, float* gw, float* gb);
/* Network inputs of a pore geometry (no counterpart in the reference):
 * walls nz*ny*nx (x fastest, non-zero = solid, at least one solid and one
 * fluid voxel, fewer than 2^31 voxels); x nz*ny*nx*2: the solid mask (1 / 0) and the signed
 * Euclidean distance between voxel centres to the nearest voxel of the other
 * kind (positive in the fluid, negative in solids), times sdf_scale.  Bit 0,
 * 1, 2 of periodic_xyz make x, y, z periodic (distances by the minimum
 * image).  Exact distances, computed on the device. */
int mflbm_unet_features(const int32_t* walls, int nx, int ny, int nz, int periodic_xyz,
                        float sdf_scale, float* x);
/* Bound of the tensor-core convolutions' waits for their pipeline stages,
 * in mbarrier polls (default 1048576).  A wait that runs out makes the call
 * return MFLBM_E_CUDA; the copies and MMAs still in flight are waited for
 * with the default bound before tensor memory is freed, so the device stays
 * usable.  0 makes every stage wait run out (a test of that path). */
int mflbm_unet_set_wait_limit(unsigned int polls);

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
