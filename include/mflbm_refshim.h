/*
 * mflbm_refshim.h — the reference's own GPU entry points, implemented on top
 * of the C ABI in mflbm.h (mf-lbm-cuda_gb300/csrc/refshim.cpp).
 *
 * Link the reference's host objects (src/main.cpp and the other src/*.cpp of
 * MF-LBM-CUDA) against libmflbm_refshim_<f32|f64>.a and libmflbm.so in place
 * of the reference's src/main_iteration_GPU.cu and src/Init_multiphase_GPU.cu.
 * The functions have C++ linkage and no arguments beyond the reference's,
 * exactly like the functions they replace; everything else is read from the
 * reference's globals (includes/Module_extern.h, Fluid_*_extern.h), which the
 * reference's main.cpp translation unit defines.
 *
 * Build the shim with MFLBM_REF_DOUBLE defined for the reference's
 * DOUBLE_PRECISION build.  Errors print "CUDA Assert: <message>" and exit with
 * the library's error code, as the reference's cudaErrorCheck does
 * (includes/utils_GPU.cuh:8-13).  MFLBM_FP_MODE=strict in the environment
 * selects the strict (no FMA contraction) kernels.
 */
#ifndef MFLBM_REFSHIM_H
#define MFLBM_REFSHIM_H

/* replaces src/Init_multiphase_GPU.cu:13 — device set-up: context + uploads */
void initialization_GPU();
/* replaces src/Init_multiphase_GPU.cu:43 — 1: upload walls, walls_type, s_n*; else: free */
void MemAllocate_geometry_GPU(int flag);
/* replaces src/Init_multiphase_GPU.cu:73 — 1: upload pdf, phi, cn, c_norm, curv, W_in, convective buffers; else: free */
void MemAllocate_multi_GPU(int flag);
/* replaces src/main_iteration_GPU.cu:14 — physical constants (re-read at every step as well) */
void copyConstantData();
/* replaces src/main_iteration_GPU.cu:1890 — one time step `ntime`; host arrays refreshed at output steps */
void main_iteration_kernel_GPU();

#endif
