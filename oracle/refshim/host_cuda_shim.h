/*
 * Force-included header that lets the reference's CUDA sources compile as
 * ordinary host C++ (test infrastructure for oracle/_ref only).
 *
 * - __global__/__constant__/__device__ expand to nothing, so every kernel is a
 *   plain function and every __constant__ symbol a plain global;
 * - threadIdx/blockIdx/blockDim are thread-local variables that the driver
 *   (ref_driver.cpp) sets before calling a kernel function;
 * - cudaMemcpyToSymbol on a host global becomes a memcpy;
 * - T_P / prc / pprc are defined here (the same macro set as the reference's
 *   solver_precision.h) so that REF_DOUBLE selects the FP64 build without
 *   editing the reference's header.
 */
#ifndef MFLBM_HOST_CUDA_SHIM_H
#define MFLBM_HOST_CUDA_SHIM_H

#define __global__
#define __constant__
#define __device__
#define __DEVICE_LAUNCH_PARAMETERS_H__ 1

#define SOLVER_PRECISION_H 1
#define SINGLE_PRECISION (1)
#define DOUBLE_PRECISION (2)
#ifdef REF_DOUBLE
#define PRECISION (DOUBLE_PRECISION)
#define T_P double
#define prc(x) x
#define pprc(x) x
#else
#define PRECISION (SINGLE_PRECISION)
#define T_P float
#define prc(x) x##f
#define pprc(x) f##x
#endif

#ifdef __cplusplus
#include <cstring>
#include <cuda_runtime_api.h>

struct shim_index3 { int x, y, z; };
extern thread_local shim_index3 threadIdx, blockIdx, blockDim;

template <class S>
inline cudaError_t cudaMemcpyToSymbol(S& symbol, const void* src, size_t count, size_t offset = 0,
                                      cudaMemcpyKind = cudaMemcpyHostToDevice) {
    std::memcpy(reinterpret_cast<char*>(&symbol) + offset, src, count);
    return cudaSuccess;
}
#endif
#endif
