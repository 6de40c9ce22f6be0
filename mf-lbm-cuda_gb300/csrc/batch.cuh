// Persistent launch for a batch of single-phase samples (included by
// step_kernels.cuh, so it runs the collision in each arithmetic flavour).
//
// One cooperative launch runs many time steps of every sample of a batch.
// Each step is a sequence of phases over a work list of (sample, unit)
// pairs, separated by grid barriers:
//   collision  units of `blockDim` consecutive fluid-list entries;
//   periodic   units of `blockDim` exchange items (periodic_item: z, y and
//              the z-y edges, which can run at once);
// the same device functions as the per-sample launches (collide_stream_kernel,
// periodic_kernel), so every sample's state is bit-identical to stepping it
// alone.
//
// Single phase: the host launches this only for samples whose second
// component is absent everywhere (every component-2 population exactly 0,
// no interface records) and that have no inlet, outlet or plate.  The
// collision then keeps it absent exactly (rho2 = 0 gives frac1 = 1, g1 = f,
// g2 = 0, phi = 1), so the colour-gradient pipeline of every later step
// would reproduce the zero records and unit phase field it finds: it is left
// out.  That is the single-phase permeability workload (phi = 1, body force,
// periodic y and z).
//
// Every barrier wait is bounded by a wall-clock limit (the %globaltimer
// nanosecond clock); a wait that runs out sets an error flag, every block
// returns at its next barrier, and the host reports MFLBM_E_TIMEOUT.
#pragma once
#include <algorithm>
#include <vector>

#include "collide.cuh"
#include "boundary.cuh"

namespace mflbm {
namespace MFLBM_NS {

template <class T, class E> struct BatchSample {
    CollideArgs<T, E> c;
    BcArgs<T, E> bc;
    int jper, kper;
};

enum { kPhaseCollide = 0, kPhasePeriodic = 1, kPhases = 2 };

struct BatchSync {
    unsigned* bar;                 // [0] arrivals, [1] generation
    int* error;                    // set to 1 when a wait ran out
    unsigned long long limit_ns;   // bound of one barrier wait
    unsigned nblocks;
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier with a bounded wait (arrival counter + generation word; the
// block's first thread fences, arrives and waits, as a grid-wide sync does).
// Returns false when some block's wait ran out (the caller returns).
__device__ __forceinline__ bool grid_sync(const BatchSync& s) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vbar = s.bar;
        volatile int* verr = s.error;
        const unsigned gen = vbar[1];
        __threadfence();
        if (atomicAdd(&s.bar[0], 1u) + 1u == s.nblocks) {
            atomicExch(&s.bar[0], 0u);
            __threadfence();
            atomicAdd(&s.bar[1], 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while (vbar[1] == gen) {
                if (*verr) break;
                if (global_ns() - t0 > s.limit_ns) {
                    atomicExch(s.error, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        ok = *verr == 0;
    }
    __syncthreads();
    return ok != 0;
}

// pre: kPhases arrays of (ns + 1) unit prefix sums, phase-major.  At least
// 3 resident blocks of 256 (2 in FP64): with the bare thread bound the
// compiler held the FP32 kernel to 64 registers and spilled 28 bytes; with
// this one it uses 80 without spills, as the collision kernel does.
template <class T, class E>
__global__ void __launch_bounds__(256, sizeof(T) == 8 ? 2 : 3) batch_persistent_kernel(const BatchSample<T, E>* S, int ns, const int* pre,
                                                               BatchSync sync, int ntime_begin, int nsteps) {
    for (int step = 0; step < nsteps; ++step) {
        const bool odd = ((ntime_begin + step) & 1) != 0;
        for (int ph = 0; ph < kPhases; ++ph) {
            const int* p = pre + ph * (ns + 1);
            const int total = p[ns];
            if (total == 0) continue;   // the same for every block: no barrier either
            int k = 0;
            for (int u = blockIdx.x; u < total; u += gridDim.x) {
                while (p[k + 1] <= u) ++k;   // u grows: the sample index only moves forward
                const int r = u - p[k];
                const BatchSample<T, E>& s = S[k];
                if (ph == kPhaseCollide) {
                    const int t = r * blockDim.x + threadIdx.x;
                    if (t < s.c.n) {
                        if (odd) collide_node<T, E, true, uint32_t>(s.c, t);
                        else collide_node<T, E, false, uint32_t>(s.c, t);
                    }
                } else {
                    const int item = r * blockDim.x + threadIdx.x;
                    if (item < periodic_items(s.bc.g, s.jper, s.kper)) {
                        if (odd) periodic_item<T, E, true>(s.bc, s.jper, s.kper, item);
                        else periodic_item<T, E, false>(s.bc, s.jper, s.kper, item);
                    }
                }
            }
            if (!grid_sync(sync)) return;
        }
    }
}

// *flag becomes non-zero if any stored component-2 population (decoded) of
// [0, n+1]^3 is not exactly 0.
template <class T, class E>
__global__ void __launch_bounds__(256) second_component_kernel(Grid g, PopView<T, E> P, int* flag) {
    const ll n1 = g.n1(), nxy = (ll)(g.nx + 2) * (g.ny + 2);
    for (ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x; t < n1 * 19; t += (ll)gridDim.x * blockDim.x) {
        const int q = (int)(t / n1);
        const ll r = t - (ll)q * n1;
        const int z = (int)(r / nxy);
        const ll rxy = r - (ll)z * nxy;
        const int y = (int)(rxy / (g.nx + 2)), x = (int)(rxy - (ll)y * (g.nx + 2));
        if (P.get(x, y, z, q, 1) != T(0)) {
            atomicExch(flag, 1);
            return;
        }
    }
}

template <class T, class E>
int launch_second_component(mflbm_context& c, int* flag_dev) {
    PopView<T, E> P;
    P.p = (E*)c.d.pdf;
    P.b = c.d.b;
    second_component_kernel<T, E><<<std::max(1, c.d.n_sm) * 4, 256, 0, c.stream>>>(c.d.g, P, flag_dev);
    return after_launch("second_component");
}

template <class T, class E>
BatchSample<T, E> batch_sample(const mflbm_context& c) {
    BatchSample<T, E> s;
    s.c = collide_args<T, E>(c);
    s.bc = bc_args<T, E>(c);
    s.jper = c.params.jper;
    s.kper = c.params.kper;
    return s;
}

// Host side of one persistent launch: the per-sample records are copied to
// `dev_samples` (capacity checked by the caller); the launch is cooperative,
// so every block is resident and the barriers can complete.
template <class T, class E>
int launch_batch_persistent(mflbm_context* const* ctx, int ns, void* dev_samples, const int* dev_pre, BatchSync sync,
                            int block, int grid, int ntime_begin, int nsteps, cudaStream_t stream) {
    std::vector<BatchSample<T, E>> h(ns);
    for (int i = 0; i < ns; ++i) h[i] = batch_sample<T, E>(*ctx[i]);
    MFLBM_CUDA(cudaMemcpyAsync(dev_samples, h.data(), sizeof(BatchSample<T, E>) * ns, cudaMemcpyHostToDevice, stream));
    const BatchSample<T, E>* S = (const BatchSample<T, E>*)dev_samples;
    void* args[] = {(void*)&S, (void*)&ns, (void*)&dev_pre, (void*)&sync, (void*)&ntime_begin, (void*)&nsteps};
    MFLBM_CUDA(cudaLaunchCooperativeKernel((const void*)batch_persistent_kernel<T, E>, dim3(grid), dim3(block), args, 0,
                                           stream));
    count_launch();
    MFLBM_CUDA(cudaStreamSynchronize(stream));   // keeps `h` alive until the copy is done
    return MFLBM_OK;
}

template <class T, class E>
int batch_grid(int block, int n_sm, int* grid) {
    int per_sm = 0;
    MFLBM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_persistent_kernel<T, E>, block, 0));
    if (per_sm < 1) return fail(MFLBM_E_CUDA, "batch: the persistent kernel does not fit on a multiprocessor");
    *grid = per_sm * std::max(1, n_sm);
    return MFLBM_OK;
}

template <class T, class E> constexpr size_t batch_sample_size() { return sizeof(BatchSample<T, E>); }

}  // namespace MFLBM_NS
}  // namespace mflbm
