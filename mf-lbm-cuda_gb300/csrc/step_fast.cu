// fast flavour of the step kernels (built with FMA contraction).
#define MFLBM_NS fast
#include "step_kernels.cuh"

namespace mflbm {
namespace fast {

#define MFLBM_DISPATCH(fn, ...) \
    (c.params.precision == MFLBM_FP32 ? fn<float>(__VA_ARGS__) : fn<double>(__VA_ARGS__))
// kernels that touch the populations: also by their storage
#define MFLBM_DISPATCH_POP(fn, ...)                                                              \
    (c.params.precision == MFLBM_FP64               ? fn<double, double>(__VA_ARGS__)             \
     : c.params.storage == MFLBM_STORE_F16          ? fn<float, __half>(__VA_ARGS__)              \
     : c.params.storage == MFLBM_STORE_BF16         ? fn<float, __nv_bfloat16>(__VA_ARGS__)       \
                                                    : fn<float, float>(__VA_ARGS__))

int collide(mflbm_context& c, bool odd) { return MFLBM_DISPATCH_POP(launch_collide, c, odd); }
int boundaries(mflbm_context& c, bool odd) { return MFLBM_DISPATCH_POP(launch_boundaries, c, odd); }
int gradient(mflbm_context& c) { return MFLBM_DISPATCH(launch_gradient, c); }
int export_arrays(mflbm_context& c) { return MFLBM_DISPATCH(launch_export, c); }
int refresh_aux(mflbm_context& c) { return MFLBM_DISPATCH(launch_refresh_aux, c); }
int second_component(mflbm_context& c, int* flag_dev) { return MFLBM_DISPATCH_POP(launch_second_component, c, flag_dev); }

namespace {
template <class T, class E>
int run_batch(mflbm_context* const* ctx, int n, const BatchLaunch& L) {
    BatchSync sync;
    sync.bar = L.bar;
    sync.error = L.error;
    sync.limit_ns = L.limit_ns;
    sync.nblocks = (unsigned)L.grid;
    return launch_batch_persistent<T, E>(ctx, n, L.samples, L.pre, sync, L.block, L.grid, L.ntime_begin, L.nsteps,
                                         L.stream);
}
template <class T, class E> int grid_of(int block, int n_sm, int* grid) { return batch_grid<T, E>(block, n_sm, grid); }
template <class T, class E> size_t sample_bytes() { return batch_sample_size<T, E>(); }
}  // namespace

int batch_persistent(mflbm_context* const* ctx, int n, const BatchLaunch& L) {
    const mflbm_context& c = *ctx[0];
    return MFLBM_DISPATCH_POP(run_batch, ctx, n, L);
}
int batch_grid(const mflbm_context& c, int block, int* grid) { return MFLBM_DISPATCH_POP(grid_of, block, c.d.n_sm, grid); }
size_t batch_sample_bytes(const mflbm_context& c) { return MFLBM_DISPATCH_POP(sample_bytes); }

}  // namespace fast
}  // namespace mflbm
