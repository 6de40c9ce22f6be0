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

}  // namespace fast
}  // namespace mflbm
