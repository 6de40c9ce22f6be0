// fast flavour of the step kernels (built with FMA contraction).
#define MFLBM_NS fast
#include "step_kernels.cuh"

namespace mflbm {
namespace fast {

int collide(mflbm_context& c, bool odd) {
    return c.params.precision == MFLBM_FP32 ? launch_collide<float>(c, odd) : launch_collide<double>(c, odd);
}

int boundaries(mflbm_context& c, bool odd) {
    return c.params.precision == MFLBM_FP32 ? launch_boundaries<float>(c, odd) : launch_boundaries<double>(c, odd);
}

int refresh_aux(mflbm_context& c) {
    return c.params.precision == MFLBM_FP32 ? launch_refresh_aux<float>(c) : launch_refresh_aux<double>(c);
}

int gradient(mflbm_context& c) {
    return c.params.precision == MFLBM_FP32 ? launch_gradient<float>(c) : launch_gradient<double>(c);
}

}  // namespace fast
}  // namespace mflbm
