// Device set-up entry points (setup.cu) and host set-up (host_setup.cpp).
#pragma once
#include "common.cuh"

namespace mflbm {
int preprocess_geometry(mflbm_context& c, const int32_t* walls_global_host, int iper);
int init_fields(mflbm_context& c, int option, double z0);
int monitor(mflbm_context& c, int nex_in, int nex_out, mflbm_monitor* out);
// monitor with its partials in a static device array (no allocation)
int monitor_noalloc(mflbm_context& c, int nex_in, int nex_out, mflbm_monitor* out);
// copy populations between d.staging (reference f1 layout) and d.pdf (brick layout)
int convert_populations(mflbm_context& c, bool to_bricks);
}  // namespace mflbm
