// Device set-up entry points (setup.cu) and host set-up (host_setup.cpp).
#pragma once
#include "common.cuh"

namespace mflbm {
int preprocess_geometry(mflbm_context& c, const int32_t* walls_global_host, int iper);
int init_fields(mflbm_context& c, int option, double z0);
int init_flow(mflbm_context& c, const void* rho, const void* u, const void* v, const void* w, int mrt);
// the fill from a normalised prediction y (device, nx*ny*nz*4 floats); work:
// device space for 4 arrays of n1 values of the context's precision
int init_flow_predicted(mflbm_context& c, const float* y, double nu, double g, const float* scales, int mrt,
                        void* work);
int monitor(mflbm_context& c, int nex_in, int nex_out, mflbm_monitor* out);
// per-slice monitor sums and the extra monitor scalars
int monitor_profile(mflbm_context& c, double* slices, mflbm_monitor_ext* ext, bool track_phi);
// monitor with its partials in a static device array (no allocation)
int monitor_noalloc(mflbm_context& c, int nex_in, int nex_out, mflbm_monitor* out);
// output files in the reference's formats (output.cu); d.staging must exist and,
// for VTK types 1 and 3, the reference-layout gradient arrays must be current
int write_vtk(mflbm_context& c, int vtk_type, int precision_cmd, const char* path);
int write_walls_vtk(mflbm_context& c, const char* path);
int write_checkpoint(mflbm_context& c, int ntime, const char* path);
// copy populations between the reference f1 layout (d.staging, or `f1`:
// page-locked host memory the device can address) and d.pdf (brick layout)
int convert_populations(mflbm_context& c, bool to_bricks, void* f1 = nullptr);
// the populations in the tile shape `to`, in a new device buffer (*out); d.pdf is unchanged
int relayout_populations(mflbm_context& c, const Bricks& to, void** out);
// the collision records in a new fluid-list order, dst[t] = aux[perm[t]], in a new buffer
int permute_records(mflbm_context& c, const int* perm_dev, void** out);
}  // namespace mflbm
