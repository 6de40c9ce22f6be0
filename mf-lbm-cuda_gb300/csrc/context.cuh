// The library context: device buffers in the reference layouts plus the
// node lists, stream and captured graphs.
#pragma once

#include "common.cuh"

namespace mflbm {

// Threads per block of the step kernels (chosen by mflbm_autotune).
struct Tuning {
    int collide = 128, normals = 128, curvature = 128, extrapolate = 128;
};

struct DeviceState {
    Tuning tune;
    Grid g{};
    Bricks b{};
    int precision = MFLBM_FP32;
    // populations in the tiled brick layout (common.cuh); fields in the reference layouts (s4 / s2 / s1)
    void* pdf = nullptr;
    void* staging = nullptr;        // reference-layout (f1) buffer for uploads / downloads
    void* cnv4 = nullptr;           // s2: (n_x, n_y, n_z, |grad phi|) per node
    void* aux = nullptr;            // per fluid node, fluid-list order: (n_x, n_y, n_z, 0.5*gamma*curv*c_norm)
    ll n_norm = 0;                  // walls_type <= 0 nodes on [-1, n+2]^3 (capacity of the sparse lists)
    int8_t* type8 = nullptr;        // walls_type as int8 (s4)
    bool arrays_stale = false;      // cn_x/y/z, c_norm, curv behind the records
    void* phi = nullptr;
    void* cn_x = nullptr;
    void* cn_y = nullptr;
    void* cn_z = nullptr;
    void* c_norm = nullptr;
    void* curv = nullptr;
    void* W_in = nullptr;
    void* f_cv = nullptr;
    void* g_cv = nullptr;
    void* phi_cv = nullptr;
    // geometry
    int32_t* walls = nullptr;       // s2
    int32_t* walls_type = nullptr;  // s4
    void* s_nx = nullptr;           // s4
    void* s_ny = nullptr;
    void* s_nz = nullptr;
    // node lists (packed coordinates)
    uint32_t* fluid_list = nullptr;    // walls == 0 on [1, n]^3, in population-layout order
    ll n_fluid = 0;
    uint2* list_phi_ext = nullptr;     // walls_type == 2 on [-2, n+3]^3: (packed, fluid-neighbour mask)
    ll n_phi_ext = 0;
    ll n_cn_ext = 0;                   // walls_type == 2 nodes on [0, n+1]^3 (normal extrapolation)
    double* red = nullptr;             // reduction scratch
    ll red_len = 0;
    int* zpair_off = nullptr;          // fluid-list offset of each layer of population tiles, ntz + 1 entries
    void* phi_prev = nullptr;          // phi at the previous tracking monitor call (s4)
    double* prof = nullptr;            // per-slice and per-block monitor partials
    ll prof_len = 0;
    uint32_t* dither = nullptr;        // step counter of 16-bit stochastic rounding: [0] read by odd, [1] by even steps
    int8_t* iface = nullptr;           // s2: 1 where the normal record may be non-zero (|grad phi| >= 1e-6, type <= 0)
    uint8_t* touch = nullptr;          // s2 (solid boundary nodes): tag of the last gradient pass that found a
                                       // non-zero record at one of the node's fluid neighbours, 0 when cleared
    uint32_t* snb = nullptr;           // s2 (fluid nodes): bit q where x + e_q is a solid boundary node of [0, n+1]^3
    uint16_t* pmask = nullptr;         // s4 rows x super-block columns: phi near +1 / -1 bits (gradient.cuh)
    uint8_t* fmask = nullptr;          // the same rows: fluid nodes of [1, n]^3
    uint8_t* cmask = nullptr;          // the same rows: walls_type <= 0 on [-1, n+2]^3
    int32_t* tmap = nullptr;           // s2: fluid-list index of a fluid node of [1, n]^3, else -1
    uint32_t* olist = nullptr;         // packed nodes with a non-zero normal record (capacity n_norm)
    uint32_t* nlist = nullptr;         // packed fluid nodes of the active 2x2x2 node blocks (capacity n_norm)
    int* gcount = nullptr;             // [0] olist, [1] solid normals written, [2] nlist, [4] previous olist
    // super-blocks of the normal pass: 4 x 4 x 4 phi bricks (8^3 nodes of the s4 lattice)
    int SX = 0, SY = 0, SZ = 0;        // super-blocks per axis
    int8_t* sbcode = nullptr;          // per super-block: the fluid code of its phi bricks (gradient.cuh)
    uint8_t* sbact = nullptr;          // per super-block: 1 if its phi can change at the next step (see gradient.cuh)
    uint8_t* sbslab = nullptr;         // per super-block: 1 if always processed (open or periodic faces)
    uint32_t* sblive = nullptr;        // super-blocks processed by the current pass
    int* sbinfo = nullptr;             // [0], [2] live counts of alternate passes; [1] 1: process every super-block at the next pass
    int grad_parity = 0;               // which live count the next gradient pass uses (launch_gradient)
    int* phioff = nullptr;             // offsets of each super-block's nodes in list_phi_ext
    int n_sm = 0;                      // multiprocessors of the device (grids of the list passes)
};

}  // namespace mflbm

struct mflbm_context {
    mflbm_params params{};
    mflbm::DeviceState d;
    cudaStream_t stream = nullptr;
    bool have_geometry = false;
    bool have_fields = false;
    unsigned long long generation = 0;  // bumped whenever captured launches would change
    // CUDA graph of one odd + even step pair (built lazily by mflbm_run)
    cudaGraphExec_t pair_graph = nullptr;
    int pair_graph_odd_first = -1;
    // kernel timing
    bool timing = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    double t_collide = 0, t_gradient = 0;
    int n_collide = 0, n_gradient = 0;
};
