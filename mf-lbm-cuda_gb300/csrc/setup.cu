// Device set-up: geometry preprocessing, start-up fields and the FP64
// monitor reductions.  Built with -fmad=false: the geometry and start-up
// arithmetic must be the reference's IEEE sequence so masks, solid normals
// and initial populations are bit-identical to the reference's host code.
#include <algorithm>
#include <string>
#include <type_traits>
#include <vector>

#include "context.cuh"
#include "setup.cuh"

namespace mflbm {

// ---------------------------------------------------------------------------
// Geometry preprocessing (src/Geometry_preprocessing.cpp:29-403) on a copy of
// the lattice padded by G = 10 layers: ghost fill, node classification
// (1 solid, 2 solid boundary, 0 fluid, -1 fluid boundary), four 27-point
// smoothing passes and the ISO8 solid normal at fluid boundary nodes.
// ---------------------------------------------------------------------------
namespace {

constexpr int G = 10;

struct Pad {
    int nx, ny, nz;
    __host__ __device__ int NX() const { return nx + 2 * G; }
    __host__ __device__ int NY() const { return ny + 2 * G; }
    __host__ __device__ int NZ() const { return nz + 2 * G; }
    __host__ __device__ ll n() const { return (ll)NX() * NY() * NZ(); }
    __host__ __device__ ll t(int x, int y, int z) const { return (x + G - 1) + (ll)NX() * ((y + G - 1) + (ll)NY() * (z + G - 1)); }
};

__global__ void pad_interior(Pad p, const int32_t* wg, int32_t* tmp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
    if (i > p.nx) return;
    tmp[p.t(i, j, k)] = wg[(i - 1) + (ll)p.nx * ((j - 1) + (ll)p.ny * (k - 1))];
}

// z ghosts for interior (i, j); then y ghosts for every z; then x ghosts for every (y, z)
__global__ void pad_fill_z(Pad p, int per, int32_t* tmp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, s = blockIdx.z;  // s in [0, 2G)
    if (i > p.nx) return;
    const int k = s < G ? 1 - G + s : p.nz + 1 + (s - G);
    const int src = s < G ? (per ? p.nz + k : 1) : (per ? k - p.nz : p.nz);
    tmp[p.t(i, j, k)] = tmp[p.t(i, j, src)];
}
__global__ void pad_fill_y(Pad p, int per, int32_t* tmp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = (int)blockIdx.y + 1 - G, s = blockIdx.z;
    if (i > p.nx) return;
    const int j = s < G ? 1 - G + s : p.ny + 1 + (s - G);
    const int src = s < G ? (per ? p.ny + j : 1) : (per ? j - p.ny : p.ny);
    tmp[p.t(i, j, k)] = tmp[p.t(i, src, k)];
}
__global__ void pad_fill_x(Pad p, int per, int32_t* tmp) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;  // [0, 2G)
    const int j = (int)blockIdx.y + 1 - G, k = (int)blockIdx.z + 1 - G;
    if (s >= 2 * G) return;
    const int i = s < G ? 1 - G + s : p.nx + 1 + (s - G);
    const int src = s < G ? (per ? p.nx + i : 1) : (per ? i - p.nx : p.nx);
    tmp[p.t(i, j, k)] = tmp[p.t(src, j, k)];
}

// classification on [2-G, n+G-1]: solid next to fluid -> 2, fluid next to solid -> -1
__global__ void classify(Pad p, const int32_t* tmp, int32_t* typ) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 2 - G;
    const int j = (int)blockIdx.y + 2 - G, k = (int)blockIdx.z + 2 - G;
    if (i > p.nx + G - 1) return;
    int v = tmp[p.t(i, j, k)];
    if (v == 1) {
        for (int q = 1; q <= 18; ++q)
            if (tmp[p.t(i + ex(q), j + ey(q), k + ez(q))] <= 0) { v = 2; break; }
    } else if (v == 0) {
        for (int q = 1; q <= 18; ++q)
            if (tmp[p.t(i + ex(q), j + ey(q), k + ez(q))] >= 1) { v = -1; break; }
    }
    typ[p.t(i, j, k)] = v;
}

template <class T>
__global__ void to_real(ll n, const int32_t* a, T* b, T* c) {
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) { b[t] = T(a[t]); c[t] = T(a[t]); }
}

// the 27-point neighbourhood in the reference's order (src/Geometry_preprocessing.cpp:31-33)
__device__ __constant__ const int kSx[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
__device__ __constant__ const int kSy[27] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, -1, 1, -1, 1};
__device__ __constant__ const int kSz[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1, -1, 1, 1, -1, -1, 1, 1, -1};

template <class T>
__global__ void smooth(Pad p, const T* in, T* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 2 - G;
    const int j = (int)blockIdx.y + 2 - G, k = (int)blockIdx.z + 2 - G;
    if (i > p.nx + G - 1) return;
    const T we[4] = {T(8) / T(27), T(2) / T(27), T(1) / T(54), T(1) / T(216)};
    T s = T(0);
#pragma unroll
    for (int q = 0; q < 27; ++q) {
        const int m = kSx[q] * kSx[q] + kSy[q] * kSy[q] + kSz[q] * kSz[q];
        s += in[p.t(i + kSx[q], j + kSy[q], k + kSz[q])] * we[m];
    }
    out[p.t(i, j, k)] = s;
}

// ISO8 gradient of the smoothed wall field at fluid boundary nodes
// (src/Geometry_preprocessing.cpp:226-386), in the reference's term order.
template <class T>
__global__ void solid_normals(Pad p, Grid g, const int32_t* typ, const T* S_, T* snx, T* sny, T* snz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 3;
    const int j = (int)blockIdx.y - 3, k = (int)blockIdx.z - 3;
    if (i > g.nx + 4) return;
    if (typ[p.t(i, j, k)] != -1) return;
    auto S = [&](int a, int b, int c) { return S_[p.t(a, b, c)]; };
    const T W[7] = {T(4) / T(45), T(1) / T(21), T(2) / T(105), T(5) / T(504), T(1) / T(315), T(1) / T(630), T(1) / T(5040)};
    const T nwx = W[0] * (S(i + 1, j, k) - S(i - 1, j, k)) +
        W[1] * (S(i + 1, j + 1, k) - S(i - 1, j - 1, k) + S(i + 1, j - 1, k) - S(i - 1, j + 1, k) + S(i + 1, j, k + 1) - S(i - 1, j, k - 1) + S(i + 1, j, k - 1) - S(i - 1, j, k + 1)) +
        W[2] * (S(i + 1, j + 1, k + 1) - S(i - 1, j - 1, k - 1) + S(i + 1, j + 1, k - 1) - S(i - 1, j - 1, k + 1) + S(i + 1, j - 1, k + 1) - S(i - 1, j + 1, k - 1) + S(i + 1, j - 1, k - 1) - S(i - 1, j + 1, k + 1)) +
        W[3] * (S(i + 2, j, k) - S(i - 2, j, k)) +
        W[4] * (S(i + 2, j + 1, k) - S(i - 2, j - 1, k) + S(i + 2, j - 1, k) - S(i - 2, j + 1, k) + S(i + 2, j, k + 1) - S(i - 2, j, k - 1) + S(i + 2, j, k - 1) - S(i - 2, j, k + 1) +
                S(i + 1, j + 2, k) - S(i - 1, j - 2, k) + S(i + 1, j - 2, k) - S(i - 1, j + 2, k) + S(i + 1, j, k + 2) - S(i - 1, j, k - 2) + S(i + 1, j, k - 2) - S(i - 1, j, k + 2)) +
        W[5] * (S(i + 2, j + 1, k + 1) - S(i - 2, j - 1, k - 1) + S(i + 2, j + 1, k - 1) - S(i - 2, j - 1, k + 1) + S(i + 2, j - 1, k + 1) - S(i - 2, j + 1, k - 1) + S(i + 2, j - 1, k - 1) - S(i - 2, j + 1, k + 1) +
                S(i + 1, j + 2, k + 1) - S(i - 1, j - 2, k - 1) + S(i + 1, j + 2, k - 1) - S(i - 1, j - 2, k + 1) + S(i + 1, j - 2, k + 1) - S(i - 1, j + 2, k - 1) + S(i + 1, j - 2, k - 1) - S(i - 1, j + 2, k + 1) +
                S(i + 1, j + 1, k + 2) - S(i - 1, j - 1, k - 2) + S(i + 1, j + 1, k - 2) - S(i - 1, j - 1, k + 2) + S(i + 1, j - 1, k + 2) - S(i - 1, j + 1, k - 2) + S(i + 1, j - 1, k - 2) - S(i - 1, j + 1, k + 2)) +
        W[6] * (S(i + 2, j + 2, k) - S(i - 2, j - 2, k) + S(i + 2, j - 2, k) - S(i - 2, j + 2, k) + S(i + 2, j, k + 2) - S(i - 2, j, k - 2) + S(i + 2, j, k - 2) - S(i - 2, j, k + 2));
    const T nwy = W[0] * (S(i, j + 1, k) - S(i, j - 1, k)) +
        W[1] * (S(i + 1, j + 1, k) - S(i - 1, j - 1, k) + S(i - 1, j + 1, k) - S(i + 1, j - 1, k) + S(i, j + 1, k + 1) - S(i, j - 1, k - 1) + S(i, j + 1, k - 1) - S(i, j - 1, k + 1)) +
        W[2] * (S(i + 1, j + 1, k + 1) - S(i - 1, j - 1, k - 1) + S(i + 1, j + 1, k - 1) - S(i - 1, j - 1, k + 1) + S(i - 1, j + 1, k - 1) - S(i + 1, j - 1, k + 1) + S(i - 1, j + 1, k + 1) - S(i + 1, j - 1, k - 1)) +
        W[3] * (S(i, j + 2, k) - S(i, j - 2, k)) +
        W[4] * (S(i + 2, j + 1, k) - S(i - 2, j - 1, k) + S(i - 2, j + 1, k) - S(i + 2, j - 1, k) + S(i, j + 2, k + 1) - S(i, j - 2, k - 1) + S(i, j + 2, k - 1) - S(i, j - 2, k + 1) +
                S(i + 1, j + 2, k) - S(i - 1, j - 2, k) + S(i - 1, j + 2, k) - S(i + 1, j - 2, k) + S(i, j + 1, k + 2) - S(i, j - 1, k - 2) + S(i, j + 1, k - 2) - S(i, j - 1, k + 2)) +
        W[5] * (S(i + 2, j + 1, k + 1) - S(i - 2, j - 1, k - 1) + S(i + 2, j + 1, k - 1) - S(i - 2, j - 1, k + 1) + S(i - 2, j + 1, k + 1) - S(i + 2, j - 1, k - 1) + S(i - 2, j + 1, k - 1) - S(i + 2, j - 1, k + 1) +
                S(i + 1, j + 2, k + 1) - S(i - 1, j - 2, k - 1) + S(i + 1, j + 2, k - 1) - S(i - 1, j - 2, k + 1) + S(i - 1, j + 2, k + 1) - S(i + 1, j - 2, k - 1) + S(i - 1, j + 2, k - 1) - S(i + 1, j - 2, k + 1) +
                S(i + 1, j + 1, k + 2) - S(i - 1, j - 1, k - 2) + S(i + 1, j + 1, k - 2) - S(i - 1, j - 1, k + 2) + S(i - 1, j + 1, k + 2) - S(i + 1, j - 1, k - 2) + S(i - 1, j + 1, k - 2) - S(i + 1, j - 1, k + 2)) +
        W[6] * (S(i + 2, j + 2, k) - S(i - 2, j - 2, k) + S(i - 2, j + 2, k) - S(i + 2, j - 2, k) + S(i, j + 2, k + 2) - S(i, j - 2, k - 2) + S(i, j + 2, k - 2) - S(i, j - 2, k + 2));
    const T nwz = W[0] * (S(i, j, k + 1) - S(i, j, k - 1)) +
        W[1] * (S(i, j + 1, k + 1) - S(i, j - 1, k - 1) + S(i, j - 1, k + 1) - S(i, j + 1, k - 1) + S(i + 1, j, k + 1) - S(i - 1, j, k - 1) + S(i - 1, j, k + 1) - S(i + 1, j, k - 1)) +
        W[2] * (S(i + 1, j + 1, k + 1) - S(i - 1, j - 1, k - 1) + S(i + 1, j - 1, k + 1) - S(i - 1, j + 1, k - 1) + S(i - 1, j + 1, k + 1) - S(i + 1, j - 1, k - 1) + S(i - 1, j - 1, k + 1) - S(i + 1, j + 1, k - 1)) +
        W[3] * (S(i, j, k + 2) - S(i, j, k - 2)) +
        W[4] * (S(i, j + 1, k + 2) - S(i, j - 1, k - 2) + S(i, j - 1, k + 2) - S(i, j + 1, k - 2) + S(i + 2, j, k + 1) - S(i - 2, j, k - 1) + S(i - 2, j, k + 1) - S(i + 2, j, k - 1) +
                S(i, j + 2, k + 1) - S(i, j - 2, k - 1) + S(i, j - 2, k + 1) - S(i, j + 2, k - 1) + S(i + 1, j, k + 2) - S(i - 1, j, k - 2) + S(i - 1, j, k + 2) - S(i + 1, j, k - 2)) +
        W[5] * (S(i + 2, j + 1, k + 1) - S(i - 2, j - 1, k - 1) + S(i + 2, j - 1, k + 1) - S(i - 2, j + 1, k - 1) + S(i - 2, j + 1, k + 1) - S(i + 2, j - 1, k - 1) + S(i - 2, j - 1, k + 1) - S(i + 2, j + 1, k - 1) +
                S(i + 1, j + 2, k + 1) - S(i - 1, j - 2, k - 1) + S(i + 1, j - 2, k + 1) - S(i - 1, j + 2, k - 1) + S(i - 1, j + 2, k + 1) - S(i + 1, j - 2, k - 1) + S(i - 1, j - 2, k + 1) - S(i + 1, j + 2, k - 1) +
                S(i + 1, j + 1, k + 2) - S(i - 1, j - 1, k - 2) + S(i + 1, j - 1, k + 2) - S(i - 1, j + 1, k - 2) + S(i - 1, j + 1, k + 2) - S(i + 1, j - 1, k - 2) + S(i - 1, j - 1, k + 2) - S(i + 1, j + 1, k - 2)) +
        W[6] * (S(i, j + 2, k + 2) - S(i, j - 2, k - 2) + S(i, j - 2, k + 2) - S(i, j + 2, k - 2) + S(i + 2, j, k + 2) - S(i - 2, j, k - 2) + S(i - 2, j, k + 2) - S(i + 2, j, k - 2));
    const T eps = T(1.1920928955078125e-07);  // numeric_limits<float>::epsilon() in both precisions
    const T inv = T(1) / (sqrt(nwx * nwx + nwy * nwy + nwz * nwz) + eps);
    const ll m = g.s4(i, j, k);
    snx[m] = nwx * inv; sny[m] = nwy * inv; snz[m] = nwz * inv;
}

// copy the padded work arrays out to the reference layouts (walls s2, walls_type s4)
__global__ void unpad(Pad p, Grid g, const int32_t* tmp, const int32_t* typ, int32_t* walls, int32_t* wt,
                      int8_t* type8) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 3;
    const int j = (int)blockIdx.y - 3, k = (int)blockIdx.z - 3;
    if (i > g.nx + 4) return;
    const int v = typ[p.t(i, j, k)];
    wt[g.s4(i, j, k)] = v;
    type8[g.s4(i, j, k)] = (int8_t)v;
    if (i >= -1 && i <= g.nx + 2 && j >= -1 && j <= g.ny + 2 && k >= -1 && k <= g.nz + 2)
        walls[g.s2(i, j, k)] = tmp[p.t(i, j, k)];
}

template <class T>
int preprocess_geometry_t(mflbm_context& c, const int32_t* walls_global_host, int iper) {
    DeviceState& d = c.d;
    const Grid g = d.g;
    const Pad p{g.nx, g.ny, g.nz};
    cudaStream_t s = c.stream;
    int32_t *wg = nullptr, *tmp = nullptr, *typ = nullptr;
    T *a = nullptr, *b = nullptr;
    int rc = MFLBM_OK;
    auto cleanup = [&]() { cudaFree(wg); cudaFree(tmp); cudaFree(typ); cudaFree(a); cudaFree(b); };
#define GEO_CUDA(call)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) { cleanup(); return fail(MFLBM_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); } \
    } while (0)
#define GEO_LAUNCH(name) do { if ((rc = after_launch(name)) != MFLBM_OK) { cleanup(); return rc; } } while (0)
    GEO_CUDA(cudaMalloc(&wg, sizeof(int32_t) * g.n0()));
    GEO_CUDA(cudaMalloc(&tmp, sizeof(int32_t) * p.n()));
    GEO_CUDA(cudaMalloc(&typ, sizeof(int32_t) * p.n()));
    GEO_CUDA(cudaMalloc(&a, sizeof(T) * p.n()));
    GEO_CUDA(cudaMalloc(&b, sizeof(T) * p.n()));
    GEO_CUDA(cudaMemcpyAsync(wg, walls_global_host, sizeof(int32_t) * g.n0(), cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemsetAsync(tmp, 0, sizeof(int32_t) * p.n(), s));
    const unsigned bx = grid_for(g.nx, 128);
    pad_interior<<<dim3(bx, g.ny, g.nz), 128, 0, s>>>(p, wg, tmp);
    GEO_LAUNCH("pad_interior");
    pad_fill_z<<<dim3(bx, g.ny, 2 * G), 128, 0, s>>>(p, c.params.kper, tmp);
    GEO_LAUNCH("pad_fill_z");
    pad_fill_y<<<dim3(bx, g.nz + 2 * G, 2 * G), 128, 0, s>>>(p, c.params.jper, tmp);
    GEO_LAUNCH("pad_fill_y");
    pad_fill_x<<<dim3(1, g.ny + 2 * G, g.nz + 2 * G), 32, 0, s>>>(p, iper, tmp);
    GEO_LAUNCH("pad_fill_x");
    GEO_CUDA(cudaMemcpyAsync(typ, tmp, sizeof(int32_t) * p.n(), cudaMemcpyDeviceToDevice, s));
    const dim3 gi(grid_for(g.nx + 2 * G - 2, 128), g.ny + 2 * G - 2, g.nz + 2 * G - 2);
    classify<<<gi, 128, 0, s>>>(p, tmp, typ);
    GEO_LAUNCH("classify");
    to_real<T><<<grid_for(p.n(), 256), 256, 0, s>>>(p.n(), tmp, a, b);
    GEO_LAUNCH("to_real");
    for (int it = 0; it < 4; ++it) {
        smooth<T><<<gi, 128, 0, s>>>(p, (it & 1) ? b : a, (it & 1) ? a : b);
        GEO_LAUNCH("smooth");
    }
    // four passes: a -> b -> a -> b -> a; the final field is in `a`
    const dim3 g4(grid_for(g.nx + 8, 128), g.ny + 8, g.nz + 8);
    GEO_CUDA(cudaMemsetAsync(d.s_nx, 0, sizeof(T) * g.n4(), s));
    GEO_CUDA(cudaMemsetAsync(d.s_ny, 0, sizeof(T) * g.n4(), s));
    GEO_CUDA(cudaMemsetAsync(d.s_nz, 0, sizeof(T) * g.n4(), s));
    solid_normals<T><<<g4, 128, 0, s>>>(p, g, typ, a, (T*)d.s_nx, (T*)d.s_ny, (T*)d.s_nz);
    GEO_LAUNCH("solid_normals");
    GEO_CUDA(cudaMemsetAsync(d.walls, 0, sizeof(int32_t) * g.n2(), s));
    unpad<<<g4, 128, 0, s>>>(p, g, tmp, typ, d.walls, d.walls_type, d.type8);
    GEO_LAUNCH("unpad");
    GEO_CUDA(cudaStreamSynchronize(s));
    cleanup();
#undef GEO_CUDA
#undef GEO_LAUNCH
    return MFLBM_OK;
}

// ---------------------------------------------------------------------------
// Start-up fields: initialization_new_multi options 1-5 and the equilibrium
// fill with u = v = w = 0, rho = 1 (src/Init_multiphase.cpp:299-496).
// ---------------------------------------------------------------------------
template <class T>
__global__ void init_phi(Grid g, int option, T z0, int open_z, T phi_inlet, T* phi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 3;
    const int j = (int)blockIdx.y - 3, k = (int)blockIdx.z - 3;
    if (i > g.nx + 4) return;
    T v = T(0);
    if (i >= 0 && i <= g.nx + 1 && j >= 0 && j <= g.ny + 1 && k >= 0 && k <= g.nz + 1) {
        const T x = T(i), y = T(j), z = T(k);
        auto sq = [](T a) { return a * a; };
        switch (option) {
        case 1: v = z <= z0 ? T(1) : T(-1); break;
        case 2: v = z <= z0 ? T(-1) : T(1); break;
        case 3: v = (sq(x - T(g.nx + 1) * T(0)) + sq(z - T(g.nz + 1) * T(0.5)) + sq(y - T(g.ny + 1) * T(0.5)) <= sq(z0)) ? T(1) : T(-1); break;
        case 4: v = (sq(x - T(g.nx + 1) * T(0)) + sq(z - T(g.nz + 1) * T(0.5)) + sq(y - T(g.ny + 1) * T(0.5)) <= sq(z0)) ? T(-1) : T(1); break;
        default: v = (sq(x - T(g.nx + 1) * T(0.5)) + sq(z - T(g.nz + 1) * T(0.5)) + sq(y - T(g.ny + 1) * T(0.5)) <= sq(z0)) ? T(1) : T(-1); break;
        }
    }
    if (open_z && k <= 0) v = phi_inlet;
    phi[g.s4(i, j, k)] = v;
}

// Equilibrium fill of initialization_new_multi_pdf (src/Init_multiphase.cpp:389-496):
// f_q = r w_q (1 + 3 c.u + 4.5 (c.u)^2 - 1.5 u.u) with r = rho (1 +- phi) / 2
// per component; rho, u, v, w in the (nx+2)(ny+2)(nz+2) layout, NULL for
// rho = 1 and u = v = w = 0 (the rest state of the cold start).
// mrt = 1: the energy-square moment of the total populations is set to the
// collision's own equilibrium, e2 = mrt_e2_coef1 rho + mrt_e2_coef2 j^2 (the
// MRT of collide(): 0 at rest), instead of the 3 rho that the lattice weights
// give; the correction lies along that moment's basis vector (12 rest, -4
// axis, 1 diagonal; no mass or momentum) and is shared between the two
// components in proportion to their densities.  Without it the first
// collisions relax that moment from 3 rho to 0, an impulse that shows up as a
// velocity transient of several times the flow itself.
template <class T, class E>
__global__ void init_pdf(Grid g, PopView<T, E> P, ModelConsts<T> c, const T* phi, const T* rho, const T* u,
                         const T* v, const T* w, int mrt = 0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i > g.nx + 1) return;
    const ll n1 = g.s1(i, j, k);
    const T ph = phi[g.s4(i, j, k)];
    const T rh = rho ? rho[n1] : T(1);
    const T ux = u ? u[n1] : T(0), uy = v ? v[n1] : T(0), uz = w ? w[n1] : T(0);
    const T r[2] = {rh * (T(1.0) + ph) * T(0.5), rh * (T(1.0) - ph) * T(0.5)};
    const T usqrt = ux * ux + uy * uy + uz * uz;
    T e2_shift = T(0);   // (target - current) / 252 of the total energy-square moment
    if (mrt) {
        T e2 = T(0);
        for (int q = 0; q < 19; ++q) {
            const T wq = q == 0 ? c.w0 : q < 7 ? c.w1 : c.w2;
            const T cu = T(ex(q)) * ux + T(ey(q)) * uy + T(ez(q)) * uz;
            const T feq = rh * wq * (T(1) + T(3) * cu + T(4.5) * cu * cu - T(1.5) * usqrt);
            e2 += (q == 0 ? T(12) : q < 7 ? T(-4) : T(1)) * feq;
        }
        const T jx = rh * ux, jy = rh * uy, jz = rh * uz;
        e2_shift = (c.mrt_e2_coef1 * rh + c.mrt_e2_coef2 * (jx * jx + jy * jy + jz * jz) - e2) / T(252);
    }
    for (int gg = 0; gg < 2; ++gg) {
        const T share = mrt ? r[gg] / rh : T(0);
        P.set(i, j, k, 0, gg, r[gg] * c.w0 + r[gg] * c.w0 * (T(-1.5) * usqrt) + share * T(12) * e2_shift);
        for (int q = 1; q < 19; ++q) {
            const T wq = q < 7 ? c.w1 : c.w2;
            // the reference's per-direction sums: only the non-zero components, left to right
            T cu = T(0);
            bool first = true;
            const int e3[3] = {ex(q), ey(q), ez(q)};
            const T u3[3] = {ux, uy, uz};
            for (int a = 0; a < 3; ++a) {
                if (e3[a] == 0) continue;
                const T term = e3[a] > 0 ? u3[a] : -u3[a];
                cu = first ? term : cu + term;
                first = false;
            }
            T f = r[gg] * wq + r[gg] * wq * (T(3.0) * cu + T(4.5) * cu * cu - T(1.5) * usqrt);
            if (mrt) f += share * (q < 7 ? T(-4) : T(1)) * e2_shift;
            P.set(i, j, k, q, gg, f);
        }
    }
}

template <class T, class E>
__global__ void init_convective(Grid g, PopView<T, E> P, const T* phi, T* f_cv, T* g_cv, T* phi_cv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i > g.nx + 1) return;
    for (int q = 0; q < 19; ++q) {
        f_cv[g.cnv(i, j, q)] = P.get(i, j, g.nz, q, 0);
        g_cv[g.cnv(i, j, q)] = P.get(i, j, g.nz, q, 1);
    }
    phi_cv[g.s1(i, j, 0)] = phi[g.s4(i, j, g.nz)];
}

template <class T, class E>
PopView<T, E> pop_view(const DeviceState& d) {
    PopView<T, E> P;
    P.p = (E*)d.pdf;
    P.b = d.b;
    return P;
}

template <class T, class E>
int init_fields_t(mflbm_context& c, int option, double z0) {
    DeviceState& d = c.d;
    const Grid g = d.g;
    const mflbm_params& p = c.params;
    cudaStream_t s = c.stream;
    const int open_z = p.kper == 0 && p.domain_wall_status_z_min == 0 && p.domain_wall_status_z_max == 0;
    int rc;
    init_phi<T><<<dim3(grid_for(g.nx + 8, 128), g.ny + 8, g.nz + 8), 128, 0, s>>>(g, option, T(z0), open_z, T(p.phi_inlet), (T*)d.phi);
    if ((rc = after_launch("init_phi")) != MFLBM_OK) return rc;
    init_pdf<T, E><<<dim3(grid_for(g.nx + 2, 128), g.ny + 2, g.nz + 2), 128, 0, s>>>(g, pop_view<T, E>(d), make_consts<T>(), (const T*)d.phi,
                                                                                nullptr, nullptr, nullptr, nullptr);
    if ((rc = after_launch("init_pdf")) != MFLBM_OK) return rc;
    MFLBM_CUDA(cudaMemsetAsync(d.f_cv, 0, sizeof(T) * g.plane1() * 19, s));
    MFLBM_CUDA(cudaMemsetAsync(d.g_cv, 0, sizeof(T) * g.plane1() * 19, s));
    MFLBM_CUDA(cudaMemsetAsync(d.phi_cv, 0, sizeof(T) * g.plane1(), s));
    if (p.outlet_BC == 1) {
        init_convective<T, E><<<dim3(grid_for(g.nx + 2, 128), g.ny + 2), 128, 0, s>>>(g, pop_view<T, E>(d), (const T*)d.phi, (T*)d.f_cv, (T*)d.g_cv, (T*)d.phi_cv);
        if ((rc = after_launch("init_convective")) != MFLBM_OK) return rc;
    }
    return MFLBM_OK;
}

// Equilibrium fill from given macroscopic fields over the current phi (the
// warm-start entry): rho, u, v, w are device arrays of (nx+2)(ny+2)(nz+2) T,
// any of them NULL.  The convective outlet buffers follow the new populations.
template <class T, class E>
int init_flow_t(mflbm_context& c, const void* rho, const void* u, const void* v, const void* w, int mrt) {
    DeviceState& d = c.d;
    const Grid g = d.g;
    cudaStream_t s = c.stream;
    int rc;
    init_pdf<T, E><<<dim3(grid_for(g.nx + 2, 128), g.ny + 2, g.nz + 2), 128, 0, s>>>(
        g, pop_view<T, E>(d), make_consts<T>(), (const T*)d.phi, (const T*)rho, (const T*)u, (const T*)v, (const T*)w, mrt);
    if ((rc = after_launch("init_pdf")) != MFLBM_OK) return rc;
    if (c.params.outlet_BC == 1) {
        init_convective<T, E><<<dim3(grid_for(g.nx + 2, 128), g.ny + 2), 128, 0, s>>>(g, pop_view<T, E>(d), (const T*)d.phi, (T*)d.f_cv, (T*)d.g_cv, (T*)d.phi_cv);
        if ((rc = after_launch("init_convective")) != MFLBM_OK) return rc;
    }
    return MFLBM_OK;
}

// Warm-start fields from a prediction in the network's output format (no
// counterpart in the reference): y holds, per interior node (x fastest, 4
// values per node), u nu/g, v nu/g, w nu/g and (rho - <rho>)/(3g), each
// divided by its scale.  A fluid node gets u = (y * scale) * (g/nu) and
// rho = 1 + (3g) * (y * scale); a solid node rests (rho = 1, u = 0).  Halo
// nodes of [0, n+1]^3 repeat the opposite interior layer along periodic
// axes (y: jper, z: kper) and rest elsewhere.  The prediction is FP32, and so
// is the arithmetic: the constants g/nu and 3g rounded to FP32, each product
// and sum rounded (no contraction), the result widened to T.
template <class T>
__global__ void predicted_fields_kernel(Grid g, const int32_t* __restrict__ walls, const float* __restrict__ y,
                                        float4 sc, float c_u, float c_rho, int per_y, int per_z, T* rho, T* u, T* v,
                                        T* w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i > g.nx + 1) return;
    const ll o = g.s1(i, j, k);
    int jj = j, kk = k;
    bool rest = i == 0 || i == g.nx + 1;
    if (j == 0 || j == g.ny + 1) { if (per_y) jj = j == 0 ? g.ny : 1; else rest = true; }
    if (k == 0 || k == g.nz + 1) { if (per_z) kk = k == 0 ? g.nz : 1; else rest = true; }
    if (rest || walls[g.s2(i, jj, kk)] != 0) {
        rho[o] = T(1); u[o] = T(0); v[o] = T(0); w[o] = T(0);
        return;
    }
    const float* p = y + 4 * ((i - 1) + (ll)g.nx * ((jj - 1) + (ll)g.ny * (kk - 1)));
    u[o] = (T)__fmul_rn(__fmul_rn(p[0], sc.x), c_u);
    v[o] = (T)__fmul_rn(__fmul_rn(p[1], sc.y), c_u);
    w[o] = (T)__fmul_rn(__fmul_rn(p[2], sc.z), c_u);
    rho[o] = (T)__fadd_rn(1.0f, __fmul_rn(c_rho, __fmul_rn(p[3], sc.w)));
}

// the fields into `work` (4 arrays of n1 T), then the equilibrium fill
template <class T, class E>
int init_flow_predicted_t(mflbm_context& c, const float* y, double nu, double gf, const float* scales, int mrt,
                          void* work) {
    const Grid g = c.d.g;
    T* f = (T*)work;
    const ll n1 = g.n1();
    const float4 sc = make_float4(scales[0], scales[1], scales[2], scales[3]);
    predicted_fields_kernel<T><<<dim3(grid_for(g.nx + 2, 128), g.ny + 2, g.nz + 2), 128, 0, c.stream>>>(
        g, c.d.walls, y, sc, (float)(gf / nu), (float)(3.0 * gf), c.params.jper != 0, c.params.kper != 0, f, f + n1,
        f + 2 * n1, f + 3 * n1);
    int rc = after_launch("predicted_fields");
    if (rc != MFLBM_OK) return rc;
    return init_flow_t<T, E>(c, f, f + n1, f + 2 * n1, f + 3 * n1, mrt);
}

// ---------------------------------------------------------------------------
// FP64 monitor reductions (quantities of src/Monitor.cpp:17-140, 472-495)
// over the fluid-node list, on post-even populations: per-block partials with
// warp shuffles, then one block folds the partials in a fixed order.
// ---------------------------------------------------------------------------
constexpr int NRED = 9;  // vol1, vol2, mass1, mass2, flux1, flux2, vol1_full, vol2_full, umax2

template <class T, class E>
__global__ void __launch_bounds__(256) monitor_partials(Grid g, PopView<T, E> P, const uint32_t* list, ll n, const T* phi,
                                                        const T* cnx, const T* cny, const T* cnz, const T* cnorm,
                                                        const T* curv, double gamma, double force_z, int k_lo, int k_hi,
                                                        double* partial) {
    double acc[NRED] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (ll)gridDim.x * blockDim.x) {
        int i, j, k;
        unpack_xyz(list[t], i, j, k);
        double f[19];
        const ll n1 = g.s1(i, j, k);
#pragma unroll
        for (int q = 0; q < 19; ++q) f[q] = (double)P.get(i, j, k, q, 0) + (double)P.get(i, j, k, q, 1);
        double rho = 0;
#pragma unroll
        for (int q = 0; q < 19; ++q) rho += f[q];
        const ll n2 = g.s2(i, j, k);
        const double tmp = 0.5 * gamma * (double)curv[n1] * (double)cnorm[n2];
        const double fx = tmp * cnx[n2], fy = tmp * cny[n2], fz = tmp * cnz[n2] + force_z;
        const double u = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14] - 0.5 * fx;
        const double v = f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18] - 0.5 * fy;
        const double w = f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18] - 0.5 * fz;
        const double ph = (double)phi[g.s4(i, j, k)];
        const double a1 = 0.5 * (1.0 + ph), a2 = 0.5 * (1.0 - ph);
        acc[6] += a1; acc[7] += a2;
        acc[4] += w * a1; acc[5] += w * a2;
        if (k >= k_lo && k <= k_hi) { acc[0] += a1; acc[1] += a2; acc[2] += rho * a1; acc[3] += rho * a2; }
        acc[8] = fmax(acc[8], u * u + v * v + w * w);
    }
    __shared__ double sh[NRED][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < NRED; ++r) {
        double x = acc[r];
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_down_sync(0xffffffffu, x, o);
            x = r == 8 ? fmax(x, y) : x + y;
        }
        if (lane == 0) sh[r][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x < NRED) {
        const int r = threadIdx.x;
        double x = sh[r][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) x = r == 8 ? fmax(x, sh[r][w]) : x + sh[r][w];
        partial[(ll)blockIdx.x * NRED + r] = x;
    }
}

// sum of the stored populations of both components over every node of
// [0, n+1]^3 (the tiles' padding beyond the lattice is not visited), decoded
// in T and summed in FP64
template <class T, class E>
__global__ void __launch_bounds__(256) sum_all(Grid g, PopView<T, E> P, double* partial) {
    const ll n1 = g.n1(), nxy = (ll)(g.nx + 2) * (g.ny + 2);
    double acc = 0;
    for (ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x; t < n1 * 19; t += (ll)gridDim.x * blockDim.x) {
        const int q = (int)(t / n1);
        const ll r = t - (ll)q * n1;
        const int z = (int)(r / nxy);
        const ll rxy = r - (ll)z * nxy;
        const int y = (int)(rxy / (g.nx + 2)), x = (int)(rxy - (ll)y * (g.nx + 2));
        acc += (double)P.get(x, y, z, q, 0) + (double)P.get(x, y, z, q, 1);
    }
    __shared__ double sh[8];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) x += sh[w];
        partial[blockIdx.x] = x;
    }
}

__global__ void fold_partials(int nblocks, int stride, const double* partial, double* out) {
    // one warp per quantity, fixed order
    const int r = blockIdx.x, lane = threadIdx.x;
    const bool is_max = (stride == NRED && r == 8);
    double x = is_max ? 0.0 : 0.0;
    for (int b = lane; b < nblocks; b += 32) {
        const double y = partial[(ll)b * stride + r];
        x = is_max ? fmax(x, y) : x + y;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_down_sync(0xffffffffu, x, o);
        x = is_max ? fmax(x, y) : x + y;
    }
    if (lane == 0) out[r] = x;
}

// Partial blocks of the monitor reductions: 4 per SM of the context's
// device.  mflbm_monitor_reduce and mflbm_monitor_reduce_noalloc use the same
// count, so their FP64 partial sums group the nodes alike and the two entry
// points return bit-identical results.
inline int monitor_blocks(const DeviceState& d) { return 4 * (d.n_sm > 0 ? d.n_sm : 1); }
// scratch doubles for `blocks` partial blocks: NRED per block for the monitor
// sums, one per block for the population total, NRED + 1 results
inline ll monitor_scratch_len(int blocks) { return (ll)NRED * blocks + blocks + NRED + 1; }

// The monitor reductions with their partials and results in `scratch`
// (monitor_scratch_len(blocks) doubles).
template <class T, class E>
int monitor_into(mflbm_context& c, int nex_in, int nex_out, double* scratch, int blocks, mflbm_monitor* out) {
    DeviceState& d = c.d;
    const Grid g = d.g;
    cudaStream_t s = c.stream;
    double* part = scratch;
    double* part2 = scratch + (ll)NRED * blocks;
    double* res = part2 + blocks;
    int rc;
    monitor_partials<T, E><<<blocks, 256, 0, s>>>(g, pop_view<T, E>(d), d.fluid_list, d.n_fluid, (const T*)d.phi,
                                               (const T*)d.cn_x, (const T*)d.cn_y, (const T*)d.cn_z,
                                               (const T*)d.c_norm, (const T*)d.curv, (double)T(c.params.lbm_gamma),
                                               (double)T(c.params.force_z), nex_in + 1, g.nz - nex_out, part);
    if ((rc = after_launch("monitor_partials")) != MFLBM_OK) return rc;
    fold_partials<<<NRED, 32, 0, s>>>(blocks, NRED, part, res);
    if ((rc = after_launch("fold_partials")) != MFLBM_OK) return rc;
    sum_all<T, E><<<blocks, 256, 0, s>>>(g, pop_view<T, E>(d), part2);
    if ((rc = after_launch("sum_all")) != MFLBM_OK) return rc;
    fold_partials<<<1, 32, 0, s>>>(blocks, 1, part2, res + NRED);
    if ((rc = after_launch("fold_partials")) != MFLBM_OK) return rc;
    double h[NRED + 1];
    MFLBM_CUDA(cudaMemcpyAsync(h, res, sizeof h, cudaMemcpyDeviceToHost, s));
    MFLBM_CUDA(cudaStreamSynchronize(s));
    out->vol1_sum = h[0]; out->vol2_sum = h[1];
    out->mass1_sum = h[2]; out->mass2_sum = h[3];
    out->flux1_sum = h[4]; out->flux2_sum = h[5];
    out->vol1_full = h[6]; out->vol2_full = h[7];
    out->umax = sqrt(h[8]);
    out->total_mass = h[9];
    out->saturation = h[0] / (h[0] + h[1]);
    return MFLBM_OK;
}

// mflbm_monitor_reduce: partials in the context's scratch, allocated on the
// first call.
template <class T, class E>
int monitor_t(mflbm_context& c, int nex_in, int nex_out, mflbm_monitor* out) {
    DeviceState& d = c.d;
    const int blocks = monitor_blocks(d);
    const ll need = monitor_scratch_len(blocks);
    if (d.red_len < need) {
        cudaFree(d.red);
        d.red = nullptr;
        d.red_len = 0;
        MFLBM_CUDA(cudaMalloc(&d.red, sizeof(double) * need));
        d.red_len = need;
    }
    return monitor_into<T, E>(c, nex_in, nex_out, d.red, blocks, out);
}

// ---------------------------------------------------------------------------
// Scratch of mflbm_monitor_reduce_noalloc: a fixed array in the library's
// device image instead of the context's lazily allocated partials, for callers
// that must not allocate device memory while the simulation runs (a lattice
// sized to fill the GPU's memory leaves no room for a first-call cudaMalloc,
// and cudaMalloc / cudaFree synchronise the whole device, stalling whatever
// else runs on it).
//
// Capacity: 4 partial blocks per SM for up to 256 SMs, i.e. NRED * 1024 +
// 1024 + NRED + 1 = 10,250 doubles (80 KiB).  A device with more SMs is
// rejected with MFLBM_E_ARG.  One copy exists per device, shared by every
// context on that device; nothing in it needs clearing, because each call
// writes every element before it reads it.
// ---------------------------------------------------------------------------
constexpr int kNoallocBlocksMax = 4 * 256;
constexpr ll kNoallocScratch = (ll)NRED * kNoallocBlocksMax + kNoallocBlocksMax + NRED + 1;
static __device__ __align__(256) double g_monitor_scratch[kNoallocScratch];

// Device address of g_monitor_scratch on the current device.  The first
// lookup on a device may load the library's device code there.  The address
// is looked up on every call rather than cached: a cudaDeviceReset unloads
// the module, and the next load may place the array elsewhere.
int noalloc_scratch(double** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_monitor_scratch);
    if (e != cudaSuccess)
        return fail(MFLBM_E_CUDA, std::string("mflbm_monitor_reduce_noalloc: cudaGetSymbolAddress: ") +
                                      cudaGetErrorString(e));
    *out = (double*)p;
    return MFLBM_OK;
}

// mflbm_monitor_reduce_noalloc: the same launches with the partials in
// g_monitor_scratch.
template <class T, class E>
int monitor_noalloc_t(mflbm_context& c, int nex_in, int nex_out, mflbm_monitor* out) {
    const int blocks = monitor_blocks(c.d);
    const ll need = monitor_scratch_len(blocks);
    if (need > kNoallocScratch)
        return fail(MFLBM_E_ARG, "mflbm_monitor_reduce_noalloc: " + std::to_string(c.d.n_sm) + " SMs need " +
                                     std::to_string(need) + " doubles of scratch, the static array holds " +
                                     std::to_string(kNoallocScratch) + " (at most 256 SMs)");
    double* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc != MFLBM_OK) return rc;
    return monitor_into<T, E>(c, nex_in, nex_out, scratch, blocks, out);
}

// ---------------------------------------------------------------------------
// Per-slice monitor profiles and the other monitor scalars (FP64),
// src/Monitor.cpp:17-104 (profiles, kinetic energy), :277-351 (phase-field
// steady state), :355-441 (capillary-pressure steady state), :447-466
// (breakthrough).  One block per layer of population tiles (SZ = 2 << lz
// slices; the fluid list is in tile order, hence tile-layer major): every
// sum is taken in a fixed order, so results repeat exactly.  Thresholds
// compare phi in the solver precision, as the reference.
// ---------------------------------------------------------------------------
constexpr int kProfSums = 7, kProfExt = 9;  // ext: umax2 usq1 usq2 pre_w pre_nw n_w n_nw breakthrough dphi_max

template <class T, class E, int SZ>
__global__ void __launch_bounds__(256) monitor_profile_kernel(Grid g, PopView<T, E> P, const uint32_t* list, const int* zoff,
                                                              const T* phi, T* phi_prev,
                                                              const typename Vec4<T>::type* aux, const int8_t* iface,
                                                              double force_z, int track, double* out) {
    constexpr int NACC = SZ * kProfSums + kProfExt;
    const int kp = blockIdx.x;
    double acc[NACC];
#pragma unroll
    for (int r = 0; r < NACC; ++r) acc[r] = 0.0;
    double* ext = acc + SZ * kProfSums;
    for (int t = zoff[kp] + threadIdx.x; t < zoff[kp + 1]; t += blockDim.x) {
        int i, j, k;
        unpack_xyz(list[t], i, j, k);
        double f[19];
#pragma unroll
        for (int q = 0; q < 19; ++q) f[q] = (double)P.get(i, j, k, q, 0) + (double)P.get(i, j, k, q, 1);
        double rho = 0;
#pragma unroll
        for (int q = 0; q < 19; ++q) rho += f[q];
        typename Vec4<T>::type a;
        a.x = T(0); a.y = T(0); a.z = T(0); a.w = T(0);
        if (iface[g.s2(i, j, k)]) a = aux[t];   // the zero record away from interfaces
        const double tmp = (double)a.w;
        const double fx = tmp * (double)a.x, fy = tmp * (double)a.y, fz = tmp * (double)a.z + force_z;
        const double u = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14] - 0.5 * fx;
        const double v = f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18] - 0.5 * fy;
        const double w = f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18] - 0.5 * fz;
        const ll n4 = g.s4(i, j, k);
        const T ph = phi[n4];
        const double pd = (double)ph, a1 = 0.5 * (1.0 + pd), a2 = 0.5 * (1.0 - pd);
        double* sl = acc + (k & (SZ - 1)) * kProfSums;
        sl[0] += w * a1; sl[1] += w * a2; sl[2] += a1; sl[3] += a2;
        sl[4] += rho * a1; sl[5] += rho * a2; sl[6] += rho;
        const double u2 = u * u + v * v + w * w;
        ext[0] = fmax(ext[0], u2);
        if (ph > T(0.999)) ext[1] += u2;
        else if (ph < T(-0.999)) ext[2] += u2;
        if (ph < T(-0.99)) { ext[3] += rho; ext[5] += 1.0; }
        if (ph > T(0.99)) { ext[4] += rho; ext[6] += 1.0; }
        if (k == g.nz - 1 && ph > T(0)) ext[7] += 1.0;
        if (track) {
            ext[8] = fmax(ext[8], fabs(pd - (double)phi_prev[n4]));
            phi_prev[n4] = ph;
        }
    }
    __shared__ double sh[NACC][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < NACC; ++r) {
        const bool is_max = r == SZ * kProfSums || r == SZ * kProfSums + 8;
        double x = acc[r];
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_down_sync(0xffffffffu, x, o);
            x = is_max ? fmax(x, y) : x + y;
        }
        if (lane == 0) sh[r][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x < NACC) {
        const int r = threadIdx.x;
        const bool is_max = r == SZ * kProfSums || r == SZ * kProfSums + 8;
        double x = sh[r][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) x = is_max ? fmax(x, sh[r][w]) : x + sh[r][w];
        out[(ll)kp * NACC + r] = x;
    }
}

template <class T, class E>
int monitor_profile_t(mflbm_context& c, double* slices, mflbm_monitor_ext* ext, bool track) {
    DeviceState& d = c.d;
    const Grid g = d.g;
    const int lz = d.b.lz, sz = 2 << lz;   // slices per tile layer
    if (lz > 1) return fail(MFLBM_E_STATE, "monitor profile: tiles of more than 2 brick layers");
    const int nb = d.b.ntz, per = sz * kProfSums + kProfExt;
    if (d.prof_len < (ll)nb * per) {
        if (d.prof) cudaFree(d.prof);
        d.prof = nullptr;
        d.prof_len = 0;
        MFLBM_CUDA(cudaMalloc(&d.prof, sizeof(double) * nb * per));
        d.prof_len = (ll)nb * per;
    }
    if (track && !d.phi_prev) {
        MFLBM_CUDA(cudaMalloc(&d.phi_prev, sizeof(T) * g.n4()));
        MFLBM_CUDA(cudaMemsetAsync(d.phi_prev, 0, sizeof(T) * g.n4(), c.stream));
    }
#define MFLBM_PROFILE(SZ)                                                                                         \
    monitor_profile_kernel<T, E, SZ><<<nb, 256, 0, c.stream>>>(g, pop_view<T, E>(d), d.fluid_list, d.zpair_off,  \
                                                            (const T*)d.phi, (T*)d.phi_prev,                     \
                                                            (const typename Vec4<T>::type*)d.aux, d.iface,       \
                                                            (double)T(c.params.force_z), track ? 1 : 0, d.prof)
    if (lz == 0) MFLBM_PROFILE(2);
    else MFLBM_PROFILE(4);
#undef MFLBM_PROFILE
    int rc = after_launch("monitor_profile");
    if (rc != MFLBM_OK) return rc;
    std::vector<double> h((size_t)nb * per);
    MFLBM_CUDA(cudaMemcpyAsync(h.data(), d.prof, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c.stream));
    MFLBM_CUDA(cudaStreamSynchronize(c.stream));
    for (int m = 0; m < kProfSums; ++m)
        for (int k = 1; k <= g.nz; ++k)
            slices[(size_t)m * g.nz + k - 1] = h[(size_t)(k / sz) * per + (k % sz) * kProfSums + m];
    if (ext) {
        double e[kProfExt] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int kp = 0; kp < nb; ++kp)
            for (int r = 0; r < kProfExt; ++r) {
                const double x = h[(size_t)kp * per + sz * kProfSums + r];
                e[r] = (r == 0 || r == 8) ? std::max(e[r], x) : e[r] + x;
            }
        ext->umax2 = e[0]; ext->usq1 = e[1]; ext->usq2 = e[2];
        ext->pre_w = e[3]; ext->pre_nw = e[4];
        ext->n_w = (long long)e[5]; ext->n_nw = (long long)e[6];
        ext->breakthrough = (long long)e[7];
        ext->dphi_max = e[8];
    }
    return MFLBM_OK;
}

// Populations moved from one tile shape to another, element by element
// without decoding (16-bit storage keeps its stored bits), one thread per
// (node, direction) of [0, n+1]^3.
template <class P2>
__global__ void relayout_kernel(Grid g, Bricks from, Bricks to, const P2* src, P2* dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, kq = blockIdx.z;
    const int k = kq % (g.nz + 2), q = kq / (g.nz + 2);
    if (i > g.nx + 1) return;
    dst[to.elem(i, j, k) + (ll)q * to.tile] = src[from.elem(i, j, k) + (ll)q * from.tile];
}

int relayout_impl(mflbm_context& c, const Bricks& to, void** out) {
    DeviceState& d = c.d;
    const Grid g = d.g;
    const size_t pair = c.params.storage != MFLBM_STORE_NATIVE ? 4 : (c.params.precision == MFLBM_FP32 ? 8 : 16);
    void* dst = nullptr;
    MFLBM_CUDA(cudaMalloc(&dst, pair * (size_t)to.pairs()));
    MFLBM_CUDA(cudaMemsetAsync(dst, 0, pair * (size_t)to.pairs(), c.stream));
    const dim3 grid(grid_for(g.nx + 2, 128), g.ny + 2, (unsigned)((g.nz + 2) * 19));
    if (pair == 4) relayout_kernel<uint32_t><<<grid, 128, 0, c.stream>>>(g, d.b, to, (const uint32_t*)d.pdf, (uint32_t*)dst);
    else if (pair == 8) relayout_kernel<uint2><<<grid, 128, 0, c.stream>>>(g, d.b, to, (const uint2*)d.pdf, (uint2*)dst);
    else relayout_kernel<uint4><<<grid, 128, 0, c.stream>>>(g, d.b, to, (const uint4*)d.pdf, (uint4*)dst);
    const int rc = after_launch("relayout");
    if (rc != MFLBM_OK) {
        cudaFree(dst);
        return rc;
    }
    *out = dst;
    return MFLBM_OK;
}

// Collision records gathered into a new fluid-list order: dst[t] = src[perm[t]].
template <class V>
__global__ void gather_records(const V* src, const int* perm, V* dst, ll n) {
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = src[perm[t]];
}

int permute_impl(mflbm_context& c, const int* perm_dev, void** out) {
    DeviceState& d = c.d;
    const ll n = std::max<ll>(1, d.n_fluid);
    const size_t rec = (c.params.precision == MFLBM_FP32 ? 4 : 8) * 4;
    void* dst = nullptr;
    MFLBM_CUDA(cudaMalloc(&dst, rec * n));
    if (d.n_fluid > 0) {
        if (c.params.precision == MFLBM_FP32)
            gather_records<float4><<<grid_for(d.n_fluid, 256), 256, 0, c.stream>>>((const float4*)d.aux, perm_dev, (float4*)dst, d.n_fluid);
        else
            gather_records<Double4><<<grid_for(d.n_fluid, 256), 256, 0, c.stream>>>((const Double4*)d.aux, perm_dev, (Double4*)dst, d.n_fluid);
        const int rc = after_launch("gather_records");
        if (rc != MFLBM_OK) {
            cudaFree(dst);
            return rc;
        }
    }
    *out = dst;
    return MFLBM_OK;
}

// Reference layout (f1) <-> brick layout, one thread per (node, direction).
// f1 is the staging buffer, or page-locked host memory that the kernel reads
// or writes over the host link directly.
template <class T, class E>
__global__ void f1_to_bricks(Grid g, PopView<T, E> P, const T* f1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, kq = blockIdx.z;
    const int k = kq % (g.nz + 2), q = kq / (g.nz + 2);
    if (i > g.nx + 1) return;
    const ll s = g.s1(i, j, k);
    P.set(i, j, k, q, 0, f1[s + g.n1() * q]);
    P.set(i, j, k, q, 1, f1[s + g.n1() * (q + 19)]);
}
template <class T, class E>
__global__ void bricks_to_f1(Grid g, PopView<T, E> P, T* f1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, kq = blockIdx.z;
    const int k = kq % (g.nz + 2), q = kq / (g.nz + 2);
    if (i > g.nx + 1) return;
    const ll s = g.s1(i, j, k);
    f1[s + g.n1() * q] = P.get(i, j, k, q, 0);
    f1[s + g.n1() * (q + 19)] = P.get(i, j, k, q, 1);
}

template <class T, class E>
int convert_t(mflbm_context& c, bool to_bricks, void* f1) {
    DeviceState& d = c.d;
    const Grid g = d.g;
    const dim3 grid(grid_for(g.nx + 2, 128), g.ny + 2, (g.nz + 2) * 19);
    T* src = (T*)(f1 ? f1 : d.staging);
    if (to_bricks) f1_to_bricks<T, E><<<grid, 128, 0, c.stream>>>(g, pop_view<T, E>(d), src);
    else bricks_to_f1<T, E><<<grid, 128, 0, c.stream>>>(g, pop_view<T, E>(d), src);
    return after_launch(to_bricks ? "f1_to_bricks" : "bricks_to_f1");
}

}  // namespace

// the population storage selects the element type E of the kernels that touch them
#define MFLBM_POP(fn, ...)                                                             \
    (c.params.precision == MFLBM_FP64         ? fn<double, double>(__VA_ARGS__)         \
     : c.params.storage == MFLBM_STORE_F16    ? fn<float, __half>(__VA_ARGS__)          \
     : c.params.storage == MFLBM_STORE_BF16   ? fn<float, __nv_bfloat16>(__VA_ARGS__)   \
                                              : fn<float, float>(__VA_ARGS__))

int convert_populations(mflbm_context& c, bool to_bricks, void* f1) { return MFLBM_POP(convert_t, c, to_bricks, f1); }
int relayout_populations(mflbm_context& c, const Bricks& to, void** out) { return relayout_impl(c, to, out); }
int permute_records(mflbm_context& c, const int* perm_dev, void** out) { return permute_impl(c, perm_dev, out); }

int preprocess_geometry(mflbm_context& c, const int32_t* walls_global, int iper) {
    return c.params.precision == MFLBM_FP32 ? preprocess_geometry_t<float>(c, walls_global, iper)
                                            : preprocess_geometry_t<double>(c, walls_global, iper);
}

int init_fields(mflbm_context& c, int option, double z0) { return MFLBM_POP(init_fields_t, c, option, z0); }
int init_flow(mflbm_context& c, const void* rho, const void* u, const void* v, const void* w, int mrt) {
    return MFLBM_POP(init_flow_t, c, rho, u, v, w, mrt);
}
int init_flow_predicted(mflbm_context& c, const float* y, double nu, double g, const float* scales, int mrt,
                        void* work) {
    return MFLBM_POP(init_flow_predicted_t, c, y, nu, g, scales, mrt, work);
}

int monitor(mflbm_context& c, int nex_in, int nex_out, mflbm_monitor* out) {
    return MFLBM_POP(monitor_t, c, nex_in, nex_out, out);
}

int monitor_profile(mflbm_context& c, double* slices, mflbm_monitor_ext* ext, bool track_phi) {
    return MFLBM_POP(monitor_profile_t, c, slices, ext, track_phi);
}

int monitor_noalloc(mflbm_context& c, int nex_in, int nex_out, mflbm_monitor* out) {
    return MFLBM_POP(monitor_noalloc_t, c, nex_in, nex_out, out);
}

}  // namespace mflbm
