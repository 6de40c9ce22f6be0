// Internal definitions shared by every translation unit of libmflbm.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/mflbm.h"

struct mflbm_context;

namespace mflbm {

// ---------------------------------------------------------------------------
// D3Q19 (the reference's ex/ey/ez/opc tables, includes/Module.h:98-101).
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int ex(int q) {
    return (q == 1 || q == 7 || q == 9 || q == 11 || q == 13) ? 1
         : (q == 2 || q == 8 || q == 10 || q == 12 || q == 14) ? -1 : 0;
}
__host__ __device__ constexpr int ey(int q) {
    return (q == 3 || q == 7 || q == 8 || q == 15 || q == 17) ? 1
         : (q == 4 || q == 9 || q == 10 || q == 16 || q == 18) ? -1 : 0;
}
__host__ __device__ constexpr int ez(int q) {
    return (q == 5 || q == 11 || q == 12 || q == 15 || q == 16) ? 1
         : (q == 6 || q == 13 || q == 14 || q == 17 || q == 18) ? -1 : 0;
}
__host__ __device__ constexpr int opp(int q) {
    return q == 0 ? 0 : (q <= 6 ? ((q & 1) ? q + 1 : q - 1)
                       : (q <= 10 ? 17 - q : (q <= 14 ? 25 - q : 33 - q)));
}

typedef long long ll;

// ---------------------------------------------------------------------------
// Padded, 1-based layouts of the reference (includes/Idx_gpu.cuh:54-70).
// ---------------------------------------------------------------------------
struct Grid {
    int nx, ny, nz;
    __host__ __device__ ll s0(ll x, ll y, ll z) const { return (x - 1) + (ll)nx * ((y - 1) + (ll)ny * (z - 1)); }
    __host__ __device__ ll s1(ll x, ll y, ll z) const { return x + (ll)(nx + 2) * (y + (ll)(ny + 2) * z); }
    __host__ __device__ ll s2(ll x, ll y, ll z) const { return (x + 1) + (ll)(nx + 4) * ((y + 1) + (ll)(ny + 4) * (z + 1)); }
    __host__ __device__ ll s4(ll x, ll y, ll z) const { return (x + 3) + (ll)(nx + 8) * ((y + 3) + (ll)(ny + 8) * (z + 3)); }
    __host__ __device__ ll f1(ll x, ll y, ll z, int e, int g) const { return s1(x, y, z) + n1() * (ll)(e + 19 * g); }
    __host__ __device__ ll cnv(ll x, ll y, int e) const { return x + (ll)(nx + 2) * (y + (ll)(ny + 2) * e); }
    __host__ __device__ ll n0() const { return (ll)nx * ny * nz; }
    __host__ __device__ ll n1() const { return (ll)(nx + 2) * (ny + 2) * (nz + 2); }
    __host__ __device__ ll n2() const { return (ll)(nx + 4) * (ny + 4) * (nz + 4); }
    __host__ __device__ ll n4() const { return (ll)(nx + 8) * (ny + 8) * (nz + 8); }
    __host__ __device__ ll plane1() const { return (ll)(nx + 2) * (ny + 2); }
};

// Internal population layout.  The lattice [0, n+1]^3 is cut into 2x2x2
// bricks; the 8 nodes of a brick are consecutive (bit 0 = x parity, bit 1 =
// y parity, bit 2 = z parity) and each slot holds both components (g = 0, 1)
// side by side, so one 64-byte DRAM burst (FP32) holds one brick of one
// direction.  Bricks are grouped into tiles of 2^lx x 2^ly x 2^lz bricks;
// a tile stores its 19 directions one after the other (direction q of the
// tile: TILE = 8 * 2^(lx+ly+lz) consecutive pairs, bricks x-fastest inside),
// and tiles are stored x-fastest.  A node's pulls and pushes then stay in its
// own tile's few tens of kilobytes for most directions (the odd step's
// neighbours across a z layer of bricks included when lz >= 1), instead of
// 19 arrays a slot-size apart.
//
// The pair index of (node, direction q) is ax(x) + ay(y) + az(z) + q * TILE:
// separable per axis, so a thread forms its 27 neighbour addresses from
// three values per axis.
struct Bricks {
    int nbx, nby, nbz;      // bricks per axis (cover [0, n+1])
    int lx, ly, lz;         // log2 of the tile extent in bricks
    int ntx, nty, ntz;      // tiles per axis
    ll tile;                // pairs per direction of a tile (8 << (lx + ly + lz))
    ll S;                   // pairs per direction over all tiles (padding included)
    __host__ __device__ ll ax(int x) const {
        const int b = x >> 1;
        return (ll)(b >> lx) * (19 * tile) + ((b & ((1 << lx) - 1)) << 3) + (x & 1);
    }
    __host__ __device__ ll ay(int y) const {
        const int b = y >> 1;
        return (ll)(b >> ly) * (19 * tile) * ntx + ((b & ((1 << ly) - 1)) << (3 + lx)) + ((y & 1) << 1);
    }
    __host__ __device__ ll az(int z) const {
        const int b = z >> 1;
        return (ll)(b >> lz) * (19 * tile) * ntx * nty + ((b & ((1 << lz) - 1)) << (3 + lx + ly)) + ((z & 1) << 2);
    }
    // pair index of direction 0 of node (x, y, z)
    __host__ __device__ ll elem(int x, int y, int z) const { return ax(x) + ay(y) + az(z); }
    // element index of component g of direction e of node (x, y, z)
    __host__ __device__ ll at(int x, int y, int z, int e, int g) const {
        return 2 * (elem(x, y, z) + (ll)e * tile) + g;
    }
    // pairs of the whole population array (19 directions)
    __host__ __device__ ll pairs() const { return 19 * S; }
};
// The tile extent used unless a tuning chooses another: 8 x 4 x 2 bricks
// (16 x 8 x 4 nodes).
constexpr int kTileLx = 3, kTileLy = 2, kTileLz = 1;
inline Bricks make_bricks(int nx, int ny, int nz, int lx = kTileLx, int ly = kTileLy, int lz = kTileLz) {
    Bricks b;
    b.nbx = (nx + 3) / 2;  // covers x in [0, nx+1]
    b.nby = (ny + 3) / 2;
    b.nbz = (nz + 3) / 2;
    b.lx = lx; b.ly = ly; b.lz = lz;
    b.ntx = (b.nbx + (1 << lx) - 1) >> lx;
    b.nty = (b.nby + (1 << ly) - 1) >> ly;
    b.ntz = (b.nbz + (1 << lz) - 1) >> lz;
    b.tile = (ll)8 << (lx + ly + lz);
    b.S = b.tile * b.ntx * b.nty * b.ntz;
    return b;
}

template <class T> struct Vec2;
template <> struct Vec2<float> { typedef float2 type; };
template <> struct Vec2<double> { typedef double2 type; };
struct __align__(32) Double4 { double x, y, z, w; };
template <class T> struct Vec4;
template <> struct Vec4<float> { typedef float4 type; };
template <> struct Vec4<double> { typedef Double4 type; };

// ---------------------------------------------------------------------------
// Population storage (mflbm_params.storage).  E is the stored element type:
// T itself, or __half / __nv_bfloat16 holding the shifted deviation
// s = g / w_q - 1 of the population g from its lattice weight w_q (decoded in
// T = float).  Pop2<E> is the pair (component 1, component 2) of one slot.
// ---------------------------------------------------------------------------
template <class E> struct Pop2;
template <> struct Pop2<float> { typedef float2 type; };
template <> struct Pop2<double> { typedef double2 type; };
template <> struct Pop2<__half> { typedef __half2 type; };
template <> struct Pop2<__nv_bfloat16> { typedef __nv_bfloat162 type; };

// enc rounds to nearest.  enc_dither rounds stochastically: to the upper of
// the two neighbouring 16-bit values with probability (x - lo) / (hi - lo),
// using r16 / 65536 as the uniform variate, so the stored value is unbiased
// (round-to-nearest would flush the small populations of a component near an
// interface to exactly zero, a systematic mass loss).  Exactly representable
// values, among them s = -1 of an absent component, are stored exactly.
template <class T, class E> struct PopCodec {  // native storage: identity
    __device__ __forceinline__ static T dec(E e, T, T) { return e; }
    __device__ __forceinline__ static E enc(T v, T, T) { return v; }
    __device__ __forceinline__ static E enc_dither(T v, T, T, uint32_t) { return v; }
};
template <> struct PopCodec<float, __half> {
    __device__ __forceinline__ static float dec(__half e, float w, float) { return w + w * __half2float(e); }
    __device__ __forceinline__ static __half enc(float v, float, float winv) { return __float2half_rn(v * winv - 1.0f); }
    // Stochastic rounding on the bits.  Half-normal range: a half keeps the
    // top 10 of the 23 mantissa bits; adding a 13-bit variate to the FP32
    // bits and truncating (rz) rounds the magnitude up with probability equal
    // to the dropped fraction (a carry into the exponent gives the next
    // binade's value).  Half-subnormal range (|x| < 2^-14, spacing 2^-24):
    // |x| * 2^40 (exact) plus a 16-bit variate, shifted down by 16, is the
    // subnormal's integer mantissa, which is also its bit pattern (1024 gives
    // 2^-14).  Both are formed and one is selected (values of a warp straddle
    // 2^-14, so a branch would run both anyway); at or above the largest half
    // the truncation saturates at 65504.
    __device__ __forceinline__ static __half enc_dither(float v, float, float winv, uint32_t r16) {
        const float x = v * winv - 1.0f;
        const uint32_t b = __float_as_uint(x), mag = b & 0x7fffffffu;
        const uint32_t t = (uint32_t)(__uint_as_float(min(mag, 0x387fffffu)) * 1099511627776.0f);
        const unsigned short hs = (unsigned short)(((b >> 16) & 0x8000u) | ((t + r16) >> 16));
        const unsigned short hn = __half_as_ushort(__float2half_rz(__uint_as_float(b + (r16 >> 3))));
        return __ushort_as_half(mag < 0x38800000u ? hs : hn);
    }
};
template <> struct PopCodec<float, __nv_bfloat16> {
    __device__ __forceinline__ static float dec(__nv_bfloat16 e, float w, float) { return w + w * __bfloat162float(e); }
    __device__ __forceinline__ static __nv_bfloat16 enc(float v, float, float winv) {
        return __float2bfloat16_rn(v * winv - 1.0f);
    }
    // Stochastic rounding on the bits: a BF16 is the top half of an FP32, so
    // adding a 16-bit variate to the magnitude and keeping the top half rounds
    // it up with probability equal to the dropped fraction.  Inf / NaN: round
    // to nearest.
    __device__ __forceinline__ static __nv_bfloat16 enc_dither(float v, float, float winv, uint32_t r16) {
        const float x = v * winv - 1.0f;
        const uint32_t b = __float_as_uint(x);
        if ((b & 0x7f800000u) == 0x7f800000u) return __float2bfloat16_rn(x);
        return __ushort_as_bfloat16((unsigned short)((b + r16) >> 16));
    }
};
// integer hash for the dither (a 32-bit avalanche mixer)
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
// lattice weight of direction q and its inverse, in T
template <class T> __device__ __forceinline__ T lat_w(int q) { return q == 0 ? T(1) / T(3) : (q < 7 ? T(1) / T(18) : T(1) / T(36)); }
template <class T> __device__ __forceinline__ T lat_winv(int q) { return q == 0 ? T(3) : (q < 7 ? T(18) : T(36)); }

// Element-wise access to the populations in the brick layout.
template <class T, class E> struct PopView {
    E* p;
    Bricks b;
    __device__ __forceinline__ T get(int x, int y, int z, int q, int g) const {
        return PopCodec<T, E>::dec(p[b.at(x, y, z, q, g)], lat_w<T>(q), lat_winv<T>(q));
    }
    __device__ __forceinline__ void set(int x, int y, int z, int q, int g, T v) const {
        p[b.at(x, y, z, q, g)] = PopCodec<T, E>::enc(v, lat_w<T>(q), lat_winv<T>(q));
    }
    // copy of a stored population between slots of equal weight (no decode / encode)
    __device__ __forceinline__ void copy(int x, int y, int z, int q, int g, int xs, int ys, int zs, int qs) const {
        p[b.at(x, y, z, q, g)] = p[b.at(xs, ys, zs, qs, g)];
    }
};

// Packed node coordinates of the node lists: x in bits 0-9, y 10-20, z 21-31,
// each stored with an offset of +4 so that ghost nodes down to -3 fit.
constexpr int PACK_OFF = 4;
__host__ __device__ inline uint32_t pack_xyz(int x, int y, int z) {
    return (uint32_t)(x + PACK_OFF) | ((uint32_t)(y + PACK_OFF) << 10) | ((uint32_t)(z + PACK_OFF) << 21);
}
__host__ __device__ inline void unpack_xyz(uint32_t p, int& x, int& y, int& z) {
    x = (int)(p & 1023u) - PACK_OFF;
    y = (int)((p >> 10) & 2047u) - PACK_OFF;
    z = (int)(p >> 21) - PACK_OFF;
}

// Model constants computed in T as the reference's host code computes them
// (includes/Module.h:104-126, includes/Fluid_multiphase.h:31-35).
template <class T> struct ModelConsts {
    T w0, w1, w2, rk2, iso4a, iso4b;
    T mrt_coef1, mrt_coef2, mrt_coef3, mrt_coef4, mrt_e2_coef1, mrt_e2_coef2, mrt_omega_xx;
};

// Physical parameters in the kernel precision.
template <class T> struct Phys {
    T gamma, force_z, nui1, nui2, beta, phi_inlet, sa_inject, uin_avg, relaxation, cos_theta, rho_in, rho_out;
    ModelConsts<T> c;
};

// ---------------------------------------------------------------------------
// Error handling.
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
void count_launch();

#define MFLBM_CUDA(call)                                                                     \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return ::mflbm::fail(MFLBM_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Count a launch and return its launch status as an MFLBM code.
inline int after_launch(const char* what) {
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(MFLBM_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return MFLBM_OK;
}

inline unsigned grid_for(ll n, int block) { return (unsigned)((n + block - 1) / block); }

// Programmatic dependent launch for the kernels of a time step.  A kernel
// launched by launch_pdl may be scheduled while the previous kernel of the
// stream is still running (its blocks are placed as the previous kernel's
// blocks retire, hiding the launch latency between the short dependent
// passes); it must call pdl_wait() before its first global memory access.
// pdl_wait returns once the previous kernel has completed and its writes are
// visible (griddepcontrol.wait; a no-op for a plain launch), then allows the
// next kernel to be scheduled.
__device__ __forceinline__ void pdl_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <class... KArgs, class... Args>
inline int launch_pdl(const char* what, void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s,
                      Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, args...);
    if (e != cudaSuccess) return fail(MFLBM_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return after_launch(what);
}

}  // namespace mflbm

namespace mflbm {

// Model constants and physical parameters in T, evaluated on the host with
// the reference's T_P arithmetic (includes/Module.h:104-126,
// includes/Fluid_multiphase.h:31-35).
template <class T>
inline ModelConsts<T> make_consts() {
    ModelConsts<T> c;
    c.w0 = T(1) / T(3);
    c.w1 = T(1) / T(18);
    c.w2 = T(1) / T(36);
    c.rk2 = T(1) / (T)sqrt((T)2) / T(36);
    c.iso4a = T(1) / T(6);
    c.iso4b = T(1) / T(12);
    c.mrt_coef1 = T(1) / T(19);
    c.mrt_coef2 = T(1) / T(2394);
    c.mrt_coef3 = T(1) / T(252);
    c.mrt_coef4 = T(1) / T(72);
    c.mrt_e2_coef1 = T(0);
    c.mrt_e2_coef2 = T(-475) / T(63);
    c.mrt_omega_xx = T(0);
    return c;
}

template <class T>
inline Phys<T> make_phys(const mflbm_params& p) {
    Phys<T> h;
    h.gamma = T(p.lbm_gamma);
    h.force_z = T(p.force_z);
    h.nui1 = T(p.la_nui1);
    h.nui2 = T(p.la_nui2);
    h.beta = T(p.lbm_beta);
    h.phi_inlet = T(p.phi_inlet);
    h.sa_inject = T(p.sa_inject);
    h.uin_avg = T(p.uin_avg);
    h.relaxation = T(p.relaxation);
    h.cos_theta = T(p.cos_theta);
    h.rho_in = T(p.rho_in);
    h.rho_out = T(p.rho_out);
    h.c = make_consts<T>();
    return h;
}

// One persistent run of a batch of single-phase samples (batch.cuh).
struct BatchLaunch {
    void* samples;               // device array of the flavour's per-sample records
    const int* pre;              // unit prefix sums, 2 phases x (n + 1)
    unsigned* bar;               // barrier words [arrivals, generation]
    int* error;                  // set when a barrier wait ran out
    unsigned long long limit_ns; // bound of one barrier wait
    int block, grid, ntime_begin, nsteps;
    cudaStream_t stream;
};

// Flavour entry points (step_fast.cu / step_strict.cu).
namespace fast {
int batch_persistent(mflbm_context* const* ctx, int n, const BatchLaunch& L);
int batch_grid(const mflbm_context& c, int block, int* grid);
size_t batch_sample_bytes(const mflbm_context& c);
int second_component(mflbm_context& c, int* flag_dev);
int refresh_aux(mflbm_context& c);
int export_arrays(mflbm_context& c);
int collide(mflbm_context& c, bool odd);
int boundaries(mflbm_context& c, bool odd);
int gradient(mflbm_context& c);
}
namespace strict {
int batch_persistent(mflbm_context* const* ctx, int n, const BatchLaunch& L);
int batch_grid(const mflbm_context& c, int block, int* grid);
size_t batch_sample_bytes(const mflbm_context& c);
int second_component(mflbm_context& c, int* flag_dev);
int refresh_aux(mflbm_context& c);
int export_arrays(mflbm_context& c);
int collide(mflbm_context& c, bool odd);
int boundaries(mflbm_context& c, bool odd);
int gradient(mflbm_context& c);
}

}  // namespace mflbm
