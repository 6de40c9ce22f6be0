// Collision + AA streaming of one time step (included by step_kernels.cuh).
#pragma once
#include <type_traits>

#include "context.cuh"

namespace mflbm {
namespace MFLBM_NS {

// ===========================================================================
// MRT collision (the reference's "original" rates, mrt == 2) with the CSF
// body force and Rothman-Keller recolouring for one fluid node
// (src/main_iteration_GPU.cu:115-345).  g1/g2 hold the 19 pre-collision
// populations of each component in direction order and receive the
// post-collision, recoloured ones; `force` is 0.5 * gamma * curv * c_norm
// (:147).  Returns the order parameter phi.
// ===========================================================================
template <class T>
__device__ __forceinline__ T collide(const Phys<T>& P, T (&g1)[19], T (&g2)[19], T cnx, T cny, T cnz, T force) {
    T f[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) f[q] = g1[q] + g2[q];
    T rho1 = g1[0], rho2 = g2[0];
#pragma unroll
    for (int q = 1; q < 19; ++q) rho1 = rho1 + g1[q];
#pragma unroll
    for (int q = 1; q < 19; ++q) rho2 = rho2 + g2[q];
    const T phi = (rho1 - rho2) / (rho1 + rho2);

    T tmp = force;  // 0.5 * gamma * curv * c_norm (:147)
    const T fx = tmp * cnx, fy = tmp * cny, fz = tmp * cnz + P.force_z;
    const T omega = T(1) / (T(6) / ((T(1) + phi) * P.nui1 + (T(1) - phi) * P.nui2) + T(0.5));
    const T s_nu = omega;
    constexpr T s_e = T(1.19), s_e2 = T(1.4), s_pi = T(1.4), s_q = T(1.2), s_t = T(1.98);

    const T den = rho1 + rho2;
    const T ux = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14] + T(0.5) * fx;
    const T uy = f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18] + T(0.5) * fy;
    const T uz = f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18] + T(0.5) * fz;
    const T u2 = ux * ux + uy * uy + uz * uz;

    // moments (Gram-Schmidt MRT basis of the reference)
    const T a1 = f[1] + f[2] + f[3] + f[4] + f[5] + f[6];
    const T a2 = f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14] + f[15] + f[16] + f[17] + f[18];
    const T a3 = f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
    const T a4 = f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18];
    const T a5 = f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18];
    const T a6 = T(2) * (f[1] + f[2]) - f[3] - f[4] - f[5] - f[6];
    const T a7 = f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14] - T(2) * (f[15] + f[16] + f[17] + f[18]);
    const T a8 = f[3] + f[4] - f[5] - f[6];
    const T a9 = f[7] + f[8] + f[9] + f[10] - f[11] - f[12] - f[13] - f[14];

    T m_e = T(-30) * f[0] - T(11) * a1 + T(8) * a2;
    T m_e2 = T(12) * f[0] - T(4) * a1 + a2;
    T m_jx = f[1] - f[2] + a3;
    T m_qx = T(-4) * (f[1] - f[2]) + a3;
    T m_jy = f[3] - f[4] + a4;
    T m_qy = T(-4) * (f[3] - f[4]) + a4;
    T m_jz = f[5] - f[6] + a5;
    T m_qz = T(-4) * (f[5] - f[6]) + a5;
    T m_3pxx = a6 + a7;
    T m_3pixx = T(-2) * a6 + a7;
    T m_pww = a8 + a9;
    T m_piww = T(-2) * a8 + a9;
    T m_pxy = f[7] - f[8] - f[9] + f[10];
    T m_pyz = f[15] - f[16] - f[17] + f[18];
    T m_pzx = f[11] - f[12] - f[13] + f[14];
    T m_tx = f[7] - f[8] + f[9] - f[10] - f[11] + f[12] - f[13] + f[14];
    T m_ty = -f[7] - f[8] + f[9] + f[10] + f[15] - f[16] + f[17] - f[18];
    T m_tz = f[11] + f[12] - f[13] - f[14] - f[15] - f[16] + f[17] + f[18];

    // relaxation with forcing in moment space
    constexpr T c23 = T(-0.666666666666666667), c13 = T(0.333333333333333333);
    const ModelConsts<T>& c = P.c;
    m_e = m_e - s_e * (m_e - (T(-11.0) * den + T(19.0) * u2)) + (T(38) - T(19) * s_e) * (fx * ux + fy * uy + fz * uz);
    m_e2 = m_e2 - s_e2 * (m_e2 - (c.mrt_e2_coef1 * den + c.mrt_e2_coef2 * u2)) + (T(-11) + T(5.5) * s_e2) * (fx * ux + fy * uy + fz * uz);
    m_jx = m_jx + fx;
    m_qx = m_qx - s_q * (m_qx - (c23 * ux)) + (c23 + c13 * s_q) * fx;
    m_jy = m_jy + fy;
    m_qy = m_qy - s_q * (m_qy - (c23 * uy)) + (c23 + c13 * s_q) * fy;
    m_jz = m_jz + fz;
    m_qz = m_qz - s_q * (m_qz - (c23 * uz)) + (c23 + c13 * s_q) * fz;
    m_3pxx = m_3pxx - s_nu * (m_3pxx - (T(3) * ux * ux - u2)) + (T(2) - s_nu) * (T(2) * fx * ux - fy * uy - fz * uz);
    m_3pixx = m_3pixx - s_pi * (m_3pixx - c.mrt_omega_xx * (T(3) * ux * ux - u2)) + (T(1) - T(0.5) * s_pi) * (T(-2) * fx * ux + fy * uy + fz * uz);
    m_pww = m_pww - s_nu * (m_pww - (uy * uy - uz * uz)) + (T(2) - s_nu) * (fy * uy - fz * uz);
    m_piww = m_piww - s_pi * (m_piww - c.mrt_omega_xx * (uy * uy - uz * uz)) + (T(1) - T(0.5) * s_pi) * (-fy * uy + fz * uz);
    m_pxy = m_pxy - s_nu * (m_pxy - (ux * uy)) + (T(1) - T(0.5) * s_nu) * (fx * uy + fy * ux);
    m_pyz = m_pyz - s_nu * (m_pyz - (uy * uz)) + (T(1) - T(0.5) * s_nu) * (fy * uz + fz * uy);
    m_pzx = m_pzx - s_nu * (m_pzx - (ux * uz)) + (T(1) - T(0.5) * s_nu) * (fx * uz + fz * ux);
    m_tx = m_tx - s_t * (m_tx);
    m_ty = m_ty - s_t * (m_ty);
    m_tz = m_tz - s_t * (m_tz);

    // back to populations
    const T m_rho = c.mrt_coef1 * den;
    m_e = c.mrt_coef2 * m_e;
    m_e2 = c.mrt_coef3 * m_e2;
    m_jx = T(0.1) * m_jx;
    m_qx = T(0.025) * m_qx;
    m_jy = T(0.1) * m_jy;
    m_qy = T(0.025) * m_qy;
    m_jz = T(0.1) * m_jz;
    m_qz = T(0.025) * m_qz;
    m_3pxx = T(2) * c.mrt_coef4 * m_3pxx;
    m_3pixx = c.mrt_coef4 * m_3pixx;
    m_pww = T(6) * c.mrt_coef4 * m_pww;
    m_piww = T(3) * c.mrt_coef4 * m_piww;
    m_pxy = T(0.25) * m_pxy;
    m_pyz = T(0.25) * m_pyz;
    m_pzx = T(0.25) * m_pzx;
    m_tx = T(0.125) * m_tx;
    m_ty = T(0.125) * m_ty;
    m_tz = T(0.125) * m_tz;
    const T b1 = m_rho - T(11) * m_e - T(4) * m_e2;
    const T b2 = T(2) * m_3pxx - T(4) * m_3pixx;
    const T b3 = m_pww - T(2) * m_piww;
    const T b4 = m_rho + T(8) * m_e + m_e2;
    const T b5 = m_jx + m_qx;
    const T b6 = m_jy + m_qy;
    const T b7 = m_jz + m_qz;
    const T b8 = m_3pxx + m_3pixx;
    const T b9 = m_pww + m_piww;

    f[0] = m_rho - T(30) * m_e + T(12) * m_e2;
    f[1] = b1 + m_jx - T(4) * m_qx + b2;
    f[2] = b1 - m_jx + T(4) * m_qx + b2;
    f[3] = b1 + m_jy - T(4) * m_qy - T(0.5) * b2 + b3;
    f[4] = b1 - m_jy + T(4) * m_qy - T(0.5) * b2 + b3;
    f[5] = b1 + m_jz - T(4) * m_qz - T(0.5) * b2 - b3;
    f[6] = b1 - m_jz + T(4) * m_qz - T(0.5) * b2 - b3;
    f[7] = b4 + b5 + b6 + b8 + b9 + m_pxy + m_tx - m_ty;
    f[8] = b4 - b5 + b6 + b8 + b9 - m_pxy - m_tx - m_ty;
    f[9] = b4 + b5 - b6 + b8 + b9 - m_pxy + m_tx + m_ty;
    f[10] = b4 - b5 - b6 + b8 + b9 + m_pxy - m_tx + m_ty;
    f[11] = b4 + b5 + b7 + b8 - b9 + m_pzx - m_tx + m_tz;
    f[12] = b4 - b5 + b7 + b8 - b9 - m_pzx + m_tx + m_tz;
    f[13] = b4 + b5 - b7 + b8 - b9 - m_pzx - m_tx - m_tz;
    f[14] = b4 - b5 - b7 + b8 - b9 + m_pzx + m_tx - m_tz;
    f[15] = b4 + b6 + b7 - b8 * T(2) + m_pyz + m_ty - m_tz;
    f[16] = b4 - b6 + b7 - b8 * T(2) - m_pyz - m_ty - m_tz;
    f[17] = b4 + b6 - b7 - b8 * T(2) - m_pyz + m_ty + m_tz;
    f[18] = b4 - b6 - b7 - b8 * T(2) + m_pyz - m_ty + m_tz;

    // Rothman-Keller recolouring (src/main_iteration_GPU.cu:302-345)
    const T frac1 = rho1 / den;
    g1[0] = frac1 * f[0];
    g2[0] = f[0] * (T(1) - frac1);
    tmp = rho1 * rho2 * P.beta / den;
    const T proj[19] = {T(0), cnx, -cnx, cny, -cny, cnz, -cnz,
                        cnx + cny, -cnx + cny, cnx - cny, -cnx - cny,
                        cnx + cnz, -cnx + cnz, cnx - cnz, -cnx - cnz,
                        cny + cnz, -cny + cnz, cny - cnz, -cny - cnz};
#pragma unroll
    for (int q = 1; q < 19; ++q) {
        const T wq = q < 7 ? c.w1 : c.rk2;
        g1[q] = frac1 * f[q] + wq * tmp * proj[q];
        g2[q] = f[q] - g1[q];
    }
    return phi;
}


// ===========================================================================
// Collision + AA streaming over the fluid-node list (tiled brick layout).
//   odd  step: populations pulled from slot q of node x - e_q, pushed to
//              slot opp(q) of node x + e_q (src/main_iteration_GPU.cu:75-113, 348-384)
//   even step: read from slot opp(q) of x, written to slot q of x (:414-452, 687-723)
// The pair index of a node is separable per axis (Bricks::ax/ay/az), so each
// thread forms three values per axis (x - 1, x, x + 1, ...) and every
// neighbour address is a sum of three of them.  I is the index type: 32-bit
// where the whole population array has fewer than 2^32 pairs.
// ===========================================================================
template <class T, class E> struct CollideArgs {
    typedef typename Pop2<E>::type P2;
    typedef typename Vec4<T>::type V4;
    P2* slot[19];   // direction q of tile 0: slot[q][i] is pair i + q * tile
    const uint32_t* list;
    int n;
    Bricks b;
    int NX4, NY4;
    T* phi;
    const V4* aux;  // fluid-list order: (n_x, n_y, n_z, 0.5 * gamma * curv * c_norm)
    const int8_t* iface;  // s2: the record is read only where 1 (elsewhere it is the zero record)
    int NX2, NY2;
    uint32_t* dither;  // step counter pair of stochastic rounding (16-bit storage)
    Phys<T> ph;
};

// Register budget per thread.  16-bit storage: 64 (32 warps per SM; the
// default allocation of the even step is 143-146 registers, 16 warps per SM;
// at 64 the collision takes 11-21 % less time at 256^3).  FP32: the allocation
// the compiler picks unbounded (64 even, 79 odd; capping the odd step at 64
// spills and runs 3 % slower).  FP64: unbounded.
template <class E, bool ODD> constexpr int collide_max_regs() {
    return sizeof(E) == 2 ? 64 : sizeof(E) == 4 ? (ODD ? 80 : 64) : 255;
}

// One fluid node of the list (entry t): pull, collide, push.
template <class T, class E, bool ODD, class I>
__device__ __forceinline__ void collide_node(const CollideArgs<T, E>& a, int t) {
    typedef typename Pop2<E>::type P2;
    typedef PopCodec<T, E> Codec;
    const uint32_t node = a.list[t];   // packed coordinates
    int x, y, z;
    unpack_xyz(node, x, y, z);
    const Bricks& B = a.b;
    I X1 = (I)B.ax(x), Y1 = (I)B.ay(y), Z1 = (I)B.az(z);
    const I e0 = X1 + Y1 + Z1;
    I X0 = 0, X2 = 0, Y0 = 0, Y2 = 0, Z0 = 0, Z2 = 0;
    if (ODD) {
        X0 = (I)B.ax(x - 1); X2 = (I)B.ax(x + 1);
        Y0 = (I)B.ay(y - 1); Y2 = (I)B.ay(y + 1);
        Z0 = (I)B.az(z - 1); Z2 = (I)B.az(z + 1);
    }
    auto nb = [&](int q) -> I {  // pair index (direction 0) of x + e_q
        return (ex(q) > 0 ? X2 : ex(q) < 0 ? X0 : X1) + (ey(q) > 0 ? Y2 : ey(q) < 0 ? Y0 : Y1) +
               (ez(q) > 0 ? Z2 : ez(q) < 0 ? Z0 : Z1);
    };
    T g1[19], g2[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const P2 v = ODD ? a.slot[q][nb(opp(q))] : a.slot[opp(q)][e0];
        g1[q] = Codec::dec(v.x, lat_w<T>(q), lat_winv<T>(q));
        g2[q] = Codec::dec(v.y, lat_w<T>(q), lat_winv<T>(q));
    }
    typename Vec4<T>::type av;
    av.x = T(0); av.y = T(0); av.z = T(0); av.w = T(0);
    if (a.iface[(x + 1) + a.NX2 * ((y + 1) + a.NY2 * (z + 1))]) av = a.aux[t];   // s2 index of (x, y, z)
    // dither seed of 16-bit storage: the node, the step counter and two
    // incoming populations, so that rounding directions are drawn afresh at
    // every step even in a steady flow (a state-only seed freezes them and
    // biases the steady state).  The odd kernel reads counter [0] and writes
    // [1] = [0] + 1, the even kernel the other way round: no word is read and
    // written by the same launch.
    uint32_t seed = 0;
    if (!std::is_same<T, E>::value) {
        const uint32_t step = a.dither[ODD ? 0 : 1];
        if (t == 0) a.dither[ODD ? 1 : 0] = step + 1u;
        seed = mix32(node ^ mix32(step * 0x9E3779B9u ^ __float_as_uint((float)g1[1]) ^
                                          mix32(__float_as_uint((float)g2[2]))));
    }
    const T phi = collide<T>(a.ph, g1, g2, av.x, av.y, av.z, av.w);
    if (ODD && std::is_same<E, __half>::value) {
        // FP16 storage: the push addresses are formed again from the packed
        // node, whose opaque copy is the one register kept live across the
        // collision instead of the nine per-axis terms (no spills at 64
        // registers; the FP32 odd step gains nothing from it, measured, and
        // the BF16 one spills more with it)
        uint32_t nd = node;
        asm volatile("" : "+r"(nd));
        unpack_xyz(nd, x, y, z);
        X1 = (I)B.ax(x); Y1 = (I)B.ay(y); Z1 = (I)B.az(z);
        X0 = (I)B.ax(x - 1); X2 = (I)B.ax(x + 1);
        Y0 = (I)B.ay(y - 1); Y2 = (I)B.ay(y + 1);
        Z0 = (I)B.az(z - 1); Z2 = (I)B.az(z + 1);
    }
    a.phi[(x + 3) + a.NX4 * ((y + 3) + a.NY4 * (z + 3))] = phi;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        P2 v;
        if (std::is_same<T, E>::value) {
            v.x = Codec::enc(g1[q], lat_w<T>(q), lat_winv<T>(q));
            v.y = Codec::enc(g2[q], lat_w<T>(q), lat_winv<T>(q));
        } else {
            // one multiply-xorshift round per direction over the node's seed
            uint32_t r = seed + (uint32_t)q * 0x9E3779B9u;
            r ^= r >> 16; r *= 0x7feb352du; r ^= r >> 15;
            v.x = Codec::enc_dither(g1[q], lat_w<T>(q), lat_winv<T>(q), r & 0xffffu);
            v.y = Codec::enc_dither(g2[q], lat_w<T>(q), lat_winv<T>(q), r >> 16);
        }
        if (ODD) a.slot[opp(q)][nb(q)] = v;
        else a.slot[q][e0] = v;
    }
}

template <class T, class E, bool ODD, class I>
__global__ void __launch_bounds__(256) __maxnreg__((collide_max_regs<E, ODD>())) collide_stream_kernel(const CollideArgs<T, E> a) {
    pdl_wait();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < a.n) collide_node<T, E, ODD, I>(a, t);
}

template <class T, class E>
CollideArgs<T, E> collide_args(const mflbm_context& c) {
    typedef typename Pop2<E>::type P2;
    const DeviceState& d = c.d;
    const Grid& g = d.g;
    CollideArgs<T, E> a;
    P2* pdf = (P2*)d.pdf;
    for (int q = 0; q < 19; ++q) a.slot[q] = pdf + d.b.tile * q;
    a.list = d.fluid_list;
    a.n = (int)d.n_fluid;
    a.b = d.b;
    a.NX4 = g.nx + 8; a.NY4 = g.ny + 8;
    a.phi = (T*)d.phi;
    a.aux = (const typename Vec4<T>::type*)d.aux;
    a.iface = d.iface;
    a.NX2 = g.nx + 4; a.NY2 = g.ny + 4;
    a.dither = d.dither;
    a.ph = make_phys<T>(c.params);
    return a;
}

template <class T, class E>
int launch_collide(mflbm_context& c, bool odd) {
    const DeviceState& d = c.d;
    const CollideArgs<T, E> a = collide_args<T, E>(c);
    if (a.n == 0) return MFLBM_OK;
    const int bs = d.tune.collide;
    const bool narrow = d.b.pairs() < (1ll << 32);   // 32-bit pair indices suffice
    const unsigned grid = grid_for(a.n, bs);
    if (narrow)
        return launch_pdl("collide_stream", odd ? collide_stream_kernel<T, E, true, uint32_t>
                                                : collide_stream_kernel<T, E, false, uint32_t>,
                          grid, bs, c.stream, a);
    return launch_pdl("collide_stream", odd ? collide_stream_kernel<T, E, true, unsigned long long>
                                            : collide_stream_kernel<T, E, false, unsigned long long>,
                      grid, bs, c.stream, a);
}

}  // namespace MFLBM_NS
}  // namespace mflbm
