// Kernels of one MF-LBM time step: AA-pattern collision+streaming, the
// colour-gradient / CSF / wetting pipeline and the boundary updates.
//
// This header is compiled twice: step_fast.cu (FMA contraction, the
// production flavour) and step_strict.cu (-fmad=false: every operation is
// the IEEE operation written here, in the reference's order, so the result
// is bit-identical to the reference's arithmetic).  MFLBM_NS names the
// flavour's namespace.
#pragma once
#ifndef MFLBM_NS
#error "define MFLBM_NS before including step_kernels.cuh"
#endif

#include "context.cuh"

namespace mflbm {
namespace MFLBM_NS {

// ===========================================================================
// Collision: MRT (reference's "original" rates, mrt == 2) with the CSF body
// force and Rothman-Keller recolouring for one fluid node
// (src/main_iteration_GPU.cu:115-345).  g1/g2 hold the 19 pre-collision
// populations of each component in direction order and receive the
// post-collision, recoloured ones.  Returns the order parameter phi.
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
// Collision + AA streaming over the fluid-node list (brick layout).
//   odd  step: populations pulled from slot q of node x - e_q, pushed to
//              slot opp(q) of node x + e_q (src/main_iteration_GPU.cu:75-113, 348-384)
//   even step: read from slot opp(q) of x, written to slot q of x (:414-452, 687-723)
// In the brick layout the element offset of a neighbour depends only on the
// parities of (x, y, z): each thread forms six deltas once and every access
// is slot_base + element.
// ===========================================================================
template <class T> struct CollideArgs {
    typedef typename Vec2<T>::type V2;
    typedef typename Vec4<T>::type V4;
    V2* slot[19];
    const uint32_t* list;
    int n;
    int bx8, bxy8;  // element strides of one brick step in y and z
    int nbx, nby;
    int NX4, NY4;
    T* phi;
    const V4* aux;
    Phys<T> ph;
};

template <class T>
__device__ __forceinline__ int brick_elem(const CollideArgs<T>& a, int x, int y, int z) {
    return (((x >> 1) + a.nbx * ((y >> 1) + a.nby * (z >> 1))) << 3) | (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
}

template <class T, bool ODD>
__global__ void __launch_bounds__(128) collide_stream_kernel(const CollideArgs<T> a) {
    typedef typename Vec2<T>::type V2;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n) return;
    int x, y, z;
    unpack_xyz(a.list[t], x, y, z);
    const int e0 = brick_elem(a, x, y, z);
    // element deltas of the +1 / -1 neighbour along each axis
    const int dxp = (x & 1) ? 7 : 1, dxm = (x & 1) ? -1 : -7;
    const int dyp = (y & 1) ? a.bx8 - 2 : 2, dym = (y & 1) ? -2 : 2 - a.bx8;
    const int dzp = (z & 1) ? a.bxy8 - 4 : 4, dzm = (z & 1) ? -4 : 4 - a.bxy8;
    auto delta = [&](int q) {
        return (ex(q) > 0 ? dxp : ex(q) < 0 ? dxm : 0) + (ey(q) > 0 ? dyp : ey(q) < 0 ? dym : 0) +
               (ez(q) > 0 ? dzp : ez(q) < 0 ? dzm : 0);
    };
    // delta(q) is the element offset of x + e_q; the offsets are not
    // antisymmetric (they depend on parity), so x - e_q is at delta(opp(q))
    T g1[19], g2[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const V2 v = ODD ? a.slot[q][e0 + delta(opp(q))] : a.slot[opp(q)][e0];
        g1[q] = v.x;
        g2[q] = v.y;
    }
    const typename Vec4<T>::type av = a.aux[e0];
    // aux.w = 0.5 * gamma * curv * c_norm, evaluated in that order by the gradient pass
    const T phi = collide<T>(a.ph, g1, g2, av.x, av.y, av.z, av.w);
    a.phi[(x + 3) + a.NX4 * ((y + 3) + a.NY4 * (z + 3))] = phi;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        V2 v;
        v.x = g1[q];
        v.y = g2[q];
        if (ODD) a.slot[opp(q)][e0 + delta(q)] = v;
        else a.slot[q][e0] = v;
    }
}

// ===========================================================================
// Colour-gradient pipeline (src/main_iteration_GPU.cu:732-1003), ranges of
// the reference launches (:2027-2054):
//   1. phi on solid boundary nodes (list, precomputed fluid-neighbour masks)
//   2. interface normal + |grad phi| on [-1, n+2]^3, with the geometrical
//      wetting applied in the same thread at fluid boundary nodes (the
//      wetting only reads its own node's values, so fusing it is exact)
//   3. normal on solid boundary nodes (list, masks)
//   4. curvature on [1, n]^3, plus the per-node record the collision reads
// ===========================================================================
template <class T> struct GradArgs {
    typedef typename Vec4<T>::type V4;
    Grid g;
    Bricks b;
    const int8_t* type8;
    const T *snx, *sny, *snz;
    T *phi, *cnx, *cny, *cnz, *cnorm, *curv;
    V4* aux;
    const uint2 *l_phi, *l_cn;
    int n_phi, n_cn;
    Phys<T> ph;
};

// ISO4 first derivatives along x, y, z of field F at flat index n of a padded
// array with strides (1, sy, sz), in the reference's operand order.
template <class T>
__device__ __forceinline__ T iso4_dx(const ModelConsts<T>& c, const T* F, int n, int sy, int sz) {
    return c.iso4a * (F[n + 1] - F[n - 1]) +
           c.iso4b * (F[n + 1 + sy] - F[n - 1 - sy] + F[n + 1 - sy] - F[n - 1 + sy] +
                      F[n + 1 + sz] - F[n - 1 - sz] + F[n + 1 - sz] - F[n - 1 + sz]);
}
template <class T>
__device__ __forceinline__ T iso4_dy(const ModelConsts<T>& c, const T* F, int n, int sy, int sz) {
    return c.iso4a * (F[n + sy] - F[n - sy]) +
           c.iso4b * (F[n + 1 + sy] - F[n - 1 - sy] + F[n - 1 + sy] - F[n + 1 - sy] +
                      F[n + sy + sz] - F[n - sy - sz] + F[n + sy - sz] - F[n - sy + sz]);
}
template <class T>
__device__ __forceinline__ T iso4_dz(const ModelConsts<T>& c, const T* F, int n, int sy, int sz) {
    return c.iso4a * (F[n + sz] - F[n - sz]) +
           c.iso4b * (F[n + 1 + sz] - F[n - 1 - sz] + F[n - 1 + sz] - F[n + 1 - sz] +
                      F[n + sy + sz] - F[n - sy - sz] + F[n - sy + sz] - F[n + sy - sz]);
}

template <class T> __device__ __forceinline__ T wq_of(const ModelConsts<T>& c, int q) { return q < 7 ? c.w1 : c.w2; }

// phi on solid boundary nodes = weighted mean over fluid neighbours (:732-755)
template <class T>
__global__ void __launch_bounds__(128) extrapolate_phi_kernel(const GradArgs<T> a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n_phi) return;
    const uint2 e = a.l_phi[t];
    int i, j, k;
    unpack_xyz(e.x, i, j, k);
    const int sy = a.g.nx + 8, sz = (a.g.nx + 8) * (a.g.ny + 8);
    const int n = (int)a.g.s4(i, j, k);
    T s = T(0), ws = T(0);
#pragma unroll
    for (int q = 1; q < 19; ++q) {
        if (e.y & (1u << q)) {
            s += a.phi[n + ex(q) + ey(q) * sy + ez(q) * sz] * wq_of(a.ph.c, q);
            ws += wq_of(a.ph.c, q);
        }
    }
    a.phi[n] = s / ws;
}

// geometrical wetting: secant iteration turning the interface normal towards
// the prescribed contact angle at a fluid boundary node (:809-878)
template <class T>
__device__ __forceinline__ void wetting(T cs, T nwx, T nwy, T nwz, T& cx, T& cy, T& cz) {
    const T local_eps = T(1e-6), lambda = T(0.5);
    T vcx0 = cx, vcy0 = cy, vcz0 = cz;
    T vcx1 = vcx0 - lambda * (vcx0 + nwx);
    T vcy1 = vcy0 - lambda * (vcy0 + nwy);
    T vcz1 = vcz0 - lambda * (vcz0 + nwz);
    T err0 = (nwx * vcx0 + nwy * vcy0 + nwz * vcz0) - cs;
    if (!((fabs(vcx0 + nwx) + fabs(vcy0 + nwy) + fabs(vcz0 + nwz) > local_eps ||
           fabs(vcx0 - nwx) + fabs(vcy0 - nwy) + fabs(vcz0 - nwz) > local_eps) &&
          err0 > local_eps))
        return;
    T err1 = (nwx * vcx1 + nwy * vcy1 + nwz * vcz1) - sqrt(vcx1 * vcx1 + vcy1 * vcy1 + vcz1 * vcz1) * cs;
    T inv = T(1) / (err1 - err0);
    T vcx2 = inv * (vcx0 * err1 - vcx1 * err0);
    T vcy2 = inv * (vcy0 * err1 - vcy1 * err0);
    T vcz2 = inv * (vcz0 * err1 - vcz1 * err0);
    T err2 = (nwx * vcx2 + nwy * vcy2 + nwz * vcz2) - sqrt(vcx2 * vcx2 + vcy2 * vcy2 + vcz2 * vcz2) * cs;
    if (err2 > local_eps) {
        for (int it = 2; it <= 4; ++it) {
            vcx0 = vcx1; vcy0 = vcy1; vcz0 = vcz1;
            vcx1 = vcx2; vcy1 = vcy2; vcz1 = vcz2;
            err0 = (nwx * vcx0 + nwy * vcy0 + nwz * vcz0) - sqrt(vcx0 * vcx0 + vcy0 * vcy0 + vcz0 * vcz0) * cs;
            err1 = (nwx * vcx1 + nwy * vcy1 + nwz * vcz1) - sqrt(vcx1 * vcx1 + vcy1 * vcy1 + vcz1 * vcz1) * cs;
            inv = T(1) / (err1 - err0);
            if (isinf(inv)) break;
            vcx2 = inv * (vcx0 * err1 - vcx1 * err0);
            vcy2 = inv * (vcy0 * err1 - vcy1 * err0);
            vcz2 = inv * (vcz0 * err1 - vcz1 * err0);
            err2 = (nwx * vcx2 + nwy * vcy2 + nwz * vcz2) - sqrt(vcx2 * vcx2 + vcy2 * vcy2 + vcz2 * vcz2) * cs;
        }
    }
    inv = T(1) / (T(1e-30) + sqrt(vcx2 * vcx2 + vcy2 * vcy2 + vcz2 * vcz2));
    cx = vcx2 * inv; cy = vcy2 * inv; cz = vcz2 * inv;
}

// unit interface normal and |grad phi| on [-1, n+2]^3 (:757-807) + wetting (:809-878)
template <class T>
__global__ void __launch_bounds__(128) normals_kernel(const GradArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = (int)blockIdx.y - 1, k = (int)blockIdx.z - 1;
    const Grid& g = a.g;
    if (i > g.nx + 2) return;
    const int sy4 = g.nx + 8, sz4 = (g.nx + 8) * (g.ny + 8);
    const int n4 = (int)g.s4(i, j, k);
    const T x = iso4_dx(a.ph.c, a.phi, n4, sy4, sz4);
    const T y = iso4_dy(a.ph.c, a.phi, n4, sy4, sz4);
    const T z = iso4_dz(a.ph.c, a.phi, n4, sy4, sz4);
    const T nrm = sqrt(x * x + y * y + z * z);
    const int type = a.type8[n4];
    const int n2 = (int)g.s2(i, j, k);
    if (nrm < T(1e-6) || type >= 1) {
        a.cnx[n2] = T(0); a.cny[n2] = T(0); a.cnz[n2] = T(0); a.cnorm[n2] = T(0);
        return;
    }
    T cx = x / nrm, cy = y / nrm, cz = z / nrm;
    if (type == -1 && nrm > T(1e-6)) wetting(a.ph.cos_theta, a.snx[n4], a.sny[n4], a.snz[n4], cx, cy, cz);
    a.cnx[n2] = cx; a.cny[n2] = cy; a.cnz[n2] = cz; a.cnorm[n2] = nrm;
}

// interface normal on solid boundary nodes = weighted mean over fluid neighbours (:880-906)
template <class T>
__global__ void __launch_bounds__(128) extrapolate_normal_kernel(const GradArgs<T> a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n_cn) return;
    const uint2 e = a.l_cn[t];
    int i, j, k;
    unpack_xyz(e.x, i, j, k);
    const int sy = a.g.nx + 4, sz = (a.g.nx + 4) * (a.g.ny + 4);
    const int n = (int)a.g.s2(i, j, k);
    T sx = T(0), syy = T(0), szz = T(0), ws = T(0);
#pragma unroll
    for (int q = 1; q < 19; ++q) {
        if (e.y & (1u << q)) {
            const int m = n + ex(q) + ey(q) * sy + ez(q) * sz;
            const T wq = wq_of(a.ph.c, q);
            sx += a.cnx[m] * wq;
            syy += a.cny[m] * wq;
            szz += a.cnz[m] * wq;
            ws += wq;
        }
    }
    a.cnx[n] = sx / ws; a.cny[n] = syy / ws; a.cnz[n] = szz / ws;
}

// interface curvature from the nine derivatives of the normal (:908-1003);
// one thread per node of [1, n]^3 mapped brick by brick so the per-node
// record (n, 0.5*gamma*curv*c_norm) for the collision is written contiguously.
template <class T>
__global__ void __launch_bounds__(128) curvature_kernel(const GradArgs<T> a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.b.S) return;
    const int w = t & 7, brick = t >> 3;
    const int bx = brick % a.b.nbx, byz = brick / a.b.nbx;
    const int by = byz % a.b.nby, bz = byz / a.b.nby;
    const int i = 2 * bx + (w & 1), j = 2 * by + ((w >> 1) & 1), k = 2 * bz + (w >> 2);
    const Grid& g = a.g;
    if (i < 1 || i > g.nx || j < 1 || j > g.ny || k < 1 || k > g.nz) return;
    const int sy = g.nx + 4, sz = (g.nx + 4) * (g.ny + 4);
    const int n = (int)g.s2(i, j, k);
    const ModelConsts<T>& c = a.ph.c;
    const T kxx = iso4_dx(c, a.cnx, n, sy, sz), kyy = iso4_dy(c, a.cny, n, sy, sz), kzz = iso4_dz(c, a.cnz, n, sy, sz);
    const T kxy = iso4_dy(c, a.cnx, n, sy, sz), kxz = iso4_dz(c, a.cnx, n, sy, sz);
    const T kyx = iso4_dx(c, a.cny, n, sy, sz), kyz = iso4_dz(c, a.cny, n, sy, sz);
    const T kzx = iso4_dx(c, a.cnz, n, sy, sz), kzy = iso4_dy(c, a.cnz, n, sy, sz);
    const T x = a.cnx[n], y = a.cny[n], z = a.cnz[n];
    const T cv = (x * x - T(1)) * kxx + (y * y - T(1)) * kyy + (z * z - T(1)) * kzz +
                 x * y * (kxy + kyx) + x * z * (kxz + kzx) + y * z * (kzy + kyz);
    a.curv[g.s1(i, j, k)] = cv;
    typename Vec4<T>::type r;
    r.x = x; r.y = y; r.z = z;
    r.w = T(0.5) * a.ph.gamma * cv * a.cnorm[n];
    a.aux[t] = r;
}

// Per-node records (n, 0.5*gamma*curv*c_norm) from cn / c_norm / curv arrays
// that were uploaded from the host (same mapping as curvature_kernel).
template <class T>
__global__ void __launch_bounds__(128) aux_kernel(const GradArgs<T> a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.b.S) return;
    const int w = t & 7, brick = t >> 3;
    const int bx = brick % a.b.nbx, byz = brick / a.b.nbx;
    const int by = byz % a.b.nby, bz = byz / a.b.nby;
    const int i = 2 * bx + (w & 1), j = 2 * by + ((w >> 1) & 1), k = 2 * bz + (w >> 2);
    const Grid& g = a.g;
    if (i < 1 || i > g.nx || j < 1 || j > g.ny || k < 1 || k > g.nz) return;
    const int n = (int)g.s2(i, j, k);
    typename Vec4<T>::type r;
    r.x = a.cnx[n]; r.y = a.cny[n]; r.z = a.cnz[n];
    r.w = T(0.5) * a.ph.gamma * a.curv[g.s1(i, j, k)] * a.cnorm[n];
    a.aux[t] = r;
}

// ===========================================================================
// Boundary updates (src/main_iteration_GPU.cu:1009-1882).  One thread per
// (i, j) column (inlet / outlet / plate) or (i, k) row (periodic y).
// keep(new, old, w) is the reference's  new*(1-w) + old*w  blend.
// ===========================================================================
template <class T> struct BcArgs {
    Grid g;
    Bricks b;
    const int32_t* walls;
    T *pdf, *phi, *W_in, *f_cv, *g_cv, *phi_cv;
    Phys<T> ph;
    int plate_cmd, Zplate;
};

template <class T> __device__ __forceinline__ T keep(T v_new, T v_old, int w) { return v_new * T(1 - w) + v_old * T(w); }

template <class T>
__device__ __forceinline__ void inlet_phi(const BcArgs<T>& a, int i, int j, int w) {
    const Grid& g = a.g;
    a.phi[g.s4(i, j, 0)] = a.ph.phi_inlet * T(1 - w) + a.phi[g.s4(i, j, 0)] * T(w);
    const T v = a.phi[g.s4(i, j, 0)];
    a.phi[g.s4(i, j, -1)] = v;
    a.phi[g.s4(i, j, -2)] = v;
    a.phi[g.s4(i, j, -3)] = v;
}

// (dx, dy, slot at z=0 of (i+dx, j+dy), slot at z=1 of (i, j)) for the five links crossing z = 1/2
__device__ __constant__ const int kInlet[5][4] = {{0, 0, 5, 6}, {-1, 0, 11, 14}, {1, 0, 12, 13}, {0, -1, 15, 18}, {0, 1, 16, 17}};
// (dx, dy, slot at z=nz+1 of (i+dx, j+dy), slot at z=nz of (i, j), convective buffer slot)
__device__ __constant__ const int kOutlet[5][5] = {{0, 0, 6, 5, 6}, {-1, 0, 13, 12, 13}, {1, 0, 14, 11, 14}, {0, -1, 17, 16, 17}, {0, 1, 18, 15, 18}};

// velocity inlet: bounce-back plus 6 w rho u injection, split by sa_inject (:1009-1077)
template <class T, bool AFTER_ODD>
__global__ void inlet_velocity_kernel(const BcArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > a.g.nx) return;
    const Grid& g = a.g;
    const int w = a.walls[g.s2(i, j, 1)];
    inlet_phi(a, i, j, w);
    T t2 = a.W_in[g.s1(i, j, 0)] * a.ph.relaxation;
    const T t1 = t2 * a.ph.sa_inject;
    t2 = t2 - t1;
#pragma unroll
    for (int gg = 0; gg < 2; ++gg) {
        const T inj = gg == 0 ? t1 : t2;
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            const T wq = s == 0 ? a.ph.c.w1 : a.ph.c.w2;
            const int dx = kInlet[s][0], dy = kInlet[s][1], s0 = kInlet[s][2], s1 = kInlet[s][3];
            if (!AFTER_ODD) {
                T& d = a.pdf[a.b.at(i + dx, j + dy, 0, s0, gg)];
                d = keep((a.pdf[a.b.at(i, j, 1, s1, gg)] + T(6.0) * wq * inj), d, w);
            } else {
                T& d = a.pdf[a.b.at(i, j, 1, s1, gg)];
                d = keep((a.pdf[a.b.at(i + dx, j + dy, 0, s0, gg)] + T(6.0) * wq * inj), d, w);
            }
        }
    }
}

// Zou-He pressure inlet per component (:1085-1241)
template <class T, bool AFTER_ODD>
__global__ void inlet_pressure_kernel(const BcArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > a.g.nx) return;
    const Grid& g = a.g;
    const int w = a.walls[g.s2(i, j, 1)];
    inlet_phi(a, i, j, w);
    T r2 = a.ph.rho_in;
    const T r1 = a.ph.rho_in * a.ph.sa_inject;
    r2 = r2 - r1;
    const T c3 = T(0.333333333333333333), c6 = T(0.166666666666666667);
#pragma unroll
    for (int gg = 0; gg < 2; ++gg) {
        auto F = [&](int u, int v, int k, int e) -> T& { return a.pdf[a.b.at(u, v, k, e, gg)]; };
        const T rc = gg == 0 ? r1 : r2;
        if (!AFTER_ODD) {
            const T t = (rc - (F(i, j, 1, 0) + F(i - 1, j, 1, 1) + F(i + 1, j, 1, 2) + F(i, j - 1, 1, 3) +
                               F(i, j + 1, 1, 4) + F(i - 1, j - 1, 1, 7) + F(i + 1, j - 1, 1, 8) +
                               F(i - 1, j + 1, 1, 9) + F(i + 1, j + 1, 1, 10) +
                               T(2) * (F(i, j, 2, 6) + F(i + 1, j, 2, 14) + F(i - 1, j, 2, 13) +
                                       F(i, j + 1, 2, 18) + F(i, j - 1, 2, 17)))) * a.ph.relaxation;
            const T tnx = T(0.5) * (F(i - 1, j, 1, 1) + F(i - 1, j - 1, 1, 7) + F(i - 1, j + 1, 1, 9) -
                                    (F(i + 1, j, 1, 2) + F(i + 1, j - 1, 1, 8) + F(i + 1, j + 1, 1, 10)));
            const T tny = T(0.5) * (F(i, j - 1, 1, 3) + F(i - 1, j - 1, 1, 7) + F(i + 1, j - 1, 1, 8) -
                                    (F(i, j + 1, 1, 4) + F(i + 1, j + 1, 1, 10) + F(i - 1, j + 1, 1, 9)));
            F(i, j, 0, 5) = keep((F(i, j, 2, 6) + c3 * t), F(i, j, 0, 5), w);
            F(i - 1, j, 0, 11) = keep((F(i + 1, j, 2, 14) + c6 * t - tnx), F(i - 1, j, 0, 11), w);
            F(i + 1, j, 0, 12) = keep((F(i - 1, j, 2, 13) + c6 * t + tnx), F(i + 1, j, 0, 12), w);
            F(i, j - 1, 0, 15) = keep((F(i, j + 1, 2, 18) + c6 * t - tny), F(i, j - 1, 0, 15), w);
            F(i, j + 1, 0, 16) = keep((F(i, j - 1, 2, 17) + c6 * t + tny), F(i, j + 1, 0, 16), w);
        } else {
            const T t = (rc - (F(i, j, 1, 0) + F(i, j, 1, 2) + F(i, j, 1, 1) + F(i, j, 1, 4) + F(i, j, 1, 3) +
                               F(i, j, 1, 8) + F(i, j, 1, 7) + F(i, j, 1, 10) + F(i, j, 1, 9) +
                               T(2) * (F(i, j, 1, 5) + F(i, j, 1, 11) + F(i, j, 1, 12) + F(i, j, 1, 15) +
                                       F(i, j, 1, 16)))) * a.ph.relaxation;
            const T tnx = T(0.5) * (F(i, j, 1, 2) + F(i, j, 1, 8) + F(i, j, 1, 10) -
                                    (F(i, j, 1, 1) + F(i, j, 1, 7) + F(i, j, 1, 9)));
            const T tny = T(0.5) * (F(i, j, 1, 4) + F(i, j, 1, 9) + F(i, j, 1, 10) -
                                    (F(i, j, 1, 3) + F(i, j, 1, 8) + F(i, j, 1, 7)));
            F(i, j, 1, 6) = keep((F(i, j, 1, 5) + c3 * t), F(i, j, 1, 6), w);
            F(i, j, 1, 13) = keep((F(i, j, 1, 12) + c6 * t + tnx), F(i, j, 1, 13), w);
            F(i, j, 1, 14) = keep((F(i, j, 1, 11) + c6 * t - tnx), F(i, j, 1, 14), w);
            F(i, j, 1, 17) = keep((F(i, j, 1, 16) + c6 * t + tny), F(i, j, 1, 17), w);
            F(i, j, 1, 18) = keep((F(i, j, 1, 15) + c6 * t - tny), F(i, j, 1, 18), w);
        }
    }
}

// convective outflow with the previous-step buffers (:1246-1357)
template <class T, bool AFTER_ODD>
__global__ void outlet_convective_kernel(const BcArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > a.g.nx) return;
    const Grid& g = a.g;
    const int nz = g.nz;
    const T u = a.ph.uin_avg;
    const T temp = T(1) / (T(1) + u);
    const int w = a.walls[g.s2(i, j, nz)];
    T& pb = a.phi_cv[g.s1(i, j, 0)];
    a.phi[g.s4(i, j, nz + 1)] = ((pb + u * a.phi[g.s4(i, j, nz)]) * temp) * T(1 - w) + a.phi[g.s4(i, j, nz + 1)] * T(w);
    const T ph = a.phi[g.s4(i, j, nz + 1)];
    pb = ph;
    a.phi[g.s4(i, j, nz + 2)] = ph;
    a.phi[g.s4(i, j, nz + 3)] = ph;
    a.phi[g.s4(i, j, nz + 4)] = ph;
#pragma unroll
    for (int gg = 0; gg < 2; ++gg) {
        T* buf = gg == 0 ? a.f_cv : a.g_cv;
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            const int dx = kOutlet[s][0], dy = kOutlet[s][1], su = kOutlet[s][2], sd = kOutlet[s][3], sb = kOutlet[s][4];
            T& bv = buf[g.cnv(i, j, sb)];
            if (!AFTER_ODD) {
                T& d = a.pdf[a.b.at(i + dx, j + dy, nz + 1, su, gg)];
                d = ((bv + u * a.pdf[a.b.at(i + dx, j + dy, nz, su, gg)]) * temp) * T(1 - w) + d * T(w);
                bv = d;
            } else {
                T& d = a.pdf[a.b.at(i, j, nz, sd, gg)];
                d = ((bv + u * a.pdf[a.b.at(i, j, nz - 1, sd, gg)]) * temp) * T(1 - w) + d * T(w);
                bv = d;
            }
        }
    }
}

// Zou-He pressure outlet on the total density, flux split by phi (:1363-1524)
template <class T, bool AFTER_ODD>
__global__ void outlet_pressure_kernel(const BcArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > a.g.nx) return;
    const Grid& g = a.g;
    const int nz = g.nz;
    const int w = a.walls[g.s2(i, j, nz)];
    const T pz = a.phi[g.s4(i, j, nz)];
    a.phi[g.s4(i, j, nz + 1)] = pz;
    a.phi[g.s4(i, j, nz + 2)] = pz;
    a.phi[g.s4(i, j, nz + 3)] = pz;
    a.phi[g.s4(i, j, nz + 4)] = pz;
    auto F = [&](int u, int v, int k, int e, int gg) -> T& { return a.pdf[a.b.at(u, v, k, e, gg)]; };
    T t1;
    if (!AFTER_ODD) {
        t1 = (F(i, j, nz, 0, 0) + F(i - 1, j, nz, 1, 0) + F(i + 1, j, nz, 2, 0) + F(i, j - 1, nz, 3, 0) +
              F(i, j + 1, nz, 4, 0) + F(i - 1, j - 1, nz, 7, 0) + F(i + 1, j - 1, nz, 8, 0) +
              F(i - 1, j + 1, nz, 9, 0) + F(i + 1, j + 1, nz, 10, 0) +
              T(2) * (F(i, j, nz - 1, 5, 0) + F(i - 1, j, nz - 1, 11, 0) + F(i + 1, j, nz - 1, 12, 0) +
                      F(i, j - 1, nz - 1, 15, 0) + F(i, j + 1, nz - 1, 16, 0)) +
              F(i, j, nz, 0, 1) + F(i - 1, j, nz, 1, 1) + F(i + 1, j, nz, 2, 1) + F(i, j - 1, nz, 3, 1) +
              F(i, j + 1, nz, 4, 1) + F(i - 1, j - 1, nz, 7, 1) + F(i + 1, j - 1, nz, 8, 1) +
              F(i - 1, j + 1, nz, 9, 1) + F(i + 1, j + 1, nz, 10, 1) +
              T(2) * (F(i, j, nz - 1, 5, 1) + F(i - 1, j, nz - 1, 11, 1) + F(i + 1, j, nz - 1, 12, 1) +
                      F(i, j - 1, nz - 1, 15, 1) + F(i, j + 1, nz - 1, 16, 1))) - a.ph.rho_out;
    } else {
        t1 = (F(i, j, nz, 0, 0) + F(i, j, nz, 2, 0) + F(i, j, nz, 1, 0) + F(i, j, nz, 4, 0) + F(i, j, nz, 3, 0) +
              F(i, j, nz, 8, 0) + F(i, j, nz, 7, 0) + F(i, j, nz, 10, 0) + F(i, j, nz, 9, 0) +
              T(2) * (F(i, j, nz, 6, 0) + F(i, j, nz, 14, 0) + F(i, j, nz, 13, 0) + F(i, j, nz, 18, 0) +
                      F(i, j, nz, 17, 0)) +
              F(i, j, nz, 0, 1) + F(i, j, nz, 2, 1) + F(i, j, nz, 1, 1) + F(i, j, nz, 4, 1) + F(i, j, nz, 3, 1) +
              F(i, j, nz, 8, 1) + F(i, j, nz, 7, 1) + F(i, j, nz, 10, 1) + F(i, j, nz, 9, 1) +
              T(2) * (F(i, j, nz, 6, 1) + F(i, j, nz, 14, 1) + F(i, j, nz, 13, 1) + F(i, j, nz, 18, 1) +
                      F(i, j, nz, 17, 1))) - a.ph.rho_out;
    }
    const T t2 = t1 * T(0.5) * (T(1) - pz);
    t1 = t1 - t2;
    const T c3 = T(0.333333333333333333), c6 = T(0.166666666666666667);
#pragma unroll
    for (int gg = 0; gg < 2; ++gg) {
        const T t = gg == 0 ? t1 : t2;
        if (!AFTER_ODD) {
            const T tnx = T(0.5) * (F(i - 1, j, nz, 1, gg) + F(i - 1, j - 1, nz, 7, gg) + F(i - 1, j + 1, nz, 9, gg) -
                                    (F(i + 1, j, nz, 2, gg) + F(i + 1, j - 1, nz, 8, gg) + F(i + 1, j + 1, nz, 10, gg)));
            const T tny = T(0.5) * (F(i, j - 1, nz, 3, gg) + F(i - 1, j - 1, nz, 7, gg) + F(i + 1, j - 1, nz, 8, gg) -
                                    (F(i, j + 1, nz, 4, gg) + F(i + 1, j + 1, nz, 10, gg) + F(i - 1, j + 1, nz, 9, gg)));
            F(i, j, nz + 1, 6, gg) = keep((F(i, j, nz - 1, 5, gg) - c3 * t), F(i, j, nz + 1, 6, gg), w);
            F(i - 1, j, nz + 1, 13, gg) = keep((F(i + 1, j, nz - 1, 12, gg) - c6 * t - tnx), F(i - 1, j, nz + 1, 13, gg), w);
            F(i + 1, j, nz + 1, 14, gg) = keep((F(i - 1, j, nz - 1, 11, gg) - c6 * t + tnx), F(i + 1, j, nz + 1, 14, gg), w);
            F(i, j - 1, nz + 1, 17, gg) = keep((F(i, j + 1, nz - 1, 16, gg) - c6 * t - tny), F(i, j - 1, nz + 1, 17, gg), w);
            F(i, j + 1, nz + 1, 18, gg) = keep((F(i, j - 1, nz - 1, 15, gg) - c6 * t + tny), F(i, j + 1, nz + 1, 18, gg), w);
        } else {
            const T tnx = T(0.5) * (F(i, j, nz, 2, gg) + F(i, j, nz, 8, gg) + F(i, j, nz, 10, gg) -
                                    (F(i, j, nz, 1, gg) + F(i, j, nz, 7, gg) + F(i, j, nz, 9, gg)));
            const T tny = T(0.5) * (F(i, j, nz, 4, gg) + F(i, j, nz, 10, gg) + F(i, j, nz, 9, gg) -
                                    (F(i, j, nz, 3, gg) + F(i, j, nz, 7, gg) + F(i, j, nz, 8, gg)));
            F(i, j, nz, 5, gg) = keep((F(i, j, nz, 6, gg) - c3 * t), F(i, j, nz, 5, gg), w);
            F(i, j, nz, 11, gg) = keep((F(i, j, nz, 14, gg) - c6 * t + tnx), F(i, j, nz, 11, gg), w);
            F(i, j, nz, 12, gg) = keep((F(i, j, nz, 13, gg) - c6 * t - tnx), F(i, j, nz, 12, gg), w);
            F(i, j, nz, 15, gg) = keep((F(i, j, nz, 18, gg) - c6 * t + tny), F(i, j, nz, 15, gg), w);
            F(i, j, nz, 16, gg) = keep((F(i, j, nz, 17, gg) - c6 * t - tny), F(i, j, nz, 16, gg), w);
        }
    }
}

// Periodic copies across z = 1 / nz, y = 1 / ny and the zy edges (:1529-1733).
// Directions leaving through the upper face: (ez or ey) = -1 ... see tables.
__device__ __constant__ const int kZup[5] = {6, 14, 13, 18, 17}, kZdn[5] = {5, 11, 12, 15, 16};
__device__ __constant__ const int kYup[5] = {4, 10, 9, 16, 18}, kYdn[5] = {3, 7, 8, 15, 17};

template <class T, bool ODD>
__global__ void periodic_z_kernel(const BcArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > a.g.nx) return;
    const Grid& g = a.g;
    const int nz = g.nz;
#pragma unroll
    for (int gg = 0; gg < 2; ++gg)
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            if (!ODD) {
                a.pdf[a.b.at(i, j, nz + 1, kZup[s], gg)] = a.pdf[a.b.at(i, j, 1, kZup[s], gg)];
                a.pdf[a.b.at(i, j, 0, kZdn[s], gg)] = a.pdf[a.b.at(i, j, nz, kZdn[s], gg)];
            } else {
                a.pdf[a.b.at(i, j, 1, kZup[s], gg)] = a.pdf[a.b.at(i, j, nz + 1, kZup[s], gg)];
                a.pdf[a.b.at(i, j, nz, kZdn[s], gg)] = a.pdf[a.b.at(i, j, 0, kZdn[s], gg)];
            }
        }
    for (int k = 1; k <= 4; ++k) {
        a.phi[g.s4(i, j, k + nz)] = a.phi[g.s4(i, j, k)];
        a.phi[g.s4(i, j, k - 4)] = a.phi[g.s4(i, j, nz + k - 4)];
    }
}

template <class T, bool ODD>
__global__ void periodic_y_kernel(const BcArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > a.g.nx) return;
    const Grid& g = a.g;
    const int ny = g.ny;
#pragma unroll
    for (int gg = 0; gg < 2; ++gg)
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            if (!ODD) {
                a.pdf[a.b.at(i, ny + 1, k, kYup[s], gg)] = a.pdf[a.b.at(i, 1, k, kYup[s], gg)];
                a.pdf[a.b.at(i, 0, k, kYdn[s], gg)] = a.pdf[a.b.at(i, ny, k, kYdn[s], gg)];
            } else {
                a.pdf[a.b.at(i, 1, k, kYup[s], gg)] = a.pdf[a.b.at(i, ny + 1, k, kYup[s], gg)];
                a.pdf[a.b.at(i, ny, k, kYdn[s], gg)] = a.pdf[a.b.at(i, 0, k, kYdn[s], gg)];
            }
        }
    for (int j = 1; j <= 4; ++j) {
        a.phi[g.s4(i, j + ny, k)] = a.phi[g.s4(i, j, k)];
        a.phi[g.s4(i, j - 4, k)] = a.phi[g.s4(i, ny + j - 4, k)];
    }
}

template <class T, bool ODD>
__global__ void periodic_zy_kernel(const BcArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > a.g.nx) return;
    const Grid& g = a.g;
    const int ny = g.ny, nz = g.nz;
#pragma unroll
    for (int gg = 0; gg < 2; ++gg) {
        if (!ODD) {
            a.pdf[a.b.at(i, ny + 1, nz + 1, 18, gg)] = a.pdf[a.b.at(i, 1, 1, 18, gg)];
            a.pdf[a.b.at(i, ny + 1, 0, 16, gg)] = a.pdf[a.b.at(i, 1, nz, 16, gg)];
            a.pdf[a.b.at(i, 0, nz + 1, 17, gg)] = a.pdf[a.b.at(i, ny, 1, 17, gg)];
            a.pdf[a.b.at(i, 0, 0, 15, gg)] = a.pdf[a.b.at(i, ny, nz, 15, gg)];
        } else {
            a.pdf[a.b.at(i, 1, 1, 18, gg)] = a.pdf[a.b.at(i, ny + 1, nz + 1, 18, gg)];
            a.pdf[a.b.at(i, 1, nz, 16, gg)] = a.pdf[a.b.at(i, ny + 1, 0, 16, gg)];
            a.pdf[a.b.at(i, ny, 1, 17, gg)] = a.pdf[a.b.at(i, 0, nz + 1, 17, gg)];
            a.pdf[a.b.at(i, ny, nz, 15, gg)] = a.pdf[a.b.at(i, 0, 0, 15, gg)];
        }
    }
    for (int k = 1; k <= 4; ++k)
        for (int j = 1; j <= 4; ++j) {
            a.phi[g.s4(i, j - 4, k - 4)] = a.phi[g.s4(i, ny + j - 4, nz + k - 4)];
            a.phi[g.s4(i, j + ny, k - 4)] = a.phi[g.s4(i, j, nz + k - 4)];
            a.phi[g.s4(i, j + ny, k + nz)] = a.phi[g.s4(i, j, k)];
            a.phi[g.s4(i, j - 4, k + nz)] = a.phi[g.s4(i, ny + j - 4, k)];
        }
}

// porous plate blocking one component at z = Zplate (:1744-1882); b = blocked component
template <class T, bool AFTER_ODD>
__global__ void porous_plate_kernel(const BcArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > a.g.nx) return;
    const Grid& g = a.g;
    const int zp = a.Zplate;
    if (!(zp >= 1 && zp <= g.nz) || (a.plate_cmd != 1 && a.plate_cmd != 2)) return;
    const int b = a.plate_cmd == 1 ? 0 : 1, o = 1 - b;
    auto F = [&](int u, int v, int k, int e, int gg) -> T& { return a.pdf[a.b.at(u, v, k, e, gg)]; };
    if (!AFTER_ODD) {
        F(i, j, zp, 6, b) = F(i, j, zp - 1, 5, b);
        F(i - 1, j, zp, 13, b) = F(i, j, zp - 1, 12, b);
        F(i + 1, j, zp, 14, b) = F(i, j, zp - 1, 11, b);
        F(i, j - 1, zp, 17, b) = F(i, j, zp - 1, 16, b);
        F(i, j + 1, zp, 18, b) = F(i, j, zp - 1, 15, b);
        F(i, j, zp, 5, b) = F(i, j, zp + 1, 6, b);
        F(i + 1, j, zp, 12, b) = F(i, j, zp + 1, 13, b);
        F(i - 1, j, zp, 11, b) = F(i, j, zp + 1, 14, b);
        F(i, j + 1, zp, 16, b) = F(i, j, zp + 1, 17, b);
        F(i, j - 1, zp, 15, b) = F(i, j, zp + 1, 18, b);
        F(i, j, zp, 6, o) = F(i, j, zp + 1, 6, o);
        F(i, j, zp, 13, o) = F(i, j, zp + 1, 13, o);
        F(i, j, zp, 14, o) = F(i, j, zp + 1, 14, o);
        F(i, j, zp, 17, o) = F(i, j, zp + 1, 17, o);
        F(i, j, zp, 18, o) = F(i, j, zp + 1, 18, o);
        F(i, j, zp, 5, o) = F(i, j, zp - 1, 5, o);
        F(i, j, zp, 12, o) = F(i, j, zp - 1, 12, o);
        F(i, j, zp, 11, o) = F(i, j, zp - 1, 11, o);
        F(i, j, zp, 16, o) = F(i, j, zp - 1, 16, o);
        F(i, j, zp, 15, o) = F(i, j, zp - 1, 15, o);
    } else {
        F(i, j, zp - 1, 5, b) = F(i, j, zp, 6, b);
        F(i, j, zp - 1, 12, b) = F(i - 1, j, zp, 13, b);
        F(i, j, zp - 1, 11, b) = F(i + 1, j, zp, 14, b);
        F(i, j, zp - 1, 16, b) = F(i, j - 1, zp, 17, b);
        F(i, j, zp - 1, 15, b) = F(i, j + 1, zp, 18, b);
        F(i, j, zp + 1, 6, b) = F(i, j, zp, 5, b);
        F(i, j, zp + 1, 13, b) = F(i + 1, j, zp, 12, b);
        F(i, j, zp + 1, 14, b) = F(i - 1, j, zp, 11, b);
        F(i, j, zp + 1, 17, b) = F(i, j + 1, zp, 16, b);
        F(i, j, zp + 1, 18, b) = F(i, j - 1, zp, 15, b);
        F(i, j, zp - 1, 5, o) = F(i, j, zp, 5, o);
        F(i, j, zp - 1, 12, o) = F(i, j, zp, 12, o);
        F(i, j, zp - 1, 11, o) = F(i, j, zp, 11, o);
        F(i, j, zp - 1, 16, o) = F(i, j, zp, 16, o);
        F(i, j, zp - 1, 15, o) = F(i, j, zp, 15, o);
        F(i, j, zp + 1, 6, o) = F(i, j, zp, 6, o);
        F(i, j, zp + 1, 13, o) = F(i, j, zp, 13, o);
        F(i, j, zp + 1, 14, o) = F(i, j, zp, 14, o);
        F(i, j, zp + 1, 17, o) = F(i, j, zp, 17, o);
        F(i, j, zp + 1, 18, o) = F(i, j, zp, 18, o);
    }
}

// ===========================================================================
// Host launchers.
// ===========================================================================
template <class T>
GradArgs<T> grad_args(const mflbm_context& c) {
    const DeviceState& d = c.d;
    GradArgs<T> a;
    a.g = d.g;
    a.b = d.b;
    a.type8 = d.type8;
    a.snx = (const T*)d.s_nx; a.sny = (const T*)d.s_ny; a.snz = (const T*)d.s_nz;
    a.phi = (T*)d.phi; a.cnx = (T*)d.cn_x; a.cny = (T*)d.cn_y; a.cnz = (T*)d.cn_z;
    a.cnorm = (T*)d.c_norm; a.curv = (T*)d.curv;
    a.aux = (typename Vec4<T>::type*)d.aux;
    a.l_phi = d.list_phi_ext; a.n_phi = (int)d.n_phi_ext;
    a.l_cn = d.list_cn_ext; a.n_cn = (int)d.n_cn_ext;
    a.ph = make_phys<T>(c.params);
    return a;
}

// The colour-gradient pipeline (also the start-up colour_gradient,
// src/Phase_gradient.cpp:15-216, which performs the same passes).
template <class T>
int launch_gradient(mflbm_context& c) {
    const GradArgs<T> a = grad_args<T>(c);
    const Grid& g = c.d.g;
    cudaStream_t s = c.stream;
    int rc;
    if (a.n_phi) {
        extrapolate_phi_kernel<T><<<grid_for(a.n_phi, 128), 128, 0, s>>>(a);
        if ((rc = after_launch("extrapolate_phi")) != MFLBM_OK) return rc;
    }
    normals_kernel<T><<<dim3(grid_for(g.nx + 4, 128), g.ny + 4, g.nz + 4), 128, 0, s>>>(a);
    if ((rc = after_launch("normals")) != MFLBM_OK) return rc;
    if (a.n_cn) {
        extrapolate_normal_kernel<T><<<grid_for(a.n_cn, 128), 128, 0, s>>>(a);
        if ((rc = after_launch("extrapolate_normal")) != MFLBM_OK) return rc;
    }
    curvature_kernel<T><<<grid_for(c.d.b.S, 128), 128, 0, s>>>(a);
    return after_launch("curvature");
}

template <class T>
int launch_refresh_aux(mflbm_context& c) {
    const GradArgs<T> a = grad_args<T>(c);
    aux_kernel<T><<<grid_for(c.d.b.S, 128), 128, 0, c.stream>>>(a);
    return after_launch("aux");
}

template <class T>
int launch_collide(mflbm_context& c, bool odd) {
    typedef typename Vec2<T>::type V2;
    const DeviceState& d = c.d;
    const Grid& g = d.g;
    CollideArgs<T> a;
    V2* pdf = (V2*)d.pdf;
    for (int q = 0; q < 19; ++q) a.slot[q] = pdf + d.b.S * q;
    a.list = d.fluid_list;
    a.n = (int)d.n_fluid;
    a.nbx = d.b.nbx; a.nby = d.b.nby;
    a.bx8 = 8 * d.b.nbx;
    a.bxy8 = 8 * d.b.nbx * d.b.nby;
    a.NX4 = g.nx + 8; a.NY4 = g.ny + 8;
    a.phi = (T*)d.phi;
    a.aux = (const typename Vec4<T>::type*)d.aux;
    a.ph = make_phys<T>(c.params);
    if (a.n == 0) return MFLBM_OK;
    if (odd) collide_stream_kernel<T, true><<<grid_for(a.n, 128), 128, 0, c.stream>>>(a);
    else collide_stream_kernel<T, false><<<grid_for(a.n, 128), 128, 0, c.stream>>>(a);
    return after_launch("collide_stream");
}

template <class T>
int launch_boundaries(mflbm_context& c, bool odd) {
    const DeviceState& d = c.d;
    const Grid& g = d.g;
    const mflbm_params& p = c.params;
    BcArgs<T> a;
    a.g = g;
    a.b = d.b;
    a.walls = d.walls;
    a.pdf = (T*)d.pdf; a.phi = (T*)d.phi; a.W_in = (T*)d.W_in;
    a.f_cv = (T*)d.f_cv; a.g_cv = (T*)d.g_cv; a.phi_cv = (T*)d.phi_cv;
    a.ph = make_phys<T>(p);
    a.plate_cmd = p.porous_plate_cmd; a.Zplate = p.Z_porous_plate;
    cudaStream_t s = c.stream;
    const unsigned bx = grid_for(g.nx, 128);
    int rc;
#define MFLBM_BC(kernel, gridv, name)                                             \
    do {                                                                          \
        if (odd) kernel<T, true><<<gridv, 128, 0, s>>>(a);                        \
        else kernel<T, false><<<gridv, 128, 0, s>>>(a);                           \
        if ((rc = after_launch(name)) != MFLBM_OK) return rc;                     \
    } while (0)
    if (p.kper) MFLBM_BC(periodic_z_kernel, dim3(bx, g.ny), "periodic_z");
    if (p.jper) MFLBM_BC(periodic_y_kernel, dim3(bx, g.nz), "periodic_y");
    if (p.jper && p.kper) MFLBM_BC(periodic_zy_kernel, dim3(bx, 1), "periodic_zy");
    if (p.kper == 0 && p.domain_wall_status_z_min == 0 && p.domain_wall_status_z_max == 0) {
        if (p.inlet_BC == 1) MFLBM_BC(inlet_velocity_kernel, dim3(bx, g.ny), "inlet_velocity");
        else if (p.inlet_BC == 2) MFLBM_BC(inlet_pressure_kernel, dim3(bx, g.ny), "inlet_pressure");
        if (p.outlet_BC == 1) MFLBM_BC(outlet_convective_kernel, dim3(bx, g.ny), "outlet_convective");
        else if (p.outlet_BC == 2) MFLBM_BC(outlet_pressure_kernel, dim3(bx, g.ny), "outlet_pressure");
    }
    if (p.porous_plate_cmd != 0) MFLBM_BC(porous_plate_kernel, dim3(bx, g.ny), "porous_plate");
#undef MFLBM_BC
    return MFLBM_OK;
}

}  // namespace MFLBM_NS
}  // namespace mflbm
