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
__device__ __forceinline__ T collide(const Phys<T>& P, T (&g1)[19], T (&g2)[19], T cnx, T cny, T cnz, T curv,
                                     T cnorm) {
    T f[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) f[q] = g1[q] + g2[q];
    T rho1 = g1[0], rho2 = g2[0];
#pragma unroll
    for (int q = 1; q < 19; ++q) rho1 = rho1 + g1[q];
#pragma unroll
    for (int q = 1; q < 19; ++q) rho2 = rho2 + g2[q];
    const T phi = (rho1 - rho2) / (rho1 + rho2);

    T tmp = T(0.5) * P.gamma * curv * cnorm;
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
// Collision + AA streaming over the fluid-node list.
//   odd  step: populations pulled from slot q of node x - e_q, pushed to
//              slot opp(q) of node x + e_q (src/main_iteration_GPU.cu:75-113, 348-384)
//   even step: read from slot opp(q) of x, written to slot q of x (:414-452, 687-723)
// pull[q + 19 g] / push[q + 19 g] are slot base pointers already offset by the
// streaming displacement, so every access is base + n1.
// ===========================================================================
template <class T> struct CollideArgs {
    const T* pull[38];
    T* push[38];
    const uint32_t* list;
    ll n;
    int NX1, NY1, NX2, NY2, NX4, NY4;
    T* phi;
    const T *cnx, *cny, *cnz, *cnorm, *curv;
    Phys<T> ph;
};

template <class T>
__global__ void __launch_bounds__(128) collide_stream_kernel(const CollideArgs<T> a) {
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n) return;
    int x, y, z;
    unpack_xyz(a.list[t], x, y, z);
    const int n1 = x + a.NX1 * (y + a.NY1 * z);
    T g1[19], g2[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        g1[q] = a.pull[q][n1];
        g2[q] = a.pull[19 + q][n1];
    }
    const ll n2 = (x + 1) + (ll)a.NX2 * ((y + 1) + (ll)a.NY2 * (z + 1));
    const T cnx = a.cnx[n2], cny = a.cny[n2], cnz = a.cnz[n2], cnorm = a.cnorm[n2], curv = a.curv[n1];
    const T phi = collide<T>(a.ph, g1, g2, cnx, cny, cnz, curv, cnorm);
    a.phi[(x + 3) + (ll)a.NX4 * ((y + 3) + (ll)a.NY4 * (z + 3))] = phi;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        a.push[q][n1] = g1[q];
        a.push[19 + q][n1] = g2[q];
    }
}

// ===========================================================================
// Colour-gradient pipeline (src/main_iteration_GPU.cu:732-1003), ranges of the
// reference launches (:2027-2054).  Solid / fluid boundary work runs over
// precomputed node lists.
// ===========================================================================
template <class T> struct GradArgs {
    Grid g;
    const int32_t* walls;
    const int32_t* wt;
    const T *snx, *sny, *snz;
    T *phi, *cnx, *cny, *cnz, *cnorm, *curv;
    const uint32_t *l_phi, *l_wet, *l_cn;
    ll n_phi, n_wet, n_cn;
    Phys<T> ph;
};

template <class T, class F>
__device__ __forceinline__ T dx_iso4(const ModelConsts<T>& c, F f, int i, int j, int k) {
    return c.iso4a * (f(i + 1, j, k) - f(i - 1, j, k)) +
           c.iso4b * (f(i + 1, j + 1, k) - f(i - 1, j - 1, k) + f(i + 1, j - 1, k) - f(i - 1, j + 1, k) +
                      f(i + 1, j, k + 1) - f(i - 1, j, k - 1) + f(i + 1, j, k - 1) - f(i - 1, j, k + 1));
}
template <class T, class F>
__device__ __forceinline__ T dy_iso4(const ModelConsts<T>& c, F f, int i, int j, int k) {
    return c.iso4a * (f(i, j + 1, k) - f(i, j - 1, k)) +
           c.iso4b * (f(i + 1, j + 1, k) - f(i - 1, j - 1, k) + f(i - 1, j + 1, k) - f(i + 1, j - 1, k) +
                      f(i, j + 1, k + 1) - f(i, j - 1, k - 1) + f(i, j + 1, k - 1) - f(i, j - 1, k + 1));
}
template <class T, class F>
__device__ __forceinline__ T dz_iso4(const ModelConsts<T>& c, F f, int i, int j, int k) {
    return c.iso4a * (f(i, j, k + 1) - f(i, j, k - 1)) +
           c.iso4b * (f(i + 1, j, k + 1) - f(i - 1, j, k - 1) + f(i - 1, j, k + 1) - f(i + 1, j, k - 1) +
                      f(i, j + 1, k + 1) - f(i, j - 1, k - 1) + f(i, j - 1, k + 1) - f(i, j + 1, k - 1));
}

template <class T> __device__ __forceinline__ T wq_of(const ModelConsts<T>& c, int q) { return q < 7 ? c.w1 : c.w2; }

// phi on solid boundary nodes = weighted mean over fluid neighbours (:732-755)
template <class T>
__global__ void extrapolate_phi_kernel(const GradArgs<T> a) {
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n_phi) return;
    int i, j, k;
    unpack_xyz(a.l_phi[t], i, j, k);
    T s = T(0), ws = T(0);
#pragma unroll
    for (int q = 1; q < 19; ++q) {
        const int u = i + ex(q), v = j + ey(q), w = k + ez(q);
        if (a.wt[a.g.s4(u, v, w)] <= 0) {
            s += a.phi[a.g.s4(u, v, w)] * wq_of(a.ph.c, q);
            ws += wq_of(a.ph.c, q);
        }
    }
    a.phi[a.g.s4(i, j, k)] = s / ws;
}

// unit interface normal and |grad phi| on [-1, n+2]^3 (:757-807)
template <class T>
__global__ void __launch_bounds__(128) normals_kernel(const GradArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y - 1, k = blockIdx.z - 1;
    if (i > a.g.nx + 2) return;
    const Grid& g = a.g;
    const T* phi = a.phi;
    auto F = [&](int u, int v, int w) { return phi[g.s4(u, v, w)]; };
    const T x = dx_iso4(a.ph.c, F, i, j, k);
    const T y = dy_iso4(a.ph.c, F, i, j, k);
    const T z = dz_iso4(a.ph.c, F, i, j, k);
    const T nrm = sqrt(x * x + y * y + z * z);
    const ll n = g.s2(i, j, k);
    if (nrm < T(1e-6) || a.walls[n] == 1) {
        a.cnx[n] = T(0); a.cny[n] = T(0); a.cnz[n] = T(0); a.cnorm[n] = T(0);
    } else {
        a.cnx[n] = x / nrm; a.cny[n] = y / nrm; a.cnz[n] = z / nrm; a.cnorm[n] = nrm;
    }
}

// geometrical wetting at fluid boundary nodes: secant iteration that turns the
// interface normal towards the prescribed contact angle (:809-878)
template <class T>
__global__ void wetting_kernel(const GradArgs<T> a) {
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n_wet) return;
    int i, j, k;
    unpack_xyz(a.l_wet[t], i, j, k);
    const ll n = a.g.s2(i, j, k), m = a.g.s4(i, j, k);
    const T local_eps = T(1e-6), lambda = T(0.5);
    if (!(a.cnorm[n] > local_eps)) return;
    const T cs = a.ph.cos_theta;
    const T nwx = a.snx[m], nwy = a.sny[m], nwz = a.snz[m];
    T vcx0 = a.cnx[n], vcy0 = a.cny[n], vcz0 = a.cnz[n];
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
    a.cnx[n] = vcx2 * inv; a.cny[n] = vcy2 * inv; a.cnz[n] = vcz2 * inv;
}

// interface normal on solid boundary nodes = weighted mean over fluid neighbours (:880-906)
template <class T>
__global__ void extrapolate_normal_kernel(const GradArgs<T> a) {
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n_cn) return;
    int i, j, k;
    unpack_xyz(a.l_cn[t], i, j, k);
    T sx = T(0), sy = T(0), sz = T(0), ws = T(0);
#pragma unroll
    for (int q = 1; q < 19; ++q) {
        const int u = i + ex(q), v = j + ey(q), w = k + ez(q);
        if (a.wt[a.g.s4(u, v, w)] <= 0) {
            const ll m = a.g.s2(u, v, w);
            const T wq = wq_of(a.ph.c, q);
            sx += a.cnx[m] * wq;
            sy += a.cny[m] * wq;
            sz += a.cnz[m] * wq;
            ws += wq;
        }
    }
    const ll n = a.g.s2(i, j, k);
    a.cnx[n] = sx / ws; a.cny[n] = sy / ws; a.cnz[n] = sz / ws;
}

// interface curvature from the nine derivatives of the normal (:908-1003)
template <class T>
__global__ void __launch_bounds__(128) curvature_kernel(const GradArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y + 1, k = blockIdx.z + 1;
    if (i > a.g.nx) return;
    const Grid& g = a.g;
    const T *X = a.cnx, *Y = a.cny, *Z = a.cnz;
    auto FX = [&](int u, int v, int w) { return X[g.s2(u, v, w)]; };
    auto FY = [&](int u, int v, int w) { return Y[g.s2(u, v, w)]; };
    auto FZ = [&](int u, int v, int w) { return Z[g.s2(u, v, w)]; };
    const ModelConsts<T>& c = a.ph.c;
    const T kxx = dx_iso4(c, FX, i, j, k), kyy = dy_iso4(c, FY, i, j, k), kzz = dz_iso4(c, FZ, i, j, k);
    const T kxy = dy_iso4(c, FX, i, j, k), kxz = dz_iso4(c, FX, i, j, k);
    const T kyx = dx_iso4(c, FY, i, j, k), kyz = dz_iso4(c, FY, i, j, k);
    const T kzx = dx_iso4(c, FZ, i, j, k), kzy = dy_iso4(c, FZ, i, j, k);
    const ll n = g.s2(i, j, k);
    const T x = X[n], y = Y[n], z = Z[n];
    a.curv[g.s1(i, j, k)] = (x * x - T(1)) * kxx + (y * y - T(1)) * kyy + (z * z - T(1)) * kzz +
                            x * y * (kxy + kyx) + x * z * (kxz + kzx) + y * z * (kzy + kyz);
}

// ===========================================================================
// Boundary updates (src/main_iteration_GPU.cu:1009-1882).  One thread per
// (i, j) column (inlet / outlet / plate) or (i, k) row (periodic y).
// keep(new, old, w) is the reference's  new*(1-w) + old*w  blend.
// ===========================================================================
template <class T> struct BcArgs {
    Grid g;
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
                T& d = a.pdf[g.f1(i + dx, j + dy, 0, s0, gg)];
                d = keep((a.pdf[g.f1(i, j, 1, s1, gg)] + T(6.0) * wq * inj), d, w);
            } else {
                T& d = a.pdf[g.f1(i, j, 1, s1, gg)];
                d = keep((a.pdf[g.f1(i + dx, j + dy, 0, s0, gg)] + T(6.0) * wq * inj), d, w);
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
        auto F = [&](int u, int v, int k, int e) -> T& { return a.pdf[g.f1(u, v, k, e, gg)]; };
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
                T& d = a.pdf[g.f1(i + dx, j + dy, nz + 1, su, gg)];
                d = ((bv + u * a.pdf[g.f1(i + dx, j + dy, nz, su, gg)]) * temp) * T(1 - w) + d * T(w);
                bv = d;
            } else {
                T& d = a.pdf[g.f1(i, j, nz, sd, gg)];
                d = ((bv + u * a.pdf[g.f1(i, j, nz - 1, sd, gg)]) * temp) * T(1 - w) + d * T(w);
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
    auto F = [&](int u, int v, int k, int e, int gg) -> T& { return a.pdf[g.f1(u, v, k, e, gg)]; };
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
                a.pdf[g.f1(i, j, nz + 1, kZup[s], gg)] = a.pdf[g.f1(i, j, 1, kZup[s], gg)];
                a.pdf[g.f1(i, j, 0, kZdn[s], gg)] = a.pdf[g.f1(i, j, nz, kZdn[s], gg)];
            } else {
                a.pdf[g.f1(i, j, 1, kZup[s], gg)] = a.pdf[g.f1(i, j, nz + 1, kZup[s], gg)];
                a.pdf[g.f1(i, j, nz, kZdn[s], gg)] = a.pdf[g.f1(i, j, 0, kZdn[s], gg)];
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
                a.pdf[g.f1(i, ny + 1, k, kYup[s], gg)] = a.pdf[g.f1(i, 1, k, kYup[s], gg)];
                a.pdf[g.f1(i, 0, k, kYdn[s], gg)] = a.pdf[g.f1(i, ny, k, kYdn[s], gg)];
            } else {
                a.pdf[g.f1(i, 1, k, kYup[s], gg)] = a.pdf[g.f1(i, ny + 1, k, kYup[s], gg)];
                a.pdf[g.f1(i, ny, k, kYdn[s], gg)] = a.pdf[g.f1(i, 0, k, kYdn[s], gg)];
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
            a.pdf[g.f1(i, ny + 1, nz + 1, 18, gg)] = a.pdf[g.f1(i, 1, 1, 18, gg)];
            a.pdf[g.f1(i, ny + 1, 0, 16, gg)] = a.pdf[g.f1(i, 1, nz, 16, gg)];
            a.pdf[g.f1(i, 0, nz + 1, 17, gg)] = a.pdf[g.f1(i, ny, 1, 17, gg)];
            a.pdf[g.f1(i, 0, 0, 15, gg)] = a.pdf[g.f1(i, ny, nz, 15, gg)];
        } else {
            a.pdf[g.f1(i, 1, 1, 18, gg)] = a.pdf[g.f1(i, ny + 1, nz + 1, 18, gg)];
            a.pdf[g.f1(i, 1, nz, 16, gg)] = a.pdf[g.f1(i, ny + 1, 0, 16, gg)];
            a.pdf[g.f1(i, ny, 1, 17, gg)] = a.pdf[g.f1(i, 0, nz + 1, 17, gg)];
            a.pdf[g.f1(i, ny, nz, 15, gg)] = a.pdf[g.f1(i, 0, 0, 15, gg)];
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
    auto F = [&](int u, int v, int k, int e, int gg) -> T& { return a.pdf[g.f1(u, v, k, e, gg)]; };
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
    a.walls = d.walls;
    a.wt = d.walls_type;
    a.snx = (const T*)d.s_nx; a.sny = (const T*)d.s_ny; a.snz = (const T*)d.s_nz;
    a.phi = (T*)d.phi; a.cnx = (T*)d.cn_x; a.cny = (T*)d.cn_y; a.cnz = (T*)d.cn_z;
    a.cnorm = (T*)d.c_norm; a.curv = (T*)d.curv;
    a.l_phi = d.list_phi_ext; a.n_phi = d.n_phi_ext;
    a.l_wet = d.list_wet; a.n_wet = d.n_wet;
    a.l_cn = d.list_cn_ext; a.n_cn = d.n_cn_ext;
    a.ph = make_phys<T>(c.params);
    return a;
}

// The five passes of the colour-gradient pipeline (also the start-up
// colour_gradient, src/Phase_gradient.cpp:15-216, which is identical).
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
    if (a.n_wet) {
        wetting_kernel<T><<<grid_for(a.n_wet, 128), 128, 0, s>>>(a);
        if ((rc = after_launch("wetting")) != MFLBM_OK) return rc;
    }
    if (a.n_cn) {
        extrapolate_normal_kernel<T><<<grid_for(a.n_cn, 128), 128, 0, s>>>(a);
        if ((rc = after_launch("extrapolate_normal")) != MFLBM_OK) return rc;
    }
    curvature_kernel<T><<<dim3(grid_for(g.nx, 128), g.ny, g.nz), 128, 0, s>>>(a);
    return after_launch("curvature");
}

template <class T>
int launch_collide(mflbm_context& c, bool odd) {
    const DeviceState& d = c.d;
    const Grid& g = d.g;
    CollideArgs<T> a;
    const ll S = g.n1();
    const int NX1 = g.nx + 2, NY1 = g.ny + 2;
    T* pdf = (T*)d.pdf;
    for (int gg = 0; gg < 2; ++gg)
        for (int q = 0; q < 19; ++q) {
            const ll off = ex(q) + (ll)NX1 * (ey(q) + (ll)NY1 * ez(q));
            if (odd) {
                a.pull[q + 19 * gg] = pdf + S * (q + 19 * gg) - off;
                a.push[q + 19 * gg] = pdf + S * (opp(q) + 19 * gg) + off;
            } else {
                a.pull[q + 19 * gg] = pdf + S * (opp(q) + 19 * gg);
                a.push[q + 19 * gg] = pdf + S * (q + 19 * gg);
            }
        }
    a.list = d.fluid_list;
    a.n = d.n_fluid;
    a.NX1 = NX1; a.NY1 = NY1;
    a.NX2 = g.nx + 4; a.NY2 = g.ny + 4;
    a.NX4 = g.nx + 8; a.NY4 = g.ny + 8;
    a.phi = (T*)d.phi;
    a.cnx = (const T*)d.cn_x; a.cny = (const T*)d.cn_y; a.cnz = (const T*)d.cn_z;
    a.cnorm = (const T*)d.c_norm; a.curv = (const T*)d.curv;
    a.ph = make_phys<T>(c.params);
    if (a.n == 0) return MFLBM_OK;
    collide_stream_kernel<T><<<grid_for(a.n, 128), 128, 0, c.stream>>>(a);
    return after_launch("collide_stream");
}

template <class T>
int launch_boundaries(mflbm_context& c, bool odd) {
    const DeviceState& d = c.d;
    const Grid& g = d.g;
    const mflbm_params& p = c.params;
    BcArgs<T> a;
    a.g = g;
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
