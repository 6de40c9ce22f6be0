/*
 * CPU oracle for the MF-LBM hot path — TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, on the CPU and in the reference's own padded layouts,
 * every function of the per-timestep hot path of MF-LBM-CUDA and the set-up
 * that produces its inputs.  It is the checker that the CUDA library is
 * compared against; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  It is never linked into, or called by, the
 * product library.
 *
 * Floating-point expressions keep the reference's operand order so that,
 * compiled with -ffp-contract=off, results are bit-identical to the
 * reference's kernels compiled as host code (oracle/_ref) and to the CUDA
 * library's strict mode.  pow(x, 2) of the reference is written x * x (GCC
 * folds the reference's call to exactly that).
 *
 * Parity pinning: tests/golden/ holds fixtures produced by oracle/_ref (the
 * reference's kernels and set-up compiled from its sources); the CPU tests
 * check this restatement against them bit for bit.
 *
 * All functions are stateless: the caller owns every array.  Exported with C
 * linkage as orc_<name>_f32 / orc_<name>_f64.
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/mflbm.h"

namespace {

/* D3Q19 lattice, includes/Module.h:98-101 (ex, ey, ez, opc). */
const int EX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int EY[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
const int EZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
const int OPP[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};

typedef long long ll;

/* Padded 1-based index functions, includes/Idx_cpu.h (i_s0 .. i_f1, icnv_f1). */
struct Grid {
    ll nx, ny, nz;
    ll s0(ll x, ll y, ll z) const { return (x - 1) + nx * ((y - 1) + ny * (z - 1)); }
    ll s1(ll x, ll y, ll z) const { return x + (nx + 2) * (y + (ny + 2) * z); }
    ll s2(ll x, ll y, ll z) const { return (x + 1) + (nx + 4) * ((y + 1) + (ny + 4) * (z + 1)); }
    ll s4(ll x, ll y, ll z) const { return (x + 3) + (nx + 8) * ((y + 3) + (ny + 8) * (z + 3)); }
    ll f1(ll x, ll y, ll z, int e, int g) const {
        return x + (nx + 2) * (y + (ny + 2) * (z + (nz + 2) * (ll)(e + 19 * g)));
    }
    ll cnv(ll x, ll y, int e) const { return x + (nx + 2) * (y + (ny + 2) * (ll)e); }
    ll n_s1() const { return (nx + 2) * (ny + 2) * (nz + 2); }
    ll n_s2() const { return (nx + 4) * (ny + 4) * (nz + 4); }
    ll n_s4() const { return (nx + 8) * (ny + 8) * (nz + 8); }
};

/* Model constants as the reference computes them in T_P
 * (includes/Module.h:104-126, includes/Fluid_multiphase.h:31-35). */
template <class T> struct Consts {
    T w[19];
    T w0, w1, w2, rk2, iso4a, iso4b;
    T mrt_coef1, mrt_coef2, mrt_coef3, mrt_coef4, mrt_e2_coef1, mrt_e2_coef2, mrt_omega_xx;
    T iso8[7];
    Consts() {
        w0 = T(1) / T(3);
        w1 = T(1) / T(18);
        w2 = T(1) / T(36);
        w[0] = w0;
        for (int q = 1; q <= 6; ++q) w[q] = w1;
        for (int q = 7; q <= 18; ++q) w[q] = w2;
        rk2 = T(1) / std::sqrt(T(2)) / T(36);
        iso4a = T(1) / T(6);
        iso4b = T(1) / T(12);
        mrt_coef1 = T(1) / T(19);
        mrt_coef2 = T(1) / T(2394);
        mrt_coef3 = T(1) / T(252);
        mrt_coef4 = T(1) / T(72);
        mrt_e2_coef1 = T(0);
        mrt_e2_coef2 = T(-475) / T(63);
        mrt_omega_xx = T(0);
        iso8[0] = T(4) / T(45); iso8[1] = T(1) / T(21); iso8[2] = T(2) / T(105);
        iso8[3] = T(5) / T(504); iso8[4] = T(1) / T(315); iso8[5] = T(1) / T(630);
        iso8[6] = T(1) / T(5040);
    }
};

template <class T> struct P {
    Grid g;
    int jper, kper, zmin_wall, zmax_wall, inlet_BC, outlet_BC, plate_cmd, Zplate;
    T gamma, force_z, nui1, nui2, beta, phi_inlet, sa_inject, uin_avg, relaxation, cos_theta, rho_in, rho_out;
    explicit P(const mflbm_params* p) {
        g = Grid{p->nx, p->ny, p->nz};
        jper = p->jper; kper = p->kper;
        zmin_wall = p->domain_wall_status_z_min; zmax_wall = p->domain_wall_status_z_max;
        inlet_BC = p->inlet_BC; outlet_BC = p->outlet_BC;
        plate_cmd = p->porous_plate_cmd; Zplate = p->Z_porous_plate;
        gamma = T(p->lbm_gamma); force_z = T(p->force_z); nui1 = T(p->la_nui1); nui2 = T(p->la_nui2);
        beta = T(p->lbm_beta); phi_inlet = T(p->phi_inlet); sa_inject = T(p->sa_inject);
        uin_avg = T(p->uin_avg); relaxation = T(p->relaxation); cos_theta = T(p->cos_theta);
        rho_in = T(p->rho_in); rho_out = T(p->rho_out);
    }
    bool open_z() const { return kper == 0 && zmin_wall == 0 && zmax_wall == 0; }
};

/* ---------------------------------------------------------------------------
 * ISO4 first-derivative stencils on a padded field, in the reference's
 * operand order (src/main_iteration_GPU.cu:765-791, :916-996).
 * ------------------------------------------------------------------------- */
template <class T, class F>
inline T deriv_x(const Consts<T>& c, F f, ll i, ll j, ll k) {
    return c.iso4a * (f(i + 1, j, k) - f(i - 1, j, k)) +
           c.iso4b * (f(i + 1, j + 1, k) - f(i - 1, j - 1, k) + f(i + 1, j - 1, k) - f(i - 1, j + 1, k) +
                      f(i + 1, j, k + 1) - f(i - 1, j, k - 1) + f(i + 1, j, k - 1) - f(i - 1, j, k + 1));
}
template <class T, class F>
inline T deriv_y(const Consts<T>& c, F f, ll i, ll j, ll k) {
    return c.iso4a * (f(i, j + 1, k) - f(i, j - 1, k)) +
           c.iso4b * (f(i + 1, j + 1, k) - f(i - 1, j - 1, k) + f(i - 1, j + 1, k) - f(i + 1, j - 1, k) +
                      f(i, j + 1, k + 1) - f(i, j - 1, k - 1) + f(i, j + 1, k - 1) - f(i, j - 1, k + 1));
}
template <class T, class F>
inline T deriv_z(const Consts<T>& c, F f, ll i, ll j, ll k) {
    return c.iso4a * (f(i, j, k + 1) - f(i, j, k - 1)) +
           c.iso4b * (f(i + 1, j, k + 1) - f(i - 1, j, k - 1) + f(i - 1, j, k + 1) - f(i + 1, j, k - 1) +
                      f(i, j + 1, k + 1) - f(i, j - 1, k - 1) + f(i, j - 1, k + 1) - f(i, j + 1, k - 1));
}

/* ---------------------------------------------------------------------------
 * Colour-gradient pipeline (src/main_iteration_GPU.cu:732-1003 and its host
 * twin src/Phase_gradient.cpp:15-291): five passes, same ranges as the
 * device launches of :2027-2054 (normals on [-1, n+2]; the device grid's
 * extra column at x = n+3 only aliases solid x-ghost cells and is omitted).
 * ------------------------------------------------------------------------- */
template <class T>
void extrapolate_phi_to_solid(const P<T>& p, const Consts<T>& c, const int32_t* wt, T* phi) {
    const Grid& g = p.g;
#pragma omp parallel for collapse(2) schedule(static)
    for (ll k = -2; k <= g.nz + 3; ++k)
        for (ll j = -2; j <= g.ny + 3; ++j)
            for (ll i = -2; i <= g.nx + 3; ++i) {
                if (wt[g.s4(i, j, k)] != 2) continue;
                T phi_sum = T(0), weight_sum = T(0);
                for (int q = 1; q < 19; ++q) {
                    ll a = i + EX[q], b = j + EY[q], d = k + EZ[q];
                    if (wt[g.s4(a, b, d)] <= 0) {
                        phi_sum += phi[g.s4(a, b, d)] * c.w[q];
                        weight_sum += c.w[q];
                    }
                }
                phi[g.s4(i, j, k)] = phi_sum / weight_sum;
            }
}

template <class T>
void interface_normals(const P<T>& p, const Consts<T>& c, const int32_t* walls, const T* phi,
                       T* cnx, T* cny, T* cnz, T* cnorm) {
    const Grid& g = p.g;
    auto F = [&](ll a, ll b, ll d) { return phi[g.s4(a, b, d)]; };
#pragma omp parallel for collapse(2) schedule(static)
    for (ll k = -1; k <= g.nz + 2; ++k)
        for (ll j = -1; j <= g.ny + 2; ++j)
            for (ll i = -1; i <= g.nx + 2; ++i) {
                ll n = g.s2(i, j, k);
                T x = deriv_x(c, F, i, j, k);
                T y = deriv_y(c, F, i, j, k);
                T z = deriv_z(c, F, i, j, k);
                T nrm = std::sqrt(x * x + y * y + z * z);
                if (nrm < T(1e-6) || walls[n] == 1) {
                    cnx[n] = T(0); cny[n] = T(0); cnz[n] = T(0); cnorm[n] = T(0);
                } else {
                    cnx[n] = x / nrm; cny[n] = y / nrm; cnz[n] = z / nrm; cnorm[n] = nrm;
                }
            }
}

/* Geometrical wetting: secant iteration on the interface normal at fluid
 * boundary nodes (src/main_iteration_GPU.cu:809-878). */
template <class T>
void wetting_node(T cos_theta, T nwx, T nwy, T nwz, T& cx, T& cy, T& cz) {
    const T lambda = T(0.5), local_eps = T(1e-6);
    const int iteration_max = 4;
    T vcx0 = cx, vcy0 = cy, vcz0 = cz;
    T vcx1 = vcx0 - lambda * (vcx0 + nwx);
    T vcy1 = vcy0 - lambda * (vcy0 + nwy);
    T vcz1 = vcz0 - lambda * (vcz0 + nwz);
    T err0 = (nwx * vcx0 + nwy * vcy0 + nwz * vcz0) - cos_theta;
    if ((std::fabs(vcx0 + nwx) + std::fabs(vcy0 + nwy) + std::fabs(vcz0 + nwz) > local_eps ||
         std::fabs(vcx0 - nwx) + std::fabs(vcy0 - nwy) + std::fabs(vcz0 - nwz) > local_eps) &&
        err0 > local_eps) {
        T err1 = (nwx * vcx1 + nwy * vcy1 + nwz * vcz1) - std::sqrt(vcx1 * vcx1 + vcy1 * vcy1 + vcz1 * vcz1) * cos_theta;
        T tmp = T(1) / (err1 - err0);
        T vcx2 = tmp * (vcx0 * err1 - vcx1 * err0);
        T vcy2 = tmp * (vcy0 * err1 - vcy1 * err0);
        T vcz2 = tmp * (vcz0 * err1 - vcz1 * err0);
        T err2 = (nwx * vcx2 + nwy * vcy2 + nwz * vcz2) - std::sqrt(vcx2 * vcx2 + vcy2 * vcy2 + vcz2 * vcz2) * cos_theta;
        if (err2 > local_eps) {
            for (int it = 2; it <= iteration_max; ++it) {
                vcx0 = vcx1; vcy0 = vcy1; vcz0 = vcz1;
                vcx1 = vcx2; vcy1 = vcy2; vcz1 = vcz2;
                err0 = (nwx * vcx0 + nwy * vcy0 + nwz * vcz0) - std::sqrt(vcx0 * vcx0 + vcy0 * vcy0 + vcz0 * vcz0) * cos_theta;
                err1 = (nwx * vcx1 + nwy * vcy1 + nwz * vcz1) - std::sqrt(vcx1 * vcx1 + vcy1 * vcy1 + vcz1 * vcz1) * cos_theta;
                tmp = T(1) / (err1 - err0);
                if (std::isinf(tmp)) break;
                vcx2 = tmp * (vcx0 * err1 - vcx1 * err0);
                vcy2 = tmp * (vcy0 * err1 - vcy1 * err0);
                vcz2 = tmp * (vcz0 * err1 - vcz1 * err0);
                err2 = (nwx * vcx2 + nwy * vcy2 + nwz * vcz2) - std::sqrt(vcx2 * vcx2 + vcy2 * vcy2 + vcz2 * vcz2) * cos_theta;
            }
        }
        tmp = T(1) / (T(1e-30) + std::sqrt(vcx2 * vcx2 + vcy2 * vcy2 + vcz2 * vcz2));
        cx = vcx2 * tmp; cy = vcy2 * tmp; cz = vcz2 * tmp;
    }
}

template <class T>
void wetting(const P<T>& p, const int32_t* wt, const T* snx, const T* sny, const T* snz,
             T* cnx, T* cny, T* cnz, const T* cnorm) {
    const Grid& g = p.g;
#pragma omp parallel for collapse(2) schedule(static)
    for (ll k = -1; k <= g.nz + 2; ++k)
        for (ll j = -1; j <= g.ny + 2; ++j)
            for (ll i = -1; i <= g.nx + 2; ++i) {
                if (wt[g.s4(i, j, k)] != -1) continue;
                ll n = g.s2(i, j, k), m = g.s4(i, j, k);
                if (!(cnorm[n] > T(1e-6))) continue;
                wetting_node(p.cos_theta, snx[m], sny[m], snz[m], cnx[n], cny[n], cnz[n]);
            }
}

template <class T>
void extrapolate_normal_to_solid(const P<T>& p, const Consts<T>& c, const int32_t* wt, T* cnx, T* cny, T* cnz) {
    const Grid& g = p.g;
#pragma omp parallel for collapse(2) schedule(static)
    for (ll k = 0; k <= g.nz + 1; ++k)
        for (ll j = 0; j <= g.ny + 1; ++j)
            for (ll i = 0; i <= g.nx + 1; ++i) {
                if (wt[g.s4(i, j, k)] != 2) continue;
                T sx = T(0), sy = T(0), sz = T(0), ws = T(0);
                for (int q = 1; q < 19; ++q) {
                    ll a = i + EX[q], b = j + EY[q], d = k + EZ[q];
                    if (wt[g.s4(a, b, d)] <= 0) {
                        ll m = g.s2(a, b, d);
                        sx += cnx[m] * c.w[q];
                        sy += cny[m] * c.w[q];
                        sz += cnz[m] * c.w[q];
                        ws += c.w[q];
                    }
                }
                ll n = g.s2(i, j, k);
                cnx[n] = sx / ws; cny[n] = sy / ws; cnz[n] = sz / ws;
            }
}

template <class T>
void curvature(const P<T>& p, const Consts<T>& c, const T* cnx, const T* cny, const T* cnz, T* curv) {
    const Grid& g = p.g;
    auto X = [&](ll a, ll b, ll d) { return cnx[g.s2(a, b, d)]; };
    auto Y = [&](ll a, ll b, ll d) { return cny[g.s2(a, b, d)]; };
    auto Z = [&](ll a, ll b, ll d) { return cnz[g.s2(a, b, d)]; };
#pragma omp parallel for collapse(2) schedule(static)
    for (ll k = 1; k <= g.nz; ++k)
        for (ll j = 1; j <= g.ny; ++j)
            for (ll i = 1; i <= g.nx; ++i) {
                T kxx = deriv_x(c, X, i, j, k), kyy = deriv_y(c, Y, i, j, k), kzz = deriv_z(c, Z, i, j, k);
                T kxy = deriv_y(c, X, i, j, k), kxz = deriv_z(c, X, i, j, k);
                T kyx = deriv_x(c, Y, i, j, k), kyz = deriv_z(c, Y, i, j, k);
                T kzx = deriv_x(c, Z, i, j, k), kzy = deriv_y(c, Z, i, j, k);
                ll n = g.s2(i, j, k);
                T x = cnx[n], y = cny[n], z = cnz[n];
                curv[g.s1(i, j, k)] = (x * x - T(1)) * kxx + (y * y - T(1)) * kyy + (z * z - T(1)) * kzz +
                                      x * y * (kxy + kyx) + x * z * (kxz + kzx) + y * z * (kzy + kyz);
            }
}

template <class T>
void color_gradient(const P<T>& p, const int32_t* walls, const int32_t* wt, const T* snx, const T* sny,
                    const T* snz, T* phi, T* cnx, T* cny, T* cnz, T* cnorm, T* curv) {
    Consts<T> c;
    extrapolate_phi_to_solid(p, c, wt, phi);
    interface_normals(p, c, walls, phi, cnx, cny, cnz, cnorm);
    wetting(p, wt, snx, sny, snz, cnx, cny, cnz, cnorm);
    extrapolate_normal_to_solid(p, c, wt, cnx, cny, cnz);
    curvature(p, c, cnx, cny, cnz, curv);
}

/* ---------------------------------------------------------------------------
 * MRT collision with CSF force and Rothman–Keller recolouring for one node
 * (src/main_iteration_GPU.cu:115-345; mrt == 2 rates :164-171).
 * g1/g2: the 19 pre-collision populations of each component in natural
 * direction order; on return they hold the post-collision, recoloured ones.
 * ------------------------------------------------------------------------- */
template <class T>
T collide_node(const P<T>& p, const Consts<T>& c, T* g1, T* g2, T cnx, T cny, T cnz, T curv, T cnorm) {
    T ft[19];
    for (int q = 0; q < 19; ++q) ft[q] = g1[q] + g2[q];
    T rho1 = g1[0], rho2 = g2[0];
    for (int q = 1; q < 19; ++q) rho1 = rho1 + g1[q];
    for (int q = 1; q < 19; ++q) rho2 = rho2 + g2[q];
    const T phi = (rho1 - rho2) / (rho1 + rho2);

    T tmp = T(0.5) * p.gamma * curv * cnorm;
    const T fx = tmp * cnx, fy = tmp * cny, fz = tmp * cnz + p.force_z;

    const T omega = T(1) / (T(6) / ((T(1) + phi) * p.nui1 + (T(1) - phi) * p.nui2) + T(0.5));
    const T s_nu = omega, s_e = T(1.19), s_e2 = T(1.4), s_pi = T(1.4), s_q = T(1.2), s_t = T(1.98);

    const T den = rho1 + rho2;
    const T ux = ft[1] - ft[2] + ft[7] - ft[8] + ft[9] - ft[10] + ft[11] - ft[12] + ft[13] - ft[14] + T(0.5) * fx;
    const T uy = ft[3] - ft[4] + ft[7] + ft[8] - ft[9] - ft[10] + ft[15] - ft[16] + ft[17] - ft[18] + T(0.5) * fy;
    const T uz = ft[5] - ft[6] + ft[11] + ft[12] - ft[13] - ft[14] + ft[15] + ft[16] - ft[17] - ft[18] + T(0.5) * fz;
    const T u2 = ux * ux + uy * uy + uz * uz;

    T sum1 = ft[1] + ft[2] + ft[3] + ft[4] + ft[5] + ft[6];
    T sum2 = ft[7] + ft[8] + ft[9] + ft[10] + ft[11] + ft[12] + ft[13] + ft[14] + ft[15] + ft[16] + ft[17] + ft[18];
    T sum3 = ft[7] - ft[8] + ft[9] - ft[10] + ft[11] - ft[12] + ft[13] - ft[14];
    T sum4 = ft[7] + ft[8] - ft[9] - ft[10] + ft[15] - ft[16] + ft[17] - ft[18];
    T sum5 = ft[11] + ft[12] - ft[13] - ft[14] + ft[15] + ft[16] - ft[17] - ft[18];
    T sum6 = T(2) * (ft[1] + ft[2]) - ft[3] - ft[4] - ft[5] - ft[6];
    T sum7 = ft[7] + ft[8] + ft[9] + ft[10] + ft[11] + ft[12] + ft[13] + ft[14] - T(2) * (ft[15] + ft[16] + ft[17] + ft[18]);
    T sum8 = ft[3] + ft[4] - ft[5] - ft[6];
    T sum9 = ft[7] + ft[8] + ft[9] + ft[10] - ft[11] - ft[12] - ft[13] - ft[14];

    T m_rho = den;
    T m_e = T(-30) * ft[0] - T(11) * sum1 + T(8) * sum2;
    T m_e2 = T(12) * ft[0] - T(4) * sum1 + sum2;
    T m_jx = ft[1] - ft[2] + sum3;
    T m_qx = T(-4) * (ft[1] - ft[2]) + sum3;
    T m_jy = ft[3] - ft[4] + sum4;
    T m_qy = T(-4) * (ft[3] - ft[4]) + sum4;
    T m_jz = ft[5] - ft[6] + sum5;
    T m_qz = T(-4) * (ft[5] - ft[6]) + sum5;
    T m_3pxx = sum6 + sum7;
    T m_3pixx = T(-2) * sum6 + sum7;
    T m_pww = sum8 + sum9;
    T m_piww = T(-2) * sum8 + sum9;
    T m_pxy = ft[7] - ft[8] - ft[9] + ft[10];
    T m_pyz = ft[15] - ft[16] - ft[17] + ft[18];
    T m_pzx = ft[11] - ft[12] - ft[13] + ft[14];
    T m_tx = ft[7] - ft[8] + ft[9] - ft[10] - ft[11] + ft[12] - ft[13] + ft[14];
    T m_ty = -ft[7] - ft[8] + ft[9] + ft[10] + ft[15] - ft[16] + ft[17] - ft[18];
    T m_tz = ft[11] + ft[12] - ft[13] - ft[14] - ft[15] - ft[16] + ft[17] + ft[18];

    const T c23 = T(-0.666666666666666667), c13 = T(0.333333333333333333);
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

    m_rho = c.mrt_coef1 * m_rho;
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
    sum1 = m_rho - T(11) * m_e - T(4) * m_e2;
    sum2 = T(2) * m_3pxx - T(4) * m_3pixx;
    sum3 = m_pww - T(2) * m_piww;
    sum4 = m_rho + T(8) * m_e + m_e2;
    sum5 = m_jx + m_qx;
    sum6 = m_jy + m_qy;
    sum7 = m_jz + m_qz;
    sum8 = m_3pxx + m_3pixx;
    sum9 = m_pww + m_piww;

    ft[0] = m_rho - T(30) * m_e + T(12) * m_e2;
    ft[1] = sum1 + m_jx - T(4) * m_qx + sum2;
    ft[2] = sum1 - m_jx + T(4) * m_qx + sum2;
    ft[3] = sum1 + m_jy - T(4) * m_qy - T(0.5) * sum2 + sum3;
    ft[4] = sum1 - m_jy + T(4) * m_qy - T(0.5) * sum2 + sum3;
    ft[5] = sum1 + m_jz - T(4) * m_qz - T(0.5) * sum2 - sum3;
    ft[6] = sum1 - m_jz + T(4) * m_qz - T(0.5) * sum2 - sum3;
    ft[7] = sum4 + sum5 + sum6 + sum8 + sum9 + m_pxy + m_tx - m_ty;
    ft[8] = sum4 - sum5 + sum6 + sum8 + sum9 - m_pxy - m_tx - m_ty;
    ft[9] = sum4 + sum5 - sum6 + sum8 + sum9 - m_pxy + m_tx + m_ty;
    ft[10] = sum4 - sum5 - sum6 + sum8 + sum9 + m_pxy - m_tx + m_ty;
    ft[11] = sum4 + sum5 + sum7 + sum8 - sum9 + m_pzx - m_tx + m_tz;
    ft[12] = sum4 - sum5 + sum7 + sum8 - sum9 - m_pzx + m_tx + m_tz;
    ft[13] = sum4 + sum5 - sum7 + sum8 - sum9 - m_pzx - m_tx - m_tz;
    ft[14] = sum4 - sum5 - sum7 + sum8 - sum9 + m_pzx + m_tx - m_tz;
    ft[15] = sum4 + sum6 + sum7 - sum8 * T(2) + m_pyz + m_ty - m_tz;
    ft[16] = sum4 - sum6 + sum7 - sum8 * T(2) - m_pyz - m_ty - m_tz;
    ft[17] = sum4 + sum6 - sum7 - sum8 * T(2) - m_pyz + m_ty + m_tz;
    ft[18] = sum4 - sum6 - sum7 - sum8 * T(2) + m_pyz - m_ty + m_tz;

    /* recolouring (src/main_iteration_GPU.cu:302-345) */
    const T tmp1 = rho1 / den;
    g1[0] = tmp1 * ft[0];
    g2[0] = ft[0] * (T(1) - tmp1);
    tmp = rho1 * rho2 * p.beta / den;
    const T proj[19] = {T(0), cnx, -cnx, cny, -cny, cnz, -cnz,
                        cnx + cny, -cnx + cny, cnx - cny, -cnx - cny,
                        cnx + cnz, -cnx + cnz, cnx - cnz, -cnx - cnz,
                        cny + cnz, -cny + cnz, cny - cnz, -cny - cnz};
    for (int q = 1; q < 19; ++q) {
        const T wq = q < 7 ? c.w1 : c.rk2;
        g1[q] = tmp1 * ft[q] + wq * tmp * proj[q];
        g2[q] = ft[q] - g1[q];
    }
    return phi;
}

/* Odd (pull from x - e, push to x + e, slot opp(e)) and even (in place,
 * swapped) AA steps over fluid nodes of [1, n]^3
 * (src/main_iteration_GPU.cu:56-388, :395-726). */
template <class T>
void collide_stream(const P<T>& p, bool odd, const int32_t* walls, T* pdf, T* phi, const T* cnx, const T* cny,
                    const T* cnz, const T* curv, const T* cnorm) {
    const Grid& g = p.g;
    Consts<T> c;
#pragma omp parallel for collapse(2) schedule(static)
    for (ll k = 1; k <= g.nz; ++k)
        for (ll j = 1; j <= g.ny; ++j)
            for (ll i = 1; i <= g.nx; ++i) {
                if (walls[g.s2(i, j, k)] != 0) continue;
                T g1[19], g2[19];
                for (int q = 0; q < 19; ++q) {
                    if (odd) {
                        g1[q] = pdf[g.f1(i - EX[q], j - EY[q], k - EZ[q], q, 0)];
                        g2[q] = pdf[g.f1(i - EX[q], j - EY[q], k - EZ[q], q, 1)];
                    } else {
                        g1[q] = pdf[g.f1(i, j, k, OPP[q], 0)];
                        g2[q] = pdf[g.f1(i, j, k, OPP[q], 1)];
                    }
                }
                ll n2 = g.s2(i, j, k);
                phi[g.s4(i, j, k)] = collide_node(p, c, g1, g2, cnx[n2], cny[n2], cnz[n2], curv[g.s1(i, j, k)], cnorm[n2]);
                for (int q = 0; q < 19; ++q) {
                    if (odd) {
                        pdf[g.f1(i + EX[q], j + EY[q], k + EZ[q], OPP[q], 0)] = g1[q];
                        pdf[g.f1(i + EX[q], j + EY[q], k + EZ[q], OPP[q], 1)] = g2[q];
                    } else {
                        pdf[g.f1(i, j, k, q, 0)] = g1[q];
                        pdf[g.f1(i, j, k, q, 1)] = g2[q];
                    }
                }
            }
}

/* ---------------------------------------------------------------------------
 * Periodic boundary copies (src/main_iteration_GPU.cu:1529-1733).
 * ------------------------------------------------------------------------- */
/* z faces: directions with ez = -1 leave through z = 1 and enter z = nz; ez = +1 the reverse. */
const int ZUP[5] = {6, 14, 13, 18, 17}, ZDN[5] = {5, 11, 12, 15, 16};
const int YUP[5] = {4, 10, 9, 16, 18}, YDN[5] = {3, 7, 8, 15, 17};

template <class T>
void periodic_pdf_z(const Grid& g, bool odd, T* pdf) {
    for (int gg = 0; gg < 2; ++gg)
        for (ll j = 1; j <= g.ny; ++j)
            for (ll i = 1; i <= g.nx; ++i)
                for (int s = 0; s < 5; ++s) {
                    if (!odd) {
                        pdf[g.f1(i, j, g.nz + 1, ZUP[s], gg)] = pdf[g.f1(i, j, 1, ZUP[s], gg)];
                        pdf[g.f1(i, j, 0, ZDN[s], gg)] = pdf[g.f1(i, j, g.nz, ZDN[s], gg)];
                    } else {
                        pdf[g.f1(i, j, 1, ZUP[s], gg)] = pdf[g.f1(i, j, g.nz + 1, ZUP[s], gg)];
                        pdf[g.f1(i, j, g.nz, ZDN[s], gg)] = pdf[g.f1(i, j, 0, ZDN[s], gg)];
                    }
                }
}
template <class T>
void periodic_pdf_y(const Grid& g, bool odd, T* pdf) {
    for (int gg = 0; gg < 2; ++gg)
        for (ll k = 1; k <= g.nz; ++k)
            for (ll i = 1; i <= g.nx; ++i)
                for (int s = 0; s < 5; ++s) {
                    if (!odd) {
                        pdf[g.f1(i, g.ny + 1, k, YUP[s], gg)] = pdf[g.f1(i, 1, k, YUP[s], gg)];
                        pdf[g.f1(i, 0, k, YDN[s], gg)] = pdf[g.f1(i, g.ny, k, YDN[s], gg)];
                    } else {
                        pdf[g.f1(i, 1, k, YUP[s], gg)] = pdf[g.f1(i, g.ny + 1, k, YUP[s], gg)];
                        pdf[g.f1(i, g.ny, k, YDN[s], gg)] = pdf[g.f1(i, 0, k, YDN[s], gg)];
                    }
                }
}
template <class T>
void periodic_pdf_zy(const Grid& g, bool odd, T* pdf) {
    const ll ny = g.ny, nz = g.nz;
    for (int gg = 0; gg < 2; ++gg)
        for (ll i = 1; i <= g.nx; ++i) {
            if (!odd) {
                pdf[g.f1(i, ny + 1, nz + 1, 18, gg)] = pdf[g.f1(i, 1, 1, 18, gg)];
                pdf[g.f1(i, ny + 1, 0, 16, gg)] = pdf[g.f1(i, 1, nz, 16, gg)];
                pdf[g.f1(i, 0, nz + 1, 17, gg)] = pdf[g.f1(i, ny, 1, 17, gg)];
                pdf[g.f1(i, 0, 0, 15, gg)] = pdf[g.f1(i, ny, nz, 15, gg)];
            } else {
                pdf[g.f1(i, 1, 1, 18, gg)] = pdf[g.f1(i, ny + 1, nz + 1, 18, gg)];
                pdf[g.f1(i, 1, nz, 16, gg)] = pdf[g.f1(i, ny + 1, 0, 16, gg)];
                pdf[g.f1(i, ny, 1, 17, gg)] = pdf[g.f1(i, 0, nz + 1, 17, gg)];
                pdf[g.f1(i, ny, nz, 15, gg)] = pdf[g.f1(i, 0, 0, 15, gg)];
            }
        }
}
template <class T>
void periodic_phi_z(const Grid& g, T* phi) {
    const int ov = 4;
    for (ll j = 1; j <= g.ny; ++j)
        for (ll i = 1; i <= g.nx; ++i)
            for (int k = 1; k <= ov; ++k) {
                phi[g.s4(i, j, k + g.nz)] = phi[g.s4(i, j, k)];
                phi[g.s4(i, j, k - ov)] = phi[g.s4(i, j, g.nz + k - ov)];
            }
}
template <class T>
void periodic_phi_y(const Grid& g, T* phi) {
    const int ov = 4;
    for (ll k = 1; k <= g.nz; ++k)
        for (ll i = 1; i <= g.nx; ++i)
            for (int j = 1; j <= ov; ++j) {
                phi[g.s4(i, j + g.ny, k)] = phi[g.s4(i, j, k)];
                phi[g.s4(i, j - ov, k)] = phi[g.s4(i, g.ny + j - ov, k)];
            }
}
template <class T>
void periodic_phi_zy(const Grid& g, T* phi) {
    const int ov = 4;
    const ll ny = g.ny, nz = g.nz;
    for (ll i = 1; i <= g.nx; ++i)
        for (int k = 1; k <= ov; ++k)
            for (int j = 1; j <= ov; ++j) {
                phi[g.s4(i, j - ov, k - ov)] = phi[g.s4(i, ny + j - ov, nz + k - ov)];
                phi[g.s4(i, j + ny, k - ov)] = phi[g.s4(i, j, nz + k - ov)];
                phi[g.s4(i, j + ny, k + nz)] = phi[g.s4(i, j, k)];
                phi[g.s4(i, j - ov, k + nz)] = phi[g.s4(i, ny + j - ov, k)];
            }
}

/* ---------------------------------------------------------------------------
 * Inlet / outlet boundaries (src/main_iteration_GPU.cu:1009-1524).
 * `keep(new, old, w)` is the reference's  new*(1-w) + old*w  blend.
 * ------------------------------------------------------------------------- */
template <class T> inline T keep(T v_new, T v_old, int w) { return v_new * T(1 - w) + v_old * T(w); }

/* Links that cross the inlet plane: (slot at k=0 of node (i+dx, j+dy), slot at k=1 of (i,j)). */
struct InletLink { int dx, dy, slot0, slot1; };
const InletLink IN_LINKS[5] = {{0, 0, 5, 6}, {-1, 0, 11, 14}, {1, 0, 12, 13}, {0, -1, 15, 18}, {0, 1, 16, 17}};

template <class T>
void inlet_phi(const P<T>& p, ll i, ll j, int w, T* phi) {
    const Grid& g = p.g;
    phi[g.s4(i, j, 0)] = p.phi_inlet * T(1 - w) + phi[g.s4(i, j, 0)] * T(w);
    phi[g.s4(i, j, -1)] = phi[g.s4(i, j, 0)];
    phi[g.s4(i, j, -2)] = phi[g.s4(i, j, 0)];
    phi[g.s4(i, j, -3)] = phi[g.s4(i, j, 0)];
}

template <class T>
void inlet_velocity(const P<T>& p, const Consts<T>& c, bool after_odd, const int32_t* walls, T* phi, T* pdf, const T* W_in) {
    const Grid& g = p.g;
    for (ll j = 1; j <= g.ny; ++j)
        for (ll i = 1; i <= g.nx; ++i) {
            const int w = walls[g.s2(i, j, 1)];
            inlet_phi(p, i, j, w, phi);
            T t2 = W_in[g.s1(i, j, 0)] * p.relaxation;
            T t1 = t2 * p.sa_inject;
            t2 = t2 - t1;
            for (int gg = 0; gg < 2; ++gg) {
                const T inj = gg == 0 ? t1 : t2;
                for (int s = 0; s < 5; ++s) {
                    const InletLink& L = IN_LINKS[s];
                    const T wq = s == 0 ? c.w1 : c.w2;
                    if (!after_odd) {
                        ll d = g.f1(i + L.dx, j + L.dy, 0, L.slot0, gg);
                        pdf[d] = keep((pdf[g.f1(i, j, 1, L.slot1, gg)] + T(6.0) * wq * inj), pdf[d], w);
                    } else {
                        ll d = g.f1(i, j, 1, L.slot1, gg);
                        pdf[d] = keep((pdf[g.f1(i + L.dx, j + L.dy, 0, L.slot0, gg)] + T(6.0) * wq * inj), pdf[d], w);
                    }
                }
            }
        }
}

template <class T>
void inlet_pressure(const P<T>& p, bool after_odd, const int32_t* walls, T* phi, T* pdf) {
    const Grid& g = p.g;
    const T c3 = T(0.333333333333333333), c6 = T(0.166666666666666667);
    for (ll j = 1; j <= g.ny; ++j)
        for (ll i = 1; i <= g.nx; ++i) {
            const int w = walls[g.s2(i, j, 1)];
            inlet_phi(p, i, j, w, phi);
            T r2 = p.rho_in;
            T r1 = p.rho_in * p.sa_inject;
            r2 = r2 - r1;
            for (int gg = 0; gg < 2; ++gg) {
                auto F = [&](ll a, ll b, ll k, int e) -> T& { return pdf[g.f1(a, b, k, e, gg)]; };
                const T rho_c = gg == 0 ? r1 : r2;
                if (!after_odd) {
                    T t = (rho_c - (F(i, j, 1, 0) + F(i - 1, j, 1, 1) + F(i + 1, j, 1, 2) + F(i, j - 1, 1, 3) +
                                    F(i, j + 1, 1, 4) + F(i - 1, j - 1, 1, 7) + F(i + 1, j - 1, 1, 8) +
                                    F(i - 1, j + 1, 1, 9) + F(i + 1, j + 1, 1, 10) +
                                    T(2) * (F(i, j, 2, 6) + F(i + 1, j, 2, 14) + F(i - 1, j, 2, 13) +
                                            F(i, j + 1, 2, 18) + F(i, j - 1, 2, 17)))) * p.relaxation;
                    T tnx = T(0.5) * (F(i - 1, j, 1, 1) + F(i - 1, j - 1, 1, 7) + F(i - 1, j + 1, 1, 9) -
                                      (F(i + 1, j, 1, 2) + F(i + 1, j - 1, 1, 8) + F(i + 1, j + 1, 1, 10)));
                    T tny = T(0.5) * (F(i, j - 1, 1, 3) + F(i - 1, j - 1, 1, 7) + F(i + 1, j - 1, 1, 8) -
                                      (F(i, j + 1, 1, 4) + F(i + 1, j + 1, 1, 10) + F(i - 1, j + 1, 1, 9)));
                    F(i, j, 0, 5) = keep((F(i, j, 2, 6) + c3 * t), F(i, j, 0, 5), w);
                    F(i - 1, j, 0, 11) = keep((F(i + 1, j, 2, 14) + c6 * t - tnx), F(i - 1, j, 0, 11), w);
                    F(i + 1, j, 0, 12) = keep((F(i - 1, j, 2, 13) + c6 * t + tnx), F(i + 1, j, 0, 12), w);
                    F(i, j - 1, 0, 15) = keep((F(i, j + 1, 2, 18) + c6 * t - tny), F(i, j - 1, 0, 15), w);
                    F(i, j + 1, 0, 16) = keep((F(i, j - 1, 2, 17) + c6 * t + tny), F(i, j + 1, 0, 16), w);
                } else {
                    T t = (rho_c - (F(i, j, 1, 0) + F(i, j, 1, 2) + F(i, j, 1, 1) + F(i, j, 1, 4) + F(i, j, 1, 3) +
                                    F(i, j, 1, 8) + F(i, j, 1, 7) + F(i, j, 1, 10) + F(i, j, 1, 9) +
                                    T(2) * (F(i, j, 1, 5) + F(i, j, 1, 11) + F(i, j, 1, 12) + F(i, j, 1, 15) +
                                            F(i, j, 1, 16)))) * p.relaxation;
                    T tnx = T(0.5) * (F(i, j, 1, 2) + F(i, j, 1, 8) + F(i, j, 1, 10) -
                                      (F(i, j, 1, 1) + F(i, j, 1, 7) + F(i, j, 1, 9)));
                    T tny = T(0.5) * (F(i, j, 1, 4) + F(i, j, 1, 9) + F(i, j, 1, 10) -
                                      (F(i, j, 1, 3) + F(i, j, 1, 8) + F(i, j, 1, 7)));
                    F(i, j, 1, 6) = keep((F(i, j, 1, 5) + c3 * t), F(i, j, 1, 6), w);
                    F(i, j, 1, 13) = keep((F(i, j, 1, 12) + c6 * t + tnx), F(i, j, 1, 13), w);
                    F(i, j, 1, 14) = keep((F(i, j, 1, 11) + c6 * t - tnx), F(i, j, 1, 14), w);
                    F(i, j, 1, 17) = keep((F(i, j, 1, 16) + c6 * t + tny), F(i, j, 1, 17), w);
                    F(i, j, 1, 18) = keep((F(i, j, 1, 15) + c6 * t - tny), F(i, j, 1, 18), w);
                }
            }
        }
}

/* Links that cross the outlet plane: (slot at nz+1 of (i+dx, j+dy), slot at nz of (i,j), convective buffer slot). */
struct OutletLink { int dx, dy, slot_up, slot_dn, buf; };
const OutletLink OUT_LINKS[5] = {{0, 0, 6, 5, 6}, {-1, 0, 13, 12, 13}, {1, 0, 14, 11, 14}, {0, -1, 17, 16, 17}, {0, 1, 18, 15, 18}};

template <class T>
void outlet_convective(const P<T>& p, bool after_odd, const int32_t* walls, T* phi, T* phi_cv, T* pdf, T* f_cv, T* g_cv) {
    const Grid& g = p.g;
    const ll nz = g.nz;
    for (ll j = 1; j <= g.ny; ++j)
        for (ll i = 1; i <= g.nx; ++i) {
            const T u_convec = p.uin_avg;
            const T temp = T(1) / (T(1) + u_convec);
            const int w = walls[g.s2(i, j, nz)];
            T& pb = phi_cv[g.s1(i, j, 0)];
            phi[g.s4(i, j, nz + 1)] = ((pb + u_convec * phi[g.s4(i, j, nz)]) * temp) * T(1 - w) + phi[g.s4(i, j, nz + 1)] * T(w);
            pb = phi[g.s4(i, j, nz + 1)];
            phi[g.s4(i, j, nz + 2)] = phi[g.s4(i, j, nz + 1)];
            phi[g.s4(i, j, nz + 3)] = phi[g.s4(i, j, nz + 1)];
            phi[g.s4(i, j, nz + 4)] = phi[g.s4(i, j, nz + 1)];
            for (int gg = 0; gg < 2; ++gg) {
                T* buf = gg == 0 ? f_cv : g_cv;
                for (int s = 0; s < 5; ++s) {
                    const OutletLink& L = OUT_LINKS[s];
                    if (!after_odd) {
                        ll d = g.f1(i + L.dx, j + L.dy, nz + 1, L.slot_up, gg);
                        pdf[d] = ((buf[g.cnv(i, j, L.buf)] + u_convec * pdf[g.f1(i + L.dx, j + L.dy, nz, L.slot_up, gg)]) * temp) * T(1 - w) + pdf[d] * T(w);
                    } else {
                        ll d = g.f1(i, j, nz, L.slot_dn, gg);
                        pdf[d] = ((buf[g.cnv(i, j, L.buf)] + u_convec * pdf[g.f1(i, j, nz - 1, L.slot_dn, gg)]) * temp) * T(1 - w) + pdf[d] * T(w);
                    }
                }
                for (int s = 0; s < 5; ++s) {
                    const OutletLink& L = OUT_LINKS[s];
                    buf[g.cnv(i, j, L.buf)] = after_odd ? pdf[g.f1(i, j, nz, L.slot_dn, gg)]
                                                        : pdf[g.f1(i + L.dx, j + L.dy, nz + 1, L.slot_up, gg)];
                }
            }
        }
}

template <class T>
void outlet_pressure(const P<T>& p, bool after_odd, const int32_t* walls, T* phi, T* pdf) {
    const Grid& g = p.g;
    const ll nz = g.nz;
    const T c3 = T(0.333333333333333333), c6 = T(0.166666666666666667);
    for (ll j = 1; j <= g.ny; ++j)
        for (ll i = 1; i <= g.nx; ++i) {
            const int w = walls[g.s2(i, j, nz)];
            phi[g.s4(i, j, nz + 1)] = phi[g.s4(i, j, nz)];
            phi[g.s4(i, j, nz + 2)] = phi[g.s4(i, j, nz)];
            phi[g.s4(i, j, nz + 3)] = phi[g.s4(i, j, nz)];
            phi[g.s4(i, j, nz + 4)] = phi[g.s4(i, j, nz)];
            auto F = [&](ll a, ll b, ll k, int e, int gg) -> T& { return pdf[g.f1(a, b, k, e, gg)]; };
            T t1;
            if (!after_odd) {
                t1 = (F(i, j, nz, 0, 0) + F(i - 1, j, nz, 1, 0) + F(i + 1, j, nz, 2, 0) + F(i, j - 1, nz, 3, 0) +
                      F(i, j + 1, nz, 4, 0) + F(i - 1, j - 1, nz, 7, 0) + F(i + 1, j - 1, nz, 8, 0) +
                      F(i - 1, j + 1, nz, 9, 0) + F(i + 1, j + 1, nz, 10, 0) +
                      T(2) * (F(i, j, nz - 1, 5, 0) + F(i - 1, j, nz - 1, 11, 0) + F(i + 1, j, nz - 1, 12, 0) +
                              F(i, j - 1, nz - 1, 15, 0) + F(i, j + 1, nz - 1, 16, 0)) +
                      F(i, j, nz, 0, 1) + F(i - 1, j, nz, 1, 1) + F(i + 1, j, nz, 2, 1) + F(i, j - 1, nz, 3, 1) +
                      F(i, j + 1, nz, 4, 1) + F(i - 1, j - 1, nz, 7, 1) + F(i + 1, j - 1, nz, 8, 1) +
                      F(i - 1, j + 1, nz, 9, 1) + F(i + 1, j + 1, nz, 10, 1) +
                      T(2) * (F(i, j, nz - 1, 5, 1) + F(i - 1, j, nz - 1, 11, 1) + F(i + 1, j, nz - 1, 12, 1) +
                              F(i, j - 1, nz - 1, 15, 1) + F(i, j + 1, nz - 1, 16, 1))) - p.rho_out;
            } else {
                t1 = (F(i, j, nz, 0, 0) + F(i, j, nz, 2, 0) + F(i, j, nz, 1, 0) + F(i, j, nz, 4, 0) + F(i, j, nz, 3, 0) +
                      F(i, j, nz, 8, 0) + F(i, j, nz, 7, 0) + F(i, j, nz, 10, 0) + F(i, j, nz, 9, 0) +
                      T(2) * (F(i, j, nz, 6, 0) + F(i, j, nz, 14, 0) + F(i, j, nz, 13, 0) + F(i, j, nz, 18, 0) +
                              F(i, j, nz, 17, 0)) +
                      F(i, j, nz, 0, 1) + F(i, j, nz, 2, 1) + F(i, j, nz, 1, 1) + F(i, j, nz, 4, 1) + F(i, j, nz, 3, 1) +
                      F(i, j, nz, 8, 1) + F(i, j, nz, 7, 1) + F(i, j, nz, 10, 1) + F(i, j, nz, 9, 1) +
                      T(2) * (F(i, j, nz, 6, 1) + F(i, j, nz, 14, 1) + F(i, j, nz, 13, 1) + F(i, j, nz, 18, 1) +
                              F(i, j, nz, 17, 1))) - p.rho_out;
            }
            T t2 = t1 * T(0.5) * (T(1) - phi[g.s4(i, j, nz)]);
            t1 = t1 - t2;
            for (int gg = 0; gg < 2; ++gg) {
                const T t = gg == 0 ? t1 : t2;
                if (!after_odd) {
                    T tnx = T(0.5) * (F(i - 1, j, nz, 1, gg) + F(i - 1, j - 1, nz, 7, gg) + F(i - 1, j + 1, nz, 9, gg) -
                                      (F(i + 1, j, nz, 2, gg) + F(i + 1, j - 1, nz, 8, gg) + F(i + 1, j + 1, nz, 10, gg)));
                    T tny = T(0.5) * (F(i, j - 1, nz, 3, gg) + F(i - 1, j - 1, nz, 7, gg) + F(i + 1, j - 1, nz, 8, gg) -
                                      (F(i, j + 1, nz, 4, gg) + F(i + 1, j + 1, nz, 10, gg) + F(i - 1, j + 1, nz, 9, gg)));
                    F(i, j, nz + 1, 6, gg) = keep((F(i, j, nz - 1, 5, gg) - c3 * t), F(i, j, nz + 1, 6, gg), w);
                    F(i - 1, j, nz + 1, 13, gg) = keep((F(i + 1, j, nz - 1, 12, gg) - c6 * t - tnx), F(i - 1, j, nz + 1, 13, gg), w);
                    F(i + 1, j, nz + 1, 14, gg) = keep((F(i - 1, j, nz - 1, 11, gg) - c6 * t + tnx), F(i + 1, j, nz + 1, 14, gg), w);
                    F(i, j - 1, nz + 1, 17, gg) = keep((F(i, j + 1, nz - 1, 16, gg) - c6 * t - tny), F(i, j - 1, nz + 1, 17, gg), w);
                    F(i, j + 1, nz + 1, 18, gg) = keep((F(i, j - 1, nz - 1, 15, gg) - c6 * t + tny), F(i, j + 1, nz + 1, 18, gg), w);
                } else {
                    T tnx = T(0.5) * (F(i, j, nz, 2, gg) + F(i, j, nz, 8, gg) + F(i, j, nz, 10, gg) -
                                      (F(i, j, nz, 1, gg) + F(i, j, nz, 7, gg) + F(i, j, nz, 9, gg)));
                    T tny = T(0.5) * (F(i, j, nz, 4, gg) + F(i, j, nz, 10, gg) + F(i, j, nz, 9, gg) -
                                      (F(i, j, nz, 3, gg) + F(i, j, nz, 7, gg) + F(i, j, nz, 8, gg)));
                    F(i, j, nz, 5, gg) = keep((F(i, j, nz, 6, gg) - c3 * t), F(i, j, nz, 5, gg), w);
                    F(i, j, nz, 11, gg) = keep((F(i, j, nz, 14, gg) - c6 * t + tnx), F(i, j, nz, 11, gg), w);
                    F(i, j, nz, 12, gg) = keep((F(i, j, nz, 13, gg) - c6 * t - tnx), F(i, j, nz, 12, gg), w);
                    F(i, j, nz, 15, gg) = keep((F(i, j, nz, 18, gg) - c6 * t + tny), F(i, j, nz, 15, gg), w);
                    F(i, j, nz, 16, gg) = keep((F(i, j, nz, 17, gg) - c6 * t - tny), F(i, j, nz, 16, gg), w);
                }
            }
        }
}

/* Porous plate (src/main_iteration_GPU.cu:1744-1882). `b` is the blocked
 * component, `o` the other one. */
template <class T>
void porous_plate(const P<T>& p, bool after_odd, T* pdf) {
    const Grid& g = p.g;
    const int zp = p.Zplate;
    if (!(zp >= 1 && zp <= g.nz)) return;
    if (p.plate_cmd != 1 && p.plate_cmd != 2) return;
    const int b = p.plate_cmd == 1 ? 0 : 1, o = 1 - b;
    auto F = [&](ll a, ll bb, ll k, int e, int gg) -> T& { return pdf[g.f1(a, bb, k, e, gg)]; };
    for (ll j = 1; j <= g.ny; ++j)
        for (ll i = 1; i <= g.nx; ++i) {
            if (!after_odd) {
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
}

/* One time step in the order of main_iteration_kernel_GPU
 * (src/main_iteration_GPU.cu:1890-2056). */
template <class T>
void step(const P<T>& p, int ntime, const int32_t* walls, const int32_t* wt, const T* snx, const T* sny, const T* snz,
          T* pdf, T* phi, T* cnx, T* cny, T* cnz, T* cnorm, T* curv, const T* W_in, T* f_cv, T* g_cv, T* phi_cv) {
    const Grid& g = p.g;
    Consts<T> c;
    const bool odd = (ntime % 2) != 0;
    collide_stream(p, odd, walls, pdf, phi, cnx, cny, cnz, curv, cnorm);
    if (p.kper) { periodic_pdf_z(g, odd, pdf); periodic_phi_z(g, phi); }
    if (p.jper) { periodic_pdf_y(g, odd, pdf); periodic_phi_y(g, phi); }
    if (p.jper && p.kper) { periodic_pdf_zy(g, odd, pdf); periodic_phi_zy(g, phi); }
    if (p.open_z()) {
        if (p.inlet_BC == 1) inlet_velocity(p, c, odd, walls, phi, pdf, W_in);
        else if (p.inlet_BC == 2) inlet_pressure(p, odd, walls, phi, pdf);
        if (p.outlet_BC == 1) outlet_convective(p, odd, walls, phi, phi_cv, pdf, f_cv, g_cv);
        else if (p.outlet_BC == 2) outlet_pressure(p, odd, walls, phi, pdf);
    }
    if (p.plate_cmd != 0) porous_plate(p, odd, pdf);
    color_gradient(p, walls, wt, snx, sny, snz, phi, cnx, cny, cnz, cnorm, curv);
}

/* ---------------------------------------------------------------------------
 * Set-up restatements.
 * ------------------------------------------------------------------------- */
/* Domain walls added to the .dat body (src/Misc.cpp:75-98, 139-192). */
void set_walls(const mflbm_control* ctl, const uint8_t* geo, int32_t* walls_global) {
    Grid g{ctl->nxGlobal, ctl->nyGlobal, ctl->nzGlobal};
    for (ll k = 1; k <= g.nz; ++k)
        for (ll j = 1; j <= g.ny; ++j)
            for (ll i = 1; i <= g.nx; ++i)
                walls_global[g.s0(i, j, k)] = geo ? (int32_t)geo[(i - 1) + g.ny * ((j - 1) + g.nx * (k - 1))] : 0;
    for (ll k = 1; k <= g.nz; ++k)
        for (ll j = 1; j <= g.ny; ++j)
            for (ll i = 1; i <= g.nx; ++i) {
                if (ctl->domain_wall_status_z_min == 1) walls_global[g.s0(i, j, 1)] = 1;
                if (ctl->domain_wall_status_z_max == 1) walls_global[g.s0(i, j, g.nz)] = 1;
                if (ctl->domain_wall_status_x_min == 1) walls_global[g.s0(1, j, k)] = 1;
                if (ctl->domain_wall_status_x_max == 1) walls_global[g.s0(g.nx, j, k)] = 1;
                if (ctl->domain_wall_status_y_min == 1) walls_global[g.s0(i, 1, k)] = 1;
                if (ctl->domain_wall_status_y_max == 1) walls_global[g.s0(i, g.ny, k)] = 1;
            }
}

/* geometry_preprocessing_new (src/Geometry_preprocessing.cpp:29-403). */
template <class T>
void geometry_preprocess(const mflbm_control* ctl, const int32_t* walls_global, int32_t* walls, int32_t* wt,
                         T* snx, T* sny, T* snz, mflbm_geometry_counts* cnt) {
    const Grid g{ctl->nxGlobal, ctl->nyGlobal, ctl->nzGlobal};
    const ll G = 10, NX = g.nx + 2 * G, NY = g.ny + 2 * G, NZ = g.nz + 2 * G;
    auto t = [&](ll x, ll y, ll z) { return (x + G - 1) + NX * ((y + G - 1) + NY * (z + G - 1)); };
    std::vector<int32_t> tmp(NX * NY * NZ, 0);
    std::vector<T> sm1(NX * NY * NZ), sm2(NX * NY * NZ);
    for (ll k = 1; k <= g.nz; ++k)
        for (ll j = 1; j <= g.ny; ++j)
            for (ll i = 1; i <= g.nx; ++i) tmp[t(i, j, k)] = walls_global[g.s0(i, j, k)];
    /* ghost fill: z, then y over all z, then x over all y,z (periodic or replicate) */
    for (ll j = 1; j <= g.ny; ++j)
        for (ll i = 1; i <= g.nx; ++i) {
            for (ll k = 1 - G; k <= 0; ++k) tmp[t(i, j, k)] = ctl->kper ? tmp[t(i, j, g.nz + k)] : tmp[t(i, j, 1)];
            for (ll k = g.nz + 1; k <= g.nz + G; ++k) tmp[t(i, j, k)] = ctl->kper ? tmp[t(i, j, k - g.nz)] : tmp[t(i, j, g.nz)];
        }
    for (ll k = 1 - G; k <= g.nz + G; ++k)
        for (ll i = 1; i <= g.nx; ++i) {
            for (ll j = 1 - G; j <= 0; ++j) tmp[t(i, j, k)] = ctl->jper ? tmp[t(i, g.ny + j, k)] : tmp[t(i, 1, k)];
            for (ll j = g.ny + 1; j <= g.ny + G; ++j) tmp[t(i, j, k)] = ctl->jper ? tmp[t(i, j - g.ny, k)] : tmp[t(i, g.ny, k)];
        }
    for (ll k = 1 - G; k <= g.nz + G; ++k)
        for (ll j = 1 - G; j <= g.ny + G; ++j) {
            for (ll i = 1 - G; i <= 0; ++i) tmp[t(i, j, k)] = ctl->iper ? tmp[t(g.nx + i, j, k)] : tmp[t(1, j, k)];
            for (ll i = g.nx + 1; i <= g.nx + G; ++i) tmp[t(i, j, k)] = ctl->iper ? tmp[t(i - g.nx, j, k)] : tmp[t(g.nx, j, k)];
        }
    for (ll k = -1; k <= g.nz + 2; ++k)
        for (ll j = -1; j <= g.ny + 2; ++j)
            for (ll i = -1; i <= g.nx + 2; ++i) walls[g.s2(i, j, k)] = tmp[t(i, j, k)];
    for (ll n = 0; n < NX * NY * NZ; ++n) { sm1[n] = T(tmp[n]); sm2[n] = T(tmp[n]); }
    /* classification (in place; the result does not depend on visiting order) */
    for (ll k = 2 - G; k <= g.nz + G - 1; ++k)
        for (ll j = 2 - G; j <= g.ny + G - 1; ++j)
            for (ll i = 2 - G; i <= g.nx + G - 1; ++i) {
                int32_t& v = tmp[t(i, j, k)];
                if (v == 1) {
                    for (int q = 1; q <= 18; ++q)
                        if (tmp[t(i + EX[q], j + EY[q], k + EZ[q])] <= 0) { v = 2; break; }
                }
                if (v == 0) {
                    for (int q = 1; q <= 18; ++q)
                        if (tmp[t(i + EX[q], j + EY[q], k + EZ[q])] >= 1) { v = -1; break; }
                }
            }
    for (ll k = -3; k <= g.nz + 4; ++k)
        for (ll j = -3; j <= g.ny + 4; ++j)
            for (ll i = -3; i <= g.nx + 4; ++i) wt[g.s4(i, j, k)] = tmp[t(i, j, k)];
    /* four 27-point smoothing passes, Jacobi (src/Geometry_preprocessing.cpp:187-206) */
    static const int ix[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
    static const int iy[27] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, -1, 1, -1, 1};
    static const int iz[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1, -1, 1, 1, -1, -1, 1, 1, -1};
    const T we[4] = {T(8) / T(27), T(2) / T(27), T(1) / T(54), T(1) / T(216)};
    for (int it = 0; it < 4; ++it) {
#pragma omp parallel for collapse(2) schedule(static)
        for (ll k = 2 - G; k <= g.nz + G - 1; ++k)
            for (ll j = 2 - G; j <= g.ny + G - 1; ++j)
                for (ll i = 2 - G; i <= g.nx + G - 1; ++i) {
                    T s = T(0);
                    for (int q = 0; q < 27; ++q) {
                        int m = ix[q] * ix[q] + iy[q] * iy[q] + iz[q] * iz[q];
                        s += sm1[t(i + ix[q], j + iy[q], k + iz[q])] * we[m];
                    }
                    sm2[t(i, j, k)] = s;
                }
#pragma omp parallel for collapse(2) schedule(static)
        for (ll k = 2 - G; k <= g.nz + G - 1; ++k)
            for (ll j = 2 - G; j <= g.ny + G - 1; ++j)
                for (ll i = 2 - G; i <= g.nx + G - 1; ++i) sm1[t(i, j, k)] = sm2[t(i, j, k)];
    }
    cnt->num_solid_boundary_global = cnt->num_fluid_boundary_global = 0;
    cnt->num_solid_boundary = cnt->num_fluid_boundary = 0;
    for (ll k = -3; k <= g.nz + 4; ++k)
        for (ll j = -3; j <= g.ny + 4; ++j)
            for (ll i = -3; i <= g.nx + 4; ++i) {
                int v = tmp[t(i, j, k)];
                bool in3 = i >= -2 && i <= g.nx + 3 && j >= -2 && j <= g.ny + 3 && k >= -2 && k <= g.nz + 3;
                if (v == 2) { cnt->num_solid_boundary_global++; if (in3) cnt->num_solid_boundary++; }
                if (v == -1) { cnt->num_fluid_boundary_global++; if (in3) cnt->num_fluid_boundary++; }
            }
    cnt->pore_sum = 0;
    for (ll k = 1; k <= g.nz; ++k)
        for (ll j = 1; j <= g.ny; ++j)
            for (ll i = 1; i <= g.nx; ++i) cnt->pore_sum += walls[g.s2(i, j, k)] <= 0;
    /* ISO8 solid normal at fluid boundary nodes (src/Geometry_preprocessing.cpp:226-386) */
    Consts<T> c;
    const T eps = T(std::numeric_limits<float>::epsilon());
    auto S = [&](ll a, ll b, ll d) { return sm2[t(a, b, d)]; };
#pragma omp parallel for collapse(2) schedule(static)
    for (ll k = -3; k <= g.nz + 4; ++k)
        for (ll j = -3; j <= g.ny + 4; ++j)
            for (ll i = -3; i <= g.nx + 4; ++i) {
                if (tmp[t(i, j, k)] != -1) continue;
                const T* W = c.iso8;
                T nwx = W[0] * (S(i + 1, j, k) - S(i - 1, j, k)) +
                    W[1] * (S(i + 1, j + 1, k) - S(i - 1, j - 1, k) + S(i + 1, j - 1, k) - S(i - 1, j + 1, k) + S(i + 1, j, k + 1) - S(i - 1, j, k - 1) + S(i + 1, j, k - 1) - S(i - 1, j, k + 1)) +
                    W[2] * (S(i + 1, j + 1, k + 1) - S(i - 1, j - 1, k - 1) + S(i + 1, j + 1, k - 1) - S(i - 1, j - 1, k + 1) + S(i + 1, j - 1, k + 1) - S(i - 1, j + 1, k - 1) + S(i + 1, j - 1, k - 1) - S(i - 1, j + 1, k + 1)) +
                    W[3] * (S(i + 2, j, k) - S(i - 2, j, k)) +
                    W[4] * (S(i + 2, j + 1, k) - S(i - 2, j - 1, k) + S(i + 2, j - 1, k) - S(i - 2, j + 1, k) + S(i + 2, j, k + 1) - S(i - 2, j, k - 1) + S(i + 2, j, k - 1) - S(i - 2, j, k + 1) +
                            S(i + 1, j + 2, k) - S(i - 1, j - 2, k) + S(i + 1, j - 2, k) - S(i - 1, j + 2, k) + S(i + 1, j, k + 2) - S(i - 1, j, k - 2) + S(i + 1, j, k - 2) - S(i - 1, j, k + 2)) +
                    W[5] * (S(i + 2, j + 1, k + 1) - S(i - 2, j - 1, k - 1) + S(i + 2, j + 1, k - 1) - S(i - 2, j - 1, k + 1) + S(i + 2, j - 1, k + 1) - S(i - 2, j + 1, k - 1) + S(i + 2, j - 1, k - 1) - S(i - 2, j + 1, k + 1) +
                            S(i + 1, j + 2, k + 1) - S(i - 1, j - 2, k - 1) + S(i + 1, j + 2, k - 1) - S(i - 1, j - 2, k + 1) + S(i + 1, j - 2, k + 1) - S(i - 1, j + 2, k - 1) + S(i + 1, j - 2, k - 1) - S(i - 1, j + 2, k + 1) +
                            S(i + 1, j + 1, k + 2) - S(i - 1, j - 1, k - 2) + S(i + 1, j + 1, k - 2) - S(i - 1, j - 1, k + 2) + S(i + 1, j - 1, k + 2) - S(i - 1, j + 1, k - 2) + S(i + 1, j - 1, k - 2) - S(i - 1, j + 1, k + 2)) +
                    W[6] * (S(i + 2, j + 2, k) - S(i - 2, j - 2, k) + S(i + 2, j - 2, k) - S(i - 2, j + 2, k) + S(i + 2, j, k + 2) - S(i - 2, j, k - 2) + S(i + 2, j, k - 2) - S(i - 2, j, k + 2));
                T nwy = W[0] * (S(i, j + 1, k) - S(i, j - 1, k)) +
                    W[1] * (S(i + 1, j + 1, k) - S(i - 1, j - 1, k) + S(i - 1, j + 1, k) - S(i + 1, j - 1, k) + S(i, j + 1, k + 1) - S(i, j - 1, k - 1) + S(i, j + 1, k - 1) - S(i, j - 1, k + 1)) +
                    W[2] * (S(i + 1, j + 1, k + 1) - S(i - 1, j - 1, k - 1) + S(i + 1, j + 1, k - 1) - S(i - 1, j - 1, k + 1) + S(i - 1, j + 1, k - 1) - S(i + 1, j - 1, k + 1) + S(i - 1, j + 1, k + 1) - S(i + 1, j - 1, k - 1)) +
                    W[3] * (S(i, j + 2, k) - S(i, j - 2, k)) +
                    W[4] * (S(i + 2, j + 1, k) - S(i - 2, j - 1, k) + S(i - 2, j + 1, k) - S(i + 2, j - 1, k) + S(i, j + 2, k + 1) - S(i, j - 2, k - 1) + S(i, j + 2, k - 1) - S(i, j - 2, k + 1) +
                            S(i + 1, j + 2, k) - S(i - 1, j - 2, k) + S(i - 1, j + 2, k) - S(i + 1, j - 2, k) + S(i, j + 1, k + 2) - S(i, j - 1, k - 2) + S(i, j + 1, k - 2) - S(i, j - 1, k + 2)) +
                    W[5] * (S(i + 2, j + 1, k + 1) - S(i - 2, j - 1, k - 1) + S(i + 2, j + 1, k - 1) - S(i - 2, j - 1, k + 1) + S(i - 2, j + 1, k + 1) - S(i + 2, j - 1, k - 1) + S(i - 2, j + 1, k - 1) - S(i + 2, j - 1, k + 1) +
                            S(i + 1, j + 2, k + 1) - S(i - 1, j - 2, k - 1) + S(i + 1, j + 2, k - 1) - S(i - 1, j - 2, k + 1) + S(i - 1, j + 2, k + 1) - S(i + 1, j - 2, k - 1) + S(i - 1, j + 2, k - 1) - S(i + 1, j - 2, k + 1) +
                            S(i + 1, j + 1, k + 2) - S(i - 1, j - 1, k - 2) + S(i + 1, j + 1, k - 2) - S(i - 1, j - 1, k + 2) + S(i - 1, j + 1, k + 2) - S(i + 1, j - 1, k - 2) + S(i - 1, j + 1, k - 2) - S(i + 1, j - 1, k + 2)) +
                    W[6] * (S(i + 2, j + 2, k) - S(i - 2, j - 2, k) + S(i - 2, j + 2, k) - S(i + 2, j - 2, k) + S(i, j + 2, k + 2) - S(i, j - 2, k - 2) + S(i, j + 2, k - 2) - S(i, j - 2, k + 2));
                T nwz = W[0] * (S(i, j, k + 1) - S(i, j, k - 1)) +
                    W[1] * (S(i, j + 1, k + 1) - S(i, j - 1, k - 1) + S(i, j - 1, k + 1) - S(i, j + 1, k - 1) + S(i + 1, j, k + 1) - S(i - 1, j, k - 1) + S(i - 1, j, k + 1) - S(i + 1, j, k - 1)) +
                    W[2] * (S(i + 1, j + 1, k + 1) - S(i - 1, j - 1, k - 1) + S(i + 1, j - 1, k + 1) - S(i - 1, j + 1, k - 1) + S(i - 1, j + 1, k + 1) - S(i + 1, j - 1, k - 1) + S(i - 1, j - 1, k + 1) - S(i + 1, j + 1, k - 1)) +
                    W[3] * (S(i, j, k + 2) - S(i, j, k - 2)) +
                    W[4] * (S(i, j + 1, k + 2) - S(i, j - 1, k - 2) + S(i, j - 1, k + 2) - S(i, j + 1, k - 2) + S(i + 2, j, k + 1) - S(i - 2, j, k - 1) + S(i - 2, j, k + 1) - S(i + 2, j, k - 1) +
                            S(i, j + 2, k + 1) - S(i, j - 2, k - 1) + S(i, j - 2, k + 1) - S(i, j + 2, k - 1) + S(i + 1, j, k + 2) - S(i - 1, j, k - 2) + S(i - 1, j, k + 2) - S(i + 1, j, k - 2)) +
                    W[5] * (S(i + 2, j + 1, k + 1) - S(i - 2, j - 1, k - 1) + S(i + 2, j - 1, k + 1) - S(i - 2, j + 1, k - 1) + S(i - 2, j + 1, k + 1) - S(i + 2, j - 1, k - 1) + S(i - 2, j - 1, k + 1) - S(i + 2, j + 1, k - 1) +
                            S(i + 1, j + 2, k + 1) - S(i - 1, j - 2, k - 1) + S(i + 1, j - 2, k + 1) - S(i - 1, j + 2, k - 1) + S(i - 1, j + 2, k + 1) - S(i + 1, j - 2, k - 1) + S(i - 1, j - 2, k + 1) - S(i + 1, j + 2, k - 1) +
                            S(i + 1, j + 1, k + 2) - S(i - 1, j - 1, k - 2) + S(i + 1, j - 1, k + 2) - S(i - 1, j + 1, k - 2) + S(i - 1, j + 1, k + 2) - S(i + 1, j - 1, k - 2) + S(i - 1, j - 1, k + 2) - S(i + 1, j + 1, k - 2)) +
                    W[6] * (S(i, j + 2, k + 2) - S(i, j - 2, k - 2) + S(i, j - 2, k + 2) - S(i, j + 2, k - 2) + S(i + 2, j, k + 2) - S(i - 2, j, k - 2) + S(i - 2, j, k + 2) - S(i + 2, j, k - 2));
                T tmpn = T(1) / (std::sqrt(nwx * nwx + nwy * nwy + nwz * nwz) + eps);
                ll m = g.s4(i, j, k);
                snx[m] = nwx * tmpn; sny[m] = nwy * tmpn; snz[m] = nwz * tmpn;
            }
}

/* Derivations of read_parameter_multi / initialization_basic_multi in T_P
 * (src/IO_multiphase.cpp:198-206, src/Init_multiphase.cpp:124-205,258-269). */
template <class T>
void params_from_control(const mflbm_control* ctl, int precision, int fp_mode, mflbm_params* o, mflbm_derived* d) {
    const T Pi = T(3.14159265358979323846);
    std::memset(o, 0, sizeof(*o));
    o->nx = ctl->nxGlobal; o->ny = ctl->nyGlobal; o->nz = ctl->nzGlobal;
    o->precision = precision; o->fp_mode = fp_mode;
    o->jper = ctl->jper; o->kper = ctl->kper;
    o->domain_wall_status_z_min = ctl->domain_wall_status_z_min;
    o->domain_wall_status_z_max = ctl->domain_wall_status_z_max;
    o->inlet_BC = ctl->inlet_BC; o->outlet_BC = ctl->outlet_BC;
    o->porous_plate_cmd = ctl->porous_plate_cmd; o->Z_porous_plate = ctl->Z_porous_plate;
    T theta = T(ctl->theta);
    theta = T(180) - theta;
    theta = theta * Pi / T(180);
    o->cos_theta = (double)std::cos(theta);
    const T la_nu1 = T(ctl->fluid1_viscosity), la_nu2 = T(ctl->fluid2_viscosity);
    const T gamma = T(ctl->surface_tension);
    o->lbm_gamma = (double)gamma;
    o->lbm_beta = (double)T(ctl->RK_beta);
    o->la_nui1 = (double)(T(1) / la_nu1);
    o->la_nui2 = (double)(T(1) / la_nu2);
    const T sa_inject = T(ctl->saturation_injection);
    o->sa_inject = (double)sa_inject;
    o->phi_inlet = (double)(T(2) * sa_inject - T(1));
    o->relaxation = 1.0;
    const T force_z0 = T(ctl->body_force_0);
    T force_z = force_z0, rho_out = T(1), rho_in = T(0), uin_avg = T(0);
    const T la_y = T(ctl->nyGlobal - 1) - T(0.5) - T(0.5);
    const T la_x = T(ctl->nxGlobal - 1) - T(0.5) - T(0.5);
    const T A_xy = la_x * la_y;
    T uin_avg_0 = T(0), flowrate = T(0);
    const bool open_z = ctl->kper == 0 && ctl->domain_wall_status_z_min == 0 && ctl->domain_wall_status_z_max == 0;
    if (open_z) {
        if (ctl->inlet_BC == 1) {
            force_z = T(0);
            uin_avg_0 = T(ctl->capillary_number) * gamma / la_nu1;
            uin_avg = uin_avg_0;
            flowrate = uin_avg_0 * A_xy;
        } else if (ctl->inlet_BC == 2) {
            force_z = T(0);
            const T p_gradient = -force_z0 / T(3);
            if (ctl->rho_out_BC) rho_out = T(1) - p_gradient * T(ctl->nzGlobal);
            else rho_in = rho_out - p_gradient * T(ctl->nzGlobal);
        }
    }
    o->force_z = (double)force_z;
    o->uin_avg = (double)uin_avg;
    o->rho_in = (double)rho_in;
    o->rho_out = (double)rho_out;
    if (d) {
        d->A_xy = (double)A_xy; d->uin_avg_0 = (double)uin_avg_0; d->flowrate = (double)flowrate;
        d->interface_z0 = (double)T(ctl->initial_interface_position);
    }
}

/* Uniform inlet profile then inlet_vel_profile_rectangular with 1000 terms
 * (src/Init_multiphase.cpp:270-284, src/Misc.cpp:387-419). */
inline float powT(float a, float b) { return powf(a, b); }
inline double powT(double a, double b) { return pow(a, b); }

template <class T>
void inlet_profile(const mflbm_control* ctl, T* W_in) {
    const Grid g{ctl->nxGlobal, ctl->nyGlobal, ctl->nzGlobal};
    mflbm_params prm; mflbm_derived d;
    params_from_control<T>(ctl, sizeof(T) == 4 ? MFLBM_FP32 : MFLBM_FP64, 0, &prm, &d);
    const T Pi = T(3.14159265358979323846);
    const T uin_avg = T(prm.uin_avg), vel_avg = T(d.uin_avg_0);
    for (ll n = 0; n < (g.nx + 2) * (g.ny + 2); ++n) W_in[n] = T(0);
    /* only the open velocity inlet sets a profile (src/Init_multiphase.cpp:186-189) */
    if (!(ctl->kper == 0 && ctl->domain_wall_status_z_min == 0 && ctl->domain_wall_status_z_max == 0 &&
          ctl->inlet_BC == 1))
        return;
    for (ll j = 1; j <= g.ny; ++j)
        for (ll i = 1; i <= g.nx; ++i) {
            W_in[g.s1(i, j, 0)] = T(0);
            if (i > 1 && i < g.nx && j > 1 && j < g.ny) W_in[g.s1(i, j, 0)] = uin_avg;
        }
    const int num_terms = 1000;
    const T la_y = T(g.ny - 1) - T(0.5) - T(0.5);
    const T la_x = T(g.nx - 1) - T(0.5) - T(0.5);
    const T a = T(0.5) * la_x, b = T(0.5) * la_y;
    T tmp1 = T(0);
    for (ll n = 1; n <= num_terms; n += 2) tmp1 += (std::tanh(T(0.5) * T(n) * Pi * b / a)) / powT(T(n), T(5));
    T tmp2 = T(1) - T(192) / powT(Pi, T(5)) * (a / b) * tmp1;
    tmp2 = T(-3) * vel_avg / (tmp2 * powT(a, T(2)));
    for (ll j = 1; j <= g.ny; ++j)
        for (ll i = 1; i <= g.nx; ++i) {
            if (!(i > 1 && i < g.nx && j > 1 && j < g.ny)) continue;
            const T xx = T(i) - T(1.5) - a, yy = T(j) - T(1.5) - b;
            T tmp3 = T(0);
            for (ll n = 1; n <= num_terms; n += 2)
                tmp3 += powT(T(-1), T(0.5) * T((n - 1))) * std::cos(T(0.5) * T(n) * Pi * xx / a) / powT(T(n), T(3)) *
                        (T(1) - (std::exp(T(0.5) * T(n) * Pi * (yy - b) / a) + std::exp(T(0.5) * T(n) * Pi * (-yy - b) / a)) /
                                    (T(1) + std::exp(T(0.5) * T(n) * Pi * (-b - b) / a)));
            W_in[g.s1(i, j, 0)] = tmp3 * (T(-16) * tmp2 * powT(a, T(2)) * powT(Pi, T(-3)));
        }
}

/* initialization_new_multi options 1-5 + initialization_new_multi_pdf with
 * u = v = w = 0, rho = 1, + convective buffers (src/Init_multiphase.cpp:299-496). */
template <class T>
void init_fields(const P<T>& p, int option, T z0, T* pdf, T* phi, T* f_cv, T* g_cv, T* phi_cv) {
    const Grid& g = p.g;
    Consts<T> c;
    for (ll n = 0; n < g.n_s4(); ++n) phi[n] = T(0);
    auto sq = [](T v) { return v * v; };
    for (ll k = 0; k <= g.nz + 1; ++k)
        for (ll j = 0; j <= g.ny + 1; ++j)
            for (ll i = 0; i <= g.nx + 1; ++i) {
                const T x = T(i), y = T(j), z = T(k);
                T v;
                switch (option) {
                case 1: v = z <= z0 ? T(1) : T(-1); break;
                case 2: v = z <= z0 ? T(-1) : T(1); break;
                case 3: v = (sq(x - T(g.nx + 1) * T(0)) + sq(z - T(g.nz + 1) * T(0.5)) + sq(y - T(g.ny + 1) * T(0.5)) <= sq(z0)) ? T(1) : T(-1); break;
                case 4: v = (sq(x - T(g.nx + 1) * T(0)) + sq(z - T(g.nz + 1) * T(0.5)) + sq(y - T(g.ny + 1) * T(0.5)) <= sq(z0)) ? T(-1) : T(1); break;
                default: v = (sq(x - T(g.nx + 1) * T(0.5)) + sq(z - T(g.nz + 1) * T(0.5)) + sq(y - T(g.ny + 1) * T(0.5)) <= sq(z0)) ? T(1) : T(-1); break;
                }
                phi[g.s4(i, j, k)] = v;
            }
    if (p.open_z())
        for (ll k = -3; k <= 0; ++k)
            for (ll j = -3; j <= g.ny + 4; ++j)
                for (ll i = -3; i <= g.nx + 4; ++i) phi[g.s4(i, j, k)] = p.phi_inlet;
    for (ll n = 0; n < g.n_s1() * 38; ++n) pdf[n] = T(0);
    for (ll k = 0; k <= g.nz + 1; ++k)
        for (ll j = 0; j <= g.ny + 1; ++j)
            for (ll i = 0; i <= g.nx + 1; ++i) {
                const T ph = phi[g.s4(i, j, k)];
                const T rho1 = T(1) * (T(1.0) + ph) * T(0.5);
                const T rho2 = T(1) * (T(1.0) - ph) * T(0.5);
                /* with u = v = w = 0 every term of the second-order equilibrium
                 * reduces to rho_k w_q + rho_k w_q * (c * 0 ...) evaluated below */
                const T usqrt = T(0) * T(0) + T(0) * T(0) + T(0) * T(0);
                for (int gg = 0; gg < 2; ++gg) {
                    const T r = gg == 0 ? rho1 : rho2;
                    pdf[g.f1(i, j, k, 0, gg)] = r * c.w0 + r * c.w0 * (T(-1.5) * usqrt);
                    for (int q = 1; q < 19; ++q) {
                        const T wq = q < 7 ? c.w1 : c.w2;
                        const T cu = T(0);
                        pdf[g.f1(i, j, k, q, gg)] = r * wq + r * wq * (T(3.0) * cu + T(4.5) * cu * cu - T(1.5) * usqrt);
                    }
                }
            }
    if (p.outlet_BC == 1 && f_cv && g_cv && phi_cv) {
        for (ll j = 0; j <= g.ny + 1; ++j)
            for (ll i = 0; i <= g.nx + 1; ++i) {
                for (int q = 0; q < 19; ++q) {
                    f_cv[g.cnv(i, j, q)] = pdf[g.f1(i, j, g.nz, q, 0)];
                    g_cv[g.cnv(i, j, q)] = pdf[g.f1(i, j, g.nz, q, 1)];
                }
                phi_cv[g.s1(i, j, 0)] = phi[g.s4(i, j, g.nz)];
            }
    }
}

/* compute_macro_vars (src/Misc.cpp:222-274) in T_P on post-even populations. */
template <class T>
void macro_vars(const P<T>& p, const int32_t* walls, const T* pdf, T* phi, const T* cnx, const T* cny, const T* cnz,
                const T* cnorm, const T* curv, T* rho, T* u, T* v, T* w) {
    const Grid& g = p.g;
#pragma omp parallel for collapse(2) schedule(static)
    for (ll k = 1; k <= g.nz; ++k)
        for (ll j = 1; j <= g.ny; ++j)
            for (ll i = 1; i <= g.nx; ++i) {
                const int wi = walls[g.s2(i, j, k)];
                T ft[19];
                for (int q = 0; q < 19; ++q) ft[q] = pdf[g.f1(i, j, k, q, 0)] + pdf[g.f1(i, j, k, q, 1)];
                T s = ft[0];
                for (int q = 1; q < 19; ++q) s = s + ft[q];
                const ll n1 = g.s1(i, j, k), n2 = g.s2(i, j, k);
                rho[n1] = s * T(1 - wi);
                T tmp = T(0.5) * p.gamma * curv[n1] * cnorm[n2];
                T fx = tmp * cnx[n2], fy = tmp * cny[n2], fz = tmp * cnz[n2] + p.force_z;
                u[n1] = (ft[1] - ft[2] + ft[7] - ft[8] + ft[9] - ft[10] + ft[11] - ft[12] + ft[13] - ft[14] - T(0.5) * fx) * T(1 - wi);
                v[n1] = (ft[3] - ft[4] + ft[7] + ft[8] - ft[9] - ft[10] + ft[15] - ft[16] + ft[17] - ft[18] - T(0.5) * fy) * T(1 - wi);
                w[n1] = (ft[5] - ft[6] + ft[11] + ft[12] - ft[13] - ft[14] + ft[15] + ft[16] - ft[17] - ft[18] - T(0.5) * fz) * T(1 - wi);
                phi[g.s4(i, j, k)] = T(0) * T(wi) + phi[g.s4(i, j, k)] * T(1 - wi);
            }
}

/* FP64 monitor sums (the quantities of src/Monitor.cpp:17-140, 472-495),
 * accumulated in double in (k, j, i) order. */
template <class T>
void monitor(const P<T>& p, const int32_t* walls, const T* pdf, const T* phi, const T* cnx, const T* cny,
             const T* cnz, const T* cnorm, const T* curv, int nex_in, int nex_out, mflbm_monitor* out) {
    const Grid& g = p.g;
    std::memset(out, 0, sizeof(*out));
    double umax2 = 0;
    for (ll k = 1; k <= g.nz; ++k)
        for (ll j = 1; j <= g.ny; ++j)
            for (ll i = 1; i <= g.nx; ++i) {
                if (walls[g.s2(i, j, k)] != 0) continue;
                double ft[19];
                for (int q = 0; q < 19; ++q) ft[q] = (double)pdf[g.f1(i, j, k, q, 0)] + (double)pdf[g.f1(i, j, k, q, 1)];
                double rho = 0;
                for (int q = 0; q < 19; ++q) rho += ft[q];
                const ll n1 = g.s1(i, j, k), n2 = g.s2(i, j, k);
                const double tmp = 0.5 * (double)p.gamma * (double)curv[n1] * (double)cnorm[n2];
                const double fx = tmp * cnx[n2], fy = tmp * cny[n2], fz = tmp * cnz[n2] + (double)p.force_z;
                const double u = ft[1] - ft[2] + ft[7] - ft[8] + ft[9] - ft[10] + ft[11] - ft[12] + ft[13] - ft[14] - 0.5 * fx;
                const double v = ft[3] - ft[4] + ft[7] + ft[8] - ft[9] - ft[10] + ft[15] - ft[16] + ft[17] - ft[18] - 0.5 * fy;
                const double w = ft[5] - ft[6] + ft[11] + ft[12] - ft[13] - ft[14] + ft[15] + ft[16] - ft[17] - ft[18] - 0.5 * fz;
                const double ph = (double)phi[g.s4(i, j, k)];
                const double a1 = 0.5 * (1.0 + ph), a2 = 0.5 * (1.0 - ph);
                const double u2 = u * u + v * v + w * w;
                if (u2 > umax2) umax2 = u2;
                out->vol1_full += a1; out->vol2_full += a2;
                out->flux1_sum += w * a1; out->flux2_sum += w * a2;
                if (k >= nex_in + 1 && k <= g.nz - nex_out) {
                    out->vol1_sum += a1; out->vol2_sum += a2;
                    out->mass1_sum += rho * a1; out->mass2_sum += rho * a2;
                }
            }
    double tm = 0;
    for (ll n = 0; n < g.n_s1() * 38; ++n) tm += (double)pdf[n];
    out->total_mass = tm;
    out->umax = std::sqrt(umax2);
    out->saturation = out->vol1_sum / (out->vol1_sum + out->vol2_sum);
}

/* Output files (src/IO_multiphase.cpp:252-305 save_checkpoint, :490-714
 * SwapEnd + VTK_legacy_writer_3D, :800-841 VTK_walls_bin), restated from the
 * host arrays of the reference layouts. */
template <class V> void put_be(std::string& out, V v) {
    unsigned char b[sizeof(V)];
    std::memcpy(b, &v, sizeof(V));
    for (int i = (int)sizeof(V) - 1; i >= 0; --i) out.push_back((char)b[i]);
}

inline std::string vtk_header(const Grid& g) {
    char buf[512];
    snprintf(buf, sizeof buf,
             "# vtk DataFile Version 3.0\nvtk output\nBINARY\nDATASET STRUCTURED_POINTS\nDIMENSIONS %lld %lld %lld\n"
             "ORIGIN 1 1 1\nSPACING 1 1 1\nPOINT_DATA %lld\n",
             g.nx, g.ny, g.nz, g.nx * g.ny * g.nz);
    return buf;
}

inline int save(const char* path, const std::string& bytes) {
    FILE* f = fopen(path, "wb");
    if (!f) return -1;
    const size_t n = fwrite(bytes.data(), 1, bytes.size(), f);
    return (fclose(f) == 0 && n == bytes.size()) ? 0 : -1;
}

template <class T>
int write_vtk(const P<T>& p, const int32_t* walls, const T* pdf, const T* phi_in, const T* cnx, const T* cny,
              const T* cnz, const T* cnorm, const T* curv, int type, int cmd, const char* path) {
    const Grid& g = p.g;
    std::vector<T> phi(phi_in, phi_in + g.n_s4());   /* the reference zeroes solids in its host copy */
    std::vector<T> rho, u, v, w;
    if (type == 1) {
        rho.assign(g.n_s1(), T(0)); u = rho; v = rho; w = rho;
        macro_vars<T>(p, walls, pdf, phi.data(), cnx, cny, cnz, cnorm, curv, rho.data(), u.data(), v.data(), w.data());
    } else if (type == 2) {
        for (ll k = 1; k <= g.nz; ++k)
            for (ll j = 1; j <= g.ny; ++j)
                for (ll i = 1; i <= g.nx; ++i) {
                    const int wi = walls[g.s2(i, j, k)];
                    phi[g.s4(i, j, k)] = T(0) * T(wi) + phi[g.s4(i, j, k)] * T(1 - wi);
                }
    }
    std::string out = vtk_header(g);
    const std::string fmt = type == 2 ? "float" : (cmd == 0 ? "float" : "double");
    const char* names[5] = {"phi", "density", "velocity_X", "velocity_Y", "velocity_Z"};
    const int nblk = type == 2 ? 1 : 5;
    for (int b = 0; b < nblk; ++b) {
        out += std::string("SCALARS ") + names[b] + " " + fmt + "\nLOOKUP_TABLE default\n";
        for (ll k = 1; k <= g.nz; ++k)
            for (ll j = 1; j <= g.ny; ++j)
                for (ll i = 1; i <= g.nx; ++i) {
                    const ll n1 = g.s1(i, j, k), n2 = g.s2(i, j, k), n4 = g.s4(i, j, k);
                    if (type == 2) { put_be(out, (float)phi[n4]); continue; }
                    T val;
                    if (type == 1) {
                        const T* src[5] = {nullptr, rho.data(), u.data(), v.data(), w.data()};
                        val = b == 0 ? phi[n4] : src[b][n1];
                    } else {
                        const T* src[5] = {nullptr, cnorm, cnx, cny, cnz};
                        val = b == 0 ? phi[n4] : src[b][n2];
                    }
                    put_be(out, val);
                }
    }
    return save(path, out);
}

inline int write_walls_vtk(ll nx, ll ny, ll nz, const int32_t* walls, const char* path) {
    const Grid g{nx, ny, nz};
    std::string out = vtk_header(g) + "SCALARS walls int\nLOOKUP_TABLE default\n";
    for (ll k = 1; k <= nz; ++k)
        for (ll j = 1; j <= ny; ++j)
            for (ll i = 1; i <= nx; ++i) put_be(out, (int32_t)walls[g.s2(i, j, k)]);
    return save(path, out);
}

template <class T>
int write_checkpoint(const P<T>& p, int ntime, const T* pdf, const T* phi, const T* f_cv, const T* g_cv,
                     const T* phi_cv, const char* path) {
    const Grid& g = p.g;
    std::string out;
    const int nt = ntime + 1;
    out.append((const char*)&nt, sizeof nt);
    out.append((const char*)&p.force_z, sizeof(T));
    out.append((const char*)&p.rho_in, sizeof(T));
    out.append((const char*)pdf, sizeof(T) * g.n_s1() * 38);
    out.append((const char*)phi, sizeof(T) * g.n_s4());
    if (p.outlet_BC == 1) {
        const ll pl = (g.nx + 2) * (g.ny + 2);
        out.append((const char*)f_cv, sizeof(T) * pl * 19);
        out.append((const char*)g_cv, sizeof(T) * pl * 19);
        out.append((const char*)phi_cv, sizeof(T) * pl);
    }
    return save(path, out);
}

} // namespace

/* ---------------------------------------------------------------------------
 * C entry points.
 * ------------------------------------------------------------------------- */
#define ORC_EXPORT extern "C" __attribute__((visibility("default")))

#define ORC_TYPED(T, SUF)                                                                                          \
    ORC_EXPORT void orc_geometry_preprocess_##SUF(const mflbm_control* ctl, const int32_t* wg, int32_t* walls,     \
                                                  int32_t* wt, T* snx, T* sny, T* snz, mflbm_geometry_counts* c) { \
        geometry_preprocess<T>(ctl, wg, walls, wt, snx, sny, snz, c);                                              \
    }                                                                                                              \
    ORC_EXPORT void orc_params_from_control_##SUF(const mflbm_control* ctl, int fp_mode, mflbm_params* o,          \
                                                  mflbm_derived* d) {                                              \
        params_from_control<T>(ctl, sizeof(T) == 4 ? MFLBM_FP32 : MFLBM_FP64, fp_mode, o, d);                      \
    }                                                                                                              \
    ORC_EXPORT void orc_inlet_profile_##SUF(const mflbm_control* ctl, T* W_in) { inlet_profile<T>(ctl, W_in); }    \
    ORC_EXPORT void orc_init_fields_##SUF(const mflbm_params* prm, int option, double z0, T* pdf, T* phi, T* f_cv, \
                                          T* g_cv, T* phi_cv) {                                                    \
        init_fields<T>(P<T>(prm), option, T(z0), pdf, phi, f_cv, g_cv, phi_cv);                                    \
    }                                                                                                              \
    ORC_EXPORT void orc_color_gradient_##SUF(const mflbm_params* prm, const int32_t* walls, const int32_t* wt,     \
                                             const T* snx, const T* sny, const T* snz, T* phi, T* cnx, T* cny,     \
                                             T* cnz, T* cnorm, T* curv) {                                          \
        color_gradient<T>(P<T>(prm), walls, wt, snx, sny, snz, phi, cnx, cny, cnz, cnorm, curv);                   \
    }                                                                                                              \
    ORC_EXPORT void orc_step_##SUF(const mflbm_params* prm, int ntime, const int32_t* walls, const int32_t* wt,    \
                                   const T* snx, const T* sny, const T* snz, T* pdf, T* phi, T* cnx, T* cny,       \
                                   T* cnz, T* cnorm, T* curv, const T* W_in, T* f_cv, T* g_cv, T* phi_cv) {        \
        step<T>(P<T>(prm), ntime, walls, wt, snx, sny, snz, pdf, phi, cnx, cny, cnz, cnorm, curv, W_in, f_cv,      \
                g_cv, phi_cv);                                                                                     \
    }                                                                                                              \
    ORC_EXPORT void orc_run_##SUF(const mflbm_params* prm, int ntime0, int nsteps, const int32_t* walls,           \
                                  const int32_t* wt, const T* snx, const T* sny, const T* snz, T* pdf, T* phi,     \
                                  T* cnx, T* cny, T* cnz, T* cnorm, T* curv, const T* W_in, T* f_cv, T* g_cv,      \
                                  T* phi_cv) {                                                                     \
        const P<T> p(prm);                                                                                         \
        for (int s = 0; s < nsteps; ++s)                                                                           \
            step<T>(p, ntime0 + s, walls, wt, snx, sny, snz, pdf, phi, cnx, cny, cnz, cnorm, curv, W_in, f_cv,     \
                    g_cv, phi_cv);                                                                                 \
    }                                                                                                              \
    ORC_EXPORT void orc_collide_##SUF(const mflbm_params* prm, int odd, const int32_t* walls, T* pdf, T* phi,      \
                                      const T* cnx, const T* cny, const T* cnz, const T* curv, const T* cnorm) {   \
        collide_stream<T>(P<T>(prm), odd != 0, walls, pdf, phi, cnx, cny, cnz, curv, cnorm);                       \
    }                                                                                                              \
    ORC_EXPORT void orc_macro_vars_##SUF(const mflbm_params* prm, const int32_t* walls, const T* pdf, T* phi,      \
                                         const T* cnx, const T* cny, const T* cnz, const T* cnorm, const T* curv,  \
                                         T* rho, T* u, T* v, T* w) {                                               \
        macro_vars<T>(P<T>(prm), walls, pdf, phi, cnx, cny, cnz, cnorm, curv, rho, u, v, w);                       \
    }                                                                                                              \
    ORC_EXPORT void orc_monitor_##SUF(const mflbm_params* prm, const int32_t* walls, const T* pdf, const T* phi,   \
                                      const T* cnx, const T* cny, const T* cnz, const T* cnorm, const T* curv,     \
                                      int nex_in, int nex_out, mflbm_monitor* out) {                               \
        monitor<T>(P<T>(prm), walls, pdf, phi, cnx, cny, cnz, cnorm, curv, nex_in, nex_out, out);                  \
    }

#define ORC_TYPED_IO(T, SUF)                                                                                       \
    ORC_EXPORT int orc_write_vtk_##SUF(const mflbm_params* prm, const int32_t* walls, const T* pdf, const T* phi,  \
                                       const T* cnx, const T* cny, const T* cnz, const T* cnorm, const T* curv,    \
                                       int type, int cmd, const char* path) {                                      \
        return write_vtk<T>(P<T>(prm), walls, pdf, phi, cnx, cny, cnz, cnorm, curv, type, cmd, path);              \
    }                                                                                                              \
    ORC_EXPORT int orc_write_checkpoint_##SUF(const mflbm_params* prm, int ntime, const T* pdf, const T* phi,      \
                                              const T* f_cv, const T* g_cv, const T* phi_cv, const char* path) {   \
        return write_checkpoint<T>(P<T>(prm), ntime, pdf, phi, f_cv, g_cv, phi_cv, path);                          \
    }

ORC_TYPED(float, f32)
ORC_TYPED_IO(float, f32)
ORC_TYPED_IO(double, f64)
ORC_TYPED(double, f64)

ORC_EXPORT void orc_set_walls(const mflbm_control* ctl, const uint8_t* geo, int32_t* walls_global) {
    set_walls(ctl, geo, walls_global);
}

ORC_EXPORT int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

ORC_EXPORT int orc_write_walls_vtk(long long nx, long long ny, long long nz, const int32_t* walls, const char* path) {
    return write_walls_vtk(nx, ny, nz, walls, path);
}
