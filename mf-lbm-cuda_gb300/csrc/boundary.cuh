// Boundary updates of one time step (included by step_kernels.cuh).
#pragma once
#include "context.cuh"

namespace mflbm {
namespace MFLBM_NS {

// ===========================================================================
// Boundary updates (src/main_iteration_GPU.cu:1009-1882).  One thread per
// (i, j) column (inlet / outlet / plate) or (i, k) row (periodic y).
// keep(new, old, w) is the reference's  new*(1-w) + old*w  blend.
// ===========================================================================
template <class T, class E> struct BcArgs {
    Grid g;
    PopView<T, E> P;  // populations
    const int32_t* walls;
    T *phi, *W_in, *f_cv, *g_cv, *phi_cv;
    Phys<T> ph;
    int plate_cmd, Zplate;
};

template <class T> __device__ __forceinline__ T keep(T v_new, T v_old, int w) { return v_new * T(1 - w) + v_old * T(w); }

// Column (i, j) of a thread of the face kernels: a block of 128 threads
// covers 16 x 8 columns, a warp 16 x 2, so that the warp's accesses to a z
// plane use half of each 2 x 2 x 2 population brick it touches (a warp
// along one x row would use a quarter).
__device__ __forceinline__ void face_column(int& i, int& j) {
    i = blockIdx.x * 16 + (threadIdx.x & 15) + 1;
    j = blockIdx.y * 8 + (threadIdx.x >> 4) + 1;
}
inline dim3 face_grid(const Grid& g) { return dim3((g.nx + 15) / 16, (g.ny + 7) / 8); }

template <class T, class E>
__device__ __forceinline__ void inlet_phi(const BcArgs<T, E>& a, int i, int j, int w) {
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

// velocity inlet: bounce-back plus 6 w rho u injection, split by sa_inject
// (:1009-1077).  One link s (kInlet) of component gg; the links of a column
// touch distinct slots, so they can run in separate threads.
template <class T, class E, bool AFTER_ODD>
__device__ __forceinline__ void inlet_velocity_link(const BcArgs<T, E>& a, int i, int j, int gg, int s) {
    const Grid& g = a.g;
    const int w = a.walls[g.s2(i, j, 1)];
    T t2 = a.W_in[g.s1(i, j, 0)] * a.ph.relaxation;
    const T t1 = t2 * a.ph.sa_inject;
    t2 = t2 - t1;
    const T inj = gg == 0 ? t1 : t2;
    const T wq = s == 0 ? a.ph.c.w1 : a.ph.c.w2;
    const int dx = kInlet[s][0], dy = kInlet[s][1], s0 = kInlet[s][2], s1 = kInlet[s][3];
    if (!AFTER_ODD) {
        const T d = a.P.get(i + dx, j + dy, 0, s0, gg);
        a.P.set(i + dx, j + dy, 0, s0, gg, keep((a.P.get(i, j, 1, s1, gg) + T(6.0) * wq * inj), d, w));
    } else {
        const T d = a.P.get(i, j, 1, s1, gg);
        a.P.set(i, j, 1, s1, gg, keep((a.P.get(i + dx, j + dy, 0, s0, gg) + T(6.0) * wq * inj), d, w));
    }
}
template <class T, class E, bool AFTER_ODD>
__device__ __forceinline__ void inlet_velocity_at(const BcArgs<T, E>& a, int i, int j) {
    inlet_phi(a, i, j, a.walls[a.g.s2(i, j, 1)]);
#pragma unroll
    for (int gg = 0; gg < 2; ++gg)
#pragma unroll
        for (int s = 0; s < 5; ++s) inlet_velocity_link<T, E, AFTER_ODD>(a, i, j, gg, s);
}

// Zou-He pressure inlet per component (:1085-1241)
template <class T, class E, bool AFTER_ODD>
__device__ __forceinline__ void inlet_pressure_at(const BcArgs<T, E>& a, int i, int j) {
    const Grid& g = a.g;
    const int w = a.walls[g.s2(i, j, 1)];
    inlet_phi(a, i, j, w);
    T r2 = a.ph.rho_in;
    const T r1 = a.ph.rho_in * a.ph.sa_inject;
    r2 = r2 - r1;
    const T c3 = T(0.333333333333333333), c6 = T(0.166666666666666667);
#pragma unroll
    for (int gg = 0; gg < 2; ++gg) {
        auto F = [&](int u, int v, int k, int e) { return a.P.get(u, v, k, e, gg); };
        auto S = [&](int u, int v, int k, int e, T x) { a.P.set(u, v, k, e, gg, x); };
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
            S(i, j, 0, 5, keep((F(i, j, 2, 6) + c3 * t), F(i, j, 0, 5), w));
            S(i - 1, j, 0, 11, keep((F(i + 1, j, 2, 14) + c6 * t - tnx), F(i - 1, j, 0, 11), w));
            S(i + 1, j, 0, 12, keep((F(i - 1, j, 2, 13) + c6 * t + tnx), F(i + 1, j, 0, 12), w));
            S(i, j - 1, 0, 15, keep((F(i, j + 1, 2, 18) + c6 * t - tny), F(i, j - 1, 0, 15), w));
            S(i, j + 1, 0, 16, keep((F(i, j - 1, 2, 17) + c6 * t + tny), F(i, j + 1, 0, 16), w));
        } else {
            const T t = (rc - (F(i, j, 1, 0) + F(i, j, 1, 2) + F(i, j, 1, 1) + F(i, j, 1, 4) + F(i, j, 1, 3) +
                               F(i, j, 1, 8) + F(i, j, 1, 7) + F(i, j, 1, 10) + F(i, j, 1, 9) +
                               T(2) * (F(i, j, 1, 5) + F(i, j, 1, 11) + F(i, j, 1, 12) + F(i, j, 1, 15) +
                                       F(i, j, 1, 16)))) * a.ph.relaxation;
            const T tnx = T(0.5) * (F(i, j, 1, 2) + F(i, j, 1, 8) + F(i, j, 1, 10) -
                                    (F(i, j, 1, 1) + F(i, j, 1, 7) + F(i, j, 1, 9)));
            const T tny = T(0.5) * (F(i, j, 1, 4) + F(i, j, 1, 9) + F(i, j, 1, 10) -
                                    (F(i, j, 1, 3) + F(i, j, 1, 8) + F(i, j, 1, 7)));
            S(i, j, 1, 6, keep((F(i, j, 1, 5) + c3 * t), F(i, j, 1, 6), w));
            S(i, j, 1, 13, keep((F(i, j, 1, 12) + c6 * t + tnx), F(i, j, 1, 13), w));
            S(i, j, 1, 14, keep((F(i, j, 1, 11) + c6 * t - tnx), F(i, j, 1, 14), w));
            S(i, j, 1, 17, keep((F(i, j, 1, 16) + c6 * t + tny), F(i, j, 1, 17), w));
            S(i, j, 1, 18, keep((F(i, j, 1, 15) + c6 * t - tny), F(i, j, 1, 18), w));
        }
    }
}

// convective outflow with the previous-step buffers (:1246-1357): the phi
// ghost layers of column (i, j), and one link s (kOutlet) of component gg
// (the links touch distinct slots and buffer entries)
template <class T, class E>
__device__ __forceinline__ void outlet_convective_phi(const BcArgs<T, E>& a, int i, int j) {
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
}
template <class T, class E, bool AFTER_ODD>
__device__ __forceinline__ void outlet_convective_link(const BcArgs<T, E>& a, int i, int j, int gg, int s) {
    const Grid& g = a.g;
    const int nz = g.nz;
    const T u = a.ph.uin_avg;
    const T temp = T(1) / (T(1) + u);
    const int w = a.walls[g.s2(i, j, nz)];
    T* buf = gg == 0 ? a.f_cv : a.g_cv;
    const int dx = kOutlet[s][0], dy = kOutlet[s][1], su = kOutlet[s][2], sd = kOutlet[s][3], sb = kOutlet[s][4];
    T& bv = buf[g.cnv(i, j, sb)];
    if (!AFTER_ODD) {
        const T d = ((bv + u * a.P.get(i + dx, j + dy, nz, su, gg)) * temp) * T(1 - w) +
                    a.P.get(i + dx, j + dy, nz + 1, su, gg) * T(w);
        a.P.set(i + dx, j + dy, nz + 1, su, gg, d);
        bv = d;
    } else {
        const T d = ((bv + u * a.P.get(i, j, nz - 1, sd, gg)) * temp) * T(1 - w) + a.P.get(i, j, nz, sd, gg) * T(w);
        a.P.set(i, j, nz, sd, gg, d);
        bv = d;
    }
}
template <class T, class E, bool AFTER_ODD>
__device__ __forceinline__ void outlet_convective_at(const BcArgs<T, E>& a, int i, int j) {
    outlet_convective_phi<T, E>(a, i, j);
#pragma unroll
    for (int gg = 0; gg < 2; ++gg)
#pragma unroll
        for (int s = 0; s < 5; ++s) outlet_convective_link<T, E, AFTER_ODD>(a, i, j, gg, s);
}

// Zou-He pressure outlet on the total density, flux split by phi (:1363-1524)
template <class T, class E, bool AFTER_ODD>
__device__ __forceinline__ void outlet_pressure_at(const BcArgs<T, E>& a, int i, int j) {
    const Grid& g = a.g;
    const int nz = g.nz;
    const int w = a.walls[g.s2(i, j, nz)];
    const T pz = a.phi[g.s4(i, j, nz)];
    a.phi[g.s4(i, j, nz + 1)] = pz;
    a.phi[g.s4(i, j, nz + 2)] = pz;
    a.phi[g.s4(i, j, nz + 3)] = pz;
    a.phi[g.s4(i, j, nz + 4)] = pz;
    auto F = [&](int u, int v, int k, int e, int gg) { return a.P.get(u, v, k, e, gg); };
    auto S = [&](int u, int v, int k, int e, int gg, T x) { a.P.set(u, v, k, e, gg, x); };
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
            S(i, j, nz + 1, 6, gg, keep((F(i, j, nz - 1, 5, gg) - c3 * t), F(i, j, nz + 1, 6, gg), w));
            S(i - 1, j, nz + 1, 13, gg, keep((F(i + 1, j, nz - 1, 12, gg) - c6 * t - tnx), F(i - 1, j, nz + 1, 13, gg), w));
            S(i + 1, j, nz + 1, 14, gg, keep((F(i - 1, j, nz - 1, 11, gg) - c6 * t + tnx), F(i + 1, j, nz + 1, 14, gg), w));
            S(i, j - 1, nz + 1, 17, gg, keep((F(i, j + 1, nz - 1, 16, gg) - c6 * t - tny), F(i, j - 1, nz + 1, 17, gg), w));
            S(i, j + 1, nz + 1, 18, gg, keep((F(i, j - 1, nz - 1, 15, gg) - c6 * t + tny), F(i, j + 1, nz + 1, 18, gg), w));
        } else {
            const T tnx = T(0.5) * (F(i, j, nz, 2, gg) + F(i, j, nz, 8, gg) + F(i, j, nz, 10, gg) -
                                    (F(i, j, nz, 1, gg) + F(i, j, nz, 7, gg) + F(i, j, nz, 9, gg)));
            const T tny = T(0.5) * (F(i, j, nz, 4, gg) + F(i, j, nz, 10, gg) + F(i, j, nz, 9, gg) -
                                    (F(i, j, nz, 3, gg) + F(i, j, nz, 7, gg) + F(i, j, nz, 8, gg)));
            S(i, j, nz, 5, gg, keep((F(i, j, nz, 6, gg) - c3 * t), F(i, j, nz, 5, gg), w));
            S(i, j, nz, 11, gg, keep((F(i, j, nz, 14, gg) - c6 * t + tnx), F(i, j, nz, 11, gg), w));
            S(i, j, nz, 12, gg, keep((F(i, j, nz, 13, gg) - c6 * t - tnx), F(i, j, nz, 12, gg), w));
            S(i, j, nz, 15, gg, keep((F(i, j, nz, 18, gg) - c6 * t + tny), F(i, j, nz, 15, gg), w));
            S(i, j, nz, 16, gg, keep((F(i, j, nz, 17, gg) - c6 * t - tny), F(i, j, nz, 16, gg), w));
        }
    }
}

// Periodic copies across z = 1 / nz, y = 1 / ny and the zy edges (:1529-1733).
// Directions leaving through the upper face: (ez or ey) = -1 ... see tables.
// Inlet (1 velocity, 2 pressure, 0 none) and outlet (1 convective, 2 pressure,
// 0 none) of column (i, j) in one launch.  The inlet reads and writes the z
// planes 0 .. 2, the outlet nz - 1 .. nz + 1 (and the phi ghosts beyond
// each): with nz >= 4 they touch no common location, so running them
// together gives the reference's result of running them one after the other.
template <class T, class E, bool AFTER_ODD>
__global__ void inlet_outlet_kernel(const BcArgs<T, E> a, int inlet, int outlet) {
    pdl_wait();
    int i, j;
    face_column(i, j);
    if (i > a.g.nx || j > a.g.ny) return;
    if (inlet == 1) inlet_velocity_at<T, E, AFTER_ODD>(a, i, j);
    else if (inlet == 2) inlet_pressure_at<T, E, AFTER_ODD>(a, i, j);
    if (outlet == 1) outlet_convective_at<T, E, AFTER_ODD>(a, i, j);
    else if (outlet == 2) outlet_pressure_at<T, E, AFTER_ODD>(a, i, j);
}

// The velocity inlet and the convective outlet (the usual pair) with 11
// threads per column: the 10 links (2 components x 5 directions) of each face
// and the phi ghost layers.  The links of a column touch distinct slots, so
// this gives the column kernel's results; eleven times the threads hide the
// latency of the scattered plane accesses.  Items are link-major (a warp:
// one link of 32 columns, 16 x 2 of them).
template <class T, class E, bool AFTER_ODD>
__global__ void inlet_outlet_links_kernel(const BcArgs<T, E> a, int inlet, int outlet, int ntx, int ncolp) {
    pdl_wait();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int item = t / ncolp, c = t - item * ncolp;
    if (item >= 11) return;
    const int lane = c & 31, tile = c >> 5;
    const int i = (tile % ntx) * 16 + (lane & 15) + 1, j = (tile / ntx) * 2 + (lane >> 4) + 1;
    if (i > a.g.nx || j > a.g.ny) return;
    if (item == 10) {
        if (inlet == 1) inlet_phi(a, i, j, a.walls[a.g.s2(i, j, 1)]);
        if (outlet == 1) outlet_convective_phi<T, E>(a, i, j);
        return;
    }
    const int gg = item / 5, s = item - 5 * gg;
    if (inlet == 1) inlet_velocity_link<T, E, AFTER_ODD>(a, i, j, gg, s);
    if (outlet == 1) outlet_convective_link<T, E, AFTER_ODD>(a, i, j, gg, s);
}

__device__ __constant__ const int kZup[5] = {6, 14, 13, 18, 17}, kZdn[5] = {5, 11, 12, 15, 16};
__device__ __constant__ const int kYup[5] = {4, 10, 9, 16, 18}, kYdn[5] = {3, 7, 8, 15, 17};

// Periodic exchanges (:1529-1735).  The reference runs z, then y, then the
// z-y edges.  Their sources are never another exchange's destinations
// (before the odd step they copy interior slots to ghosts, after it ghost
// slots to the interior), and their destinations meet only after the odd
// step, at the four corner slots of each x column where z and y both write
// and the edge copy writes last.  `edges` (periodic y and z) makes z and y
// leave those four slots to the edge copy, so the three can run at once
// with the reference's result.
template <class T, class E, bool ODD>
__device__ __forceinline__ void periodic_z_at(const BcArgs<T, E>& a, int i, int j, bool edges = false) {
    const Grid& g = a.g;
    const int nz = g.nz;
#pragma unroll
    for (int gg = 0; gg < 2; ++gg)
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            if (!ODD) {
                a.P.copy(i, j, nz + 1, kZup[s], gg, i, j, 1, kZup[s]);
                a.P.copy(i, j, 0, kZdn[s], gg, i, j, nz, kZdn[s]);
            } else {
                const bool up = !(edges && ((j == 1 && kZup[s] == 18) || (j == g.ny && kZup[s] == 17)));
                const bool dn = !(edges && ((j == 1 && kZdn[s] == 16) || (j == g.ny && kZdn[s] == 15)));
                if (up) a.P.copy(i, j, 1, kZup[s], gg, i, j, nz + 1, kZup[s]);
                if (dn) a.P.copy(i, j, nz, kZdn[s], gg, i, j, 0, kZdn[s]);
            }
        }
    for (int k = 1; k <= 4; ++k) {
        a.phi[g.s4(i, j, k + nz)] = a.phi[g.s4(i, j, k)];
        a.phi[g.s4(i, j, k - 4)] = a.phi[g.s4(i, j, nz + k - 4)];
    }
}

// periodic y of row (i, k), i, k >= 1
template <class T, class E, bool ODD>
__device__ __forceinline__ void periodic_y_at(const BcArgs<T, E>& a, int i, int k, bool edges = false) {
    const Grid& g = a.g;
    const int ny = g.ny;
#pragma unroll
    for (int gg = 0; gg < 2; ++gg)
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            if (!ODD) {
                a.P.copy(i, ny + 1, k, kYup[s], gg, i, 1, k, kYup[s]);
                a.P.copy(i, 0, k, kYdn[s], gg, i, ny, k, kYdn[s]);
            } else {
                const bool up = !(edges && ((k == 1 && kYup[s] == 18) || (k == g.nz && kYup[s] == 16)));
                const bool dn = !(edges && ((k == 1 && kYdn[s] == 17) || (k == g.nz && kYdn[s] == 15)));
                if (up) a.P.copy(i, 1, k, kYup[s], gg, i, ny + 1, k, kYup[s]);
                if (dn) a.P.copy(i, ny, k, kYdn[s], gg, i, 0, k, kYdn[s]);
            }
        }
    for (int j = 1; j <= 4; ++j) {
        a.phi[g.s4(i, j + ny, k)] = a.phi[g.s4(i, j, k)];
        a.phi[g.s4(i, j - 4, k)] = a.phi[g.s4(i, ny + j - 4, k)];
    }
}

// periodic z-y edges of column i >= 1
template <class T, class E, bool ODD>
__device__ __forceinline__ void periodic_zy_at(const BcArgs<T, E>& a, int i) {
    const Grid& g = a.g;
    const int ny = g.ny, nz = g.nz;
#pragma unroll
    for (int gg = 0; gg < 2; ++gg) {
        if (!ODD) {
            a.P.copy(i, ny + 1, nz + 1, 18, gg, i, 1, 1, 18);
            a.P.copy(i, ny + 1, 0, 16, gg, i, 1, nz, 16);
            a.P.copy(i, 0, nz + 1, 17, gg, i, ny, 1, 17);
            a.P.copy(i, 0, 0, 15, gg, i, ny, nz, 15);
        } else {
            a.P.copy(i, 1, 1, 18, gg, i, ny + 1, nz + 1, 18);
            a.P.copy(i, 1, nz, 16, gg, i, ny + 1, 0, 16);
            a.P.copy(i, ny, 1, 17, gg, i, 0, nz + 1, 17);
            a.P.copy(i, ny, nz, 15, gg, i, 0, 0, 15);
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
// Work item r of the periodic exchanges (0 <= r < periodic_items): z for
// (i, j) when kper, then y for (i, k) when jper, then the edges for i when
// both.
__host__ __device__ __forceinline__ int periodic_items(const Grid& g, int jper, int kper) {
    return (kper ? g.nx * g.ny : 0) + (jper ? g.nx * g.nz : 0) + (jper && kper ? g.nx : 0);
}
template <class T, class E, bool ODD>
__device__ __forceinline__ void periodic_item(const BcArgs<T, E>& a, int jper, int kper, int r) {
    const Grid& g = a.g;
    const bool edges = jper && kper;
    const int nzr = kper ? g.nx * g.ny : 0, nyr = jper ? g.nx * g.nz : 0;
    if (r < nzr) periodic_z_at<T, E, ODD>(a, r % g.nx + 1, r / g.nx + 1, edges);
    else if (r < nzr + nyr) periodic_y_at<T, E, ODD>(a, (r - nzr) % g.nx + 1, (r - nzr) / g.nx + 1, edges);
    else periodic_zy_at<T, E, ODD>(a, r - nzr - nyr + 1);
}
// all periodic exchanges of a step in one launch
template <class T, class E, bool ODD>
__global__ void periodic_kernel(const BcArgs<T, E> a, int jper, int kper, int n) {
    pdl_wait();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) periodic_item<T, E, ODD>(a, jper, kper, r);
}

// porous plate blocking one component at z = Zplate (:1744-1882); b = blocked component
template <class T, class E, bool AFTER_ODD>
__global__ void porous_plate_kernel(const BcArgs<T, E> a) {
    pdl_wait();
    int i, j;
    face_column(i, j);
    if (i > a.g.nx || j > a.g.ny) return;
    const Grid& g = a.g;
    const int zp = a.Zplate;
    if (!(zp >= 1 && zp <= g.nz) || (a.plate_cmd != 1 && a.plate_cmd != 2)) return;
    const int b = a.plate_cmd == 1 ? 0 : 1, o = 1 - b;
    auto F = [&](int u, int v, int k, int e, int gg, int us, int vs, int ks, int es) {
        a.P.copy(u, v, k, e, gg, us, vs, ks, es);
    };
    if (!AFTER_ODD) {
        F(i, j, zp, 6, b, i, j, zp - 1, 5);
        F(i - 1, j, zp, 13, b, i, j, zp - 1, 12);
        F(i + 1, j, zp, 14, b, i, j, zp - 1, 11);
        F(i, j - 1, zp, 17, b, i, j, zp - 1, 16);
        F(i, j + 1, zp, 18, b, i, j, zp - 1, 15);
        F(i, j, zp, 5, b, i, j, zp + 1, 6);
        F(i + 1, j, zp, 12, b, i, j, zp + 1, 13);
        F(i - 1, j, zp, 11, b, i, j, zp + 1, 14);
        F(i, j + 1, zp, 16, b, i, j, zp + 1, 17);
        F(i, j - 1, zp, 15, b, i, j, zp + 1, 18);
        F(i, j, zp, 6, o, i, j, zp + 1, 6);
        F(i, j, zp, 13, o, i, j, zp + 1, 13);
        F(i, j, zp, 14, o, i, j, zp + 1, 14);
        F(i, j, zp, 17, o, i, j, zp + 1, 17);
        F(i, j, zp, 18, o, i, j, zp + 1, 18);
        F(i, j, zp, 5, o, i, j, zp - 1, 5);
        F(i, j, zp, 12, o, i, j, zp - 1, 12);
        F(i, j, zp, 11, o, i, j, zp - 1, 11);
        F(i, j, zp, 16, o, i, j, zp - 1, 16);
        F(i, j, zp, 15, o, i, j, zp - 1, 15);
    } else {
        F(i, j, zp - 1, 5, b, i, j, zp, 6);
        F(i, j, zp - 1, 12, b, i - 1, j, zp, 13);
        F(i, j, zp - 1, 11, b, i + 1, j, zp, 14);
        F(i, j, zp - 1, 16, b, i, j - 1, zp, 17);
        F(i, j, zp - 1, 15, b, i, j + 1, zp, 18);
        F(i, j, zp + 1, 6, b, i, j, zp, 5);
        F(i, j, zp + 1, 13, b, i + 1, j, zp, 12);
        F(i, j, zp + 1, 14, b, i - 1, j, zp, 11);
        F(i, j, zp + 1, 17, b, i, j + 1, zp, 16);
        F(i, j, zp + 1, 18, b, i, j - 1, zp, 15);
        F(i, j, zp - 1, 5, o, i, j, zp, 5);
        F(i, j, zp - 1, 12, o, i, j, zp, 12);
        F(i, j, zp - 1, 11, o, i, j, zp, 11);
        F(i, j, zp - 1, 16, o, i, j, zp, 16);
        F(i, j, zp - 1, 15, o, i, j, zp, 15);
        F(i, j, zp + 1, 6, o, i, j, zp, 6);
        F(i, j, zp + 1, 13, o, i, j, zp, 13);
        F(i, j, zp + 1, 14, o, i, j, zp, 14);
        F(i, j, zp + 1, 17, o, i, j, zp, 17);
        F(i, j, zp + 1, 18, o, i, j, zp, 18);
    }
}


template <class T, class E>
BcArgs<T, E> bc_args(const mflbm_context& c) {
    const DeviceState& d = c.d;
    const mflbm_params& p = c.params;
    BcArgs<T, E> a;
    a.g = d.g;
    a.P.p = (E*)d.pdf;
    a.P.b = d.b;
    a.walls = d.walls;
    a.phi = (T*)d.phi; a.W_in = (T*)d.W_in;
    a.f_cv = (T*)d.f_cv; a.g_cv = (T*)d.g_cv; a.phi_cv = (T*)d.phi_cv;
    a.ph = make_phys<T>(p);
    a.plate_cmd = p.porous_plate_cmd; a.Zplate = p.Z_porous_plate;
    return a;
}

template <class T, class E>
int launch_boundaries(mflbm_context& c, bool odd) {
    const DeviceState& d = c.d;
    const Grid& g = d.g;
    const mflbm_params& p = c.params;
    const BcArgs<T, E> a = bc_args<T, E>(c);
    cudaStream_t s = c.stream;
    int rc;
    if (p.jper || p.kper) {
        const int n = periodic_items(g, p.jper, p.kper);
        rc = launch_pdl("periodic", odd ? periodic_kernel<T, E, true> : periodic_kernel<T, E, false>,
                        grid_for(n, 128), 128, s, a, p.jper, p.kper, n);
        if (rc != MFLBM_OK) return rc;
    }
    if (p.kper == 0 && p.domain_wall_status_z_min == 0 && p.domain_wall_status_z_max == 0) {
        const int in = p.inlet_BC == 1 || p.inlet_BC == 2 ? p.inlet_BC : 0;
        const int out = p.outlet_BC == 1 || p.outlet_BC == 2 ? p.outlet_BC : 0;
        if ((in == 0 || in == 1) && (out == 0 || out == 1) && (in || out)) {
            const int ntx = (g.nx + 15) / 16, ncolp = ntx * 16 * ((g.ny + 1) / 2 * 2);
            rc = launch_pdl("inlet_outlet",
                            odd ? inlet_outlet_links_kernel<T, E, true> : inlet_outlet_links_kernel<T, E, false>,
                            grid_for((ll)ncolp * 11, 128), 128, s, a, in, out, ntx, ncolp);
            if (rc != MFLBM_OK) return rc;
        } else if (in || out) {
            rc = launch_pdl("inlet_outlet", odd ? inlet_outlet_kernel<T, E, true> : inlet_outlet_kernel<T, E, false>,
                            face_grid(g), 128, s, a, in, out);
            if (rc != MFLBM_OK) return rc;
        }
    }
    if (p.porous_plate_cmd != 0)
        return launch_pdl("porous_plate", odd ? porous_plate_kernel<T, E, true> : porous_plate_kernel<T, E, false>,
                          face_grid(g), 128, s, a);
    return MFLBM_OK;
}

}  // namespace MFLBM_NS
}  // namespace mflbm
