// Colour-gradient pipeline of one time step (included by step_kernels.cuh):
// src/main_iteration_GPU.cu:732-1003 with the ranges of the reference's
// launches (:2027-2054).
//
//   1. phi on solid boundary nodes (list with precomputed fluid-neighbour masks)
//   2. unit interface normal + |grad phi| at the fluid nodes of [-1, n+2]^3
//      (list in brick order), with the geometrical wetting applied in the
//      same thread at fluid boundary nodes (it only reads its own node's
//      values, so fusing it is exact); stored as one record
//      (n_x, n_y, n_z, |grad phi|) per node of the s2 layout.  Solid nodes
//      keep the zero record the reference writes there every step (records
//      are zeroed when the geometry is set and when arrays are packed).
//      The fluid nodes of [1, n]^3 with a non-zero record are appended to a
//      compact list (the interface nodes of this step).
//   3. normal on solid boundary nodes (list with masks)
//   4. curvature at the interface nodes and the record the collision reads,
//      (n_x, n_y, n_z, 0.5 * gamma * curv * c_norm), stored in fluid-list
//      order so that the collision reads it contiguously
//
// The reference-layout arrays cn_x/y/z, c_norm and curv (curvature on all of
// [1, n]^3, solid nodes included) are produced from the records only when the
// host asks for them (export), and records are rebuilt from such arrays when
// the host uploads them (pack).
#pragma once
#include "context.cuh"

namespace mflbm {
namespace MFLBM_NS {

template <class T> struct GradArgs {
    typedef typename Vec4<T>::type V4;
    Grid g;
    const int8_t* type8;
    const T *snx, *sny, *snz;
    T* phi;
    V4* cn;    // s2: (n_x, n_y, n_z, |grad phi|)
    V4* aux;   // fluid-list order: (n_x, n_y, n_z, 0.5 * gamma * curv * c_norm)
    int8_t* iface;  // s2 (fluid nodes): 1 where the record may be non-zero; 0: the zero record
    int8_t* phib;   // per 2x2x2 brick of the s4 lattice: 1 all phi = +1, 2 all phi = -1, else 0
    const int32_t* tmap;   // s2 -> fluid-list index (or -1)
    uint32_t* ilist;       // interface nodes of this step (fluid-list indices), appended by the normal pass
    int* ilist_n;
    T *cnx, *cny, *cnz, *cnorm, *curv;  // reference-layout arrays (export / pack)
    const uint2 *l_phi, *l_cn;
    const uint32_t *l_fluid, *l_norm;
    int n_phi, n_cn, n_fluid, n_norm;
    Phys<T> ph;
};

template <class T> __device__ __forceinline__ T wq_of(const ModelConsts<T>& c, int q) { return q < 7 ? c.w1 : c.w2; }

// phi on solid boundary nodes = weighted mean over fluid neighbours (:732-755)
template <class T>
__global__ void __launch_bounds__(256) extrapolate_phi_kernel(const GradArgs<T> a) {
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

// ISO4 first derivatives of a scalar field at flat index n of an array with
// strides (1, sy, sz), in the reference's operand order (:765-791).
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

// Bulk detection for the normal pass: per 2x2x2 brick of the s4 lattice
// (s4-local coordinates 2b, 2b + 1 on each axis; positions past the lattice
// end are ignored), 1 if every phi is exactly +1, 2 if every phi is exactly -1,
// 0 otherwise.  Away from interfaces phi is exactly +-1 (one component is
// exactly zero), so most bricks are uniform.
template <class T>
__global__ void __launch_bounds__(256) phi_brick_kernel(const GradArgs<T> a) {
    typedef typename Vec2<T>::type P;
    const int NX = a.g.nx + 8, NY = a.g.ny + 8, NZ = a.g.nz + 8;
    const int BX = (NX + 1) >> 1, BY = (NY + 1) >> 1, BZ = (NZ + 1) >> 1;
    const ll b = (ll)blockIdx.x * blockDim.x + threadIdx.x;   // bricks in x-fastest order
    if (b >= (ll)BX * BY * BZ) return;
    const int bx = (int)(b % BX), by = (int)((b / BX) % BY), bz = (int)(b / ((ll)BX * BY));
    bool plus = true, minus = true;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int y = 2 * by + (e & 1), z = 2 * bz + (e >> 1);
        if (y >= NY || z >= NZ) continue;
        const T* row = a.phi + (ll)NX * (y + (ll)NY * z);
        T v0, v1;
        if (!(NX & 1)) {            // even rows: every row starts on a pair boundary
            const P v = reinterpret_cast<const P*>(row)[bx];
            v0 = v.x;
            v1 = v.y;
        } else {
            v0 = row[2 * bx];
            v1 = 2 * bx + 1 < NX ? row[2 * bx + 1] : v0;
        }
        plus = plus && v0 == T(1) && v1 == T(1);
        minus = minus && v0 == T(-1) && v1 == T(-1);
    }
    a.phib[b] = plus ? 1 : minus ? 2 : 0;
}

// the normal record of node (i, j, k) of walls_type <= 0 (:757-807) + wetting
// (:809-878): the unit normal and |grad phi|, or the zero record where
// |grad phi| < 1e-6
template <class T>
__device__ __forceinline__ bool normal_at(const GradArgs<T>& a, int i, int j, int k, int type) {
    const Grid& g = a.g;
    const int sy4 = g.nx + 8, sz4 = (g.nx + 8) * (g.ny + 8);
    const int n4 = (int)g.s4(i, j, k);
    const T x = iso4_dx(a.ph.c, a.phi, n4, sy4, sz4);
    const T y = iso4_dy(a.ph.c, a.phi, n4, sy4, sz4);
    const T z = iso4_dz(a.ph.c, a.phi, n4, sy4, sz4);
    const T nrm = sqrt(x * x + y * y + z * z);
    typename Vec4<T>::type r;
    if (nrm < T(1e-6) || type >= 1) {
        r.x = T(0); r.y = T(0); r.z = T(0); r.w = T(0);
    } else {
        T cx = x / nrm, cy = y / nrm, cz = z / nrm;
        if (type == -1 && nrm > T(1e-6)) wetting(a.ph.cos_theta, a.snx[n4], a.sny[n4], a.snz[n4], cx, cy, cz);
        r.x = cx; r.y = cy; r.z = cz; r.w = nrm;
    }
    const ll n2 = g.s2(i, j, k);
    a.cn[n2] = r;
    a.iface[n2] = r.w != T(0) ? 1 : 0;
    return r.w != T(0);
}

// unit interface normal and |grad phi| at the fluid nodes of [-1, n+2]^3
// (:757-807) + wetting (:809-878)
template <class T>
__global__ void __launch_bounds__(256) normals_kernel(const GradArgs<T> a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n_norm) return;
    int i, j, k;
    unpack_xyz(a.l_norm[t], i, j, k);
    const Grid& g = a.g;
    const int n4 = (int)g.s4(i, j, k);
    const ll n2 = g.s2(i, j, k);
    const int8_t was = a.iface[n2];   // issued with the brick loads below
    {
        // The stencil (s4-local i+2 .. i+4 on each axis) lies in the 2x2x2
        // bricks (i+2)>>1 .. +1: if they are uniform with one value, every
        // difference in the ISO4 sums is +0, |grad phi| = 0 and the record is
        // the zero record -- written without reading the 18 neighbours.
        const int BX = (g.nx + 9) >> 1, BY = (g.ny + 9) >> 1;
        const int bx = (i + 2) >> 1, by = (j + 2) >> 1, bz = (k + 2) >> 1;
        const int8_t* pb = a.phib + bx + (ll)BX * (by + (ll)BY * bz);
        const int8_t c0 = pb[0];
        if (c0 != 0 && pb[1] == c0 && pb[BX] == c0 && pb[BX + 1] == c0 && pb[(ll)BX * BY] == c0 &&
            pb[(ll)BX * BY + 1] == c0 && pb[(ll)BX * BY + BX] == c0 && pb[(ll)BX * BY + BX + 1] == c0) {
            // a record is non-zero only where the interface flag is set: only
            // those are cleared, every other one is already the zero record
            if (was) {
                typename Vec4<T>::type r;
                r.x = T(0); r.y = T(0); r.z = T(0); r.w = T(0);
                a.cn[n2] = r;
                a.iface[n2] = 0;
            }
            return;
        }
    }
    const bool on = normal_at<T>(a, i, j, k, a.type8[n4]);
    // fluid nodes of [1, n]^3 with a non-zero record join the curvature's list
    // (one atomic per warp; the order of the list does not matter)
    const int tf = on ? a.tmap[n2] : -1;
    const unsigned act = __activemask();
    const unsigned want = __ballot_sync(act, tf >= 0);
    if (want) {
        const int lane = threadIdx.x & 31, leader = __ffs(want) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(a.ilist_n, __popc(want));
        base = __shfl_sync(act, base, leader);
        if (tf >= 0) a.ilist[base + __popc(want & ((1u << lane) - 1u))] = (uint32_t)tf;
    }
}

// interface normal on solid boundary nodes = weighted mean over fluid neighbours (:880-906)
template <class T>
__global__ void __launch_bounds__(256) extrapolate_normal_kernel(const GradArgs<T> a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n_cn) return;
    const uint2 e = a.l_cn[t];
    int i, j, k;
    unpack_xyz(e.x, i, j, k);
    const int sy = a.g.nx + 4, sz = (a.g.nx + 4) * (a.g.ny + 4);
    const int n = (int)a.g.s2(i, j, k);
    // fluid neighbours whose record is the zero record (interface flag 0)
    // contribute +0 to every sum: when all of them are such, the mean is +0
    // and only the flags (1 byte each) are read
    bool any = false;
#pragma unroll
    for (int q = 1; q < 19; ++q)
        if (e.y & (1u << q)) any = any || a.iface[n + ex(q) + ey(q) * sy + ez(q) * sz];
    // |grad phi| of a solid node is 0 in every record (the geometry set-up and
    // the array packing write solid records as zero records; only the
    // direction is extrapolated), so the record is written without reading it
    typename Vec4<T>::type r;
    r.w = T(0);
    if (!any) {
        r.x = T(0); r.y = T(0); r.z = T(0);
        a.cn[n] = r;
        return;
    }
    T sx = T(0), syy = T(0), szz = T(0), ws = T(0);
#pragma unroll
    for (int q = 1; q < 19; ++q) {
        if (e.y & (1u << q)) {
            const typename Vec4<T>::type v = a.cn[n + ex(q) + ey(q) * sy + ez(q) * sz];
            const T wq = wq_of(a.ph.c, q);
            sx += v.x * wq;
            syy += v.y * wq;
            szz += v.z * wq;
            ws += wq;
        }
    }
    r.x = sx / ws; r.y = syy / ws; r.z = szz / ws;
    a.cn[n] = r;
}

// curvature at node n (s2 index) from the nine ISO4 derivatives of the
// normal (:916-1002); the 18 neighbour records are loaded once.
template <class T>
__device__ __forceinline__ T curvature_at(const ModelConsts<T>& c, const typename Vec4<T>::type* cn, int n, int sy,
                                          int sz, typename Vec4<T>::type& ctr) {
    typedef typename Vec4<T>::type V4;
    ctr = cn[n];
    const V4 xp = cn[n + 1], xm = cn[n - 1], yp = cn[n + sy], ym = cn[n - sy], zp = cn[n + sz], zm = cn[n - sz];
    const V4 xpyp = cn[n + 1 + sy], xmym = cn[n - 1 - sy], xpym = cn[n + 1 - sy], xmyp = cn[n - 1 + sy];
    const V4 xpzp = cn[n + 1 + sz], xmzm = cn[n - 1 - sz], xpzm = cn[n + 1 - sz], xmzp = cn[n - 1 + sz];
    const V4 ypzp = cn[n + sy + sz], ymzm = cn[n - sy - sz], ypzm = cn[n + sy - sz], ymzp = cn[n - sy + sz];
#define MFLBM_DX(C) (c.iso4a * (xp.C - xm.C) + c.iso4b * (xpyp.C - xmym.C + xpym.C - xmyp.C + xpzp.C - xmzm.C + xpzm.C - xmzp.C))
#define MFLBM_DY(C) (c.iso4a * (yp.C - ym.C) + c.iso4b * (xpyp.C - xmym.C + xmyp.C - xpym.C + ypzp.C - ymzm.C + ypzm.C - ymzp.C))
#define MFLBM_DZ(C) (c.iso4a * (zp.C - zm.C) + c.iso4b * (xpzp.C - xmzm.C + xmzp.C - xpzm.C + ypzp.C - ymzm.C + ymzp.C - ypzm.C))
    const T kxx = MFLBM_DX(x), kyy = MFLBM_DY(y), kzz = MFLBM_DZ(z);
    const T kxy = MFLBM_DY(x), kxz = MFLBM_DZ(x);
    const T kyx = MFLBM_DX(y), kyz = MFLBM_DZ(y);
    const T kzx = MFLBM_DX(z), kzy = MFLBM_DY(z);
#undef MFLBM_DX
#undef MFLBM_DY
#undef MFLBM_DZ
    const T x = ctr.x, y = ctr.y, z = ctr.z;
    return (x * x - T(1)) * kxx + (y * y - T(1)) * kyy + (z * z - T(1)) * kzz +
           x * y * (kxy + kyx) + x * z * (kxz + kzx) + y * z * (kzy + kyz);
}

// Curvature and the collision's record (fluid-list order) at this step's
// interface nodes: the list the normal pass appended (fluid nodes with a
// non-zero normal record).  Away from interfaces |grad phi| is exactly 0 and
// the normal record is all zeros; the collision's force 0.5 gamma curv
// |grad phi| n and its recolouring direction are then zero whatever the
// curvature, and the collision reads the record only where the interface
// flag is set.  Grid-stride loop over the list (its length is on the device).
template <class T>
__global__ void __launch_bounds__(256) curvature_kernel(const GradArgs<T> a) {
    const Grid& g = a.g;
    const int sy = g.nx + 4, sz = (g.nx + 4) * (g.ny + 4);
    const int n = *a.ilist_n;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int t = (int)a.ilist[p];
        int i, j, k;
        unpack_xyz(a.l_fluid[t], i, j, k);
        typename Vec4<T>::type ctr, r;
        const T cv = curvature_at<T>(a.ph.c, a.cn, (int)g.s2(i, j, k), sy, sz, ctr);
        r.x = ctr.x; r.y = ctr.y; r.z = ctr.z;
        r.w = T(0.5) * a.ph.gamma * cv * ctr.w;
        a.aux[t] = r;
    }
}

// curvature on all of [1, n]^3 into the reference-layout curv array (export)
template <class T>
__global__ void __launch_bounds__(128) curvature_export_kernel(const GradArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y + 1, k = blockIdx.z + 1;
    const Grid& g = a.g;
    if (i > g.nx) return;
    const int sy = g.nx + 4, sz = (g.nx + 4) * (g.ny + 4);
    typename Vec4<T>::type ctr;
    a.curv[g.s1(i, j, k)] = curvature_at<T>(a.ph.c, a.cn, (int)g.s2(i, j, k), sy, sz, ctr);
}

// records -> reference arrays cn_x/y/z, c_norm on the s2 range
template <class T>
__global__ void __launch_bounds__(256) split_normals_kernel(const GradArgs<T> a, int n2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n2) return;
    const typename Vec4<T>::type v = a.cn[t];
    a.cnx[t] = v.x; a.cny[t] = v.y; a.cnz[t] = v.z; a.cnorm[t] = v.w;
}

// reference arrays (uploaded by the host) -> records; solid nodes get the
// zero record that the next gradient pass of the reference would leave there
template <class T>
__global__ void __launch_bounds__(128) pack_normals_kernel(const GradArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = (int)blockIdx.y - 1, k = (int)blockIdx.z - 1;
    const Grid& g = a.g;
    if (i > g.nx + 2) return;
    const ll n = g.s2(i, j, k);
    typename Vec4<T>::type v;
    if (a.type8[g.s4(i, j, k)] >= 1) {
        v.x = T(0); v.y = T(0); v.z = T(0); v.w = T(0);
    } else {
        v.x = a.cnx[n]; v.y = a.cny[n]; v.z = a.cnz[n]; v.w = a.cnorm[n];
    }
    a.cn[n] = v;
    // 1 where the record may be non-zero: uploaded arrays can carry a normal
    // with c_norm = 0, and the next normal pass must clear it
    a.iface[n] = (v.x != T(0) || v.y != T(0) || v.z != T(0) || v.w != T(0)) ? 1 : 0;
}
template <class T>
__global__ void __launch_bounds__(128) aux_from_arrays_kernel(const GradArgs<T> a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n_fluid) return;
    int i, j, k;
    unpack_xyz(a.l_fluid[t], i, j, k);
    const ll n2 = a.g.s2(i, j, k);
    typename Vec4<T>::type r;
    r.x = a.cnx[n2]; r.y = a.cny[n2]; r.z = a.cnz[n2];
    r.w = T(0.5) * a.ph.gamma * a.curv[a.g.s1(i, j, k)] * a.cnorm[n2];
    a.aux[t] = r;
}

// ---------------------------------------------------------------------------
template <class T>
GradArgs<T> grad_args(const mflbm_context& c) {
    const DeviceState& d = c.d;
    GradArgs<T> a;
    a.g = d.g;
    a.type8 = d.type8;
    a.snx = (const T*)d.s_nx; a.sny = (const T*)d.s_ny; a.snz = (const T*)d.s_nz;
    a.phi = (T*)d.phi;
    a.cn = (typename Vec4<T>::type*)d.cnv4;
    a.aux = (typename Vec4<T>::type*)d.aux;
    a.iface = d.iface;
    a.phib = d.phib;
    a.tmap = d.tmap; a.ilist = d.ilist; a.ilist_n = d.ilist_n;
    a.cnx = (T*)d.cn_x; a.cny = (T*)d.cn_y; a.cnz = (T*)d.cn_z;
    a.cnorm = (T*)d.c_norm; a.curv = (T*)d.curv;
    a.l_phi = d.list_phi_ext; a.n_phi = (int)d.n_phi_ext;
    a.l_cn = d.list_cn_ext; a.n_cn = (int)d.n_cn_ext;
    a.l_fluid = d.fluid_list; a.n_fluid = (int)d.n_fluid;
    a.l_norm = d.list_norm; a.n_norm = (int)d.n_norm;
    a.ph = make_phys<T>(c.params);
    return a;
}

// The per-step pipeline (also the start-up colour_gradient,
// src/Phase_gradient.cpp:15-216, which performs the same passes).
template <class T>
int launch_gradient(mflbm_context& c) {
    const GradArgs<T> a = grad_args<T>(c);
    const Tuning& tn = c.d.tune;
    cudaStream_t s = c.stream;
    int rc;
    if (a.n_phi) {
        extrapolate_phi_kernel<T><<<grid_for(a.n_phi, tn.extrapolate), tn.extrapolate, 0, s>>>(a);
        if ((rc = after_launch("extrapolate_phi")) != MFLBM_OK) return rc;
    }
    MFLBM_CUDA(cudaMemsetAsync(c.d.ilist_n, 0, sizeof(int), s));
    if (a.n_norm) {
        const Grid& g = c.d.g;
        phi_brick_kernel<T><<<grid_for((ll)((g.nx + 9) / 2) * ((g.ny + 9) / 2) * ((g.nz + 9) / 2), 256), 256, 0, s>>>(a);
        if ((rc = after_launch("phi_brick")) != MFLBM_OK) return rc;
        normals_kernel<T><<<grid_for(a.n_norm, tn.normals), tn.normals, 0, s>>>(a);
        if ((rc = after_launch("normals")) != MFLBM_OK) return rc;
    }
    if (a.n_cn) {
        extrapolate_normal_kernel<T><<<grid_for(a.n_cn, tn.extrapolate), tn.extrapolate, 0, s>>>(a);
        if ((rc = after_launch("extrapolate_normal")) != MFLBM_OK) return rc;
    }
    if (!a.n_fluid) return MFLBM_OK;
    // a fixed grid (the interface count is known only on the device)
    const int blocks = (int)std::min<ll>(grid_for(a.n_fluid, tn.curvature), 152 * 8);
    curvature_kernel<T><<<blocks, tn.curvature, 0, s>>>(a);
    return after_launch("curvature");
}

// Reference-layout cn_x/y/z, c_norm, curv from the records.
template <class T>
int launch_export(mflbm_context& c) {
    const GradArgs<T> a = grad_args<T>(c);
    const Grid& g = c.d.g;
    split_normals_kernel<T><<<grid_for(g.n2(), 256), 256, 0, c.stream>>>(a, (int)g.n2());
    int rc = after_launch("split_normals");
    if (rc != MFLBM_OK) return rc;
    curvature_export_kernel<T><<<dim3(grid_for(g.nx, 128), g.ny, g.nz), 128, 0, c.stream>>>(a);
    return after_launch("curvature_export");
}

// Records from reference-layout arrays supplied by the host.
template <class T>
int launch_refresh_aux(mflbm_context& c) {
    const GradArgs<T> a = grad_args<T>(c);
    const Grid& g = c.d.g;
    pack_normals_kernel<T><<<dim3(grid_for(g.nx + 4, 128), g.ny + 4, g.nz + 4), 128, 0, c.stream>>>(a);
    int rc = after_launch("pack_normals");
    if (rc != MFLBM_OK || !a.n_fluid) return rc;
    aux_from_arrays_kernel<T><<<grid_for(a.n_fluid, 128), 128, 0, c.stream>>>(a);
    return after_launch("aux_from_arrays");
}

}  // namespace MFLBM_NS
}  // namespace mflbm
