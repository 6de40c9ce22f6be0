// Colour-gradient pipeline of one time step (included by step_kernels.cuh):
// src/main_iteration_GPU.cu:732-1003 with the ranges of the reference's
// launches (:2027-2054).
//
//   1. phi on solid boundary nodes (list with precomputed fluid-neighbour masks)
//   2. unit interface normal + |grad phi| at the fluid nodes of [-1, n+2]^3,
//      with the geometrical wetting applied in the same thread at fluid
//      boundary nodes (it only reads its own node's values, so fusing it is
//      exact); stored as one record (n_x, n_y, n_z, |grad phi|) per node of
//      the s2 layout.  Solid nodes keep the zero record the reference writes
//      there every step (records are zeroed when the geometry is set and when
//      arrays are packed).
//   3. normal on solid boundary nodes: weighted mean of the fluid
//      neighbours' normals
//   4. curvature at the interface nodes and the record the collision reads,
//      (n_x, n_y, n_z, 0.5 * gamma * curv * c_norm), stored in fluid-list
//      order so that the collision reads it contiguously
//
// Sparse passes.  Away from interfaces phi is exactly +1 or -1, every
// difference in an ISO4 sum is +0 and the normal record is the zero record;
// so are the extrapolated normals of solid nodes whose fluid neighbours all
// have zero records.  The pipeline keeps the list of the fluid nodes whose
// record is non-zero (olist) between passes.  A pass resets those records to
// zero, lists the fluid nodes whose stencil is not all (to within 7e-7) +1
// or -1 (nlist, from per-row bit masks of phi), recomputes the normals of
// those nodes only (rebuilding olist), extrapolates normals to the solid
// boundary nodes of the super-blocks where phi can have changed and computes
// the curvature at the fluid nodes of olist.  Every fluid record outside the
// list is the zero record and every solid record is the dense passes' value,
// as in the reference.
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
    uint8_t* touch;        // s2 (solid boundary nodes): tag of the last pass with a non-zero record next to it
    const uint32_t* snb;   // s2 (fluid nodes): bit q where x + e_q is a solid boundary node of [0, n+1]^3
    int tag;               // this pass's tag, 1 or 2 (alternating); the previous pass had the other
    uint16_t* pmask;       // s4 rows (y, z) x super-block columns: phi near +1 bits (low byte), near -1 (high byte)
    const uint8_t* fmask;  // the same rows: fluid nodes of [1, n]^3
    const uint8_t* cmask;  // the same rows: walls_type <= 0 on [-1, n+2]^3 (the nodes whose normal may be non-zero)
    const int32_t* tmap;   // s2 -> fluid-list index (or -1)
    uint32_t* olist;       // packed coordinates of the nodes whose record is non-zero (interface flag set)
    uint32_t* nlist;       // packed fluid nodes whose normal this pass recomputes
    int* gcount;           // [0] olist, [2] nlist lengths, [1] solid nodes given a non-zero normal by this
                           // pass; [4] the previous pass's [0]; [5] 1: this pass processes every node
    T *cnx, *cny, *cnz, *cnorm, *curv;  // reference-layout arrays (export / pack)
    const uint2* l_phi;
    const uint32_t* l_fluid;
    int n_phi, n_cn, n_fluid, n_norm;
    // super-blocks (4 x 4 x 4 phi bricks)
    int SX, SY, SZ;
    int8_t* sbcode;        // fluid code of the super-block (below)
    uint8_t* sbact;        // 1: the super-block's phi may change at the next step
    uint32_t* sblive;      // super-blocks of this pass
    int* sbinfo;           // [1] 1: every super-block (consumed by this pass)
    int* live_n;           // number of super-blocks of this pass (sbinfo[0] or [2], alternating)
    int* live_next;        // the next pass's count, zeroed by this pass
    const int* phioff;     // list_phi_ext offsets of each super-block
    int slab_z, slab_y;    // 1: the two super-block rows at each z (y) face are always processed
    Phys<T> ph;
};

template <class T> __device__ __forceinline__ T wq_of(const ModelConsts<T>& c, int q) { return q < 7 ? c.w1 : c.w2; }

// Distance from +-1 within which a stencil value counts as +-1 for the node
// listing (phi_mask_kernel): 3 * 2^-22, exact in FP32 and FP64.
constexpr double kNearOne = 7.152557373046875e-07;

// Append `value` to `list` (capacity `cap`) where `want` is set: one atomic
// per warp, the order within the list is arbitrary.  Every list is sized for
// the most entries a pass can produce; the capacity checks here and the
// clamped lengths of the readers keep every access inside the buffers even
// if a count were not reset.
__device__ __forceinline__ void warp_append(bool want, uint32_t value, uint32_t* list, int* count, int cap) {
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, want);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(act, base, leader);
    const int idx = base + __popc(m & ((1u << lane) - 1u));
    if (want && idx < cap) list[idx] = value;
}

// Reserve `cnt` consecutive slots of a list per thread (warp prefix sum, one
// atomic per warp); returns the thread's first slot.  Every lane of the warp
// must call it.
__device__ __forceinline__ int warp_reserve(int cnt, int* count) {
    const int lane = threadIdx.x & 31;
    int incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int base = 0;
    if (lane == 31 && total) base = atomicAdd(count, total);
    return __shfl_sync(0xffffffffu, base, 31) + incl - cnt;
}


// phi on solid boundary nodes = weighted mean over fluid neighbours (:732-755)
template <class T>
__device__ __forceinline__ void extrapolate_phi_at(const GradArgs<T>& a, int t) {
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

// ---------------------------------------------------------------------------
// Super-blocks.  The dense passes (phi on solid boundary nodes, phi row
// masks, node listing) run only over super-blocks of 4 x 4 x 4 phi bricks
// (8^3 nodes of the s4 lattice) where phi can have changed since the last
// pass.  Away from the interfaces phi is exactly +1 or -1 and a fluid node
// keeps its value exactly as long as its fluid D3Q19 neighbours hold the
// same value: the absent component's populations are exactly 0 there, and
// collision, recolouring, streaming and bounce-back keep them 0.  A
// super-block's fluid code is 1 (2) when all its fluid nodes hold +1 (-1),
// 3 when it has no fluid node, 0 otherwise; the previous pass flagged it
// (`sbact`) when its code is 0 or it holds fluid of one sign next to a
// super-block with fluid of the other.  A fluid node whose phi can change is
// then in a flagged super-block or one node from one.  Solid and ghost nodes
// do not count in the codes: the phi of a solid node is extrapolated from
// fluid nodes within two nodes, and a node's row-mask bits and listing
// depend on phi within one node, so every change lies within four nodes of a
// flagged super-block: inside the 3 x 3 x 3 super-blocks around it, which
// this pass processes.  Super-blocks at open (inlet / outlet) or periodic
// faces, whose ghost layers the boundary updates rewrite every step, are
// always processed, and so is everything after the host set or uploaded a
// state.
// Elsewhere phi, the row masks and the zero records are those of the last
// pass that processed the super-block.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) sb_live_kernel(const GradArgs<T> a) {
    pdl_wait();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    bool live = false;
    if (s < a.SX * a.SY * a.SZ) {
        const int sx = s % a.SX, sy = (s / a.SX) % a.SY, sz = s / (a.SX * a.SY);
        live = a.sbinfo[1] != 0 || (a.slab_z && (sz <= 1 || sz >= a.SZ - 2)) ||
               (a.slab_y && (sy <= 1 || sy >= a.SY - 2));
        unsigned any = 0;
#pragma unroll
        for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                for (int dx = -1; dx <= 1; ++dx) {
                    const int x = sx + dx, y = sy + dy, z = sz + dz;
                    if (x >= 0 && x < a.SX && y >= 0 && y < a.SY && z >= 0 && z < a.SZ)
                        any |= a.sbact[x + a.SX * (y + a.SY * z)];
                }
        live = live || any != 0;
    }
    if (s == 0) {
        *a.live_next = 0;
        // the node lists restart; the previous olist length stays for the
        // reset of its records (clear_records)
        a.gcount[4] = a.gcount[0];
        a.gcount[0] = a.gcount[1] = a.gcount[2] = 0;
        a.gcount[5] = a.sbinfo[1] != 0 ? 1 : 0;
    }
    warp_append(live, (uint32_t)s, a.sblive, a.live_n, a.SX * a.SY * a.SZ);
}

// sbact of super-block s from this pass's codes (run by the node-listing
// kernel over every super-block)
template <class T>
__device__ __forceinline__ void sb_active_at(const GradArgs<T>& a, int s) {
    const int sx = s % a.SX, sy = (s / a.SX) % a.SY, sz = s / (a.SX * a.SY);
    const int8_t c = a.sbcode[s];
    unsigned seen = 0;   // bit c: code c occurs in the 3 x 3 x 3 super-blocks around
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
                const int x = sx + dx, y = sy + dy, z = sz + dz;
                if (x >= 0 && x < a.SX && y >= 0 && y < a.SY && z >= 0 && z < a.SZ)
                    seen |= 1u << a.sbcode[x + a.SX * (y + a.SY * z)];
            }
    // flagged: mixed fluid nodes, or fluid of one sign next to fluid of the
    // other (fluid neighbours lie in the same or adjacent super-blocks)
    const bool act = c == 0 || (c != 3 && (seen & 6u) == 6u);
    a.sbact[s] = act ? 1 : 0;
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

// Reset the records of the previous pass's interface list to the zero record
// (and their flags), so that every fluid record outside this pass's list is
// zero.  Grid-stride, run by the threads of the mask pass.
template <class T>
__device__ __forceinline__ void clear_records(const GradArgs<T>& a, int tid, int nthreads) {
    const int no = min(a.gcount[4], a.n_norm);
    typename Vec4<T>::type z;
    z.x = T(0); z.y = T(0); z.z = T(0); z.w = T(0);
    for (int p = tid; p < no; p += nthreads) {
        int i, j, k;
        unpack_xyz(a.olist[p], i, j, k);
        const ll n2 = a.g.s2(i, j, k);
        a.cn[n2] = z;
        a.iface[n2] = 0;
    }
}

// Per super-block of this pass (one block of 64 threads): the phi of its
// solid boundary nodes (extrapolated from fluid neighbours, which this
// kernel does not write, so the super-blocks are independent), then the row
// masks of the s4 lattice: for row (y, z) and byte b (x = 8b .. 8b + 7, the
// x extent of super-block column b), pmask holds bit x & 7 where phi is
// within kNearOne of +1 (low byte) and of -1 (high byte).  One row of 8
// nodes per thread; the super-block's fluid code follows from the rows'
// fluid masks (fmask) and exact comparisons with +-1.  The threads also
// reset the records of the previous pass's lists.
//
// Why "within kNearOne" suffices: with every stencil value phi_q = s + e_q,
// s = +-1 and |e_q| <= d, the ISO4 gradient is 3 sum_q w_q e_q e_q-vector,
// whose length is at most d * max over sign choices |sum_q 3 w_q (+-e_q)| =
// d * sqrt(14) / 3 = 1.2472 d (attained along (1, 2/3, 1/3)).  In the
// arithmetic of iso4_d*: the face difference is exact (Sterbenz), the
// running edge sum rounds at most three times by half an ulp of 1 (2^-24 in
// FP32), times iso4b = 1/12, and the products and the final sum round
// values of order d; so the computed |grad phi| is below 1.2472 d + 3e-8.
// With d = 3 * 2^-22 (7.15e-7, exact in FP32) that is below 9.3e-7 < 1e-6,
// the cut-off under which the normal pass writes the zero record: such a
// node need not be listed.  Away from interfaces phi is exactly +-1 or
// within a few ulps of it, so most stencils qualify.
template <class T>
__global__ void __launch_bounds__(64) phi_mask_kernel(const GradArgs<T> a) {
    pdl_wait();
    clear_records<T>(a, (int)(blockIdx.x * blockDim.x + threadIdx.x), (int)(gridDim.x * blockDim.x));
    const int NX = a.g.nx + 8, NY = a.g.ny + 8, NZ = a.g.nz + 8;
    const int nl = min(*a.live_n, a.SX * a.SY * a.SZ);
    const int ly = threadIdx.x & 7, lz = threadIdx.x >> 3;
    for (int w = blockIdx.x; w < nl; w += gridDim.x) {
        const int sb = (int)a.sblive[w];
        // phi of the super-block's solid boundary nodes (from fluid phi only),
        // then its rows
        if (a.n_phi) {
            for (int t = a.phioff[sb] + threadIdx.x; t < a.phioff[sb + 1]; t += blockDim.x) extrapolate_phi_at<T>(a, t);
            __syncthreads();
        }
        const int sx = sb % a.SX, y = 8 * ((sb / a.SX) % a.SY) + ly, z = 8 * (sb / (a.SX * a.SY)) + lz;
        unsigned F = 0, P = 0, M = 0, NP = 0, NM = 0;   // exactly +-1 (codes), within kNearOne (listing)
        if (y < NY && z < NZ) {
            const ll r = sx + (ll)a.SX * (y + (ll)NY * z);
            const T* row = a.phi + (ll)NX * (y + (ll)NY * z) + 8 * sx;
            const int nb = min(8, NX - 8 * sx);
            const T d = T(kNearOne);
#pragma unroll
            for (int b = 0; b < 8; ++b)
                if (b < nb) {
                    const T v = row[b];
                    P |= (v == T(1) ? 1u : 0u) << b;
                    M |= (v == T(-1) ? 1u : 0u) << b;
                    NP |= (v >= T(1) - d && v <= T(1) + d ? 1u : 0u) << b;
                    NM |= (v >= T(-1) - d && v <= T(-1) + d ? 1u : 0u) << b;
                }
            a.pmask[r] = (uint16_t)(NP | (NM << 8));
            F = a.fmask[r];
        }
        // fluid code: 3 without fluid nodes, 1 (2) when all of them are +1 (-1), else 0
        const int anyf = __syncthreads_or(F != 0);
        const int notp = __syncthreads_or((F & ~P) != 0);
        const int notm = __syncthreads_or((F & ~M) != 0);
        if (threadIdx.x == 0) a.sbcode[sb] = !anyf ? 3 : !notp ? 1 : !notm ? 2 : 0;
    }
}

// 24-bit windows of a row's +1 and -1 masks around byte b: bytes b - 1, b,
// b + 1 (0 past the row ends) at bits 0, 8, 16.
__device__ __forceinline__ void mask_window(const uint16_t* pm, ll r, int b, int SX, uint32_t& wp, uint32_t& wm) {
    const uint32_t c = pm[r], l = b > 0 ? pm[r - 1] : 0u, h = b + 1 < SX ? pm[r + 1] : 0u;
    wp = (l & 0xFFu) | ((c & 0xFFu) << 8) | ((h & 0xFFu) << 16);
    wm = (l >> 8) | ((c >> 8) << 8) | ((h >> 8) << 16);
}

// The nodes whose normal this pass recomputes: the candidates (walls_type <=
// 0 on [-1, n+2]^3, cmask) whose ISO4 stencil (the node and its 18 D3Q19
// neighbours) is not all within kNearOne of +1 or all within it of -1;
// elsewhere |grad phi| < 1e-6 and the record is the zero record
// (phi_mask_kernel gives the bound).  Per
// row of 8 nodes, bit-parallel: with a window w of a row's mask (byte b at
// bits 8..15), w >> 8, w >> 7 and w >> 9 hold x, x - 1 and x + 1; the
// stencil is x +- 1 of row (y, z), x and x +- 1 of rows (y +- 1, z) and
// (y, z +- 1), and x of rows (y +- 1, z +- 1).  Appended to nlist (one atomic
// per warp).  One block of 64 threads per super-block of this pass.  The
// same launch first flags every super-block for the next pass (sb_active_at:
// it needs the codes of this pass, which the mask kernel has written).
template <class T>
__global__ void __launch_bounds__(64) active_nodes_kernel(const GradArgs<T> a) {
    pdl_wait();
    const int NY = a.g.ny + 8, NZ = a.g.nz + 8;
    const int nl = min(*a.live_n, a.SX * a.SY * a.SZ);
    const int ly = threadIdx.x & 7, lz = threadIdx.x >> 3;
    const ll RY = a.SX, RZ = (ll)a.SX * NY;   // row strides of the masks
    const int nsb = a.SX * a.SY * a.SZ;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsb; s += gridDim.x * blockDim.x) sb_active_at<T>(a, s);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.sbinfo[1] = 0;   // the every-super-block request is consumed
    if (!a.n_norm) return;
    for (int w = blockIdx.x; w < nl; w += gridDim.x) {
        const int sb = (int)a.sblive[w];
        const int sx = sb % a.SX, y = 8 * ((sb / a.SX) % a.SY) + ly, z = 8 * (sb / (a.SX * a.SY)) + lz;
        unsigned sel = 0;   // bit b: node x = 8 sx + b of the row is listed
        if (y >= 1 && y < NY - 1 && z >= 1 && z < NZ - 1) {
            const ll r = sx + RY * y + RZ * z;
            const unsigned cand = a.cmask[r];
            if (cand) {
                uint32_t up = 0xFFFFFFFFu, um = 0xFFFFFFFFu, wp, wm;
                mask_window(a.pmask, r, sx, a.SX, wp, wm);
                up &= (wp >> 7) & (wp >> 8) & (wp >> 9);
                um &= (wm >> 7) & (wm >> 8) & (wm >> 9);
                const ll side[4] = {-RY, RY, -RZ, RZ};
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    mask_window(a.pmask, r + side[e], sx, a.SX, wp, wm);
                    up &= (wp >> 7) & (wp >> 8) & (wp >> 9);
                    um &= (wm >> 7) & (wm >> 8) & (wm >> 9);
                }
                const ll diag[4] = {-RY - RZ, RY - RZ, -RY + RZ, RY + RZ};
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const uint32_t c = a.pmask[r + diag[e]];
                    up &= c;
                    um &= c >> 8;
                }
                sel = cand & ~(up | um) & 0xFFu;
            }
        }
        int base = warp_reserve(__popc(sel), &a.gcount[2]);
        for (int b = 0; b < 8; ++b)
            if (sel & (1u << b)) {
                if (base < a.n_norm) a.nlist[base] = pack_xyz(8 * sx + b - 3, y - 3, z - 3);
                ++base;
            }
    }
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

// unit interface normal and |grad phi| (:757-807) + wetting (:809-878) at the
// nodes of nlist; nodes with a non-zero record are appended to olist (one
// atomic per warp) and give their solid boundary neighbours (snb) this
// pass's tag: plain byte stores of one value, so concurrent writers agree.
template <class T>
__global__ void __launch_bounds__(256, 8) normals_kernel(const GradArgs<T> a) {
    pdl_wait();
    const Grid& g = a.g;
    const int nt = min(a.gcount[2], a.n_norm);
    const int iters = (nt + gridDim.x * blockDim.x - 1) / (gridDim.x * blockDim.x);
    for (int it = 0; it < iters; ++it) {
        const int p = (it * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x;
        uint32_t packed = 0;
        bool on = false;
        if (p < nt) {
            int i, j, k;
            packed = a.nlist[p];
            unpack_xyz(packed, i, j, k);
            on = normal_at<T>(a, i, j, k, a.type8[g.s4(i, j, k)]);
            if (on) {
                const ll n2 = g.s2(i, j, k);
                const uint32_t m = a.snb[n2];
                if (m) {
                    const ll sy = g.nx + 4, sz = (ll)(g.nx + 4) * (g.ny + 4);
#pragma unroll
                    for (int q = 1; q < 19; ++q)
                        if (m & (1u << q)) a.touch[n2 + ex(q) + ey(q) * sy + ez(q) * sz] = (uint8_t)a.tag;
                }
            }
        }
        warp_append(on, packed, a.olist, &a.gcount[0], a.n_norm);
    }
}

// Interface normal on the solid boundary nodes (walls_type 2) of [0, n+1]^3
// = weighted mean over the fluid neighbours (walls_type <= 0), in direction
// order (:880-906), for every solid boundary node of this pass's
// super-blocks: zero or not, its record is written, so no list of the solid
// nodes that received a normal is kept.  A solid node's normal depends on the
// records of its fluid neighbours, which change only within two nodes of a
// phi that changed: within three nodes of a flagged super-block, inside the
// processed ones.  Neighbours whose interface flag is clear hold the zero
// record: their +0 terms are skipped (only their weights are summed), which
// leaves every sum bit-identical.
// The non-zero fluid records after a pass are exactly those of its olist, so
// a solid node's record can differ from its last written value only if a
// fluid neighbour is in this pass's olist (the normal pass tagged it with
// this pass's tag) or in the previous one's (the previous tag).  Only those
// are recomputed; a node that carries the previous tag has no non-zero
// neighbour left, so it gets the zero record and its tag is cleared.  A node
// tagged two passes ago and not since carries the current tag value again
// and is recomputed once more, which is harmless.  A pass after the host set
// the state recomputes every node.  Each block takes a run of consecutive
// live super-blocks (about live / grid of them) and lays their solid nodes
// out as one index range (offsets in shared memory); a thread loads the list
// entries and then the tags of kNodes nodes before it handles any of them,
// so the loads of a block overlap instead of following each other per
// super-block.  gcount[1] counts the non-zero results.
template <class T>
__global__ void __launch_bounds__(256) extrapolate_normal_kernel(const GradArgs<T> a) {
    pdl_wait();
    typedef typename Vec4<T>::type V4;
    constexpr int kMaxSB = 32;   // super-blocks per batch (one warp's scan)
    constexpr int kNodes = 4;    // list entries per thread per round
    __shared__ int s_beg[kMaxSB + 1], s_off[kMaxSB];
    __shared__ int s_dn[19];     // s2 offset of direction q
    const Grid& g = a.g;
    const int sy = g.nx + 4, sz = (g.nx + 4) * (g.ny + 4);
    if (threadIdx.x < 19) {
        const int q = threadIdx.x;
        s_dn[q] = ex(q) + ey(q) * sy + ez(q) * sz;
    }
    const int nl = min(*a.live_n, a.SX * a.SY * a.SZ);
    const bool all = a.gcount[5] != 0;
    const uint8_t tag = (uint8_t)a.tag, prev = (uint8_t)(3 - a.tag);
    const int per = min(kMaxSB, max(1, (nl + (int)gridDim.x - 1) / (int)gridDim.x));
    int nonzero = 0;
    for (int w0 = blockIdx.x * per; w0 < nl; w0 += gridDim.x * per) {
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            int cnt = 0, off = 0;
            if (lane < per && w0 + lane < nl) {
                const uint32_t sb = a.sblive[w0 + lane];
                off = a.phioff[sb];
                cnt = a.phioff[sb + 1] - off;
            }
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            if (lane < per) { s_off[lane] = off; s_beg[lane + 1] = incl; }
            if (lane == 0) s_beg[0] = 0;
        }
        __syncthreads();
        const int total = s_beg[per];
        for (int t0 = threadIdx.x; t0 < total; t0 += kNodes * blockDim.x) {
            int n[kNodes];
            uint32_t nb[kNodes];
#pragma unroll
            for (int u = 0; u < kNodes; ++u) {
                const int t = t0 + u * (int)blockDim.x;
                n[u] = -1;
                nb[u] = 0;
                if (t < total) {
                    int lo = 0, hi = per;   // s_beg[lo] <= t < s_beg[hi]
                    while (hi - lo > 1) {
                        const int mid = (lo + hi) >> 1;
                        if (s_beg[mid] <= t) lo = mid; else hi = mid;
                    }
                    const uint2 e = a.l_phi[s_off[lo] + t - s_beg[lo]];
                    int i, j, k;
                    unpack_xyz(e.x, i, j, k);
                    if (i >= 0 && j >= 0 && k >= 0 && i <= g.nx + 1 && j <= g.ny + 1 && k <= g.nz + 1) {
                        n[u] = (int)g.s2(i, j, k);
                        nb[u] = e.y;
                    }
                }
            }
            uint8_t tv[kNodes];
#pragma unroll
            for (int u = 0; u < kNodes; ++u) tv[u] = (n[u] >= 0 && !all) ? a.touch[n[u]] : tag;
#pragma unroll
            for (int u = 0; u < kNodes; ++u) {
                if (n[u] < 0) continue;
                if (tv[u] != tag) {
                    if (tv[u] == prev) {
                        V4 z;
                        z.x = T(0); z.y = T(0); z.z = T(0); z.w = T(0);
                        a.cn[n[u]] = z;
                        a.touch[n[u]] = 0;
                    }
                    continue;
                }
                // the fluid neighbours in direction order (lowest bit first)
                T sx = T(0), syy = T(0), szz = T(0), ws = T(0);
                uint32_t m = nb[u] & 0x7FFFEu;
                while (m) {
                    const int q = __ffs(m) - 1;
                    m &= m - 1;
                    const int mm = n[u] + s_dn[q];
                    const T wq = wq_of(a.ph.c, q);
                    if (a.iface[mm]) {
                        const V4 v = a.cn[mm];
                        sx += v.x * wq;
                        syy += v.y * wq;
                        szz += v.z * wq;
                    }
                    ws += wq;
                }
                V4 r;
                r.x = sx / ws; r.y = syy / ws; r.z = szz / ws; r.w = T(0);
                a.cn[n[u]] = r;
                nonzero += (r.x != T(0) || r.y != T(0) || r.z != T(0)) ? 1 : 0;
            }
        }
        __syncthreads();   // s_beg / s_off of the next batch
    }
    // one atomic per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nonzero += __shfl_xor_sync(0xffffffffu, nonzero, o);
    if ((threadIdx.x & 31) == 0 && nonzero) atomicAdd(&a.gcount[1], nonzero);
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
// interface nodes: the fluid nodes of [1, n]^3 in olist (non-zero normal
// record).  Away from interfaces |grad phi| is exactly 0 and the normal
// record is all zeros; the collision's force 0.5 gamma curv |grad phi| n and
// its recolouring direction are then zero whatever the curvature, and the
// collision reads the record only where the interface flag is set.
// Grid-stride loop over the list (its length is on the device).
template <class T>
__global__ void __launch_bounds__(256) curvature_kernel(const GradArgs<T> a) {
    pdl_wait();
    const Grid& g = a.g;
    const int sy = g.nx + 4, sz = (g.nx + 4) * (g.ny + 4);
    const int n = min(a.gcount[0], a.n_norm);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int i, j, k;
        unpack_xyz(a.olist[p], i, j, k);
        const int n2 = (int)g.s2(i, j, k);
        const int t = a.tmap[n2];
        if (t < 0) continue;   // ghost layers and nodes outside the fluid list
        typename Vec4<T>::type ctr, r;
        const T cv = curvature_at<T>(a.ph.c, a.cn, n2, sy, sz, ctr);
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
    // 1 where the record is non-zero (uploaded arrays can carry a normal with
    // c_norm = 0); such nodes form olist, which the next pass clears first.
    // Solid records are zero here; the next pass (every super-block) extrapolates them.
    const bool nz = v.x != T(0) || v.y != T(0) || v.z != T(0) || v.w != T(0);
    a.iface[n] = nz ? 1 : 0;
    if (nz) {
        const int at = atomicAdd(&a.gcount[0], 1);
        if (at < a.n_norm) a.olist[at] = pack_xyz(i, j, k);
    }
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
    a.touch = d.touch; a.snb = d.snb; a.tag = 1;
    a.pmask = d.pmask; a.fmask = d.fmask; a.cmask = d.cmask;
    a.tmap = d.tmap;
    a.olist = d.olist; a.nlist = d.nlist; a.gcount = d.gcount;
    a.cnx = (T*)d.cn_x; a.cny = (T*)d.cn_y; a.cnz = (T*)d.cn_z;
    a.cnorm = (T*)d.c_norm; a.curv = (T*)d.curv;
    a.l_phi = d.list_phi_ext; a.n_phi = (int)d.n_phi_ext;
    a.n_cn = (int)d.n_cn_ext;
    a.l_fluid = d.fluid_list; a.n_fluid = (int)d.n_fluid;
    a.n_norm = (int)d.n_norm;
    a.SX = d.SX; a.SY = d.SY; a.SZ = d.SZ;
    a.sbcode = d.sbcode; a.sbact = d.sbact; a.sblive = (uint32_t*)d.sblive; a.sbinfo = d.sbinfo;
    a.live_n = a.live_next = nullptr;   // set by launch_gradient
    a.phioff = d.phioff;
    const mflbm_params& p = c.params;
    a.slab_z = p.kper || (p.domain_wall_status_z_min == 0 && p.domain_wall_status_z_max == 0);
    a.slab_y = p.jper;
    a.ph = make_phys<T>(c.params);
    return a;
}

// The per-step pipeline (also the start-up colour_gradient,
// src/Phase_gradient.cpp:15-216, which performs the same passes).  Every
// kernel is launched with programmatic dependent launch (launch_pdl); the
// list counters are reset inside the kernels (the super-block count of the
// next pass by sb_live, the node lists by sb_active), so no memset breaks
// the chain.
template <class T>
int launch_gradient(mflbm_context& c) {
    GradArgs<T> a = grad_args<T>(c);
    a.live_n = c.d.sbinfo + (c.d.grad_parity ? 2 : 0);
    a.live_next = c.d.sbinfo + (c.d.grad_parity ? 0 : 2);
    a.tag = 1 + c.d.grad_parity;
    c.d.grad_parity ^= 1;
    const Tuning& tn = c.d.tune;
    cudaStream_t s = c.stream;
    int rc;
    // the list passes run one wave of resident blocks (grid-stride loops: the
    // list lengths are known only on the device; blocks beyond the resident
    // ones would start only after the first wave has walked the whole list)
    auto wave = [&](const void* kernel, int bs) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, bs, 0) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        return (unsigned)(std::max(1, c.d.n_sm) * per_sm);
    };
    const int nsb = a.SX * a.SY * a.SZ;
    // this pass's super-blocks
    if ((rc = launch_pdl("sb_live", sb_live_kernel<T>, grid_for(nsb, 64), 64, s, a)) != MFLBM_OK) return rc;
    // solid phi + row masks + super-block codes + reset of the previous lists' records
    if ((rc = launch_pdl("phi_mask", phi_mask_kernel<T>, wave((const void*)phi_mask_kernel<T>, 64), 64, s, a)) !=
        MFLBM_OK)
        return rc;
    // flags for the next pass + node listing
    rc = launch_pdl("active_nodes", active_nodes_kernel<T>, wave((const void*)active_nodes_kernel<T>, 64), 64, s, a);
    if (rc != MFLBM_OK) return rc;
    if (a.n_norm) {
        rc = launch_pdl("normals", normals_kernel<T>, wave((const void*)normals_kernel<T>, tn.normals), tn.normals, s, a);
        if (rc != MFLBM_OK) return rc;
        if (a.n_cn && (rc = launch_pdl("extrapolate_normal", extrapolate_normal_kernel<T>,
                                       wave((const void*)extrapolate_normal_kernel<T>, tn.extrapolate), tn.extrapolate,
                                       s, a)) != MFLBM_OK)
            return rc;
    }
    if (!a.n_fluid) return MFLBM_OK;
    return launch_pdl("curvature", curvature_kernel<T>, wave((const void*)curvature_kernel<T>, tn.curvature),
                      tn.curvature, s, a);
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
    MFLBM_CUDA(cudaMemsetAsync(c.d.gcount, 0, 3 * sizeof(int), c.stream));
    pack_normals_kernel<T><<<dim3(grid_for(g.nx + 4, 128), g.ny + 4, g.nz + 4), 128, 0, c.stream>>>(a);
    int rc = after_launch("pack_normals");
    if (rc != MFLBM_OK || !a.n_fluid) return rc;
    aux_from_arrays_kernel<T><<<grid_for(a.n_fluid, 128), 128, 0, c.stream>>>(a);
    return after_launch("aux_from_arrays");
}

}  // namespace MFLBM_NS
}  // namespace mflbm
