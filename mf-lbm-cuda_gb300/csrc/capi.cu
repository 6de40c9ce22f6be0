// The C ABI of libmflbm (include/mflbm.h).
#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstring>
#include <string>
#include <vector>

#include "context.cuh"
#include "setup.cuh"

namespace mflbm {

namespace {
thread_local std::string g_last_error;
std::atomic<unsigned long long> g_launches{0};

struct TimingPool {
    std::vector<cudaEvent_t> ev;  // 4 per timed step: collide start/end, gradient start/end
    size_t used = 0;
};
TimingPool& timing_pool(mflbm_context* c);
}  // namespace

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

namespace {

size_t tsize(const mflbm_context* c) { return c->params.precision == MFLBM_FP32 ? 4 : 8; }

int check_params(const mflbm_params* p) {
    if (!p) return fail(MFLBM_E_ARG, "null params");
    if (p->precision != MFLBM_FP32 && p->precision != MFLBM_FP64) return fail(MFLBM_E_ARG, "precision must be MFLBM_FP32 or MFLBM_FP64");
    if (p->fp_mode != MFLBM_FAST && p->fp_mode != MFLBM_STRICT) return fail(MFLBM_E_ARG, "fp_mode must be MFLBM_FAST or MFLBM_STRICT");
    if (p->nx < 3 || p->ny < 3 || p->nz < 4) return fail(MFLBM_E_ARG, "lattice must be at least 3 x 3 x 4");
    if (p->nx + 8 >= 1024 || p->ny + 8 >= 2048 || p->nz + 8 >= 2048)
        return fail(MFLBM_E_ARG, "lattice too large for packed node coordinates (nx <= 1015, ny, nz <= 2039)");
    const ll n1 = (p->nx + 2) * (p->ny + 2) * (p->nz + 2);
    if (n1 >= (1ll << 31)) return fail(MFLBM_E_ARG, "lattice too large: (nx+2)(ny+2)(nz+2) must be below 2^31");
    if (p->inlet_BC < 0 || p->inlet_BC > 2 || p->outlet_BC < 0 || p->outlet_BC > 2) return fail(MFLBM_E_ARG, "inlet_BC/outlet_BC must be 0, 1 or 2");
    if (p->porous_plate_cmd < 0 || p->porous_plate_cmd > 2) return fail(MFLBM_E_ARG, "porous_plate_cmd must be 0, 1 or 2");
    if (p->storage < MFLBM_STORE_NATIVE || p->storage > MFLBM_STORE_BF16)
        return fail(MFLBM_E_ARG, "storage must be MFLBM_STORE_NATIVE, MFLBM_STORE_F16 or MFLBM_STORE_BF16");
    if (p->storage != MFLBM_STORE_NATIVE && p->precision != MFLBM_FP32)
        return fail(MFLBM_E_ARG, "16-bit population storage needs MFLBM_FP32 (the collision computes in FP32)");
    return MFLBM_OK;
}

void free_all(mflbm_context* c) {
    DeviceState& d = c->d;
    void* ptrs[] = {d.pdf, d.phi, d.cn_x, d.cn_y, d.cn_z, d.c_norm, d.curv, d.W_in, d.f_cv, d.g_cv, d.phi_cv,
                    d.walls, d.walls_type, d.s_nx, d.s_ny, d.s_nz, d.fluid_list, d.list_phi_ext,
                    d.red, d.staging, d.aux, d.type8, d.cnv4, d.zpair_off,
                    d.phi_prev, d.prof, d.dither, d.iface, d.touch, d.snb, d.pmask, d.fmask, d.cmask, d.tmap, d.olist, d.nlist, d.gcount,
                    d.sbcode, d.sbact, d.sblive, d.sbinfo, d.phioff};
    for (void* p : ptrs) if (p) cudaFree(p);
    d = DeviceState{};
    if (c->pair_graph) cudaGraphExecDestroy(c->pair_graph);
    c->pair_graph = nullptr;
}

int alloc_zero(void** p, size_t bytes, cudaStream_t s) {
    MFLBM_CUDA(cudaMalloc(p, bytes));
    MFLBM_CUDA(cudaMemsetAsync(*p, 0, bytes, s));
    return MFLBM_OK;
}

// The next gradient pass processes every super-block: the host has set or
// replaced phi or the populations (gradient.cuh, super-blocks).
int request_full_pass(mflbm_context* c) {
    static const int one = 1;
    if (!c->d.sbinfo) return MFLBM_OK;
    MFLBM_CUDA(cudaMemcpyAsync(c->d.sbinfo + 1, &one, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    return MFLBM_OK;
}

template <class V>
int upload_list(V** dptr, ll* n, const std::vector<V>& h) {
    if (*dptr) cudaFree(*dptr);
    *dptr = nullptr;
    *n = (ll)h.size();
    if (h.empty()) return MFLBM_OK;
    MFLBM_CUDA(cudaMalloc(dptr, sizeof(V) * h.size()));
    MFLBM_CUDA(cudaMemcpy(*dptr, h.data(), sizeof(V) * h.size(), cudaMemcpyHostToDevice));
    return MFLBM_OK;
}

// The fluid list in the order of the population layout (consecutive threads
// touch consecutive pairs), the fluid-list index of each node (tmap) and the
// list offset of each layer of population tiles (zpair_off).  With `perm`,
// perm[t] receives the position in the previous list of the node now at t.
int order_fluid_list(mflbm_context* c, const std::vector<uint32_t>& nodes, std::vector<int>* perm) {
    DeviceState& d = c->d;
    const Grid g = d.g;
    std::vector<std::pair<ll, uint32_t>> fe;
    fe.reserve(nodes.size());
    for (uint32_t p : nodes) {
        int x, y, z;
        unpack_xyz(p, x, y, z);
        fe.emplace_back(d.b.elem(x, y, z), p);
    }
    std::sort(fe.begin(), fe.end());
    std::vector<uint32_t> fl(fe.size());
    for (size_t n = 0; n < fe.size(); ++n) fl[n] = fe[n].second;
    // layout order is tile-layer major: offsets of each layer of tiles
    // (slices 2^(lz+1) kt .. 2^(lz+1) (kt + 1) - 1)
    std::vector<int> zoff(d.b.ntz + 1, 0);
    for (size_t n = 0; n < fe.size(); ++n) {
        int x, y, z;
        unpack_xyz(fe[n].second, x, y, z);
        zoff[((z >> 1) >> d.b.lz) + 1]++;
    }
    for (int kt = 0; kt < d.b.ntz; ++kt) zoff[kt + 1] += zoff[kt];
    std::vector<int32_t> tm(g.n2(), -1);
    if (perm) {
        // the previous order from the previous tmap
        std::vector<int32_t> old(g.n2(), -1);
        if (d.tmap) MFLBM_CUDA(cudaMemcpy(old.data(), d.tmap, sizeof(int32_t) * g.n2(), cudaMemcpyDeviceToHost));
        perm->assign(fl.size(), 0);
        for (size_t n = 0; n < fl.size(); ++n) {
            int x, y, z;
            unpack_xyz(fl[n], x, y, z);
            (*perm)[n] = old[g.s2(x, y, z)];
            if ((*perm)[n] < 0) return fail(MFLBM_E_STATE, "fluid list: a node is missing from the previous order");
        }
    }
    for (size_t n = 0; n < fl.size(); ++n) {
        int x, y, z;
        unpack_xyz(fl[n], x, y, z);
        tm[g.s2(x, y, z)] = (int32_t)n;
    }
    int rc;
    if ((rc = upload_list(&d.fluid_list, &d.n_fluid, fl)) != MFLBM_OK) return rc;
    ll ntm = 0, nzo = 0;
    if ((rc = upload_list(&d.tmap, &ntm, tm)) != MFLBM_OK) return rc;
    if ((rc = upload_list(&d.zpair_off, &nzo, zoff)) != MFLBM_OK) return rc;
    return MFLBM_OK;
}

// Node lists from the device geometry: the fluid nodes of [1, n]^3 in the
// order of the population layout (order_fluid_list), and the solid boundary
// nodes with an 18-bit mask of their fluid neighbours (bit q set when
// neighbour x + e_q has walls_type <= 0).
int build_lists(mflbm_context* c) {
    DeviceState& d = c->d;
    const Grid g = d.g;
    std::vector<int32_t> walls(g.n2()), wt(g.n4());
    MFLBM_CUDA(cudaMemcpy(walls.data(), d.walls, sizeof(int32_t) * g.n2(), cudaMemcpyDeviceToHost));
    MFLBM_CUDA(cudaMemcpy(wt.data(), d.walls_type, sizeof(int32_t) * g.n4(), cudaMemcpyDeviceToHost));
    std::vector<uint32_t> nodes;
    for (int k = 1; k <= g.nz; ++k)
        for (int j = 1; j <= g.ny; ++j)
            for (int i = 1; i <= g.nx; ++i)
                if (walls[g.s2(i, j, k)] == 0) nodes.push_back(pack_xyz(i, j, k));
    std::vector<uint2> lphi;
    ll ncn = 0;   // walls_type == 2 nodes of [0, n+1]^3: the nodes of the normal extrapolation
    for (int k = -2; k <= g.nz + 3; ++k)
        for (int j = -2; j <= g.ny + 3; ++j)
            for (int i = -2; i <= g.nx + 3; ++i) {
                if (wt[g.s4(i, j, k)] != 2) continue;
                uint32_t mask = 0;
                for (int q = 1; q < 19; ++q)
                    if (wt[g.s4(i + ex(q), j + ey(q), k + ez(q))] <= 0) mask |= 1u << q;
                const uint2 e = make_uint2(pack_xyz(i, j, k), mask);
                lphi.push_back(e);
                if (i >= 0 && i <= g.nx + 1 && j >= 0 && j <= g.ny + 1 && k >= 0 && k <= g.nz + 1) ++ncn;
            }
    int rc;
    if ((rc = order_fluid_list(c, nodes, nullptr)) != MFLBM_OK) return rc;
    // the nodes whose normal the step may need: walls_type <= 0 on
    // [-1, n+2]^3 (their count bounds the sparse lists)
    d.n_norm = 0;
    for (int k = -1; k <= g.nz + 2; ++k)
        for (int j = -1; j <= g.ny + 2; ++j)
            for (int i = -1; i <= g.nx + 2; ++i)
                if (wt[g.s4(i, j, k)] <= 0) ++d.n_norm;
    {
        // row masks over the s4 lattice (row (y, z), byte b: x = 8b .. 8b + 7):
        // the fluid nodes of [1, n]^3 (super-block codes) and the nodes whose
        // normal may be non-zero (walls_type <= 0 on [-1, n+2]^3)
        const int NY4 = g.ny + 8, NZ4 = g.nz + 8;
        std::vector<uint8_t> fm((size_t)d.SX * NY4 * NZ4, 0), cm(fm.size(), 0);
        auto at = [&](int i, int j, int k) { return (size_t)((i + 3) >> 3) + (size_t)d.SX * ((j + 3) + (size_t)NY4 * (k + 3)); };
        for (int k = -1; k <= g.nz + 2; ++k)
            for (int j = -1; j <= g.ny + 2; ++j)
                for (int i = -1; i <= g.nx + 2; ++i) {
                    const uint8_t bit = (uint8_t)(1u << ((i + 3) & 7));
                    if (wt[g.s4(i, j, k)] <= 0) cm[at(i, j, k)] |= bit;
                    if (i >= 1 && i <= g.nx && j >= 1 && j <= g.ny && k >= 1 && k <= g.nz && walls[g.s2(i, j, k)] == 0)
                        fm[at(i, j, k)] |= bit;
                }
        ll nfm = 0;
        if ((rc = upload_list(&d.fmask, &nfm, fm)) != MFLBM_OK) return rc;
        if ((rc = upload_list(&d.cmask, &nfm, cm)) != MFLBM_OK) return rc;
    }
    {
        // solid boundary nodes grouped by super-block (4 x 4 x 4 phi bricks),
        // in scan order within each
        const int nsb = d.SX * d.SY * d.SZ;
        auto sb_of = [&](uint32_t p) {
            int x, y, z;
            unpack_xyz(p, x, y, z);
            return ((x + 3) >> 3) + d.SX * (((y + 3) >> 3) + d.SY * ((z + 3) >> 3));
        };
        std::stable_sort(lphi.begin(), lphi.end(), [&](const uint2& u, const uint2& v) { return sb_of(u.x) < sb_of(v.x); });
        std::vector<int> off(nsb + 1, 0);
        for (const uint2& e : lphi) off[sb_of(e.x) + 1]++;
        for (int b = 0; b < nsb; ++b) off[b + 1] += off[b];
        ll noff = 0;
        if ((rc = upload_list(&d.phioff, &noff, off)) != MFLBM_OK) return rc;
    }
    if ((rc = upload_list(&d.list_phi_ext, &d.n_phi_ext, lphi)) != MFLBM_OK) return rc;
    d.n_cn_ext = ncn;
    {
        // per fluid node of [-1, n+2]^3: its neighbours whose normal record
        // the solid-normal extrapolation writes (walls_type 2 on [0, n+1]^3),
        // for the tags of the normal pass
        std::vector<uint32_t> nb(g.n2(), 0u);
        for (int k = -1; k <= g.nz + 2; ++k)
            for (int j = -1; j <= g.ny + 2; ++j)
                for (int i = -1; i <= g.nx + 2; ++i) {
                    if (wt[g.s4(i, j, k)] > 0) continue;
                    uint32_t m = 0;
                    for (int q = 1; q < 19; ++q) {
                        const int x = i + ex(q), y = j + ey(q), z = k + ez(q);
                        if (x >= 0 && x <= g.nx + 1 && y >= 0 && y <= g.ny + 1 && z >= 0 && z <= g.nz + 1 &&
                            wt[g.s4(x, y, z)] == 2)
                            m |= 1u << q;
                    }
                    nb[g.s2(i, j, k)] = m;
                }
        ll nnb = 0;
        if ((rc = upload_list(&d.snb, &nnb, nb)) != MFLBM_OK) return rc;
    }
    {
        // lists of the sparse gradient passes (all records start as zero records)
        int dev = 0;
        MFLBM_CUDA(cudaGetDevice(&dev));
        MFLBM_CUDA(cudaDeviceGetAttribute(&d.n_sm, cudaDevAttrMultiProcessorCount, dev));
        for (void** p : {(void**)&d.olist, (void**)&d.nlist, (void**)&d.gcount}) {
            if (*p) cudaFree(*p);
            *p = nullptr;
        }
        MFLBM_CUDA(cudaMalloc(&d.olist, sizeof(uint32_t) * std::max<ll>(1, d.n_norm)));
        MFLBM_CUDA(cudaMalloc(&d.nlist, sizeof(uint32_t) * std::max<ll>(1, d.n_norm)));
        MFLBM_CUDA(cudaMalloc(&d.gcount, 8 * sizeof(int)));
        MFLBM_CUDA(cudaMemset(d.gcount, 0, 8 * sizeof(int)));
    }
    if (d.phi_prev) cudaFree(d.phi_prev);
    d.phi_prev = nullptr;
    if (d.aux) cudaFree(d.aux);
    d.aux = nullptr;
    const size_t rec = (c->params.precision == MFLBM_FP32 ? 4 : 8) * 4;
    MFLBM_CUDA(cudaMalloc(&d.aux, rec * std::max<ll>(1, d.n_fluid)));
    MFLBM_CUDA(cudaMemset(d.aux, 0, rec * std::max<ll>(1, d.n_fluid)));
    // solid nodes keep a zero normal record (only fluid nodes are rewritten per step)
    MFLBM_CUDA(cudaMemset(d.cnv4, 0, rec * g.n2()));
    MFLBM_CUDA(cudaMemset(d.iface, 0, g.n2()));
    MFLBM_CUDA(cudaMemset(d.touch, 0, g.n2()));
    c->pair_graph_odd_first = -1;  // kernels are launched with the list sizes
    c->generation++;
    return request_full_pass(c);
}

int ensure_staging(mflbm_context* c) {
    if (c->d.staging) return MFLBM_OK;
    const size_t bytes = (c->params.precision == MFLBM_FP32 ? 4 : 8) * c->d.g.n1() * 38;
    MFLBM_CUDA(cudaMalloc(&c->d.staging, bytes));
    return MFLBM_OK;
}

int flavour_collide(mflbm_context* c, bool odd) {
    return c->params.fp_mode == MFLBM_STRICT ? strict::collide(*c, odd) : fast::collide(*c, odd);
}
int flavour_boundaries(mflbm_context* c, bool odd) {
    return c->params.fp_mode == MFLBM_STRICT ? strict::boundaries(*c, odd) : fast::boundaries(*c, odd);
}
int flavour_gradient(mflbm_context* c) {
    c->d.arrays_stale = true;
    return c->params.fp_mode == MFLBM_STRICT ? strict::gradient(*c) : fast::gradient(*c);
}

// Materialise the reference-layout cn_x/y/z, c_norm and curv arrays from the
// per-node records (only needed when the host reads them).
int export_arrays(mflbm_context* c) {
    if (!c->d.arrays_stale) return MFLBM_OK;
    int rc = c->params.fp_mode == MFLBM_STRICT ? strict::export_arrays(*c) : fast::export_arrays(*c);
    if (rc == MFLBM_OK) c->d.arrays_stale = false;
    return rc;
}

TimingPool& timing_pool(mflbm_context* c) {
    static thread_local std::vector<std::pair<mflbm_context*, TimingPool*>> pools;
    for (auto& p : pools) if (p.first == c) return *p.second;
    pools.emplace_back(c, new TimingPool());
    return *pools.back().second;
}

cudaEvent_t next_event(mflbm_context* c) {
    TimingPool& tp = timing_pool(c);
    if (tp.used == tp.ev.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        tp.ev.push_back(e);
    }
    return tp.ev[tp.used++];
}

int one_step(mflbm_context* c, int ntime) {
    const bool odd = (ntime % 2) != 0;
    int rc;
    if (c->timing) cudaEventRecord(next_event(c), c->stream);
    if ((rc = flavour_collide(c, odd)) != MFLBM_OK) return rc;
    if (c->timing) cudaEventRecord(next_event(c), c->stream);
    if ((rc = flavour_boundaries(c, odd)) != MFLBM_OK) return rc;
    if (c->timing) cudaEventRecord(next_event(c), c->stream);
    if ((rc = flavour_gradient(c)) != MFLBM_OK) return rc;
    if (c->timing) cudaEventRecord(next_event(c), c->stream);
    return MFLBM_OK;
}

int require_ready(mflbm_context* c) {
    if (!c) return fail(MFLBM_E_ARG, "null context");
    if (!c->have_geometry) return fail(MFLBM_E_STATE, "geometry not set (mflbm_preprocess_geometry / mflbm_upload_geometry)");
    if (!c->have_fields) return fail(MFLBM_E_STATE, "fields not set (mflbm_init_fields / mflbm_upload_fields)");
    return MFLBM_OK;
}

int capture_pair(mflbm_context* c, int first_ntime) {
    if (c->pair_graph) {
        cudaGraphExecDestroy(c->pair_graph);
        c->pair_graph = nullptr;
    }
    cudaGraph_t graph;
    // a captured pair runs two gradient passes, so the live-count parity is
    // back where it started after the capture; a failed capture runs nothing
    const int parity = c->d.grad_parity;
    MFLBM_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = one_step(c, first_ntime);
    if (rc == MFLBM_OK) rc = one_step(c, first_ntime + 1);
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (rc != MFLBM_OK || e != cudaSuccess) c->d.grad_parity = parity;
    if (rc != MFLBM_OK) { if (e == cudaSuccess) cudaGraphDestroy(graph); return rc; }
    if (e != cudaSuccess) return fail(MFLBM_E_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&c->pair_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(MFLBM_E_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    c->pair_graph_odd_first = first_ntime & 1;
    return MFLBM_OK;
}

}  // namespace
}  // namespace mflbm

using namespace mflbm;

struct mflbm_batch {
    std::vector<mflbm_context*> ctx;
    std::vector<unsigned long long> gen;  // generations at capture
    cudaStream_t origin = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraphExec_t exec = nullptr;
    // persistent launch
    int mode = MFLBM_BATCH_AUTO, block = 128;
    double wait_s = 2.0;
    int used_mode = 0, grid = 0;
    void* dev_samples = nullptr;
    size_t samples_cap = 0;
    int* dev_pre = nullptr;
    size_t pre_cap = 0;
    unsigned* dev_bar = nullptr;   // [arrivals, generation]
    int* dev_err = nullptr;        // [timeout flag, second-component flag]
};

namespace mflbm {
namespace {

// One graph: fork from the batch stream to every context's stream, an odd and
// an even step on each, join back.
int capture_batch(mflbm_batch* b) {
    if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
    cudaGraph_t graph;
    std::vector<int> parity(b->ctx.size());   // restored if the capture fails (capture_pair)
    for (size_t i = 0; i < b->ctx.size(); ++i) parity[i] = b->ctx[i]->d.grad_parity;
    MFLBM_CUDA(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal));
    int rc = MFLBM_OK;
    cudaError_t e = cudaEventRecord(b->fork, b->origin);
    for (size_t i = 0; i < b->ctx.size() && rc == MFLBM_OK && e == cudaSuccess; ++i) {
        mflbm_context* c = b->ctx[i];
        e = cudaStreamWaitEvent(c->stream, b->fork, 0);
        if (e != cudaSuccess) break;
        if ((rc = one_step(c, 1)) != MFLBM_OK) break;
        if ((rc = one_step(c, 2)) != MFLBM_OK) break;
        if ((e = cudaEventRecord(b->join[i], c->stream)) != cudaSuccess) break;
        e = cudaStreamWaitEvent(b->origin, b->join[i], 0);
    }
    const cudaError_t e2 = cudaStreamEndCapture(b->origin, &graph);
    if (rc != MFLBM_OK || e != cudaSuccess || e2 != cudaSuccess)
        for (size_t i = 0; i < b->ctx.size(); ++i) b->ctx[i]->d.grad_parity = parity[i];
    if (rc != MFLBM_OK) { if (e2 == cudaSuccess) cudaGraphDestroy(graph); return rc; }
    if (e != cudaSuccess) { if (e2 == cudaSuccess) cudaGraphDestroy(graph); return fail(MFLBM_E_CUDA, std::string("batch capture: ") + cudaGetErrorString(e)); }
    if (e2 != cudaSuccess) return fail(MFLBM_E_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e2));
    e = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(MFLBM_E_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    for (size_t i = 0; i < b->ctx.size(); ++i) b->gen[i] = b->ctx[i]->generation;
    return MFLBM_OK;
}

int set_tiling(mflbm_context* c, int lx, int ly, int lz);

// Everything a step writes (populations, phi, records, convective buffers,
// sparse-set lists), copied aside in the context's current tile shape.
struct SavedState {
    char* buf = nullptr;
    int lx = 0, ly = 0, lz = 0;
    bool stale = false;
};
struct Span { void* p; size_t n; };
std::vector<Span> state_spans(mflbm_context* c) {
    DeviceState& d = c->d;
    const Grid& g = d.g;
    const size_t T = tsize(c), pl = (size_t)g.plane1();
    const size_t pop_e = c->params.storage == MFLBM_STORE_NATIVE ? T : 2;
    return std::vector<Span>{{d.pdf, pop_e * d.b.S * 38}, {d.phi, T * g.n4()},
                             {d.aux, T * 4 * std::max<ll>(1, d.n_fluid)}, {d.cnv4, T * 4 * g.n2()},
                             {d.f_cv, T * pl * 19}, {d.g_cv, T * pl * 19}, {d.phi_cv, T * pl},
                             {d.dither, 2 * sizeof(uint32_t)}, {d.iface, (size_t)g.n2()},
                             {d.olist, sizeof(uint32_t) * std::max<ll>(1, d.n_norm)},
                             {d.gcount, 8 * sizeof(int)}};
}
int save_state(mflbm_context* c, SavedState* s) {
    const std::vector<Span> st = state_spans(c);
    size_t total = 0;
    for (auto& x : st) total += (x.n + 255) / 256 * 256;
    MFLBM_CUDA(cudaMalloc(&s->buf, total));
    size_t off = 0;
    for (auto& x : st) {
        MFLBM_CUDA(cudaMemcpyAsync(s->buf + off, x.p, x.n, cudaMemcpyDeviceToDevice, c->stream));
        off += (x.n + 255) / 256 * 256;
    }
    s->lx = c->d.b.lx; s->ly = c->d.b.ly; s->lz = c->d.b.lz;
    s->stale = c->d.arrays_stale;
    MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    return MFLBM_OK;
}
// Back to the saved tile shape and state; frees the copy.
int restore_state(mflbm_context* c, SavedState* s) {
    int rc = set_tiling(c, s->lx, s->ly, s->lz);
    if (rc == MFLBM_OK) {
        const std::vector<Span> st = state_spans(c);
        size_t off = 0;
        for (auto& x : st) {
            cudaMemcpyAsync(x.p, s->buf + off, x.n, cudaMemcpyDeviceToDevice, c->stream);
            off += (x.n + 255) / 256 * 256;
        }
        MFLBM_CUDA(cudaStreamSynchronize(c->stream));
        c->d.arrays_stale = s->stale;
        rc = request_full_pass(c);
    }
    cudaFree(s->buf);
    s->buf = nullptr;
    if (c->pair_graph) { cudaGraphExecDestroy(c->pair_graph); c->pair_graph = nullptr; }
    c->generation++;
    return rc;
}

// Whether a batch can run as one persistent launch (batch.cuh): the same
// precision, storage and flavour everywhere, 32-bit population indices, no
// inlet, outlet or plate, no interface records, and every component-2
// population exactly 0.  `why` receives the first reason it cannot.
int batch_persistent_ok(mflbm_batch* b, bool* ok, std::string* why) {
    *ok = false;
    const mflbm_context* c0 = b->ctx[0];
    for (mflbm_context* c : b->ctx) {
        const mflbm_params& p = c->params;
        if (p.precision != c0->params.precision || p.storage != c0->params.storage || p.fp_mode != c0->params.fp_mode) {
            *why = "contexts differ in precision, storage or arithmetic flavour";
            return MFLBM_OK;
        }
        if (p.kper == 0 && p.domain_wall_status_z_min == 0 && p.domain_wall_status_z_max == 0 &&
            (p.inlet_BC != 0 || p.outlet_BC != 0)) {
            *why = "a context has an inlet or outlet boundary";
            return MFLBM_OK;
        }
        if (p.porous_plate_cmd != 0) { *why = "a context has a porous plate"; return MFLBM_OK; }
        if (c->d.b.pairs() >= (1ll << 32)) { *why = "a context needs 64-bit population indices"; return MFLBM_OK; }
    }
    MFLBM_CUDA(cudaMemsetAsync(b->dev_err + 1, 0, sizeof(int), b->origin));
    MFLBM_CUDA(cudaStreamSynchronize(b->origin));
    for (mflbm_context* c : b->ctx) {
        int h[3] = {0, 0, 0};
        MFLBM_CUDA(cudaMemcpy(h, c->d.gcount, sizeof(h), cudaMemcpyDeviceToHost));
        if (h[0] != 0 || h[1] != 0) { *why = "a context has interface records (two phases)"; return MFLBM_OK; }
        const int rc = c->params.fp_mode == MFLBM_STRICT ? strict::second_component(*c, b->dev_err + 1)
                                                         : fast::second_component(*c, b->dev_err + 1);
        if (rc != MFLBM_OK) return rc;
        MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    }
    int flag = 0;
    MFLBM_CUDA(cudaMemcpy(&flag, b->dev_err + 1, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) { *why = "a context holds the second component"; return MFLBM_OK; }
    *ok = true;
    return MFLBM_OK;
}

// ntime_begin .. ntime_begin + nsteps - 1 of every context as persistent
// launches of at most 100 steps.
int batch_run_persistent(mflbm_batch* b, int ntime_begin, int nsteps) {
    const int ns = (int)b->ctx.size(), bs = b->block;
    // phase 0: collision units of bs list entries; phase 1: periodic exchange items
    std::vector<int> pre(2 * (ns + 1), 0);
    int max_units = 1;
    for (int ph = 0; ph < 2; ++ph) {
        for (int i = 0; i < ns; ++i) {
            const mflbm_context& c = *b->ctx[i];
            const Grid& g = c.d.g;
            const ll items = ph == 0 ? c.d.n_fluid
                                     : (ll)(c.params.kper ? g.nx * g.ny : 0) + (c.params.jper ? g.nx * g.nz : 0) +
                                           (c.params.jper && c.params.kper ? g.nx : 0);
            pre[ph * (ns + 1) + i + 1] = pre[ph * (ns + 1) + i] + (int)((items + bs - 1) / bs);
        }
        max_units = std::max(max_units, pre[ph * (ns + 1) + ns]);
    }
    if (b->pre_cap < pre.size()) {
        if (b->dev_pre) cudaFree(b->dev_pre);
        b->dev_pre = nullptr;
        b->pre_cap = 0;
        MFLBM_CUDA(cudaMalloc(&b->dev_pre, sizeof(int) * pre.size()));
        b->pre_cap = pre.size();
    }
    MFLBM_CUDA(cudaMemcpyAsync(b->dev_pre, pre.data(), sizeof(int) * pre.size(), cudaMemcpyHostToDevice, b->origin));
    const mflbm_context& c0 = *b->ctx[0];
    const bool strict_mode = c0.params.fp_mode == MFLBM_STRICT;
    const size_t need = (strict_mode ? strict::batch_sample_bytes(c0) : fast::batch_sample_bytes(c0)) * ns;
    if (b->samples_cap < need) {
        if (b->dev_samples) cudaFree(b->dev_samples);
        b->dev_samples = nullptr;
        b->samples_cap = 0;
        MFLBM_CUDA(cudaMalloc(&b->dev_samples, need));
        b->samples_cap = need;
    }
    int grid = 0;
    int rc = strict_mode ? strict::batch_grid(c0, bs, &grid) : fast::batch_grid(c0, bs, &grid);
    if (rc != MFLBM_OK) return rc;
    grid = std::min(grid, max_units);
    BatchLaunch L;
    L.samples = b->dev_samples;
    L.pre = b->dev_pre;
    L.bar = b->dev_bar;
    L.error = b->dev_err;
    L.limit_ns = (unsigned long long)(b->wait_s * 1e9);
    L.block = bs;
    L.grid = grid;
    L.stream = b->origin;
    for (int done = 0; done < nsteps;) {
        const int chunk = std::min(100, nsteps - done);
        L.ntime_begin = ntime_begin + done;
        L.nsteps = chunk;
        MFLBM_CUDA(cudaMemsetAsync(b->dev_bar, 0, 2 * sizeof(unsigned), b->origin));
        MFLBM_CUDA(cudaMemsetAsync(b->dev_err, 0, sizeof(int), b->origin));
        rc = strict_mode ? strict::batch_persistent(b->ctx.data(), ns, L) : fast::batch_persistent(b->ctx.data(), ns, L);
        if (rc != MFLBM_OK) return rc;
        int err = 0;
        MFLBM_CUDA(cudaMemcpy(&err, b->dev_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) return fail(MFLBM_E_TIMEOUT, "mflbm_batch_run: a grid-barrier wait of the persistent launch ran out after " +
                                                  std::to_string(b->wait_s) + " s; the contexts' states are undefined");
        done += chunk;
    }
    b->grid = grid;
    for (mflbm_context* c : b->ctx) {
        c->d.arrays_stale = true;
        if ((rc = request_full_pass(c)) != MFLBM_OK) return rc;
    }
    return MFLBM_OK;
}

int check_block(int v) { return v == 0 || v == 64 || v == 128 || v == 256; }

// log2 of a tile extent (a power of two, 1 .. max); false otherwise
bool tile_shift(int extent, int max, int* out) {
    for (int l = 0; (1 << l) <= max; ++l)
        if (extent == (1 << l)) { *out = l; return true; }
    return false;
}
bool tile_shifts(int tx, int ty, int tz, int* lx, int* ly, int* lz) {
    return tile_shift(tx, 32, lx) && tile_shift(ty, 32, ly) && tile_shift(tz, 2, lz);
}

void fill_tuning(const mflbm_context& c, mflbm_tuning* out) {
    const Tuning& t = c.d.tune;
    out->collide_block = t.collide; out->normals_block = t.normals;
    out->curvature_block = t.curvature; out->extrapolate_block = t.extrapolate;
    out->tile_x = 1 << c.d.b.lx; out->tile_y = 1 << c.d.b.ly; out->tile_z = 1 << c.d.b.lz;
}

// Switch the population layout to tiles of 2^lx x 2^ly x 2^lz bricks.  The
// populations move element by element and the collision records follow the
// fluid list's new order, so the state, and every later step, is unchanged
// (bit for bit).
int set_tiling(mflbm_context* c, int lx, int ly, int lz) {
    DeviceState& d = c->d;
    if (lx == d.b.lx && ly == d.b.ly && lz == d.b.lz) return MFLBM_OK;
    const Bricks to = make_bricks(d.g.nx, d.g.ny, d.g.nz, lx, ly, lz);
    void* pdf = nullptr;
    int rc = relayout_populations(*c, to, &pdf);
    if (rc != MFLBM_OK) return rc;
    MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    cudaFree(d.pdf);
    d.pdf = pdf;
    d.b = to;
    if (d.fluid_list && d.n_fluid > 0) {
        std::vector<uint32_t> nodes((size_t)d.n_fluid);
        MFLBM_CUDA(cudaMemcpy(nodes.data(), d.fluid_list, sizeof(uint32_t) * nodes.size(), cudaMemcpyDeviceToHost));
        std::vector<int> perm;
        if ((rc = order_fluid_list(c, nodes, &perm)) != MFLBM_OK) return rc;
        int* perm_dev = nullptr;
        MFLBM_CUDA(cudaMalloc(&perm_dev, sizeof(int) * perm.size()));
        MFLBM_CUDA(cudaMemcpy(perm_dev, perm.data(), sizeof(int) * perm.size(), cudaMemcpyHostToDevice));
        void* aux = nullptr;
        rc = permute_records(*c, perm_dev, &aux);
        cudaStreamSynchronize(c->stream);
        cudaFree(perm_dev);
        if (rc != MFLBM_OK) return rc;
        cudaFree(d.aux);
        d.aux = aux;
    }
    if (c->pair_graph) { cudaGraphExecDestroy(c->pair_graph); c->pair_graph = nullptr; }
    c->pair_graph_odd_first = -1;
    c->generation++;
    return MFLBM_OK;
}

}  // namespace
}  // namespace mflbm

extern "C" {

int mflbm_abi_version(void) { return MFLBM_ABI_VERSION; }
const char* mflbm_last_error(void) { return g_last_error.c_str(); }
unsigned long long mflbm_kernel_launch_count(void) { return g_launches.load(); }

int mflbm_create(const mflbm_params* params, mflbm_context** out) {
    if (!out) return fail(MFLBM_E_ARG, "mflbm_create: null output pointer");
    *out = nullptr;
    int rc = check_params(params);
    if (rc != MFLBM_OK) return rc;
    mflbm_context* c = new mflbm_context();
    c->params = *params;
    DeviceState& d = c->d;
    d.g = Grid{(int)params->nx, (int)params->ny, (int)params->nz};
    d.b = make_bricks(d.g.nx, d.g.ny, d.g.nz);
    d.precision = params->precision;
    const Grid& g = d.g;
    const size_t T = tsize(c);
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return fail(MFLBM_E_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e)); }
    // super-blocks of 4 x 4 x 4 phi bricks over the s4 lattice
    d.SX = ((g.nx + 9) / 2 + 3) / 4;
    d.SY = ((g.ny + 9) / 2 + 3) / 4;
    d.SZ = ((g.nz + 9) / 2 + 3) / 4;
    const size_t nsb = (size_t)d.SX * d.SY * d.SZ;
    struct { void** p; size_t bytes; } allocs[] = {
        {&d.pdf, (params->storage == MFLBM_STORE_NATIVE ? T : 2) * d.b.S * 38}, {&d.cnv4, T * 4 * g.n2()},
        {(void**)&d.type8, (size_t)g.n4()},
        {&d.phi, T * g.n4()}, {&d.cn_x, T * g.n2()}, {&d.cn_y, T * g.n2()},
        {&d.cn_z, T * g.n2()}, {&d.c_norm, T * g.n2()}, {&d.curv, T * g.n1()}, {&d.W_in, T * g.plane1()},
        {&d.f_cv, T * g.plane1() * 19}, {&d.g_cv, T * g.plane1() * 19}, {&d.phi_cv, T * g.plane1()},
        {(void**)&d.walls, sizeof(int32_t) * g.n2()}, {(void**)&d.walls_type, sizeof(int32_t) * g.n4()},
        {&d.s_nx, T * g.n4()}, {&d.s_ny, T * g.n4()}, {&d.s_nz, T * g.n4()},
        {(void**)&d.dither, 2 * sizeof(uint32_t)}, {(void**)&d.iface, (size_t)g.n2()}, {(void**)&d.touch, (size_t)g.n2()},
        {(void**)&d.pmask, sizeof(uint16_t) * (size_t)d.SX * (g.ny + 8) * (g.nz + 8)},
        {(void**)&d.sbcode, nsb}, {(void**)&d.sbact, nsb}, {(void**)&d.sblive, sizeof(uint32_t) * nsb},
        {(void**)&d.sbinfo, 4 * sizeof(int)}};
    for (auto& a : allocs) {
        if ((rc = alloc_zero(a.p, a.bytes, c->stream)) != MFLBM_OK) {
            free_all(c);
            cudaStreamDestroy(c->stream);
            delete c;
            return rc == MFLBM_E_CUDA ? MFLBM_E_NOMEM : rc;
        }
    }
    if ((rc = request_full_pass(c)) != MFLBM_OK) { free_all(c); cudaStreamDestroy(c->stream); delete c; return rc; }
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { free_all(c); cudaStreamDestroy(c->stream); delete c; return fail(MFLBM_E_CUDA, cudaGetErrorString(e)); }
    *out = c;
    return MFLBM_OK;
}

int mflbm_destroy(mflbm_context* c) {
    if (!c) return MFLBM_OK;
    cudaStreamSynchronize(c->stream);
    free_all(c);
    TimingPool& tp = timing_pool(c);
    for (auto e : tp.ev) cudaEventDestroy(e);
    tp.ev.clear();
    tp.used = 0;
    cudaStreamDestroy(c->stream);
    delete c;
    return MFLBM_OK;
}

int mflbm_set_params(mflbm_context* c, const mflbm_params* p) {
    if (!c) return fail(MFLBM_E_ARG, "null context");
    int rc = check_params(p);
    if (rc != MFLBM_OK) return rc;
    if (p->nx != c->params.nx || p->ny != c->params.ny || p->nz != c->params.nz || p->precision != c->params.precision ||
        p->storage != c->params.storage)
        return fail(MFLBM_E_ARG, "mflbm_set_params cannot change the lattice size, precision or storage");
    c->params = *p;
    if (c->pair_graph) { cudaGraphExecDestroy(c->pair_graph); c->pair_graph = nullptr; }
    c->generation++;
    return MFLBM_OK;
}

int mflbm_get_params(mflbm_context* c, mflbm_params* out) {
    if (!c || !out) return fail(MFLBM_E_ARG, "mflbm_get_params: null argument");
    *out = c->params;
    return MFLBM_OK;
}

int mflbm_preprocess_geometry(mflbm_context* c, const int32_t* walls_global, int32_t* walls, int32_t* walls_type,
                              void* s_nx, void* s_ny, void* s_nz, mflbm_geometry_counts* counts) {
    if (!c || !walls_global) return fail(MFLBM_E_ARG, "mflbm_preprocess_geometry: null argument");
    int rc = preprocess_geometry(*c, walls_global, 0);
    if (rc != MFLBM_OK) return rc;
    if ((rc = build_lists(c)) != MFLBM_OK) return rc;
    c->have_geometry = true;
    const Grid& g = c->d.g;
    const size_t T = tsize(c);
    if (walls) MFLBM_CUDA(cudaMemcpy(walls, c->d.walls, sizeof(int32_t) * g.n2(), cudaMemcpyDeviceToHost));
    if (walls_type) MFLBM_CUDA(cudaMemcpy(walls_type, c->d.walls_type, sizeof(int32_t) * g.n4(), cudaMemcpyDeviceToHost));
    if (s_nx) MFLBM_CUDA(cudaMemcpy(s_nx, c->d.s_nx, T * g.n4(), cudaMemcpyDeviceToHost));
    if (s_ny) MFLBM_CUDA(cudaMemcpy(s_ny, c->d.s_ny, T * g.n4(), cudaMemcpyDeviceToHost));
    if (s_nz) MFLBM_CUDA(cudaMemcpy(s_nz, c->d.s_nz, T * g.n4(), cudaMemcpyDeviceToHost));
    if (counts) {
        std::vector<int32_t> wt(g.n4()), w(g.n2());
        MFLBM_CUDA(cudaMemcpy(wt.data(), c->d.walls_type, sizeof(int32_t) * g.n4(), cudaMemcpyDeviceToHost));
        MFLBM_CUDA(cudaMemcpy(w.data(), c->d.walls, sizeof(int32_t) * g.n2(), cudaMemcpyDeviceToHost));
        *counts = mflbm_geometry_counts{};
        for (int k = -3; k <= g.nz + 4; ++k)
            for (int j = -3; j <= g.ny + 4; ++j)
                for (int i = -3; i <= g.nx + 4; ++i) {
                    const int v = wt[g.s4(i, j, k)];
                    const bool in3 = i >= -2 && i <= g.nx + 3 && j >= -2 && j <= g.ny + 3 && k >= -2 && k <= g.nz + 3;
                    if (v == 2) { counts->num_solid_boundary_global++; if (in3) counts->num_solid_boundary++; }
                    if (v == -1) { counts->num_fluid_boundary_global++; if (in3) counts->num_fluid_boundary++; }
                }
        counts->pore_sum = c->d.n_fluid;
    }
    return MFLBM_OK;
}

int mflbm_upload_geometry(mflbm_context* c, const int32_t* walls, const int32_t* walls_type, const void* s_nx,
                          const void* s_ny, const void* s_nz) {
    if (!c || !walls || !walls_type || !s_nx || !s_ny || !s_nz) return fail(MFLBM_E_ARG, "mflbm_upload_geometry: null argument");
    const Grid& g = c->d.g;
    const size_t T = tsize(c);
    MFLBM_CUDA(cudaMemcpy(c->d.walls, walls, sizeof(int32_t) * g.n2(), cudaMemcpyHostToDevice));
    MFLBM_CUDA(cudaMemcpy(c->d.walls_type, walls_type, sizeof(int32_t) * g.n4(), cudaMemcpyHostToDevice));
    MFLBM_CUDA(cudaMemcpy(c->d.s_nx, s_nx, T * g.n4(), cudaMemcpyHostToDevice));
    MFLBM_CUDA(cudaMemcpy(c->d.s_ny, s_ny, T * g.n4(), cudaMemcpyHostToDevice));
    MFLBM_CUDA(cudaMemcpy(c->d.s_nz, s_nz, T * g.n4(), cudaMemcpyHostToDevice));
    std::vector<int8_t> t8(g.n4());
    for (ll n = 0; n < g.n4(); ++n) t8[n] = (int8_t)walls_type[n];
    MFLBM_CUDA(cudaMemcpy(c->d.type8, t8.data(), g.n4(), cudaMemcpyHostToDevice));
    int rc = build_lists(c);
    if (rc != MFLBM_OK) return rc;
    c->have_geometry = true;
    return MFLBM_OK;
}

int mflbm_init_fields(mflbm_context* c, int option, double interface_z0, const void* W_in) {
    if (!c) return fail(MFLBM_E_ARG, "null context");
    if (!c->have_geometry) return fail(MFLBM_E_STATE, "geometry must be set before mflbm_init_fields");
    if (option < 1 || option > 5) return fail(MFLBM_E_ARG, "initial_fluid_distribution_option must be 1-5");
    const Grid& g = c->d.g;
    if (W_in) MFLBM_CUDA(cudaMemcpyAsync(c->d.W_in, W_in, tsize(c) * g.plane1(), cudaMemcpyHostToDevice, c->stream));
    int rc = init_fields(*c, option, interface_z0);
    if (rc != MFLBM_OK) return rc;
    if ((rc = request_full_pass(c)) != MFLBM_OK) return rc;
    if ((rc = flavour_gradient(c)) != MFLBM_OK) return rc;
    MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    c->have_fields = true;
    return MFLBM_OK;
}

static int init_flow_entry(mflbm_context* c, const void* rho, const void* u, const void* v, const void* w, int mrt) {
    if (!c) return fail(MFLBM_E_ARG, "null context");
    if (!c->have_fields) return fail(MFLBM_E_STATE, "mflbm_init_flow needs phi (mflbm_init_fields or mflbm_upload_fields first)");
    const Grid& g = c->d.g;
    const size_t T = tsize(c), n = T * g.n1();
    int rc = ensure_staging(c);
    if (rc != MFLBM_OK) return rc;
    const void* host[4] = {rho, u, v, w};
    const void* dev[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int a = 0; a < 4; ++a) {
        if (!host[a]) continue;
        void* dst = (char*)c->d.staging + a * n;
        MFLBM_CUDA(cudaMemcpyAsync(dst, host[a], n, cudaMemcpyHostToDevice, c->stream));
        dev[a] = dst;
    }
    if ((rc = init_flow(*c, dev[0], dev[1], dev[2], dev[3], mrt)) != MFLBM_OK) return rc;
    MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    c->d.arrays_stale = true;
    return request_full_pass(c);
}

int mflbm_init_flow_predicted(mflbm_context* c, const float* y, double nu, double g, const float* scales, int mrt) {
    if (!c || !y || !scales) return fail(MFLBM_E_ARG, "mflbm_init_flow_predicted: null argument");
    if (!c->have_fields)
        return fail(MFLBM_E_STATE, "mflbm_init_flow_predicted needs phi (mflbm_init_fields or mflbm_upload_fields first)");
    if (!(nu > 0) || !std::isfinite(g)) return fail(MFLBM_E_ARG, "mflbm_init_flow_predicted: nu must be > 0, g finite");
    const Grid& gr = c->d.g;
    int rc = ensure_staging(c);
    if (rc != MFLBM_OK) return rc;
    // the staging buffer (38 n1 values) holds the prediction (4 floats per
    // interior node) and, 256-byte aligned after it, the four fields
    const size_t ybytes = sizeof(float) * 4 * (size_t)gr.n0();
    float* ydev = (float*)c->d.staging;
    void* work = (char*)c->d.staging + ((ybytes + 255) / 256) * 256;
    MFLBM_CUDA(cudaMemcpyAsync(ydev, y, ybytes, cudaMemcpyHostToDevice, c->stream));
    if ((rc = init_flow_predicted(*c, ydev, nu, g, scales, mrt ? 1 : 0, work)) != MFLBM_OK) return rc;
    MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    c->d.arrays_stale = true;
    return request_full_pass(c);
}

int mflbm_init_flow(mflbm_context* c, const void* rho, const void* u, const void* v, const void* w) {
    return init_flow_entry(c, rho, u, v, w, 0);
}

int mflbm_init_flow_mrt(mflbm_context* c, const void* rho, const void* u, const void* v, const void* w) {
    return init_flow_entry(c, rho, u, v, w, 1);
}

// The device address of a page-locked host range [p, p + bytes) (allocated
// or registered with CUDA, so the device can read and write it over the host
// link), or nullptr for other memory.
void* device_view(const void* p, size_t bytes) {
    if (!p || !bytes) return nullptr;
    cudaPointerAttributes a, b;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess || a.type != cudaMemoryTypeHost || !a.devicePointer ||
        cudaPointerGetAttributes(&b, (const char*)p + bytes - 1) != cudaSuccess || b.type != cudaMemoryTypeHost ||
        (const char*)b.devicePointer - (const char*)a.devicePointer != (ptrdiff_t)(bytes - 1)) {
        cudaGetLastError();   // an unregistered pointer may leave an error behind
        return nullptr;
    }
    return a.devicePointer;
}

int mflbm_upload_fields(mflbm_context* c, const void* pdf, const void* phi, const void* cn_x, const void* cn_y,
                        const void* cn_z, const void* c_norm, const void* curv, const void* W_in,
                        const void* f_convec_bc, const void* g_convec_bc, const void* phi_convec_bc) {
    if (!c || !pdf || !phi) return fail(MFLBM_E_ARG, "mflbm_upload_fields: pdf and phi are required");
    if (!c->have_geometry) return fail(MFLBM_E_STATE, "geometry must be set before mflbm_upload_fields");
    DeviceState& d = c->d;
    const Grid& g = d.g;
    const size_t T = tsize(c);
    cudaStream_t s = c->stream;
    int rc = request_full_pass(c);
    if (rc != MFLBM_OK) return rc;
    // populations: page-locked host memory is read by the relayout kernel
    // directly over the host link (132 against 83 GB/s for a copy into the
    // staging buffer plus the relayout, measured); other memory goes through
    // the staging buffer
    if (void* dv = device_view(pdf, T * g.n1() * 38)) {
        if ((rc = convert_populations(*c, true, dv)) != MFLBM_OK) return rc;
    } else {
        if ((rc = ensure_staging(c)) != MFLBM_OK) return rc;
        MFLBM_CUDA(cudaMemcpyAsync(d.staging, pdf, T * g.n1() * 38, cudaMemcpyHostToDevice, s));
        if ((rc = convert_populations(*c, true)) != MFLBM_OK) return rc;
    }
    MFLBM_CUDA(cudaMemcpyAsync(d.phi, phi, T * g.n4(), cudaMemcpyHostToDevice, s));
    if (W_in) MFLBM_CUDA(cudaMemcpyAsync(d.W_in, W_in, T * g.plane1(), cudaMemcpyHostToDevice, s));
    const bool have_grad = cn_x && cn_y && cn_z && c_norm && curv;
    if (f_convec_bc) MFLBM_CUDA(cudaMemcpyAsync(d.f_cv, f_convec_bc, T * g.plane1() * 19, cudaMemcpyHostToDevice, s));
    if (g_convec_bc) MFLBM_CUDA(cudaMemcpyAsync(d.g_cv, g_convec_bc, T * g.plane1() * 19, cudaMemcpyHostToDevice, s));
    if (phi_convec_bc) MFLBM_CUDA(cudaMemcpyAsync(d.phi_cv, phi_convec_bc, T * g.plane1(), cudaMemcpyHostToDevice, s));
    // the collision reads per-node records (n, 0.5*gamma*curv*c_norm): build
    // them from the uploaded arrays, or run the gradient pass when they are absent
    if (have_grad) {
        MFLBM_CUDA(cudaMemcpyAsync(d.cn_x, cn_x, T * g.n2(), cudaMemcpyHostToDevice, s));
        MFLBM_CUDA(cudaMemcpyAsync(d.cn_y, cn_y, T * g.n2(), cudaMemcpyHostToDevice, s));
        MFLBM_CUDA(cudaMemcpyAsync(d.cn_z, cn_z, T * g.n2(), cudaMemcpyHostToDevice, s));
        MFLBM_CUDA(cudaMemcpyAsync(d.c_norm, c_norm, T * g.n2(), cudaMemcpyHostToDevice, s));
        MFLBM_CUDA(cudaMemcpyAsync(d.curv, curv, T * g.n1(), cudaMemcpyHostToDevice, s));
        rc = c->params.fp_mode == MFLBM_STRICT ? strict::refresh_aux(*c) : fast::refresh_aux(*c);
        c->d.arrays_stale = false;
    } else {
        rc = flavour_gradient(c);
    }
    if (rc != MFLBM_OK) return rc;
    MFLBM_CUDA(cudaStreamSynchronize(s));
    c->have_fields = true;
    return MFLBM_OK;
}

int mflbm_download_fields(mflbm_context* c, void* pdf, void* phi, void* cn_x, void* cn_y, void* cn_z, void* c_norm,
                          void* curv, void* f_convec_bc, void* g_convec_bc, void* phi_convec_bc) {
    if (!c) return fail(MFLBM_E_ARG, "null context");
    DeviceState& d = c->d;
    const Grid& g = d.g;
    const size_t T = tsize(c);
    cudaStream_t s = c->stream;
    // populations: relayout into the staging buffer, then one copy (a copy
    // engine writes page-locked host memory faster than the relayout
    // kernel's stores over the host link: 168 against 132 GB/s measured)
    if (pdf) {
        int rc = ensure_staging(c);
        if (rc != MFLBM_OK) return rc;
        if ((rc = convert_populations(*c, false)) != MFLBM_OK) return rc;
    }
    if (cn_x || cn_y || cn_z || c_norm || curv) {
        int rc = export_arrays(c);
        if (rc != MFLBM_OK) return rc;
    }
    struct { void* dst; const void* src; size_t n; } cp[] = {
        {pdf, d.staging, T * g.n1() * 38}, {phi, d.phi, T * g.n4()}, {cn_x, d.cn_x, T * g.n2()}, {cn_y, d.cn_y, T * g.n2()},
        {cn_z, d.cn_z, T * g.n2()}, {c_norm, d.c_norm, T * g.n2()}, {curv, d.curv, T * g.n1()},
        {f_convec_bc, d.f_cv, T * g.plane1() * 19}, {g_convec_bc, d.g_cv, T * g.plane1() * 19},
        {phi_convec_bc, d.phi_cv, T * g.plane1()}};
    for (auto& x : cp)
        if (x.dst) MFLBM_CUDA(cudaMemcpyAsync(x.dst, x.src, x.n, cudaMemcpyDeviceToHost, s));
    MFLBM_CUDA(cudaStreamSynchronize(s));
    return MFLBM_OK;
}

int mflbm_step(mflbm_context* c, int ntime) {
    int rc = require_ready(c);
    if (rc != MFLBM_OK) return rc;
    return one_step(c, ntime);
}

int mflbm_run(mflbm_context* c, int ntime_begin, int nsteps) {
    int rc = require_ready(c);
    if (rc != MFLBM_OK) return rc;
    if (nsteps <= 0) return MFLBM_OK;
    if (c->timing || nsteps < 4) {
        for (int s = 0; s < nsteps; ++s)
            if ((rc = one_step(c, ntime_begin + s)) != MFLBM_OK) return rc;
        return MFLBM_OK;
    }
    int nt = ntime_begin, left = nsteps;
    c->d.arrays_stale = true;  // graph replays do not pass through the host-side gradient launch
    // the graph holds an (odd, even) pair
    if ((nt & 1) == 0) {
        if ((rc = one_step(c, nt)) != MFLBM_OK) return rc;
        ++nt; --left;
    }
    if (!c->pair_graph || c->pair_graph_odd_first != 1)
        if ((rc = capture_pair(c, nt)) != MFLBM_OK) return rc;
    while (left >= 2) {
        MFLBM_CUDA(cudaGraphLaunch(c->pair_graph, c->stream));
        nt += 2; left -= 2;
    }
    if (left == 1 && (rc = one_step(c, nt)) != MFLBM_OK) return rc;
    return MFLBM_OK;
}

int mflbm_synchronize(mflbm_context* c) {
    if (!c) return fail(MFLBM_E_ARG, "null context");
    MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    return MFLBM_OK;
}

int mflbm_interface_stats(mflbm_context* c, long long* interface_nodes, long long* solid_normals,
                          long long* active_nodes) {
    int rc = require_ready(c);
    if (rc != MFLBM_OK) return rc;
    int h[3] = {0, 0, 0};
    if (c->d.gcount) {
        MFLBM_CUDA(cudaMemcpyAsync(h, c->d.gcount, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
        MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    }
    if (interface_nodes) *interface_nodes = h[0];
    if (solid_normals) *solid_normals = h[1];
    if (active_nodes) *active_nodes = h[2];
    return MFLBM_OK;
}

int mflbm_super_block_stats(mflbm_context* c, long long* processed, long long* flagged, long long* total) {
    int rc = require_ready(c);
    if (rc != MFLBM_OK) return rc;
    const DeviceState& d = c->d;
    const size_t nsb = (size_t)d.SX * d.SY * d.SZ;
    int live[4] = {0, 0, 0, 0};
    std::vector<uint8_t> act(nsb);
    MFLBM_CUDA(cudaMemcpyAsync(live, d.sbinfo, sizeof(live), cudaMemcpyDeviceToHost, c->stream));
    MFLBM_CUDA(cudaMemcpyAsync(act.data(), d.sbact, nsb, cudaMemcpyDeviceToHost, c->stream));
    MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    // the last pass counted into the slot the next pass does not use
    if (processed) *processed = live[d.grad_parity ? 0 : 2];
    if (flagged) {
        long long n = 0;
        for (uint8_t v : act) n += v != 0;
        *flagged = n;
    }
    if (total) *total = (long long)nsb;
    return MFLBM_OK;
}

int mflbm_monitor_reduce(mflbm_context* c, int n_exclude_inlet, int n_exclude_outlet, mflbm_monitor* out) {
    int rc = require_ready(c);
    if (rc != MFLBM_OK) return rc;
    if (!out) return fail(MFLBM_E_ARG, "null output");
    if ((rc = export_arrays(c)) != MFLBM_OK) return rc;
    return monitor(*c, n_exclude_inlet, n_exclude_outlet, out);
}

int mflbm_monitor_reduce_noalloc(mflbm_context* c, int n_exclude_inlet, int n_exclude_outlet, mflbm_monitor* out) {
    int rc = require_ready(c);
    if (rc != MFLBM_OK) return rc;
    if (!out) return fail(MFLBM_E_ARG, "null output");
    if ((rc = export_arrays(c)) != MFLBM_OK) return rc;
    return monitor_noalloc(*c, n_exclude_inlet, n_exclude_outlet, out);
}

int mflbm_write_vtk(mflbm_context* c, int vtk_type, int output_fieldData_precision_cmd, const char* path) {
    int rc = require_ready(c);
    if (rc != MFLBM_OK) return rc;
    if (!path) return fail(MFLBM_E_ARG, "mflbm_write_vtk: null path");
    if (vtk_type < 1 || vtk_type > 3) return fail(MFLBM_E_ARG, "mflbm_write_vtk: vtk_type must be 1, 2 or 3");
    if ((rc = ensure_staging(c)) != MFLBM_OK) return rc;
    if (vtk_type != 2 && (rc = export_arrays(c)) != MFLBM_OK) return rc;
    return write_vtk(*c, vtk_type, output_fieldData_precision_cmd, path);
}

int mflbm_write_walls_vtk(mflbm_context* c, const char* path) {
    if (!c || !path) return fail(MFLBM_E_ARG, "mflbm_write_walls_vtk: null argument");
    if (!c->have_geometry) return fail(MFLBM_E_STATE, "geometry not set (mflbm_preprocess_geometry / mflbm_upload_geometry)");
    int rc = ensure_staging(c);
    if (rc != MFLBM_OK) return rc;
    return write_walls_vtk(*c, path);
}

int mflbm_write_checkpoint(mflbm_context* c, int ntime, const char* path) {
    int rc = require_ready(c);
    if (rc != MFLBM_OK) return rc;
    if (!path) return fail(MFLBM_E_ARG, "mflbm_write_checkpoint: null path");
    if ((rc = ensure_staging(c)) != MFLBM_OK) return rc;
    return write_checkpoint(*c, ntime, path);
}

int mflbm_read_checkpoint(mflbm_context* c, const char* path, const void* W_in, int* ntime0) {
    if (!c || !path) return fail(MFLBM_E_ARG, "mflbm_read_checkpoint: null argument");
    if (!c->have_geometry) return fail(MFLBM_E_STATE, "geometry must be set before mflbm_read_checkpoint");
    const Grid& g = c->d.g;
    const size_t T = tsize(c), pl = (size_t)g.plane1();
    const bool convec = c->params.outlet_BC == 1;
    const size_t expect = sizeof(int) + 2 * T + T * ((size_t)g.n1() * 38 + (size_t)g.n4()) + (convec ? T * pl * 39 : 0);
    FILE* f = fopen(path, "rb");
    if (!f) return fail(MFLBM_E_ARG, std::string("checkpoint not found: ") + path);
    std::vector<unsigned char> buf(expect + 1);
    const size_t got = fread(buf.data(), 1, buf.size(), f);
    fclose(f);
    if (got != expect)
        return fail(MFLBM_E_ARG, std::string("checkpoint ") + path + " has " + std::to_string(got) + " bytes, expected " +
                                     std::to_string(expect) + " for this lattice, precision and outlet_BC");
    int nt_next;
    std::memcpy(&nt_next, buf.data(), sizeof(int));
    const unsigned char* p = buf.data() + sizeof(int);
    mflbm_params np = c->params;
    if (T == 4) {
        float fz, rin;
        std::memcpy(&fz, p, 4); std::memcpy(&rin, p + 4, 4);
        np.force_z = fz; np.rho_in = rin;
    } else {
        std::memcpy(&np.force_z, p, 8); std::memcpy(&np.rho_in, p + 8, 8);
    }
    p += 2 * T;
    int rc = mflbm_set_params(c, &np);
    if (rc != MFLBM_OK) return rc;
    const unsigned char* pdf = p;
    const unsigned char* phi = pdf + T * (size_t)g.n1() * 38;
    const unsigned char* cv = phi + T * (size_t)g.n4();
    rc = mflbm_upload_fields(c, pdf, phi, nullptr, nullptr, nullptr, nullptr, nullptr, W_in,
                             convec ? cv : nullptr, convec ? cv + T * pl * 19 : nullptr,
                             convec ? cv + T * pl * 38 : nullptr);
    if (rc != MFLBM_OK) return rc;
    if (ntime0) *ntime0 = nt_next - 1;
    return MFLBM_OK;
}

int mflbm_monitor_profile(mflbm_context* c, double* slices, mflbm_monitor_ext* ext, int track_phi) {
    int rc = require_ready(c);
    if (rc != MFLBM_OK) return rc;
    if (!slices) return fail(MFLBM_E_ARG, "mflbm_monitor_profile: null slices");
    return monitor_profile(*c, slices, ext, track_phi != 0);
}

int mflbm_set_tuning(mflbm_context* c, const mflbm_tuning* t) {
    if (!c || !t) return fail(MFLBM_E_ARG, "mflbm_set_tuning: null argument");
    if (!check_block(t->collide_block) || !check_block(t->normals_block) || !check_block(t->curvature_block) ||
        !check_block(t->extrapolate_block))
        return fail(MFLBM_E_ARG, "mflbm_set_tuning: block sizes must be 64, 128, 256 or 0");
    const bool tile = t->tile_x || t->tile_y || t->tile_z;
    int lx = 0, ly = 0, lz = 0;
    if (tile && !tile_shifts(t->tile_x, t->tile_y, t->tile_z, &lx, &ly, &lz))
        return fail(MFLBM_E_ARG, "mflbm_set_tuning: tile extents must be powers of two, x and y 1-32, z 1 or 2 "
                                 "(all three, or all three 0)");
    if (tile) {
        const int rc = set_tiling(c, lx, ly, lz);
        if (rc != MFLBM_OK) return rc;
    }
    Tuning& tn = c->d.tune;
    if (t->collide_block) tn.collide = t->collide_block;
    if (t->normals_block) tn.normals = t->normals_block;
    if (t->curvature_block) tn.curvature = t->curvature_block;
    if (t->extrapolate_block) tn.extrapolate = t->extrapolate_block;
    if (c->pair_graph) { cudaGraphExecDestroy(c->pair_graph); c->pair_graph = nullptr; }
    c->generation++;
    return MFLBM_OK;
}

int mflbm_get_tuning(mflbm_context* c, mflbm_tuning* out) {
    if (!c || !out) return fail(MFLBM_E_ARG, "mflbm_get_tuning: null argument");
    fill_tuning(*c, out);
    out->step_ms_before = out->step_ms_after = 0.0;
    return MFLBM_OK;
}

int mflbm_autotune(mflbm_context* c, int reps, mflbm_tuning* out) {
    int rc = require_ready(c);
    if (rc != MFLBM_OK) return rc;
    if (c->timing) return fail(MFLBM_E_STATE, "mflbm_autotune: switch kernel timing off first");
    if (reps < 1) reps = 1;
    DeviceState& d = c->d;
    SavedState saved;
    if ((rc = save_state(c, &saved)) != MFLBM_OK) return rc;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto measure = [&](const Tuning& t, double* ms) -> int {
        d.tune = t;
        int r;
        if ((r = one_step(c, 1)) != MFLBM_OK || (r = one_step(c, 2)) != MFLBM_OK) return r;   // warm-up pair
        MFLBM_CUDA(cudaEventRecord(e0, c->stream));
        for (int k = 0; k < reps; ++k)
            if ((r = one_step(c, 1)) != MFLBM_OK || (r = one_step(c, 2)) != MFLBM_OK) return r;
        MFLBM_CUDA(cudaEventRecord(e1, c->stream));
        MFLBM_CUDA(cudaEventSynchronize(e1));
        float f = 0;
        MFLBM_CUDA(cudaEventElapsedTime(&f, e0, e1));
        *ms = f / (2.0 * reps);
        return MFLBM_OK;
    };
    Tuning best = d.tune;
    double before = 0, best_ms = 0;
    rc = measure(best, &before);
    best_ms = before;
    // tile shape of the population layout (with the entry block sizes), then
    // block sizes, one kernel family at a time
    int blx = saved.lx, bly = saved.ly, blz = saved.lz;
    static const int kTiles[][3] = {{3, 2, 1}, {3, 3, 1}, {1, 1, 1}, {3, 1, 1}, {4, 1, 1}, {2, 2, 1}};
    for (const auto& tl : kTiles) {
        if (rc != MFLBM_OK) break;
        if (tl[0] == saved.lx && tl[1] == saved.ly && tl[2] == saved.lz) continue;
        if ((rc = set_tiling(c, tl[0], tl[1], tl[2])) != MFLBM_OK) break;
        double ms = 0;
        if ((rc = measure(best, &ms)) != MFLBM_OK) break;
        if (ms < best_ms) { best_ms = ms; blx = tl[0]; bly = tl[1]; blz = tl[2]; }
    }
    if (rc == MFLBM_OK) rc = set_tiling(c, blx, bly, blz);
    for (int f = 0; f < 4 && rc == MFLBM_OK; ++f)
        for (int bs : {64, 128, 256}) {
            Tuning t = best;
            int* tf[4] = {&t.collide, &t.normals, &t.curvature, &t.extrapolate};
            if (*tf[f] == bs) continue;
            *tf[f] = bs;
            double ms = 0;
            if ((rc = measure(t, &ms)) != MFLBM_OK) break;
            if (ms < best_ms) { best_ms = ms; best = t; }
        }
    d.tune = best;
    int rc2 = restore_state(c, &saved);   // the entry layout and state
    if (rc == MFLBM_OK && rc2 == MFLBM_OK) rc2 = set_tiling(c, blx, bly, blz);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (c->pair_graph) { cudaGraphExecDestroy(c->pair_graph); c->pair_graph = nullptr; }
    c->generation++;
    if (rc != MFLBM_OK) return rc;
    if (rc2 != MFLBM_OK) return rc2;
    if (out) {
        fill_tuning(*c, out);
        out->step_ms_before = before; out->step_ms_after = best_ms;
    }
    return MFLBM_OK;
}

int mflbm_batch_autotune(mflbm_batch* b, int reps, mflbm_tuning* out) {
    if (!b) return fail(MFLBM_E_ARG, "null batch");
    if (reps < 1) reps = 1;
    for (mflbm_context* c : b->ctx) {
        if (c->timing) return fail(MFLBM_E_STATE, "mflbm_batch_autotune: kernel timing is on for a context");
        MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    }
    bool ok = false;
    std::string why;
    int rc = batch_persistent_ok(b, &ok, &why);
    if (rc != MFLBM_OK) return rc;
    if (!ok) return fail(MFLBM_E_STATE, "mflbm_batch_autotune: no persistent launch: " + why);
    const size_t n = b->ctx.size();
    std::vector<SavedState> saved(n);
    for (size_t i = 0; i < n && rc == MFLBM_OK; ++i) rc = save_state(b->ctx[i], &saved[i]);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto tile_all = [&](int lx, int ly, int lz) -> int {
        for (mflbm_context* c : b->ctx) {
            const int r = set_tiling(c, lx, ly, lz);
            if (r != MFLBM_OK) return r;
        }
        return MFLBM_OK;
    };
    auto measure = [&](int block, double* ms) -> int {
        b->block = block;
        int r;
        if ((r = batch_run_persistent(b, 1, 2)) != MFLBM_OK) return r;   // warm-up pair
        MFLBM_CUDA(cudaEventRecord(e0, b->origin));
        if ((r = batch_run_persistent(b, 1, 2 * reps)) != MFLBM_OK) return r;
        MFLBM_CUDA(cudaEventRecord(e1, b->origin));
        MFLBM_CUDA(cudaEventSynchronize(e1));
        float f = 0;
        MFLBM_CUDA(cudaEventElapsedTime(&f, e0, e1));
        *ms = f / (2.0 * reps);
        return MFLBM_OK;
    };
    const int entry_block = b->block;
    double before = 0, best_ms = 0;
    if (rc == MFLBM_OK) rc = measure(entry_block, &before);
    best_ms = before;
    int best_block = entry_block, blx = saved[0].lx, bly = saved[0].ly, blz = saved[0].lz;
    static const int kTiles[][3] = {{3, 2, 1}, {1, 1, 1}, {3, 3, 1}};
    for (const auto& tl : kTiles) {
        if (rc != MFLBM_OK) break;
        if ((rc = tile_all(tl[0], tl[1], tl[2])) != MFLBM_OK) break;
        for (int bs : {64, 128, 256}) {
            double ms = 0;
            if ((rc = measure(bs, &ms)) != MFLBM_OK) break;
            if (ms < best_ms) { best_ms = ms; best_block = bs; blx = tl[0]; bly = tl[1]; blz = tl[2]; }
        }
    }
    b->block = best_block;
    int rc2 = MFLBM_OK;
    for (size_t i = 0; i < n; ++i) {
        if (!saved[i].buf) continue;
        const int r = restore_state(b->ctx[i], &saved[i]);
        if (rc2 == MFLBM_OK) rc2 = r;
    }
    if (rc == MFLBM_OK && rc2 == MFLBM_OK) rc2 = tile_all(blx, bly, blz);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != MFLBM_OK) return rc;
    if (rc2 != MFLBM_OK) return rc2;
    if (out) {
        fill_tuning(*b->ctx[0], out);
        out->collide_block = best_block;
        out->step_ms_before = before; out->step_ms_after = best_ms;
    }
    return MFLBM_OK;
}

int mflbm_batch_create(mflbm_context* const* ctxs, int n, mflbm_batch** out) {
    if (!ctxs || n < 1 || !out) return fail(MFLBM_E_ARG, "mflbm_batch_create: need n >= 1 contexts and an output pointer");
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        int rc = require_ready(ctxs[i]);
        if (rc != MFLBM_OK) return rc;
        if (ctxs[i]->timing) return fail(MFLBM_E_STATE, "mflbm_batch_create: kernel timing is on for a context");
        for (int j = 0; j < i; ++j)
            if (ctxs[j] == ctxs[i]) return fail(MFLBM_E_ARG, "mflbm_batch_create: a context appears twice");
    }
    mflbm_batch* b = new mflbm_batch();
    b->ctx.assign(ctxs, ctxs + n);
    b->gen.assign(n, ~0ull);
    b->join.assign(n, nullptr);
    cudaError_t e = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->dev_bar, 2 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&b->dev_err, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming);
    if (e != cudaSuccess) { mflbm_batch_destroy(b); return fail(MFLBM_E_CUDA, std::string("mflbm_batch_create: ") + cudaGetErrorString(e)); }
    *out = b;
    return MFLBM_OK;
}

int mflbm_batch_run(mflbm_batch* b, int ntime_begin, int nsteps) {
    if (!b) return fail(MFLBM_E_ARG, "null batch");
    if ((ntime_begin & 1) == 0 || (nsteps & 1) != 0 || nsteps < 0)
        return fail(MFLBM_E_ARG, "mflbm_batch_run: ntime_begin must be odd and nsteps even");
    if (nsteps == 0) return MFLBM_OK;
    bool stale = !b->exec;
    for (size_t i = 0; i < b->ctx.size(); ++i) {
        mflbm_context* c = b->ctx[i];
        if (c->timing) return fail(MFLBM_E_STATE, "mflbm_batch_run: kernel timing is on for a context");
        MFLBM_CUDA(cudaStreamSynchronize(c->stream));
        stale = stale || b->gen[i] != c->generation;
        c->d.arrays_stale = true;
    }
    int rc;
    bool retry = b->mode == MFLBM_BATCH_AUTO;
    while (b->mode != MFLBM_BATCH_GRAPH) {
        bool ok = false;
        std::string why;
        if ((rc = batch_persistent_ok(b, &ok, &why)) != MFLBM_OK) return rc;
        if (ok) {
            b->used_mode = MFLBM_BATCH_PERSISTENT;
            return batch_run_persistent(b, ntime_begin, nsteps);
        }
        if (b->mode == MFLBM_BATCH_PERSISTENT) return fail(MFLBM_E_STATE, "mflbm_batch_run: no persistent launch: " + why);
        // AUTO: a single-phase state straight from the start-up may still
        // carry normal records at ghost nodes (the start-up colour gradient
        // sees the periodic ghost layers before the first exchange fills
        // them); one graph-launched step pair clears them, then check again.
        if (!retry || nsteps < 4) break;
        retry = false;
        if (stale && (rc = capture_batch(b)) != MFLBM_OK) return rc;
        stale = false;
        MFLBM_CUDA(cudaGraphLaunch(b->exec, b->origin));
        MFLBM_CUDA(cudaStreamSynchronize(b->origin));
        ntime_begin += 2;
        nsteps -= 2;
    }
    b->used_mode = MFLBM_BATCH_GRAPH;
    if (stale && (rc = capture_batch(b)) != MFLBM_OK) return rc;
    for (int s = 0; s < nsteps; s += 2) MFLBM_CUDA(cudaGraphLaunch(b->exec, b->origin));
    MFLBM_CUDA(cudaStreamSynchronize(b->origin));
    return MFLBM_OK;
}

int mflbm_batch_set_options(mflbm_batch* b, const mflbm_batch_options* o) {
    if (!b || !o) return fail(MFLBM_E_ARG, "mflbm_batch_set_options: null argument");
    if (o->mode < MFLBM_BATCH_AUTO || o->mode > MFLBM_BATCH_PERSISTENT)
        return fail(MFLBM_E_ARG, "mflbm_batch_set_options: mode must be MFLBM_BATCH_AUTO, _GRAPH or _PERSISTENT");
    if (o->block != 64 && o->block != 128 && o->block != 256)
        return fail(MFLBM_E_ARG, "mflbm_batch_set_options: block must be 64, 128 or 256");
    if (!(o->wait_limit_s > 0.0) || o->wait_limit_s > 60.0)
        return fail(MFLBM_E_ARG, "mflbm_batch_set_options: wait_limit_s must be in (0, 60]");
    b->mode = o->mode;
    b->block = o->block;
    b->wait_s = o->wait_limit_s;
    return MFLBM_OK;
}

int mflbm_batch_get_options(mflbm_batch* b, mflbm_batch_options* o) {
    if (!b || !o) return fail(MFLBM_E_ARG, "mflbm_batch_get_options: null argument");
    o->mode = b->mode;
    o->block = b->block;
    o->wait_limit_s = b->wait_s;
    o->used_mode = b->used_mode;
    o->grid = b->grid;
    return MFLBM_OK;
}

int mflbm_batch_destroy(mflbm_batch* b) {
    if (!b) return MFLBM_OK;
    if (b->origin) cudaStreamSynchronize(b->origin);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->fork) cudaEventDestroy(b->fork);
    for (auto e : b->join) if (e) cudaEventDestroy(e);
    if (b->origin) cudaStreamDestroy(b->origin);
    for (void* p : {(void*)b->dev_samples, (void*)b->dev_pre, (void*)b->dev_bar, (void*)b->dev_err})
        if (p) cudaFree(p);
    delete b;
    return MFLBM_OK;
}

int mflbm_node_counts(mflbm_context* c, long long counts[2]) {
    if (!c || !counts) return fail(MFLBM_E_ARG, "null argument");
    counts[0] = c->d.n_fluid;
    counts[1] = c->d.g.n0();
    return MFLBM_OK;
}

void* mflbm_stream(mflbm_context* c) { return c ? (void*)c->stream : nullptr; }

int mflbm_set_kernel_timing(mflbm_context* c, int enable) {
    if (!c) return fail(MFLBM_E_ARG, "null context");
    MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    c->timing = enable != 0;
    timing_pool(c).used = 0;
    return MFLBM_OK;
}

int mflbm_kernel_times(mflbm_context* c, double* collide_ms_total, double* gradient_ms_total, int* n_collide,
                       int* n_gradient) {
    if (!c) return fail(MFLBM_E_ARG, "null context");
    MFLBM_CUDA(cudaStreamSynchronize(c->stream));
    TimingPool& tp = timing_pool(c);
    double tc = 0, tg = 0;
    int n = 0;
    for (size_t b = 0; b + 4 <= tp.used; b += 4) {
        float a = 0, g = 0;
        MFLBM_CUDA(cudaEventElapsedTime(&a, tp.ev[b], tp.ev[b + 1]));
        MFLBM_CUDA(cudaEventElapsedTime(&g, tp.ev[b + 2], tp.ev[b + 3]));
        tc += a; tg += g; ++n;
    }
    if (collide_ms_total) *collide_ms_total = tc;
    if (gradient_ms_total) *gradient_ms_total = tg;
    if (n_collide) *n_collide = n;
    if (n_gradient) *n_gradient = n;
    return n;
}

}  // extern "C"
