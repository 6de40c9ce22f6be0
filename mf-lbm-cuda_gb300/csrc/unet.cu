// 3-D U-Net warm start (no counterpart in the reference): network, training
// step and C ABI.  4 levels of 16 / 32 / 64 / 128 channels, two 3x3x3
// convolutions with ReLU per level, average pooling down, nearest
// up-sampling and concatenation with the encoder's output up, a final 3x3x3
// convolution to the 4 outputs (u, v, w, p).  Activations and weights BF16,
// accumulation FP32 (unet_kernels.cuh), FP32 master weights with Adam.
//
// Inputs carry 2 channels (solid mask, signed distance) and outputs 4; both
// are stored with 16 channels so every convolution has a multiple of 16 on
// each side (the padding channels are zero and stay zero: their weights get
// zero gradients).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "common.cuh"
#include <cudaTypedefs.h>

#include "unet_halo.cuh"
#include "unet_kernels.cuh"
#include "unet_tc.cuh"

using mflbm::fail;
namespace U = mflbm::unet;
typedef U::bf16 bf16;

namespace {

constexpr int kIn = 2, kOut = 4, kPad = 16;
inline unsigned nblk(size_t n, int b = 256) { return (unsigned)((n + b - 1) / b); }

struct DevBuf {
    void* p = nullptr;
    size_t n = 0;
    ~DevBuf() { if (p) cudaFree(p); }
    int alloc(size_t bytes) {
        if (p) cudaFree(p);
        p = nullptr;
        n = bytes;
        MFLBM_CUDA(cudaMalloc(&p, bytes));
        MFLBM_CUDA(cudaMemset(p, 0, bytes));
        return MFLBM_OK;
    }
    template <class X> X* as() const { return (X*)p; }
};

struct Tensor {  // D x H x W x C, BF16, with its gradient
    U::Dims d;
    int c = 0;
    DevBuf v, g;
    size_t count() const { return (size_t)d.D * d.H * d.W * c; }
    int alloc(U::Dims dd, int cc) {
        d = dd;
        c = cc;
        int rc = v.alloc(count() * sizeof(bf16));
        return rc == MFLBM_OK ? g.alloc(count() * sizeof(bf16)) : rc;
    }
};

struct Conv {
    int cin, cout;
    bool relu;
    DevBuf w32, w16, wt, b, gw, gb, mw, vw, mb, vb;
    size_t nw() const { return (size_t)cout * 27 * cin; }
};

template <int NT>
int configure_tc() {
    static bool done = false;
    if (!done) {
        constexpr int smem = U::tc_smem_bytes<NT>();
        MFLBM_CUDA(cudaFuncSetAttribute(U::conv3d_fwd_tc_kernel<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        MFLBM_CUDA(cudaFuncSetAttribute(U::conv3d_wgrad_tc_kernel<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        done = true;
    }
    return MFLBM_OK;
}

// the N tile of a channel count: the count itself (one tile) when it is one
// of the instantiated sizes, else the largest instantiated divisor
int tc_tile(int c) {
    static const int sizes[] = {192, 128, 96, 64, 48, 32, 16};
    for (int t : sizes)
        if (c == t) return t;
    for (int t : sizes)
        if (t <= 128 && c % t == 0) return t;
    return 0;
}

template <int NT>
int conv_tc(const U::Dims& d, const bf16* x, int cin, const bf16* w, const float* b, bf16* y, float* y32, int cout,
            bool relu, int* err, DevBuf& split, cudaStream_t s) {
    int rc = configure_tc<NT>();
    if (rc != MFLBM_OK) return rc;
    const int V = d.vox();
    const unsigned gx = nblk((size_t)V, U::TC_M), gy = cout / NT;
    // split K over the taps when the grid would leave most SMs idle (deep levels)
    const int chunks = 27 * (cin / 16);
    int ksplit = 1;
    const long long base = (long long)gx * gy;
    if (base < 2 * 152) ksplit = (int)std::min<long long>((2 * 152 + base - 1) / base, (chunks + 3) / 4);
    float* part = nullptr;
    if (ksplit > 1) {
        const size_t bytes = sizeof(float) * (size_t)ksplit * V * cout;
        if (split.n < bytes && (rc = split.alloc(bytes)) != MFLBM_OK) return rc;
        part = split.as<float>();
    }
    U::conv3d_fwd_tc_kernel<NT><<<dim3(gx, gy, ksplit), 128, U::tc_smem_bytes<NT>(), s>>>(
        d, x, cin, w, b, y, y32, cout, relu, ksplit, part, err);
    MFLBM_CUDA(cudaGetLastError());
    mflbm::count_launch();
    if (ksplit > 1) {
        const size_t n = (size_t)V * cout;
        U::splitk_reduce_kernel<<<nblk(n), 256, 0, s>>>(part, ksplit, n, cout, b, relu, y, y32);
        MFLBM_CUDA(cudaGetLastError());
        mflbm::count_launch();
    }
    return MFLBM_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// multiprocessors of the current device (0 if the query fails)
int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            n = 0;
    }
    return n;
}

// CTAs of the halo-tiled kernel per multiprocessor: shared memory (with the
// per-block reservation), 16 blocks of 128 threads, 512 tensor-memory columns
int halo_per_sm(int cin, int cout, int tz, int nbuf) {
    static int smem_sm = 0, reserved = 0;
    if (!smem_sm) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess)
            return 0;
    }
    const int bytes = U::halo_smem_bytes(cin, cout, tz, nbuf);
    if (bytes > 227 * 1024) return 0;
    const int by_smem = smem_sm / (bytes + reserved);
    return std::min(std::min(by_smem, 16), 512 / U::halo_tmem_cols(cout, tz));
}

struct HaloPlan {
    int tz = 0, nbuf = 2;
};

// The halo-tiled kernel's z extent and halo buffers for a convolution, or
// tz = 0 where it cannot take it: cout must be one instantiated tile (16, 32
// or 48), the weights of all taps and the halo buffers must fit in shared
// memory, the tensor map needs a 16-byte aligned input, and there must be at
// least one tile per multiprocessor.  Two halo buffers unless one buffer
// lets more CTAs share a multiprocessor (one issuing thread each).  Among the
// extents that qualify, the one with the fewest z slices per CTA (rounds of
// resident CTAs x tz) wins, the larger extent on a tie.
HaloPlan halo_plan(const U::Dims& d, const bf16* x, int cin, int cout) {
    HaloPlan best;
    if (cout != 16 && cout != 32 && cout != 48) return best;
    if (reinterpret_cast<uintptr_t>(x) % 16 || !tensor_map_encoder()) return best;
    const int nsm = sm_count();
    if (nsm <= 0) return best;
    const long long txy = (long long)((d.W + 7) / 8) * ((d.H + 15) / 16);
    long long best_cost = 0;
    for (int tz : {4, 2, 1}) {
        const int two = halo_per_sm(cin, cout, tz, 2), one = halo_per_sm(cin, cout, tz, 1);
        const int nbuf = two >= 2 || two >= one ? 2 : 1;
        const int per_sm = nbuf == 2 ? two : one;
        const long long tiles = txy * ((d.D + tz - 1) / tz);
        if (per_sm < 1 || tiles < nsm) continue;
        const long long resident = (long long)per_sm * nsm;
        const long long cost = (tiles + resident - 1) / resident * tz;
        if (!best.tz || cost < best_cost) { best.tz = tz; best.nbuf = nbuf; best_cost = cost; }
    }
    return best;
}

template <int NT>
int conv_halo(const U::Dims& d, const bf16* x, int cin, const HaloPlan& plan, const bf16* w, const float* b, bf16* y,
              float* y32, bool relu, int* err, DevBuf& scratch, cudaStream_t s) {
    static bool configured = false;
    if (!configured) {
        MFLBM_CUDA(cudaFuncSetAttribute(U::conv3d_halo_tc_kernel<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        227 * 1024));
        configured = true;
    }
    const int tz = plan.tz;
    // the weights' shared-memory image
    const int rows = 27 * (cin / 8) * NT;
    int rc;
    if (scratch.n < (size_t)rows * 16 && (rc = scratch.alloc((size_t)rows * 16)) != MFLBM_OK) return rc;
    U::arrange_halo_weights_kernel<<<nblk(rows), 256, 0, s>>>(w, cin, NT, scratch.as<bf16>());
    MFLBM_CUDA(cudaGetLastError());
    mflbm::count_launch();
    CUtensorMap map;
    const cuuint64_t dims[4] = {(cuuint64_t)cin, (cuuint64_t)d.W, (cuuint64_t)d.H, (cuuint64_t)d.D};
    const cuuint64_t strides[3] = {(cuuint64_t)cin * 2, (cuuint64_t)cin * 2 * d.W, (cuuint64_t)cin * 2 * d.W * d.H};
    const cuuint32_t box[4] = {8, U::HALO_X, U::HALO_Y, (cuuint32_t)(tz + 2)};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult cr = tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)x, dims, strides, box,
                                             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return fail(MFLBM_E_CUDA, "cuTensorMapEncodeTiled failed for the convolution input");
    const int smem = U::halo_smem_bytes(cin, NT, tz, plan.nbuf);
    const int per_sm = halo_per_sm(cin, NT, tz, plan.nbuf);
    if (per_sm < 1) return fail(MFLBM_E_CUDA, "halo convolution does not fit on a multiprocessor");
    const long long tiles = (long long)((d.W + 7) / 8) * ((d.H + 15) / 16) * ((d.D + tz - 1) / tz);
    const int grid = (int)std::min<long long>(tiles, (long long)per_sm * sm_count());
    U::conv3d_halo_tc_kernel<NT><<<grid, 128, smem, s>>>(map, d, cin, tz, plan.nbuf, scratch.as<bf16>(), b, y, y32,
                                                         relu ? 1 : 0, err);
    MFLBM_CUDA(cudaGetLastError());
    mflbm::count_launch();
    return MFLBM_OK;
}

// y = act(conv(x, w) + b) on the tensor cores; cin and cout multiples of 16
int launch_conv(const U::Dims& d, const bf16* x, int cin, const bf16* w, const float* b, bf16* y, float* y32,
                int cout, bool relu, int* err, DevBuf& split, cudaStream_t s) {
    if (cin % 16 || cout % 16 || cin <= 0 || cout <= 0)
        return fail(MFLBM_E_ARG, "convolution channels must be positive multiples of 16");
    const HaloPlan plan = halo_plan(d, x, cin, cout);
    if (plan.tz) {
        switch (cout) {
        case 16: return conv_halo<16>(d, x, cin, plan, w, b, y, y32, relu, err, split, s);
        case 32: return conv_halo<32>(d, x, cin, plan, w, b, y, y32, relu, err, split, s);
        default: return conv_halo<48>(d, x, cin, plan, w, b, y, y32, relu, err, split, s);
        }
    }
    switch (tc_tile(cout)) {
    case 192: return conv_tc<192>(d, x, cin, w, b, y, y32, cout, relu, err, split, s);
    case 128: return conv_tc<128>(d, x, cin, w, b, y, y32, cout, relu, err, split, s);
    case 96: return conv_tc<96>(d, x, cin, w, b, y, y32, cout, relu, err, split, s);
    case 64: return conv_tc<64>(d, x, cin, w, b, y, y32, cout, relu, err, split, s);
    case 48: return conv_tc<48>(d, x, cin, w, b, y, y32, cout, relu, err, split, s);
    case 32: return conv_tc<32>(d, x, cin, w, b, y, y32, cout, relu, err, split, s);
    default: return conv_tc<16>(d, x, cin, w, b, y, y32, cout, relu, err, split, s);
    }
}

template <int NT>
int wgrad_tc(const U::Dims& d, const bf16* x, int cin, const bf16* gy, int cout, int chunk, int chunks, float* part,
             int* err, cudaStream_t s) {
    int rc = configure_tc<NT>();
    if (rc != MFLBM_OK) return rc;
    const int groups = (27 + 128 / cout - 1) / (128 / cout);
    U::conv3d_wgrad_tc_kernel<NT><<<dim3(chunks, groups, cin / NT), 128, U::tc_smem_bytes<NT>(), s>>>(
        d, x, cin, gy, cout, chunk, part, err);
    MFLBM_CUDA(cudaGetLastError());
    mflbm::count_launch();
    return MFLBM_OK;
}

// gradients of a convolution: gw, gb from (x, gy); gx = conv(gy, flipped w).
// Weight-gradient partials per chunk of voxels on the tensor cores (chunks of
// 256..2048 voxels, enough to occupy the GPU), folded in chunk order.
int conv_backward(const U::Dims& d, const bf16* x, int cin, const bf16* w, bf16* wt, const bf16* gy, int cout,
                  float* gw, float* gb, bf16* gx, DevBuf& work, DevBuf& split, int* err, cudaStream_t s) {
    if (cout != 16 && cout != 32 && cout != 64 && cout != 128)
        return fail(MFLBM_E_ARG, "weight gradient: output channels must be 16, 32, 64 or 128");
    if (cin % 16 || cin <= 0) return fail(MFLBM_E_ARG, "weight gradient: input channels must be a multiple of 16");
    const int V = d.vox();
    const int groups = (27 + 128 / cout - 1) / (128 / cout);
    int chunk = 2048;
    while (chunk > 256 && (long long)((V + chunk - 1) / chunk) * groups < 2 * 152) chunk >>= 1;
    const int chunks = (V + chunk - 1) / chunk;
    const size_t nw = (size_t)cout * 27 * cin;
    const size_t need = sizeof(float) * (chunks * nw + (size_t)chunks * cout);
    int rc;
    if (work.n < need && (rc = work.alloc(need)) != MFLBM_OK) return rc;
    float* part = work.as<float>();
    switch (tc_tile(cin)) {
    case 192: rc = wgrad_tc<192>(d, x, cin, gy, cout, chunk, chunks, part, err, s); break;
    case 128: rc = wgrad_tc<128>(d, x, cin, gy, cout, chunk, chunks, part, err, s); break;
    case 96: rc = wgrad_tc<96>(d, x, cin, gy, cout, chunk, chunks, part, err, s); break;
    case 64: rc = wgrad_tc<64>(d, x, cin, gy, cout, chunk, chunks, part, err, s); break;
    case 48: rc = wgrad_tc<48>(d, x, cin, gy, cout, chunk, chunks, part, err, s); break;
    case 32: rc = wgrad_tc<32>(d, x, cin, gy, cout, chunk, chunks, part, err, s); break;
    default: rc = wgrad_tc<16>(d, x, cin, gy, cout, chunk, chunks, part, err, s); break;
    }
    if (rc != MFLBM_OK) return rc;
    U::sum_chunks_kernel<<<nblk(nw), 256, 0, s>>>(part, chunks, nw, gw);
    float* bpart = part + chunks * nw;
    U::bias_grad_kernel<<<chunks, 256, 0, s>>>(gy, V, cout, chunk, bpart);
    U::sum_chunks_kernel<<<nblk(cout), 256, 0, s>>>(bpart, chunks, cout, gb);
    MFLBM_CUDA(cudaGetLastError());
    mflbm::count_launch();
    if (gx) {
        U::flip_weights_kernel<<<nblk(nw), 256, 0, s>>>(w, cout, cin, cout, wt);
        MFLBM_CUDA(cudaGetLastError());
        return launch_conv(d, gy, cout, wt, nullptr, gx, nullptr, cin, false, err, split, s);
    }
    return MFLBM_OK;
}

}  // namespace

struct mflbm_unet {
    U::Dims d[4];
    cudaStream_t s = nullptr;
    std::vector<std::unique_ptr<Conv>> conv;  // enc 0a 0b 1a 1b 2a 2b 3a 3b, dec 2a 2b 1a 1b 0a 0b, final
    // activations: x, e[l][0..1], p[l], c[l] (concat), dd[l][0..1], out
    Tensor x, e[4][2], p[4], cc[3], dd[3][2], out;
    DevBuf out32, tgt, mask, mse_part, work, split, err;  // err: time-out flag of the tensor-core pipelines
    DevBuf raw;                                           // host-layout staging (D*H*W*4 FP32)
    int step = 0;
};

namespace {

int add_conv(mflbm_unet* n, int cin, int cout, bool relu, std::mt19937_64& rng) {
    auto c = std::make_unique<Conv>();
    c->cin = cin; c->cout = cout; c->relu = relu;
    const size_t nw = c->nw();
    int rc;
    for (DevBuf* b : {&c->w32, &c->gw, &c->mw, &c->vw})
        if ((rc = b->alloc(sizeof(float) * nw)) != MFLBM_OK) return rc;
    for (DevBuf* b : {&c->w16, &c->wt})
        if ((rc = b->alloc(sizeof(bf16) * nw)) != MFLBM_OK) return rc;
    for (DevBuf* b : {&c->b, &c->gb, &c->mb, &c->vb})
        if ((rc = b->alloc(sizeof(float) * cout)) != MFLBM_OK) return rc;
    // He initialisation over the real fan-in; padding channels start (and stay) zero
    const int real_in = cin == kPad && n->conv.empty() ? kIn : cin;
    const int real_out = cout == kPad && c->relu == false ? kOut : cout;
    std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (27.0f * real_in)));
    std::vector<float> w(nw, 0.0f);
    for (int co = 0; co < real_out; ++co)
        for (int t = 0; t < 27; ++t)
            for (int ci = 0; ci < real_in; ++ci) w[((size_t)co * 27 + t) * cin + ci] = nd(rng);
    MFLBM_CUDA(cudaMemcpy(c->w32.p, w.data(), sizeof(float) * nw, cudaMemcpyHostToDevice));
    U::f32_to_bf16_kernel<<<nblk(nw), 256, 0, n->s>>>(c->w32.as<float>(), c->w16.as<bf16>(), nw);
    MFLBM_CUDA(cudaGetLastError());
    n->conv.push_back(std::move(c));
    return MFLBM_OK;
}

int conv_fwd(mflbm_unet* n, int li, const Tensor& in, Tensor& out, float* y32 = nullptr) {
    Conv& c = *n->conv[li];
    return launch_conv(in.d, in.v.as<bf16>(), c.cin, c.w16.as<bf16>(), c.b.as<float>(), out.v.as<bf16>(), y32,
                       c.cout, c.relu, n->err.as<int>(), n->split, n->s);
}

// gradient of the layer's output in out.g (ReLU applied here); accumulates nothing
int conv_bwd(mflbm_unet* n, int li, Tensor& in, Tensor& out, bool need_gx) {
    Conv& c = *n->conv[li];
    if (c.relu) {
        U::relu_grad_kernel<<<nblk(out.count()), 256, 0, n->s>>>(out.g.as<bf16>(), out.v.as<bf16>(), out.count());
        MFLBM_CUDA(cudaGetLastError());
    }
    return conv_backward(in.d, in.v.as<bf16>(), c.cin, c.w16.as<bf16>(), c.wt.as<bf16>(), out.g.as<bf16>(), c.cout,
                         c.gw.as<float>(), c.gb.as<float>(), need_gx ? in.g.as<bf16>() : nullptr, n->work,
                         n->split, n->err.as<int>(), n->s);
}

int forward(mflbm_unet* n) {
    int rc, li = 0;
    const Tensor* in = &n->x;
    for (int l = 0; l < 4; ++l) {
        if (l > 0) {
            const Tensor& src = n->e[l - 1][1];
            U::pool_fwd_kernel<<<nblk(n->p[l].count()), 256, 0, n->s>>>(src.d, src.v.as<bf16>(), src.c, n->p[l].v.as<bf16>());
            MFLBM_CUDA(cudaGetLastError());
            in = &n->p[l];
        }
        if ((rc = conv_fwd(n, li++, *in, n->e[l][0])) != MFLBM_OK) return rc;
        if ((rc = conv_fwd(n, li++, n->e[l][0], n->e[l][1])) != MFLBM_OK) return rc;
    }
    const Tensor* low = &n->e[3][1];
    for (int l = 2; l >= 0; --l) {
        Tensor& cat = n->cc[l];
        U::up_fwd_kernel<<<nblk((size_t)cat.d.vox() * low->c), 256, 0, n->s>>>(cat.d, low->v.as<bf16>(), low->c,
                                                                                cat.v.as<bf16>(), cat.c, 0);
        const Tensor& skip = n->e[l][1];
        U::copy_channels_kernel<<<nblk((size_t)cat.d.vox() * skip.c), 256, 0, n->s>>>(
            skip.v.as<bf16>(), skip.c, 0, cat.v.as<bf16>(), cat.c, low->c, skip.c, (size_t)cat.d.vox());
        MFLBM_CUDA(cudaGetLastError());
        if ((rc = conv_fwd(n, li++, cat, n->dd[l][0])) != MFLBM_OK) return rc;
        if ((rc = conv_fwd(n, li++, n->dd[l][0], n->dd[l][1])) != MFLBM_OK) return rc;
        low = &n->dd[l][1];
    }
    return conv_fwd(n, li, n->dd[0][1], n->out, n->out32.as<float>());
}

int backward(mflbm_unet* n) {
    int rc;
    const int last = (int)n->conv.size() - 1;
    if ((rc = conv_bwd(n, last, n->dd[0][1], n->out, true)) != MFLBM_OK) return rc;
    int li = last - 1;
    for (int l = 0; l <= 2; ++l) {
        // decoder level l: dd[l][1] <- dd[l][0] <- cat[l]
        if ((rc = conv_bwd(n, li--, n->dd[l][0], n->dd[l][1], true)) != MFLBM_OK) return rc;
        if ((rc = conv_bwd(n, li--, n->cc[l], n->dd[l][0], true)) != MFLBM_OK) return rc;
        Tensor& cat = n->cc[l];
        Tensor& low = l < 2 ? n->dd[l + 1][1] : n->e[3][1];
        Tensor& skip = n->e[l][1];
        U::up_bwd_kernel<<<nblk(low.count()), 256, 0, n->s>>>(cat.d, cat.g.as<bf16>(), cat.c, 0, low.c, low.g.as<bf16>());
        // skip gradient: stored now, the pooling gradient is added when its level is reached
        U::copy_channels_kernel<<<nblk(skip.count()), 256, 0, n->s>>>(cat.g.as<bf16>(), cat.c, low.c, skip.g.as<bf16>(),
                                                                     skip.c, 0, skip.c, (size_t)skip.d.vox());
        MFLBM_CUDA(cudaGetLastError());
    }
    // encoder, deepest first; e[3][1].g came from the up-sampling of level 2
    for (int l = 3; l >= 0; --l) {
        const int la = 2 * l, lb = 2 * l + 1;
        if ((rc = conv_bwd(n, lb, n->e[l][0], n->e[l][1], true)) != MFLBM_OK) return rc;
        Tensor& in = l > 0 ? n->p[l] : n->x;
        if ((rc = conv_bwd(n, la, in, n->e[l][0], l > 0)) != MFLBM_OK) return rc;
        if (l > 0) {
            // e[l-1][1] feeds the pool of level l and the concatenation of level l-1
            Tensor& prev = n->e[l - 1][1];
            U::pool_bwd_add_kernel<<<nblk(prev.count()), 256, 0, n->s>>>(prev.d, n->p[l].g.as<bf16>(), prev.c, prev.g.as<bf16>());
            MFLBM_CUDA(cudaGetLastError());
        }
    }
    return MFLBM_OK;
}

int adam(mflbm_unet* n, float lr) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    n->step++;
    const float c1 = 1.0f / (1.0f - std::pow(b1, (float)n->step)), c2 = 1.0f / (1.0f - std::pow(b2, (float)n->step));
    for (auto& cp : n->conv) {
        Conv& c = *cp;
        const size_t nw = c.nw();
        U::adam_kernel<<<nblk(nw), 256, 0, n->s>>>(c.w32.as<float>(), c.w16.as<bf16>(), c.gw.as<float>(), c.mw.as<float>(),
                                                   c.vw.as<float>(), nw, lr, b1, b2, c1, c2, eps);
        U::adam_kernel<<<nblk(c.cout), 256, 0, n->s>>>(c.b.as<float>(), nullptr, c.gb.as<float>(), c.mb.as<float>(),
                                                       c.vb.as<float>(), c.cout, lr, b1, b2, c1, c2, eps);
        MFLBM_CUDA(cudaGetLastError());
    }
    return MFLBM_OK;
}

// host (D*H*W*k, FP32) -> device (D*H*W*16, BF16), padded on the device
int upload_padded(mflbm_unet* n, const float* h, int k, Tensor& t) {
    const size_t V = (size_t)t.d.vox();
    MFLBM_CUDA(cudaMemcpyAsync(n->raw.p, h, V * k * sizeof(float), cudaMemcpyHostToDevice, n->s));
    U::pad_input_kernel<<<nblk(V * kPad), 256, 0, n->s>>>(n->raw.as<float>(), k, V, t.v.as<bf16>());
    MFLBM_CUDA(cudaGetLastError());
    return MFLBM_OK;
}

// the time-out flag of the tensor-core pipelines (after a synchronisation)
int check_pipeline_flag(const DevBuf& err) {
    int h = 0;
    MFLBM_CUDA(cudaMemcpy(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) return fail(MFLBM_E_CUDA, "tensor-core convolution: an mbarrier wait timed out");
    return MFLBM_OK;
}

// masked MSE of the 4 outputs and the gradients of every layer (no update)
int loss_and_gradients(mflbm_unet* n, const float* x, const float* target, const float* mask, float* loss) {
    int rc = upload_padded(n, x, kIn, n->x);
    if (rc != MFLBM_OK) return rc;
    const size_t V = (size_t)n->d[0].vox();
    double count = 0;
    for (size_t v = 0; v < V; ++v) count += mask[v];
    MFLBM_CUDA(cudaMemcpyAsync(n->raw.p, target, V * kOut * sizeof(float), cudaMemcpyHostToDevice, n->s));
    U::pad_target_kernel<<<nblk(V * kPad), 256, 0, n->s>>>(n->raw.as<float>(), kOut, V, n->tgt.as<float>());
    MFLBM_CUDA(cudaGetLastError());
    MFLBM_CUDA(cudaMemcpyAsync(n->mask.p, mask, V * sizeof(float), cudaMemcpyHostToDevice, n->s));
    if ((rc = forward(n)) != MFLBM_OK) return rc;
    const unsigned nb = nblk(V * kPad);
    const double norm = 1.0 / (std::max(count, 1.0) * kOut);
    U::mse_kernel<<<nb, 256, 0, n->s>>>(n->out32.as<float>(), n->tgt.as<float>(), n->mask.as<float>(), kPad, V,
                                        (float)norm, n->out.g.as<bf16>(), n->mse_part.as<float>());
    MFLBM_CUDA(cudaGetLastError());
    if ((rc = backward(n)) != MFLBM_OK) return rc;
    std::vector<float> part(nb);
    MFLBM_CUDA(cudaMemcpyAsync(part.data(), n->mse_part.p, nb * sizeof(float), cudaMemcpyDeviceToHost, n->s));
    MFLBM_CUDA(cudaStreamSynchronize(n->s));
    if ((rc = check_pipeline_flag(n->err)) != MFLBM_OK) return rc;
    double s = 0;
    for (float p : part) s += p;
    if (loss) *loss = (float)(s * norm);
    return MFLBM_OK;
}

}  // namespace

extern "C" {

int mflbm_unet_create(int D, int H, int W, unsigned long long seed, mflbm_unet** out) {
    if (!out) return fail(MFLBM_E_ARG, "mflbm_unet_create: null output");
    *out = nullptr;
    if (D < 8 || H < 8 || W < 8 || D % 8 || H % 8 || W % 8)
        return fail(MFLBM_E_ARG, "mflbm_unet_create: dimensions must be multiples of 8 (three poolings)");
    auto n = std::make_unique<mflbm_unet>();
    MFLBM_CUDA(cudaStreamCreateWithFlags(&n->s, cudaStreamNonBlocking));
    static const int ch[4] = {16, 32, 64, 128};
    for (int l = 0; l < 4; ++l) n->d[l] = U::Dims{D >> l, H >> l, W >> l};
    std::mt19937_64 rng(seed);
    int rc;
    if ((rc = n->x.alloc(n->d[0], kPad)) != MFLBM_OK) return rc;
    for (int l = 0; l < 4; ++l) {
        if (l > 0 && (rc = n->p[l].alloc(n->d[l], ch[l - 1])) != MFLBM_OK) return rc;
        if ((rc = add_conv(n.get(), l == 0 ? kPad : ch[l - 1], ch[l], true, rng)) != MFLBM_OK) return rc;
        if ((rc = add_conv(n.get(), ch[l], ch[l], true, rng)) != MFLBM_OK) return rc;
        for (int k = 0; k < 2; ++k)
            if ((rc = n->e[l][k].alloc(n->d[l], ch[l])) != MFLBM_OK) return rc;
    }
    for (int l = 2; l >= 0; --l) {
        const int low = l == 2 ? ch[3] : ch[l + 1];
        if ((rc = n->cc[l].alloc(n->d[l], low + ch[l])) != MFLBM_OK) return rc;
        if ((rc = add_conv(n.get(), low + ch[l], ch[l], true, rng)) != MFLBM_OK) return rc;
        if ((rc = add_conv(n.get(), ch[l], ch[l], true, rng)) != MFLBM_OK) return rc;
        for (int k = 0; k < 2; ++k)
            if ((rc = n->dd[l][k].alloc(n->d[l], ch[l])) != MFLBM_OK) return rc;
    }
    if ((rc = add_conv(n.get(), ch[0], kPad, false, rng)) != MFLBM_OK) return rc;
    if ((rc = n->out.alloc(n->d[0], kPad)) != MFLBM_OK) return rc;
    const size_t V = (size_t)D * H * W;
    if ((rc = n->out32.alloc(sizeof(float) * V * kPad)) != MFLBM_OK) return rc;
    if ((rc = n->tgt.alloc(sizeof(float) * V * kPad)) != MFLBM_OK) return rc;
    if ((rc = n->mask.alloc(sizeof(float) * V)) != MFLBM_OK) return rc;
    if ((rc = n->mse_part.alloc(sizeof(float) * nblk(V * kPad))) != MFLBM_OK) return rc;
    if ((rc = n->err.alloc(sizeof(int))) != MFLBM_OK) return rc;
    if ((rc = n->raw.alloc(sizeof(float) * V * kOut)) != MFLBM_OK) return rc;
    MFLBM_CUDA(cudaStreamSynchronize(n->s));
    *out = n.release();
    return MFLBM_OK;
}

int mflbm_unet_destroy(mflbm_unet* n) {
    if (!n) return MFLBM_OK;
    cudaStreamSynchronize(n->s);
    cudaStream_t s = n->s;
    delete n;
    cudaStreamDestroy(s);
    return MFLBM_OK;
}

int mflbm_unet_param_count(mflbm_unet* n, long long* count) {
    if (!n || !count) return fail(MFLBM_E_ARG, "mflbm_unet_param_count: null argument");
    long long c = 0;
    for (auto& cp : n->conv) c += (long long)cp->nw() + cp->cout;
    *count = c;
    return MFLBM_OK;
}

int mflbm_unet_get_params(mflbm_unet* n, float* params) {
    if (!n || !params) return fail(MFLBM_E_ARG, "mflbm_unet_get_params: null argument");
    MFLBM_CUDA(cudaStreamSynchronize(n->s));
    for (auto& cp : n->conv) {
        MFLBM_CUDA(cudaMemcpy(params, cp->w32.p, cp->nw() * sizeof(float), cudaMemcpyDeviceToHost));
        params += cp->nw();
        MFLBM_CUDA(cudaMemcpy(params, cp->b.p, cp->cout * sizeof(float), cudaMemcpyDeviceToHost));
        params += cp->cout;
    }
    return MFLBM_OK;
}

// loads weights and biases and restarts the optimiser (moments zero, step 0)
int mflbm_unet_set_params(mflbm_unet* n, const float* params) {
    if (!n || !params) return fail(MFLBM_E_ARG, "mflbm_unet_set_params: null argument");
    for (auto& cp : n->conv) {
        Conv& c = *cp;
        MFLBM_CUDA(cudaMemcpyAsync(c.w32.p, params, c.nw() * sizeof(float), cudaMemcpyHostToDevice, n->s));
        params += c.nw();
        MFLBM_CUDA(cudaMemcpyAsync(c.b.p, params, c.cout * sizeof(float), cudaMemcpyHostToDevice, n->s));
        params += c.cout;
        U::f32_to_bf16_kernel<<<nblk(c.nw()), 256, 0, n->s>>>(c.w32.as<float>(), c.w16.as<bf16>(), c.nw());
        MFLBM_CUDA(cudaGetLastError());
        for (DevBuf* b : {&c.mw, &c.vw, &c.mb, &c.vb}) MFLBM_CUDA(cudaMemsetAsync(b->p, 0, b->n, n->s));
    }
    n->step = 0;
    MFLBM_CUDA(cudaStreamSynchronize(n->s));
    return MFLBM_OK;
}

int mflbm_unet_forward(mflbm_unet* n, const float* x, float* y) {
    if (!n || !x || !y) return fail(MFLBM_E_ARG, "mflbm_unet_forward: null argument");
    int rc = upload_padded(n, x, kIn, n->x);
    if (rc != MFLBM_OK || (rc = forward(n)) != MFLBM_OK) return rc;
    const size_t V = (size_t)n->d[0].vox();
    U::take_outputs_kernel<<<nblk(V * kOut), 256, 0, n->s>>>(n->out32.as<float>(), V, kOut, n->raw.as<float>());
    MFLBM_CUDA(cudaGetLastError());
    MFLBM_CUDA(cudaMemcpyAsync(y, n->raw.p, V * kOut * sizeof(float), cudaMemcpyDeviceToHost, n->s));
    MFLBM_CUDA(cudaStreamSynchronize(n->s));
    return check_pipeline_flag(n->err);
}

int mflbm_unet_train_step(mflbm_unet* n, const float* x, const float* target, const float* mask, float lr, float* loss) {
    if (!n || !x || !target || !mask) return fail(MFLBM_E_ARG, "mflbm_unet_train_step: null argument");
    int rc = loss_and_gradients(n, x, target, mask, loss);
    return rc != MFLBM_OK ? rc : adam(n, lr);
}

int mflbm_unet_gradients(mflbm_unet* n, const float* x, const float* target, const float* mask, float* grads,
                         float* loss) {
    if (!n || !x || !target || !mask || !grads) return fail(MFLBM_E_ARG, "mflbm_unet_gradients: null argument");
    int rc = loss_and_gradients(n, x, target, mask, loss);
    if (rc != MFLBM_OK) return rc;
    for (auto& cp : n->conv) {
        MFLBM_CUDA(cudaMemcpyAsync(grads, cp->gw.p, cp->nw() * sizeof(float), cudaMemcpyDeviceToHost, n->s));
        grads += cp->nw();
        MFLBM_CUDA(cudaMemcpyAsync(grads, cp->gb.p, cp->cout * sizeof(float), cudaMemcpyDeviceToHost, n->s));
        grads += cp->cout;
    }
    MFLBM_CUDA(cudaStreamSynchronize(n->s));
    return MFLBM_OK;
}

// One convolution and its gradients on host arrays (checks against a CPU
// restatement): x D*H*W*cin, w cout*27*cin, b cout, gy D*H*W*cout, all FP32
// (rounded to BF16 on the device); outputs y (FP32 before rounding), gx, gw, gb.
// Network inputs of a geometry (solid mask, signed distance times sdf_scale)
// from its wall array, on the device: three separable passes of the exact
// distance transform (both signs at once) and one pass forming the inputs.
// All work is on the legacy default stream, in order with the allocations.
int mflbm_unet_features(const int32_t* walls, int nx, int ny, int nz, int periodic_xyz, float sdf_scale, float* x) {
    if (!walls || !x) return fail(MFLBM_E_ARG, "mflbm_unet_features: null argument");
    if (nx < 1 || ny < 1 || nz < 1 || nx > 4096 || ny > 4096 || nz > 4096)
        return fail(MFLBM_E_ARG, "mflbm_unet_features: extents must be in [1, 4096]");
    const size_t V = (size_t)nx * ny * nz;
    if (V >= (size_t)1 << 31) return fail(MFLBM_E_ARG, "mflbm_unet_features: at most 2^31 - 1 voxels");
    const U::Dims d{nz, ny, nx};
    size_t solids = 0;
    for (size_t i = 0; i < V; ++i) solids += walls[i] != 0;
    if (solids == 0 || solids == V)
        return fail(MFLBM_E_ARG, "mflbm_unet_features: the geometry needs both solid and fluid voxels");
    DevBuf w, a, b, out;
    int rc;
    if ((rc = w.alloc(V * sizeof(int32_t))) != MFLBM_OK || (rc = a.alloc(V * sizeof(int2))) != MFLBM_OK ||
        (rc = b.alloc(V * sizeof(int2))) != MFLBM_OK || (rc = out.alloc(V * 2 * sizeof(float))) != MFLBM_OK)
        return rc;
    MFLBM_CUDA(cudaMemcpy(w.p, walls, V * sizeof(int32_t), cudaMemcpyHostToDevice));
    const unsigned g = nblk(V, 128);
    U::edt_axis_kernel<<<g, 128>>>(w.as<int32_t>(), nullptr, a.as<int2>(), d, 0, periodic_xyz & 1);
    U::edt_axis_kernel<<<g, 128>>>(w.as<int32_t>(), a.as<int2>(), b.as<int2>(), d, 1, (periodic_xyz >> 1) & 1);
    U::edt_axis_kernel<<<g, 128>>>(w.as<int32_t>(), b.as<int2>(), a.as<int2>(), d, 2, (periodic_xyz >> 2) & 1);
    U::edt_features_kernel<<<nblk(V), 256>>>(w.as<int32_t>(), a.as<int2>(), V, (double)sdf_scale, out.as<float>());
    MFLBM_CUDA(cudaGetLastError());
    MFLBM_CUDA(cudaMemcpy(x, out.p, V * 2 * sizeof(float), cudaMemcpyDeviceToHost));
    return MFLBM_OK;
}

int mflbm_unet_set_wait_limit(unsigned int polls) {
    MFLBM_CUDA(cudaMemcpyToSymbol(U::g_tc_stage_wait, &polls, sizeof(polls)));
    return MFLBM_OK;
}

int mflbm_unet_conv_check(int D, int H, int W, int cin, int cout, const float* x, const float* w, const float* b,
                          int relu, const float* gy, float* y, float* gx, float* gw, float* gb) {
    if (cin % 16 || cout % 16 || cin <= 0 || cout <= 0)
        return fail(MFLBM_E_ARG, "mflbm_unet_conv_check: channels must be positive multiples of 16");
    const U::Dims d{D, H, W};
    const size_t V = (size_t)D * H * W, nw = (size_t)cout * 27 * cin;
    DevBuf dx, dw, db, dy, dy32, dgy, dgx, dgw, dgb, dwt, f32, work, split, derr;
    int rc;
    const size_t ci = (size_t)cin, co = (size_t)cout;
    struct { DevBuf* b; size_t n; } al[] = {{&dx, V * ci * 2}, {&dw, nw * 2}, {&db, co * 4}, {&dy, V * co * 2},
                                            {&dy32, V * co * 4}, {&dgy, V * co * 2}, {&dgx, V * ci * 2},
                                            {&dgw, nw * 4}, {&dgb, co * 4}, {&dwt, nw * 2},
                                            {&f32, std::max(V * std::max(ci, co), nw) * 4}, {&derr, sizeof(int)}};
    for (auto& a : al)
        if ((rc = a.b->alloc(a.n)) != MFLBM_OK) return rc;
    auto up16 = [&](const float* h, size_t cnt, DevBuf& dst) -> int {
        MFLBM_CUDA(cudaMemcpy(f32.p, h, cnt * 4, cudaMemcpyHostToDevice));
        U::f32_to_bf16_kernel<<<nblk(cnt), 256>>>(f32.as<float>(), dst.as<bf16>(), cnt);
        MFLBM_CUDA(cudaGetLastError());
        return MFLBM_OK;
    };
    if ((rc = up16(x, V * cin, dx)) != MFLBM_OK || (rc = up16(w, nw, dw)) != MFLBM_OK) return rc;
    MFLBM_CUDA(cudaMemcpy(db.p, b, cout * 4, cudaMemcpyHostToDevice));
    if ((rc = launch_conv(d, dx.as<bf16>(), cin, dw.as<bf16>(), db.as<float>(), dy.as<bf16>(), dy32.as<float>(), cout,
                          relu != 0, derr.as<int>(), split, 0)) != MFLBM_OK)
        return rc;
    if (gy) {
        if ((rc = up16(gy, V * cout, dgy)) != MFLBM_OK) return rc;
        if ((rc = conv_backward(d, dx.as<bf16>(), cin, dw.as<bf16>(), dwt.as<bf16>(), dgy.as<bf16>(), cout,
                                dgw.as<float>(), dgb.as<float>(), dgx.as<bf16>(), work, split, derr.as<int>(), 0)) != MFLBM_OK)
            return rc;
    }
    MFLBM_CUDA(cudaDeviceSynchronize());
    if ((rc = check_pipeline_flag(derr)) != MFLBM_OK) return rc;
    if (y) MFLBM_CUDA(cudaMemcpy(y, dy32.p, V * cout * 4, cudaMemcpyDeviceToHost));
    if (gy) {
        std::vector<bf16> h(V * cin);
        MFLBM_CUDA(cudaMemcpy(h.data(), dgx.p, h.size() * 2, cudaMemcpyDeviceToHost));
        if (gx)
            for (size_t i = 0; i < h.size(); ++i) gx[i] = __bfloat162float(h[i]);
        if (gw) MFLBM_CUDA(cudaMemcpy(gw, dgw.p, nw * 4, cudaMemcpyDeviceToHost));
        if (gb) MFLBM_CUDA(cudaMemcpy(gb, dgb.p, cout * 4, cudaMemcpyDeviceToHost));
    }
    return MFLBM_OK;
}

}  // extern "C"
