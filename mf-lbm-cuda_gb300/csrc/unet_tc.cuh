// 3x3x3 convolution as an implicit GEMM on the 5th-generation tensor cores
// (tcgen05): M = 128 voxels per CTA, N = an output-channel tile of 16..128,
// K = 27 taps x Cin, in stages of 64 (four 16-channel chunks).  The threads
// gather a stage of the A (activations) and B (weights) operands into shared
// memory in the canonical K-major layout without swizzle; one thread issues
// the tcgen05.mma instructions (BF16 x BF16 -> FP32, accumulator in tensor
// memory) and commits them to the stage's mbarrier, so the gather of the next
// stage overlaps the MMAs of this one (two stages).  The epilogue reads the
// accumulator with tcgen05.ld (one row per thread), adds the bias, applies
// the ReLU and writes BF16 (and optionally FP32) outputs.
//
// Operand tiles of R rows (M or N) x 64 K (BF16) in shared memory, without
// swizzle: core matrices of 128 bytes, the one of row group g = r / 8 and K
// group kg = k / 8 at g * 1024 + kg * 128 (K-group byte offset 128, row-group
// byte offset 1024).  K-major: the core matrix holds 8 rows of 8 K values
// (16 bytes per row); MN-major: 8 K rows of 8 M (or N) values.
//
// Every wait on an mbarrier is bounded; on a time-out the kernel records an
// error in *err, waits (bounded) for the MMAs it issued, frees its tensor
// memory and returns.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#include "unet_kernels.cuh"

namespace mflbm {
namespace unet {

constexpr int TC_M = 128;          // voxels per CTA (accumulator lanes)
constexpr int TC_K = 64;           // K per stage (four 16-channel chunks)
constexpr int TC_A_BYTES = TC_M * TC_K * 2;
constexpr uint32_t TC_WAIT_LIMIT = 1u << 20;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of tcgen05 (no swizzle): start address,
// leading and stride byte offsets (all >> 4), descriptor version 1 at bit 46.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of tcgen05.mma kind::f16: D FP32 (bits 4-5 = 1),
// A and B BF16 (bits 7-9 and 10-12 = 1), A / B K-major (bit 15 / 16 = 0) or
// MN-major (= 1), N / 8 at bits 17-22, M / 16 at bits 24-28.
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int m, int n, bool a_mn = false, bool b_mn = false) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
           ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// tensor-memory columns of an M = 128 x N FP32 accumulator (a power of two >= 32)
template <int NT>
__host__ __device__ constexpr uint32_t tc_ncols() {
    return NT <= 32 ? 32u : NT <= 64 ? 64u : NT <= 128 ? 128u : 256u;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bound of the waits for pipeline stages (polls; mflbm_unet_set_wait_limit
// lowers it to exercise the error path).  The waits for copies and MMAs
// still in flight on the way out always use TC_WAIT_LIMIT, so a short bound
// never frees tensor or shared memory under an operation.
__device__ uint32_t g_tc_stage_wait = TC_WAIT_LIMIT;

// bounded wait for the phase of the given parity; false on time-out
__device__ __forceinline__ bool mbar_wait_for(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// the drain waits (full bound)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    return mbar_wait_for(bar, parity, TC_WAIT_LIMIT);
}
// the waits of the pipeline stages
__device__ __forceinline__ bool mbar_wait_stage(uint64_t* bar, uint32_t parity) {
    return mbar_wait_for(bar, parity, *(volatile uint32_t*)&g_tc_stage_wait);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t tc_setup(uint32_t* tslot, uint64_t* bars, uint32_t ncols) {
    if ((threadIdx.x >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    return *tslot;
}

// one thread waits (bounded) for the phase of a stage's barrier, then the
// block synchronises on the result, so the other threads do not spend issue
// slots polling; false (for every thread) on a time-out
__device__ __forceinline__ bool tc_wait_stage(uint64_t* bar, uint32_t parity) {
    bool ok = true;
    if (threadIdx.x == 0) ok = mbar_wait_stage(bar, parity);
    return __syncthreads_and(ok);
}

// after `issued` stages (stage s committed to bars[s & 1]): wait (bounded)
// for the last commit of each barrier; uniform over the block
__device__ __forceinline__ bool tc_drain(uint64_t* bars, int issued) {
    bool done = true;
    if (threadIdx.x == 0)
        for (int b = 0; b < 2; ++b) {
            const int uses = (issued + 1 - b) >> 1;
            if (uses > 0 && !mbar_wait(&bars[b], (uses - 1) & 1)) done = false;
        }
    return __syncthreads_and(done);
}

__device__ __forceinline__ void tc_teardown(uint32_t tmem, uint32_t ncols) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

// thread 0: the four K = 16 MMAs of a stage (fewer on the last), then the commit
__device__ __forceinline__ void tc_issue(uint32_t tmem, const uint8_t* A, const uint8_t* B, uint32_t idesc, int nk,
                                         bool first, uint64_t* bar) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t a0 = smem_addr(A), b0 = smem_addr(B);
    for (int k = 0; k < nk; ++k)
        tc_mma(tmem, tc_desc(a0 + k * 256, 128, 1024), tc_desc(b0 + k * 256, 128, 1024), idesc,
               (!first || k > 0) ? 1u : 0u);
    tc_commit(bar);
}

// y = act(conv(x, w) + b).  M = 128 voxels per CTA (blockIdx.x), N = NT
// output channels (tile blockIdx.y), K = the 16-channel chunks (tap, c0) of
// the range of split blockIdx.z: [z * chunks / ksplit, (z + 1) * chunks /
// ksplit) with chunks = 27 * cin / 16.  A and B are K-major.  With ksplit > 1
// the raw FP32 sums go to part[z][v][cout] (splitk_reduce_kernel finishes).
template <int NT>
__global__ void __launch_bounds__(128) conv3d_fwd_tc_kernel(Dims d, const bf16* __restrict__ x, int cin,
                                                            const bf16* __restrict__ w, const float* __restrict__ bias,
                                                            bf16* __restrict__ y, float* __restrict__ y32, int cout,
                                                            int relu, int ksplit, float* __restrict__ part,
                                                            int* __restrict__ err) {
    constexpr int STAGE = TC_A_BYTES + NT * TC_K * 2;
    constexpr uint32_t NCOLS = tc_ncols<NT>();
    constexpr uint32_t IDESC = tc_idesc_bf16(TC_M, NT);
    extern __shared__ __align__(1024) uint8_t sm[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + 2 * STAGE);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 2 * STAGE + 16);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int V = d.vox();
    const int m0 = blockIdx.x * TC_M, n0 = blockIdx.y * NT;
    const uint32_t tmem = tc_setup(tslot, bars, NCOLS);

    const int cpt = cin >> 4;                 // 16-channel chunks per tap
    const int chunks = 27 * cpt;
    const int cb = (int)(((long long)blockIdx.z * chunks) / ksplit), ce = (int)(((long long)(blockIdx.z + 1) * chunks) / ksplit);
    const int stages = (ce - cb + 3) >> 2;
    const int v = m0 + tid;                   // the A row this thread gathers
    const int vx = v % d.W, vy = (v / d.W) % d.H, vz = v / (d.W * d.H);
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    bool ok = true;
    int issued = 0;
    for (int s = 0; s < stages && ok; ++s) {
        const int st = s & 1;
        uint8_t* A = sm + st * STAGE;
        uint8_t* B = A + TC_A_BYTES;
        // the stage's previous MMAs must be done before it is overwritten
        if (s >= 2 && !tc_wait_stage(&bars[st], ((s - 2) >> 1) & 1)) { ok = false; break; }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int ch = cb + 4 * s + i;
            uint4 lo = zero, hi = zero;
            if (ch < ce && v < V) {
                const int tap = ch / cpt, c0 = (ch - tap * cpt) << 4;
                const int xx = vx + tap % 3 - 1, yy = vy + (tap / 3) % 3 - 1, zz = vz + tap / 9 - 1;
                if (xx >= 0 && yy >= 0 && zz >= 0 && xx < d.W && yy < d.H && zz < d.D) {
                    const uint4* src =
                        reinterpret_cast<const uint4*>(x + (((size_t)zz * d.H + yy) * d.W + xx) * cin + c0);
                    lo = src[0];
                    hi = src[1];
                }
            }
            uint8_t* dst = A + ((tid >> 3) * 8 + 2 * i) * 128 + (tid & 7) * 16;
            *reinterpret_cast<uint4*>(dst) = lo;
            *reinterpret_cast<uint4*>(dst + 128) = hi;
        }
        for (int it = tid; it < NT * 8; it += 128) {
            const int n = it >> 3, kc = it & 7;
            const int ch = cb + 4 * s + (kc >> 1), co = n0 + n;
            uint4 val = zero;
            if (ch < ce && co < cout) {
                const int tap = ch / cpt, c0 = (ch - tap * cpt) << 4;
                val = *reinterpret_cast<const uint4*>(w + ((size_t)co * 27 + tap) * cin + c0 + (kc & 1) * 8);
            }
            *reinterpret_cast<uint4*>(B + ((n >> 3) * 8 + kc) * 128 + (n & 7) * 16) = val;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) tc_issue(tmem, A, B, IDESC, min(4, ce - cb - 4 * s), s == 0, &bars[st]);
        ++issued;
    }
    const bool done = tc_drain(bars, issued);
    if (!ok || !done) {
        if (tid == 0) atomicExch(err, 1);
    } else if (issued > 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int vo = m0 + warp * 32 + (tid & 31);
        for (int c = 0; c < NT / 8; ++c) {
            float acc[8];
            tc_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 8), acc);
            const int co = n0 + c * 8;
            if (vo >= V || co >= cout) continue;
            if (ksplit > 1) {
                float4* o = reinterpret_cast<float4*>(part + ((size_t)blockIdx.z * V + vo) * cout + co);
                o[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
                o[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
                continue;
            }
            uint32_t packed[4];
#pragma unroll
            for (int j = 0; j < 8; j += 2) {
                float r0 = acc[j] + (bias ? bias[co + j] : 0.0f), r1 = acc[j + 1] + (bias ? bias[co + j + 1] : 0.0f);
                if (relu) { r0 = fmaxf(r0, 0.0f); r1 = fmaxf(r1, 0.0f); }
                acc[j] = r0;
                acc[j + 1] = r1;
                packed[j >> 1] = pack_bf16(__float2bfloat16_rn(r0), __float2bfloat16_rn(r1));
            }
            *reinterpret_cast<uint4*>(y + (size_t)vo * cout + co) = make_uint4(packed[0], packed[1], packed[2], packed[3]);
            if (y32) {
                float4* o = reinterpret_cast<float4*>(y32 + (size_t)vo * cout + co);
                o[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
                o[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
            }
        }
    }
    tc_teardown(tmem, NCOLS);
}

// sum of the split-K partials in split order, bias, ReLU, BF16 (and FP32) output
__global__ void splitk_reduce_kernel(const float* __restrict__ part, int ksplit, size_t n, int cout,
                                     const float* __restrict__ bias, int relu, bf16* __restrict__ y,
                                     float* __restrict__ y32) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float r = 0.0f;
    for (int z = 0; z < ksplit; ++z) r += part[(size_t)z * n + i];
    if (bias) r += bias[i % cout];
    if (relu) r = fmaxf(r, 0.0f);
    y[i] = __float2bfloat16_rn(r);
    if (y32) y32[i] = r;
}

// Weight gradient on the tensor cores, partial over a chunk of voxels:
//   part[chunk][co][t][ci] = sum_{u in chunk} gy[u - off(t)][co] * x[u][ci]
// (the substitution u = v + off(t) of sum_v gy[v][co] x[v + off(t)][ci]), a
// GEMM with M = 128 rows (tl, co) for the 128 / cout taps of the tap group
// blockIdx.y, N = NT input channels (tile blockIdx.z), K = the voxels u of
// the chunk blockIdx.x in stages of 64.  Both operands are MN-major, so the
// channels-last tensors are gathered with 16-byte copies: one A core-matrix
// row is 8 output channels of gy at one voxel, one B row 8 input channels of
// x.  cout in {16, 32, 64, 128}; cin a multiple of NT; chunk_vox a multiple
// of 64.
template <int NT>
__global__ void __launch_bounds__(128) conv3d_wgrad_tc_kernel(Dims d, const bf16* __restrict__ x, int cin,
                                                              const bf16* __restrict__ gy, int cout, int chunk_vox,
                                                              float* __restrict__ part, int* __restrict__ err) {
    constexpr int STAGE = TC_A_BYTES + NT * TC_K * 2;
    constexpr uint32_t NCOLS = tc_ncols<NT>();
    constexpr uint32_t IDESC = tc_idesc_bf16(TC_M, NT, true, true);
    extern __shared__ __align__(1024) uint8_t sm[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + 2 * STAGE);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 2 * STAGE + 16);
    int* ucoord = reinterpret_cast<int*>(sm + 2 * STAGE + 32);   // 2 stages x 64 packed voxel coordinates
    const int tid = threadIdx.x, warp = tid >> 5;
    const int V = d.vox();
    const int tg = 128 / cout;                      // taps per group
    const int t0 = blockIdx.y * tg, ci0 = blockIdx.z * NT;
    const int vb = blockIdx.x * chunk_vox, ve = min(V, vb + chunk_vox);
    const uint32_t tmem = tc_setup(tslot, bars, NCOLS);
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);

    const int stages = (ve - vb + TC_K - 1) / TC_K;
    bool ok = true;
    int issued = 0;
    for (int s = 0; s < stages && ok; ++s) {
        const int st = s & 1;
        uint8_t* A = sm + st * STAGE;
        uint8_t* B = A + TC_A_BYTES;
        int* uc = ucoord + st * 64;
        const int u0 = vb + s * TC_K;
        if (s >= 2 && !tc_wait_stage(&bars[st], ((s - 2) >> 1) & 1)) { ok = false; break; }
        if (tid < 64) {
            const int u = u0 + tid;
            uc[tid] = u < ve ? ((u % d.W) | (((u / d.W) % d.H) << 10) | ((u / (d.W * d.H)) << 20)) : -1;
        }
        __syncthreads();
        // A: 16 row groups (tl, co..co+7) x 64 voxels; gy at u - off(t), zero outside the volume
        for (int it = tid; it < 16 * TC_K; it += 128) {
            const int k = it & (TC_K - 1), mg = it >> 6;
            const int tl = (mg * 8) / cout, co = mg * 8 - tl * cout, t = t0 + tl;
            const int c = uc[k];
            uint4 val = zero;
            if (c >= 0 && t < 27) {
                const int xx = (c & 1023) - (t % 3 - 1), yy = ((c >> 10) & 1023) - ((t / 3) % 3 - 1),
                          zz = (c >> 20) - (t / 9 - 1);
                if (xx >= 0 && yy >= 0 && zz >= 0 && xx < d.W && yy < d.H && zz < d.D)
                    val = *reinterpret_cast<const uint4*>(gy + (((size_t)zz * d.H + yy) * d.W + xx) * cout + co);
            }
            *reinterpret_cast<uint4*>(A + mg * 1024 + (k >> 3) * 128 + (k & 7) * 16) = val;
        }
        // B: NT / 8 row groups (ci..ci+7) x 64 voxels of x
        for (int it = tid; it < NT * 8; it += 128) {
            const int k = it & (TC_K - 1), ng = it >> 6;
            const int u = u0 + k;
            const uint4 val = u < ve ? *reinterpret_cast<const uint4*>(x + (size_t)u * cin + ci0 + ng * 8) : zero;
            *reinterpret_cast<uint4*>(B + ng * 1024 + (k >> 3) * 128 + (k & 7) * 16) = val;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) tc_issue(tmem, A, B, IDESC, 4, s == 0, &bars[st]);
        ++issued;
    }
    const bool done = tc_drain(bars, issued);
    if (!ok || !done) {
        if (tid == 0) atomicExch(err, 1);
    } else if (issued > 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int m = warp * 32 + (tid & 31);
        const int tl = m / cout, co = m - tl * cout, t = t0 + tl;
        float* out = part + (size_t)blockIdx.x * cout * 27 * cin;
        for (int c = 0; c < NT / 8; ++c) {
            float acc[8];
            tc_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 8), acc);
            if (t >= 27) continue;
            float4* o = reinterpret_cast<float4*>(out + ((size_t)co * 27 + t) * cin + ci0 + c * 8);
            o[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
            o[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
        }
    }
    tc_teardown(tmem, NCOLS);
}

// two stages, the barriers, the tensor-memory address and the wgrad voxel
// coordinates (within the first 1 KB after the stages), and 8 KB of slack so
// that no operand read of a stage can leave the block's shared memory
template <int NT>
constexpr int tc_smem_bytes() {
    return 2 * (TC_A_BYTES + NT * TC_K * 2) + 8192;
}

}  // namespace unet
}  // namespace mflbm
