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
// Layout of a K-major operand tile of R rows x 64 K (BF16) in shared memory:
// core matrices of 8 rows x 16 bytes, row r of group r / 8 and K chunk kc
// (8 elements) at ((r / 8) * 8 + kc) * 128 + (r % 8) * 16 bytes, i.e. leading
// (K) byte offset 128 and stride (row-group) byte offset 1024.
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
// A and B BF16 (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0),
// N / 8 at bits 17-22, M / 16 at bits 24-28.
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
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
// bounded wait for the phase of the given parity; false on time-out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t i = 0; i < TC_WAIT_LIMIT; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
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

template <int NT>
__global__ void __launch_bounds__(128) conv3d_fwd_tc_kernel(Dims d, const bf16* __restrict__ x, int cin,
                                                            const bf16* __restrict__ w, const float* __restrict__ bias,
                                                            bf16* __restrict__ y, float* __restrict__ y32, int cout,
                                                            int relu, int* __restrict__ err) {
    constexpr int B_BYTES = NT * TC_K * 2;
    constexpr int STAGE = TC_A_BYTES + B_BYTES;
    constexpr uint32_t NCOLS = NT < 32 ? 32 : NT;
    constexpr uint32_t IDESC = tc_idesc_bf16(TC_M, NT);
    extern __shared__ __align__(1024) uint8_t sm[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + 2 * STAGE);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 2 * STAGE + 16);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int V = d.vox();
    const int m0 = blockIdx.x * TC_M, n0 = blockIdx.y * NT;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"(NCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    const int cpt = cin >> 4;                 // 16-channel chunks per tap
    const int chunks = 27 * cpt;
    const int stages = (chunks + 3) >> 2;
    const int v = m0 + tid;                   // the A row this thread gathers
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    bool ok = true;
    int issued = 0;                           // commits issued (stage s commits to bars[s & 1])

    for (int s = 0; s < stages && ok; ++s) {
        const int st = s & 1;
        uint8_t* A = sm + st * STAGE;
        uint8_t* B = A + TC_A_BYTES;
        // the stage's previous MMAs must be done before it is overwritten
        // (the decision is made uniform over the block)
        if (s >= 2 && !__syncthreads_and(mbar_wait(&bars[st], ((s - 2) >> 1) & 1))) { ok = false; break; }
        // A: row tid, K chunks 2i, 2i+1 of chunk i of this stage
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int ch = 4 * s + i;
            uint4 lo = zero, hi = zero;
            if (ch < chunks && v < V) {
                const int tap = ch / cpt, c0 = (ch - tap * cpt) << 4;
                const int nb = neighbour(d, v, tap);
                if (nb >= 0) {
                    const uint4* src = reinterpret_cast<const uint4*>(x + (size_t)nb * cin + c0);
                    lo = src[0];
                    hi = src[1];
                }
            }
            uint8_t* dst = A + ((tid >> 3) * 8 + 2 * i) * 128 + (tid & 7) * 16;
            *reinterpret_cast<uint4*>(dst) = lo;
            *reinterpret_cast<uint4*>(dst + 128) = hi;
        }
        // B: NT rows x 8 K chunks
        for (int it = tid; it < NT * 8; it += 128) {
            const int n = it >> 3, kc = it & 7;
            const int ch = 4 * s + (kc >> 1), co = n0 + n;
            uint4 val = zero;
            if (ch < chunks && co < cout) {
                const int tap = ch / cpt, c0 = (ch - tap * cpt) << 4;
                val = *reinterpret_cast<const uint4*>(w + ((size_t)co * 27 + tap) * cin + c0 + (kc & 1) * 8);
            }
            *reinterpret_cast<uint4*>(B + ((n >> 3) * 8 + kc) * 128 + (n & 7) * 16) = val;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int nk = min(4, chunks - 4 * s);
            const uint32_t a0 = smem_addr(A), b0 = smem_addr(B);
            for (int k = 0; k < nk; ++k)
                tc_mma(tmem, tc_desc(a0 + k * 256, 128, 1024), tc_desc(b0 + k * 256, 128, 1024), IDESC,
                       (s > 0 || k > 0) ? 1u : 0u);
            tc_commit(&bars[st]);
        }
        ++issued;
    }
    // the last commit of each barrier: wait for all MMAs before reading (or freeing) the accumulator
    bool done = true;
    for (int b = 0; b < 2; ++b) {
        const int uses = (issued + 1 - b) >> 1;   // commits to bars[b]
        if (uses > 0 && !mbar_wait(&bars[b], (uses - 1) & 1)) done = false;
    }
    done = __syncthreads_and(done);
    if (!ok || !done) {
        if (tid == 0) atomicExch(err, 1);
    } else {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int vo = m0 + warp * 32 + (tid & 31);
        for (int c = 0; c < NT / 8; ++c) {
            float acc[8];
            tc_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 8), acc);
            const int co = n0 + c * 8;
            if (vo >= V || co >= cout) continue;
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
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOLS) : "memory");
}

// two stages, the barriers and the tensor-memory address, and 8 KB of slack
// so that no operand read of a stage can leave the block's shared memory
template <int NT>
constexpr int tc_smem_bytes() {
    return 2 * (TC_A_BYTES + NT * TC_K * 2) + 8192;
}

}  // namespace unet
}  // namespace mflbm
