// 3x3x3 convolution, halo-tiled, on the 5th-generation tensor cores: every
// input voxel is loaded into shared memory once per output tile instead of
// once per tap.
//
// A CTA computes output tiles of 8 (x) x 16 (y) x TZ (z) voxels with all
// Cout = NT output channels.  Each z slice of a tile is one M = 128
// accumulator in tensor memory (row m = 8 * y + x).  Per tile, one TMA
// load per 8-channel group brings the input halo of (8+2) x (16+2) x (TZ+2)
// voxels into shared memory, laid out [z][y][x][8 channels] per group: a
// 16-byte row per voxel, so eight consecutive x voxels form one core matrix
// of the canonical K-major layout without swizzle.  The A operand of tap
// (dx, dy, dz) for z slice zi is then a shifted view of the halo: start
// (((zi + dz) * 18 + dy) * 10 + dx) * 16, row groups (y rows) 160 bytes
// apart (SBO), channel groups a plane apart (LBO): no gather at all.  Out of
// volume voxels are zero-filled by the TMA (the convolution's zero padding).
// The weights of all 27 taps stay in shared memory for the CTA's life, in
// the K-major layout [tap][channel group][n][8 channels].
//
// The CTA is persistent over tiles; the halo is double-buffered, so the TMA
// of the next tile overlaps the MMAs and the epilogue of this one.  One
// thread issues the TMA loads and the 27 * Cin / 16 MMAs per z slice (kind::f16,
// BF16 x BF16 -> FP32) and commits them to an mbarrier; the epilogue reads
// the accumulators with tcgen05.ld (one row per thread), adds the bias,
// applies the ReLU and writes BF16 (and FP32) outputs, as the gather kernel
// does.  Every wait is bounded: on a time-out the kernel records an error,
// waits (bounded) for its TMA loads and MMAs in flight, frees its tensor
// memory and returns.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cstdint>

#include "unet_tc.cuh"

namespace mflbm {
namespace unet {

constexpr int HALO_X = 10, HALO_Y = 18;   // 8 x 16 outputs + 1 voxel each side

// bytes of one 8-channel plane of the halo (rounded up to 128 for the TMA
// destination alignment)
__host__ __device__ constexpr int halo_plane_bytes(int tz) { return (HALO_X * HALO_Y * (tz + 2) * 16 + 127) / 128 * 128; }
__host__ __device__ constexpr int halo_weight_bytes(int cin, int nt) { return (27 * cin * nt * 2 + 1023) / 1024 * 1024; }
// weights, two halo buffers, then 64 bytes of barriers and the TMEM slot
__host__ __device__ constexpr int halo_smem_bytes(int cin, int nt, int tz) {
    return halo_weight_bytes(cin, nt) + 2 * (cin / 8) * halo_plane_bytes(tz) + 64;
}

__device__ __forceinline__ void tma_expect(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
        : "memory");
}

// y = act(conv(x, w) + b) for cout == NT.  x is read through `xmap`: a 4-D
// tensor map over (channel, x, y, z) of the BF16 input with a box of
// (8, 10, 18, tz + 2).  Tiles: ceil(W / 8) x ceil(H / 16) x ceil(D / tz).
template <int NT>
__global__ void __launch_bounds__(128) conv3d_halo_tc_kernel(const __grid_constant__ CUtensorMap xmap, Dims d, int cin,
                                                             int tz, const bf16* __restrict__ w,
                                                             const float* __restrict__ bias, bf16* __restrict__ y,
                                                             float* __restrict__ y32, int relu, int* __restrict__ err) {
    constexpr uint32_t IDESC = tc_idesc_bf16(TC_M, NT);
    extern __shared__ __align__(1024) uint8_t sm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int KG = cin >> 3;                      // 8-channel groups
    const int WB = halo_weight_bytes(cin, NT), P = halo_plane_bytes(tz);
    const int HB = KG * P;                        // one halo buffer
    uint8_t* halo = sm + WB;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + WB + 2 * HB);   // [0], [1] TMA per buffer, [2] MMA
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 4);
    const uint32_t ncols = tz * NT <= 32 ? 32u : tz * NT <= 64 ? 64u : tz * NT <= 128 ? 128u : tz * NT <= 256 ? 256u : 512u;

    // tensor memory, barriers
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int b = 0; b < 3; ++b) mbar_init(&bars[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&xmap)) : "memory");
    }
    // weights of all taps: [tap][group][n][8 channels], 16 bytes per row
    for (int i = tid; i < 27 * KG * NT; i += blockDim.x) {
        const int n = i % NT, r = i / NT, kg = r % KG, t = r / KG;
        *reinterpret_cast<uint4*>(sm + (size_t)i * 16) =
            *reinterpret_cast<const uint4*>(w + ((size_t)n * 27 + t) * cin + kg * 8);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    const int TXn = (d.W + 7) >> 3, TYn = (d.H + 15) >> 4, TZn = (d.D + tz - 1) / tz;
    const int ntiles = TXn * TYn * TZn;
    const int mine = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const uint32_t tx_bytes = (uint32_t)(KG * HALO_X * HALO_Y * (tz + 2) * 16);
    auto origin = [&](int tile, int& x0, int& y0, int& z0) {
        x0 = (tile % TXn) * 8;
        y0 = ((tile / TXn) % TYn) * 16;
        z0 = (tile / (TXn * TYn)) * tz;
    };
    auto load = [&](int i) {   // thread 0: the halo of this CTA's i-th tile into buffer i & 1
        int x0, y0, z0;
        origin(blockIdx.x + i * gridDim.x, x0, y0, z0);
        uint64_t* bar = &bars[i & 1];
        tma_expect(bar, tx_bytes);
        const uint32_t dst = smem_addr(halo + (i & 1) * HB);
        for (int kg = 0; kg < KG; ++kg) tma_load_4d(dst + kg * P, &xmap, kg * 8, x0 - 1, y0 - 1, z0 - 1, bar);
    };

    int loads = 0, mmas = 0;   // issued by thread 0 (TMA loads, MMA commits)
    bool ok = true;
    if (tid == 0 && mine > 0) { load(0); ++loads; }
    for (int i = 0; i < mine && ok; ++i) {
        if (tid == 0) {
            if (i + 1 < mine) { load(i + 1); ++loads; }   // its buffer's MMAs (tile i - 1) are done
            if (!mbar_wait(&bars[i & 1], (i >> 1) & 1)) {
                ok = false;
            } else {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a0 = smem_addr(halo + (i & 1) * HB), b0 = smem_addr(sm);
                for (int zi = 0; zi < tz; ++zi) {
                    bool first = true;
                    for (int t = 0; t < 27; ++t) {
                        const int dx = t % 3, dy = (t / 3) % 3, dz = t / 9;
                        const uint32_t at = a0 + (uint32_t)((((zi + dz) * HALO_Y + dy) * HALO_X + dx) * 16);
                        for (int cc = 0; cc < KG; cc += 2) {
                            tc_mma(tmem + (uint32_t)(zi * NT), tc_desc(at + cc * P, P, HALO_X * 16),
                                   tc_desc(b0 + (uint32_t)(((t * KG + cc) * NT) * 16), NT * 16, 128), IDESC,
                                   first ? 0u : 1u);
                            first = false;
                        }
                    }
                }
                tc_commit(&bars[2]);
                ++mmas;
            }
        }
        if (!__syncthreads_and(ok)) { ok = false; break; }
        if (!tc_wait_stage(&bars[2], i & 1)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // epilogue: row m = 32 * warp + lane of every z slice
        int x0, y0, z0;
        origin(blockIdx.x + i * gridDim.x, x0, y0, z0);
        const int m = warp * 32 + (tid & 31);
        const int vx = x0 + (m & 7), vy = y0 + (m >> 3);
        for (int zi = 0; zi < tz; ++zi) {
            const int vz = z0 + zi;
            const bool in = vx < d.W && vy < d.H && vz < d.D;
            const size_t vo = ((size_t)vz * d.H + vy) * d.W + vx;
            for (int c = 0; c < NT / 8; ++c) {
                float acc[8];
                tc_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(zi * NT + c * 8), acc);
                if (!in) continue;
                const int co = c * 8;
                uint32_t packed[4];
#pragma unroll
                for (int j = 0; j < 8; j += 2) {
                    float r0 = acc[j] + (bias ? bias[co + j] : 0.0f), r1 = acc[j + 1] + (bias ? bias[co + j + 1] : 0.0f);
                    if (relu) { r0 = fmaxf(r0, 0.0f); r1 = fmaxf(r1, 0.0f); }
                    acc[j] = r0;
                    acc[j + 1] = r1;
                    packed[j >> 1] = pack_bf16(__float2bfloat16_rn(r0), __float2bfloat16_rn(r1));
                }
                *reinterpret_cast<uint4*>(y + vo * NT + co) = make_uint4(packed[0], packed[1], packed[2], packed[3]);
                if (y32) {
                    float4* o = reinterpret_cast<float4*>(y32 + vo * NT + co);
                    o[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
                    o[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
                }
            }
        }
        // the accumulators are read before the next tile's MMAs overwrite them
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
    }
    if (!ok) {
        // time-out: record it, then wait (bounded) for what is still in flight
        if (tid == 0) {
            atomicExch(err, 1);
            // TMA loads: the i-th load completes phase (i >> 1) & 1 of bars[i & 1]
            for (int i = loads - 2 < 0 ? 0 : loads - 2; i < loads; ++i) mbar_wait(&bars[i & 1], (i >> 1) & 1);
            if (mmas > 0) mbar_wait(&bars[2], (mmas - 1) & 1);
        }
        __syncthreads();
    }
    tc_teardown(tmem, ncols);
}

}  // namespace unet
}  // namespace mflbm
