// 3x3x3 convolution, halo-tiled, on the 5th-generation tensor cores: every
// input voxel is loaded into shared memory once per output tile instead of
// once per tap.
//
// A CTA computes output tiles of 8 (x) x 16 (y) x TZ (z) voxels with all
// Cout = NT output channels.  Each z slice of a tile is an M = 128 block
// (row m = 8 * y + x).  Per tile, one TMA load per 8-channel group brings the
// input halo of (8+2) x (16+2) x (TZ+2) voxels into shared memory, laid out
// [z][y][x][8 channels] per group: a 16-byte row per voxel, so eight
// consecutive x voxels form one core matrix of the canonical K-major layout
// without swizzle.  The A operand of tap (dx, dy, dz) for z slice zi is then
// a shifted view of the halo: start (((zi + dz) * 18 + dy) * 10 + dx) * 16,
// row groups (y rows) 160 bytes apart (SBO), channel groups a plane apart
// (LBO): no gather at all.  Out-of-volume voxels are zero-filled by the TMA
// (the convolution's zero padding).  The weights of all 27 taps stay in
// shared memory for the CTA's life, in the K-major layout
// [tap][channel group][n][8 channels], brought in by one bulk copy of an
// image that arrange_halo_weights_kernel prepares.
//
// An M = 128, N = 16..48, K = 16 MMA is short: one thread issuing a chain of
// them into one accumulator is bound by the issue and the accumulation
// latency, not by the tensor pipe.  So the taps of a z slice are spread over
// S partial accumulators (tap t into partial t % S, summed in partial order
// by the epilogue) and the MMAs of the z slices and partials are interleaved,
// giving tz * S >= 4 independent chains; the descriptors advance by
// precomputed increments.  Several CTAs share a multiprocessor, each with its
// own issuing thread.
//
// The CTA is persistent over tiles.  With two halo buffers the TMA of the
// next tile overlaps the MMAs and the epilogue of this one; with one (wide
// inputs, so that two CTAs fit on a multiprocessor) it overlaps the
// epilogue.  The epilogue reads the accumulators with tcgen05.ld (one row
// per thread), adds the bias, applies the ReLU and writes BF16 (and FP32)
// outputs.  Every wait is bounded: on a time-out the kernel records an
// error, waits (bounded) for its copies and MMAs in flight, frees its tensor
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
// partial accumulators per z slice
__host__ __device__ constexpr int halo_splits(int tz) { return tz >= 4 ? 1 : 4 / tz; }
// tensor-memory columns of a CTA (a power of two >= 32)
__host__ __device__ constexpr int halo_tmem_cols(int nt, int tz) {
    return tz * halo_splits(tz) * nt <= 32 ? 32 : tz * halo_splits(tz) * nt <= 64 ? 64
         : tz * halo_splits(tz) * nt <= 128 ? 128 : tz * halo_splits(tz) * nt <= 256 ? 256 : 512;
}
// weights, nbuf halo buffers, the bias (up to 64 floats), then 64 bytes of
// barriers and the TMEM slot
__host__ __device__ constexpr int halo_smem_bytes(int cin, int nt, int tz, int nbuf) {
    return halo_weight_bytes(cin, nt) + nbuf * (cin / 8) * halo_plane_bytes(tz) + 256 + 64;
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
// contiguous global -> shared copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// The shared-memory image of the weights: img[((t * KG + g) * nt + n) * 8 + e]
// = w[(n * 27 + t) * cin + 8 * g + e] (w: [cout = nt][27][cin]).
__global__ void arrange_halo_weights_kernel(const bf16* __restrict__ w, int cin, int nt, bf16* __restrict__ img) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;   // one 16-byte row
    const int KG = cin >> 3;
    if (i >= 27 * KG * nt) return;
    const int n = i % nt, r = i / nt, g = r % KG, t = r / KG;
    reinterpret_cast<uint4*>(img)[i] = *reinterpret_cast<const uint4*>(w + ((size_t)n * 27 + t) * cin + g * 8);
}

// y = act(conv(x, w) + b) for cout == NT.  x is read through `xmap`: a 4-D
// tensor map over (channel, x, y, z) of the BF16 input with a box of
// (8, 10, 18, tz + 2); `wimg` is the weights' shared-memory image; nbuf
// halo buffers (1 or 2).  Tiles: ceil(W / 8) x ceil(H / 16) x ceil(D / tz).
template <int NT>
__global__ void __launch_bounds__(128) conv3d_halo_tc_kernel(const __grid_constant__ CUtensorMap xmap, Dims d, int cin,
                                                             int tz, int nbuf, const bf16* __restrict__ wimg,
                                                             const float* __restrict__ bias, bf16* __restrict__ y,
                                                             float* __restrict__ y32, int relu, int* __restrict__ err) {
    constexpr uint32_t IDESC = tc_idesc_bf16(TC_M, NT);
    extern __shared__ __align__(1024) uint8_t sm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int KG = cin >> 3;                      // 8-channel groups
    const int S = halo_splits(tz);
    const int WB = halo_weight_bytes(cin, NT), P = halo_plane_bytes(tz);
    const int HB = KG * P;                        // one halo buffer
    uint8_t* halo = sm + WB;
    float* sbias = reinterpret_cast<float*>(sm + WB + nbuf * HB);
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + WB + nbuf * HB + 256);   // [0], [1] halo, [2] MMA, [3] weights
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 4);
    const uint32_t ncols = (uint32_t)halo_tmem_cols(NT, tz);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int b = 0; b < 4; ++b) mbar_init(&bars[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&xmap)) : "memory");
    }
    if (tid < NT) sbias[tid] = bias ? bias[tid] : 0.0f;
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
    // tile i's halo goes to buffer i % nbuf, completing phase (i / nbuf) & 1 of its barrier
    auto load = [&](int i) {   // thread 0
        int x0, y0, z0;
        origin(blockIdx.x + i * gridDim.x, x0, y0, z0);
        uint64_t* bar = &bars[i % nbuf];
        tma_expect(bar, tx_bytes);
        const uint32_t dst = smem_addr(halo + (i % nbuf) * HB);
        for (int kg = 0; kg < KG; ++kg) tma_load_4d(dst + kg * P, &xmap, kg * 8, x0 - 1, y0 - 1, z0 - 1, bar);
    };

    bool ok = true, wready = false;
    int loads = 0, mmas = 0;   // issued by thread 0 (halo loads, MMA commits)
    if (tid == 0 && mine > 0) {
        tma_expect(&bars[3], (uint32_t)(27 * cin * NT * 2));
        bulk_load(smem_addr(sm), wimg, (uint32_t)(27 * cin * NT * 2), &bars[3]);
        load(0);
        ++loads;
    }
    for (int i = 0; i < mine && ok; ++i) {
        if (tid == 0) {
            // two buffers: the next tile's (its MMAs, of tile i - 1, are done)
            if (nbuf == 2 && i + 1 < mine) { load(i + 1); ++loads; }
            if (!wready) ok = wready = mbar_wait_stage(&bars[3], 0);
            if (ok && !mbar_wait_stage(&bars[i % nbuf], (i / nbuf) & 1)) ok = false;
            if (ok) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                // descriptors advance in 16-byte units (start address field)
                const uint64_t a0 = tc_desc(smem_addr(halo + (i % nbuf) * HB), P, HALO_X * 16);
                const uint64_t b0 = tc_desc(smem_addr(sm), NT * 16, 128);
                const uint32_t zstep = HALO_X * HALO_Y, gstep = (uint32_t)P >> 4;
                for (int t = 0; t < 27; ++t) {
                    const uint64_t at = a0 + (uint32_t)(((t / 9) * HALO_Y + (t / 3) % 3) * HALO_X + t % 3);
                    const uint64_t bt = b0 + (uint32_t)(t * KG * NT);
                    const uint32_t dcol = (uint32_t)((t % S) * NT);
                    for (int cc = 0; cc < KG; cc += 2) {
                        const uint32_t acc = (t < S && cc == 0) ? 0u : 1u;
                        const uint64_t ac = at + cc * gstep, bc = bt + (uint32_t)(cc * NT);
                        for (int zi = 0; zi < tz; ++zi)
                            tc_mma(tmem + (uint32_t)(zi * S * NT) + dcol, ac + zi * zstep, bc, IDESC, acc);
                    }
                }
                tc_commit(&bars[2]);
                ++mmas;
            }
        }
        if (!__syncthreads_and(ok)) { ok = false; break; }
        if (!tc_wait_stage(&bars[2], i & 1)) { ok = false; break; }
        // one buffer: the next tile's, now that this tile's MMAs are done
        if (tid == 0 && nbuf == 1 && i + 1 < mine) { load(i + 1); ++loads; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // epilogue: row m = 32 * warp + lane of every z slice
        int x0, y0, z0;
        origin(blockIdx.x + i * gridDim.x, x0, y0, z0);
        const int m = warp * 32 + (tid & 31);
        const int vx = x0 + (m & 7), vy = y0 + (m >> 3);
        const uint32_t lanes = tmem + ((uint32_t)(warp * 32) << 16);
        for (int zi = 0; zi < tz; ++zi) {
            const int vz = z0 + zi;
            const bool in = vx < d.W && vy < d.H && vz < d.D;
            const size_t vo = ((size_t)vz * d.H + vy) * d.W + vx;
            for (int c = 0; c < NT / 8; ++c) {
                float acc[8];
                tc_ld8(lanes + (uint32_t)(zi * S * NT + c * 8), acc);
                for (int s = 1; s < S; ++s) {
                    float part[8];
                    tc_ld8(lanes + (uint32_t)((zi * S + s) * NT + c * 8), part);
#pragma unroll
                    for (int j = 0; j < 8; ++j) acc[j] += part[j];
                }
                if (!in) continue;
                const int co = c * 8;
                uint32_t packed[4];
#pragma unroll
                for (int j = 0; j < 8; j += 2) {
                    float r0 = acc[j] + sbias[co + j], r1 = acc[j + 1] + sbias[co + j + 1];
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
            if (mine > 0 && !wready) mbar_wait(&bars[3], 0);
            // halo loads: the i-th load completes phase (i / nbuf) & 1 of bars[i % nbuf]
            for (int i = loads - nbuf < 0 ? 0 : loads - nbuf; i < loads; ++i) mbar_wait(&bars[i % nbuf], (i / nbuf) & 1);
            if (mmas > 0) mbar_wait(&bars[2], (mmas - 1) & 1);
        }
        __syncthreads();
    }
    tc_teardown(tmem, ncols);
}

}  // namespace unet
}  // namespace mflbm
