// Kernels of the 3-D U-Net warm start (no counterpart in the reference):
// 3x3x3 convolutions as implicit GEMMs on the BF16 tensor cores with FP32
// accumulation, their two gradients, pooling, up-sampling, concatenation,
// the masked MSE loss and the Adam update.
//
// Tensors are channels-last: element (z, y, x, c) of a D x H x W x C tensor is
// at ((z * H + y) * W + x) * C + c; activations and weights are BF16, bias,
// gradients of weights, loss and optimiser state FP32.  Weights of a
// convolution are [Cout][27][Cin] (tap = (dz + 1) * 9 + (dy + 1) * 3 + dx + 1),
// zero padding keeps the spatial size.  Channel counts are multiples of 16
// except the output channels of the last layer (multiple of 4).
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace mflbm {
namespace unet {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ uint32_t pack_bf16(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// D = A (16x16, row) * B (16x8, col) + C on BF16 tensor cores, FP32 accumulate.
// Fragments per the PTX ISA layout of mma.m16n8k16 (g = lane / 4, t = lane % 4):
//   a0: (g, 2t..2t+1)  a1: (g+8, 2t..)  a2: (g, 2t+8..)  a3: (g+8, 2t+8..)
//   b0: (k = 2t..2t+1, n = g)  b1: (k = 2t+8.., n = g)
//   c0, c1: (g, 2t..2t+1)  c2, c3: (g+8, 2t..2t+1)
__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct Dims {
    int D, H, W;
    __host__ __device__ __forceinline__ int vox() const { return D * H * W; }
};

// index of the neighbour of voxel v at tap, or -1 outside the volume
__device__ __forceinline__ int neighbour(const Dims& d, int v, int tap) {
    const int x = v % d.W, y = (v / d.W) % d.H, z = v / (d.W * d.H);
    const int xx = x + tap % 3 - 1, yy = y + (tap / 3) % 3 - 1, zz = z + tap / 9 - 1;
    if (xx < 0 || yy < 0 || zz < 0 || xx >= d.W || yy >= d.H || zz >= d.D) return -1;
    return (zz * d.H + yy) * d.W + xx;
}

// y = act(conv(x, w) + b).  Block: 4 warps x 16 voxels; each warp computes
// its 16 voxels for NT output channels (NT / 8 mma tiles).  Grid:
// (ceil(V / 64), ceil(Cout / NT)).  cout: real output channels (stores
// beyond it are skipped; weights of the padded channels are read as zero).
template <int NT>
__global__ void __launch_bounds__(128) conv3d_fwd_kernel(Dims d, const bf16* __restrict__ x, int cin,
                                                         const bf16* __restrict__ w, const float* __restrict__ bias,
                                                         bf16* __restrict__ y, float* __restrict__ y32, int cout,
                                                         int relu) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int V = d.vox();
    const int v0 = (blockIdx.x * 4 + warp) * 16;
    const int n0 = blockIdx.y * NT;
    const int va = v0 + g, vb = v0 + g + 8;
    float acc[NT / 8][4];
#pragma unroll
    for (int j = 0; j < NT / 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    const uint32_t* xw = reinterpret_cast<const uint32_t*>(x);   // pairs of channels
    const uint32_t* ww = reinterpret_cast<const uint32_t*>(w);
    for (int tap = 0; tap < 27; ++tap) {
        const int na = va < V ? neighbour(d, va, tap) : -1;
        const int nb = vb < V ? neighbour(d, vb, tap) : -1;
        for (int c0 = 0; c0 < cin; c0 += 16) {
            uint32_t a[4];
            a[0] = na >= 0 ? xw[((size_t)na * cin + c0) / 2 + t] : 0u;
            a[1] = nb >= 0 ? xw[((size_t)nb * cin + c0) / 2 + t] : 0u;
            a[2] = na >= 0 ? xw[((size_t)na * cin + c0 + 8) / 2 + t] : 0u;
            a[3] = nb >= 0 ? xw[((size_t)nb * cin + c0 + 8) / 2 + t] : 0u;
#pragma unroll
            for (int j = 0; j < NT / 8; ++j) {
                const int co = n0 + j * 8 + g;
                uint32_t b[2];
                const size_t wb = ((size_t)co * 27 + tap) * cin + c0;
                b[0] = co < cout ? ww[wb / 2 + t] : 0u;
                b[1] = co < cout ? ww[(wb + 8) / 2 + t] : 0u;
                mma_bf16(acc[j], a, b);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NT / 8; ++j) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int v = h ? vb : va;
            if (v >= V) continue;
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int co = n0 + j * 8 + 2 * t + e;
                if (co >= cout) continue;
                float r = acc[j][2 * h + e] + (bias ? bias[co] : 0.0f);
                if (relu) r = fmaxf(r, 0.0f);
                y[(size_t)v * cout + co] = __float2bfloat16_rn(r);
                if (y32) y32[(size_t)v * cout + co] = r;
            }
        }
    }
}

// Weight gradient, partial over a chunk of voxels:
//   part[chunk][co][tap][ci] = sum_{v in chunk} gy[v][co] * x[v + tap][ci]
// as a GEMM with M = Cout (16 per warp), N = Cin (8 per mma), K = voxels.
// Block: 4 warps, warp w takes output channels 16 w .. 16 w + 15 of the
// 64-channel tile blockIdx.y; blockIdx.x = chunk * 27 + tap; blockIdx.z: Cin
// tiles of 32.
__global__ void __launch_bounds__(128) conv3d_wgrad_kernel(Dims d, const bf16* __restrict__ x, int cin,
                                                           const bf16* __restrict__ gy, int cout, int chunk_vox,
                                                           float* __restrict__ part) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int tap = blockIdx.x % 27, chunk = blockIdx.x / 27;
    const int co0 = blockIdx.y * 64 + warp * 16;
    const int ci0 = blockIdx.z * 32;
    const int V = d.vox();
    if (co0 >= cout) return;
    float acc[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    const int vb = chunk * chunk_vox, ve = min(V, vb + chunk_vox);
    for (int k0 = vb; k0 < ve; k0 += 16) {
        // A (16 co x 16 voxels): a0 (co g, v 2t..2t+1), a1 (co g+8, ...), a2 (co g, v 2t+8..), a3 (co g+8, v 2t+8..)
        uint32_t a[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int co = co0 + g + ((r & 1) ? 8 : 0);
            const int v = k0 + 2 * t + ((r & 2) ? 8 : 0);
            const bf16 lo = (v < ve && co < cout) ? gy[(size_t)v * cout + co] : __float2bfloat16_rn(0.0f);
            const bf16 hi = (v + 1 < ve && co < cout) ? gy[(size_t)(v + 1) * cout + co] : __float2bfloat16_rn(0.0f);
            a[r] = pack_bf16(lo, hi);
        }
        int nbr[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int v = k0 + 2 * t + (r & 1) + ((r & 2) ? 8 : 0);
            nbr[r] = v < ve ? neighbour(d, v, tap) : -1;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            // B (16 voxels x 8 ci): b0 (v 2t..2t+1, ci g), b1 (v 2t+8.., ci g)
            const int ci = ci0 + j * 8 + g;
            uint32_t b[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int n_lo = nbr[2 * h], n_hi = nbr[2 * h + 1];
                const bf16 lo = (n_lo >= 0 && ci < cin) ? x[(size_t)n_lo * cin + ci] : __float2bfloat16_rn(0.0f);
                const bf16 hi = (n_hi >= 0 && ci < cin) ? x[(size_t)n_hi * cin + ci] : __float2bfloat16_rn(0.0f);
                b[h] = pack_bf16(lo, hi);
            }
            mma_bf16(acc[j], a, b);
        }
    }
    float* out = part + (size_t)chunk * cout * 27 * cin;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int co = co0 + g + 8 * h, ci = ci0 + j * 8 + 2 * t + e;
                if (co < cout && ci < cin) out[((size_t)co * 27 + tap) * cin + ci] = acc[j][2 * h + e];
            }
}

// dw[i] = sum over chunks of part[chunk][i], in chunk order (deterministic); db[co] likewise
__global__ void sum_chunks_kernel(const float* __restrict__ part, int chunks, size_t n, float* __restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.0f;
    for (int c = 0; c < chunks; ++c) s += part[(size_t)c * n + i];
    out[i] = s;
}

// bias gradient partials: one block per chunk of voxels, threads over channels
__global__ void bias_grad_kernel(const bf16* __restrict__ gy, int V, int cout, int chunk_vox, float* __restrict__ part) {
    const int vb = blockIdx.x * chunk_vox, ve = min(V, vb + chunk_vox);
    for (int co = threadIdx.x; co < cout; co += blockDim.x) {
        float s = 0.0f;
        for (int v = vb; v < ve; ++v) s += __bfloat162float(gy[(size_t)v * cout + co]);
        part[(size_t)blockIdx.x * cout + co] = s;
    }
}

// w'[ci][26 - tap][co] = w[co][tap][ci]: the data gradient is a convolution of
// the output gradient with these weights (cin' = cout, cout' = cin)
__global__ void flip_weights_kernel(const bf16* __restrict__ w, int cout, int cin, int cout_pad, bf16* __restrict__ wt) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = (size_t)cin * 27 * cout_pad;
    if (i >= n) return;
    const int co = (int)(i % cout_pad), tap = (int)((i / cout_pad) % 27), ci = (int)(i / ((size_t)cout_pad * 27));
    wt[i] = co < cout ? w[((size_t)co * 27 + (26 - tap)) * cin + ci] : __float2bfloat16_rn(0.0f);
}

// g = g * (y > 0) (ReLU backward, in place)
__global__ void relu_grad_kernel(bf16* __restrict__ g, const bf16* __restrict__ y, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && !(__bfloat162float(y[i]) > 0.0f)) g[i] = __float2bfloat16_rn(0.0f);
}

// 2 x 2 x 2 average pooling and its gradient
__global__ void pool_fwd_kernel(Dims d, const bf16* __restrict__ x, int c, bf16* __restrict__ y) {
    const int Do = d.D / 2, Ho = d.H / 2, Wo = d.W / 2;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)Do * Ho * Wo * c) return;
    const int ch = (int)(i % c);
    const size_t vo = i / c;
    const int xo = (int)(vo % Wo), yo = (int)((vo / Wo) % Ho), zo = (int)(vo / ((size_t)Wo * Ho));
    float s = 0.0f;
    for (int k = 0; k < 8; ++k) {
        const int xx = 2 * xo + (k & 1), yy = 2 * yo + ((k >> 1) & 1), zz = 2 * zo + (k >> 2);
        s += __bfloat162float(x[(((size_t)zz * d.H + yy) * d.W + xx) * c + ch]);
    }
    y[i] = __float2bfloat16_rn(0.125f * s);
}
// (gx += the pooling gradient: the pooled tensor also feeds a skip connection)
__global__ void pool_bwd_add_kernel(Dims d, const bf16* __restrict__ gy, int c, bf16* __restrict__ gx) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)d.vox() * c) return;
    const int ch = (int)(i % c);
    const size_t v = i / c;
    const int xx = (int)(v % d.W), yy = (int)((v / d.W) % d.H), zz = (int)(v / ((size_t)d.W * d.H));
    const size_t vo = ((size_t)(zz / 2) * (d.H / 2) + yy / 2) * (d.W / 2) + xx / 2;
    gx[i] = __float2bfloat16_rn(__bfloat162float(gx[i]) + 0.125f * __bfloat162float(gy[vo * c + ch]));
}

// nearest up-sampling by 2 into channels [off, off + c) of a tensor of ctot
// channels (the decoder's concatenation buffer), and its gradient
__global__ void up_fwd_kernel(Dims d, const bf16* __restrict__ x, int c, bf16* __restrict__ y, int ctot, int off) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;  // over the fine grid
    if (i >= (size_t)d.vox() * c) return;
    const int ch = (int)(i % c);
    const size_t v = i / c;
    const int xx = (int)(v % d.W), yy = (int)((v / d.W) % d.H), zz = (int)(v / ((size_t)d.W * d.H));
    const size_t vc = ((size_t)(zz / 2) * (d.H / 2) + yy / 2) * (d.W / 2) + xx / 2;
    y[v * ctot + off + ch] = x[vc * c + ch];
}
__global__ void up_bwd_kernel(Dims d, const bf16* __restrict__ gy, int ctot, int off, int c, bf16* __restrict__ gx) {
    const int Dc = d.D / 2, Hc = d.H / 2, Wc = d.W / 2;  // d: fine grid
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)Dc * Hc * Wc * c) return;
    const int ch = (int)(i % c);
    const size_t vc = i / c;
    const int xc = (int)(vc % Wc), yc = (int)((vc / Wc) % Hc), zc = (int)(vc / ((size_t)Wc * Hc));
    float s = 0.0f;
    for (int k = 0; k < 8; ++k) {
        const int xx = 2 * xc + (k & 1), yy = 2 * yc + ((k >> 1) & 1), zz = 2 * zc + (k >> 2);
        s += __bfloat162float(gy[(((size_t)zz * d.H + yy) * d.W + xx) * ctot + off + ch]);
    }
    gx[i] = __float2bfloat16_rn(s);
}
// copy channels [0, c) of src into channels [off, off + c) of dst (ctot channels), or back
__global__ void copy_channels_kernel(const bf16* __restrict__ src, int csrc, int soff, bf16* __restrict__ dst, int cdst,
                                     int doff, int c, size_t vox) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= vox * c) return;
    const int ch = (int)(i % c);
    const size_t v = i / c;
    dst[v * cdst + doff + ch] = src[v * csrc + soff + ch];
}
// masked MSE on FP32 predictions: per-block partial sums of mask * (p - t)^2
// and of the mask; the gradient 2 mask (p - t) / count is written as BF16
__global__ void mse_kernel(const float* __restrict__ pred, const float* __restrict__ tgt, const float* __restrict__ mask,
                           int c, size_t vox, float inv_count, bf16* __restrict__ grad, float* __restrict__ part) {
    __shared__ float sh[256];
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    float e = 0.0f;
    if (i < vox * c) {
        const float m = mask[i / c], r = pred[i] - tgt[i];
        e = m * r * r;
        grad[i] = __float2bfloat16_rn(2.0f * m * r * inv_count);
    }
    sh[threadIdx.x] = e;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Adam on FP32 master weights; the BF16 copy used by the convolutions follows
__global__ void adam_kernel(float* __restrict__ w, bf16* __restrict__ w16, const float* __restrict__ gw, float* __restrict__ m,
                            float* __restrict__ v, size_t n, float lr, float b1, float b2, float c1, float c2, float eps) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = gw[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi, vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    w[i] = wi;
    if (w16) w16[i] = __float2bfloat16_rn(wi);
}

__global__ void f32_to_bf16_kernel(const float* __restrict__ a, bf16* __restrict__ b, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = __float2bfloat16_rn(a[i]);
}

}  // namespace unet
}  // namespace mflbm
