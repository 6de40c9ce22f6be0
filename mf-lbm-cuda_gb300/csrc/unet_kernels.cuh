// Element-wise kernels of the 3-D U-Net warm start (no counterpart in the
// reference): chunk folds of the weight gradients, bias gradient, weight
// flip for the data gradient, ReLU gradient, pooling, up-sampling,
// concatenation, the masked MSE loss and the Adam update.  The convolutions
// themselves run on the tensor cores (unet_tc.cuh).
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

// dw[i] = sum over chunks of part[chunk][i], in chunk order (deterministic); db[co] likewise
__global__ void sum_chunks_kernel(const float* __restrict__ part, int chunks, size_t n, float* __restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.0f;
    for (int c = 0; c < chunks; ++c) s += part[(size_t)c * n + i];
    out[i] = s;
}

// bias gradient partials: one block of 256 threads per chunk of voxels;
// thread (r, c) = (tid / cout, tid % cout) sums channel c over the voxels
// r, r + 256 / cout, ... of the chunk (coalesced rows), then the rows are
// folded in shared memory in a fixed order.  cout divides 256.
__global__ void __launch_bounds__(256) bias_grad_kernel(const bf16* __restrict__ gy, int V, int cout, int chunk_vox,
                                                        float* __restrict__ part) {
    __shared__ float sh[256];
    const int rows = 256 / cout, r = threadIdx.x / cout, c = threadIdx.x - r * cout;
    const int vb = blockIdx.x * chunk_vox, ve = min(V, vb + chunk_vox);
    float s = 0.0f;
    if (r < rows)
        for (int v = vb + r; v < ve; v += rows) s += __bfloat162float(gy[(size_t)v * cout + c]);
    sh[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < cout) {
        float t = 0.0f;
        for (int k = 0; k < rows; ++k) t += sh[k * cout + threadIdx.x];
        part[(size_t)blockIdx.x * cout + threadIdx.x] = t;
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

// host-side tensors have k channels per voxel; the network's have 16
// (zero padding), BF16 for inputs, FP32 for targets and outputs
__global__ void pad_input_kernel(const float* __restrict__ raw, int k, size_t vox, bf16* __restrict__ x) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= vox * 16) return;
    const int c = (int)(i & 15);
    x[i] = __float2bfloat16_rn(c < k ? raw[(i >> 4) * k + c] : 0.0f);
}
__global__ void pad_target_kernel(const float* __restrict__ raw, int k, size_t vox, float* __restrict__ t) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= vox * 16) return;
    const int c = (int)(i & 15);
    t[i] = c < k ? raw[(i >> 4) * k + c] : 0.0f;
}
__global__ void take_outputs_kernel(const float* __restrict__ out32, size_t vox, int k, float* __restrict__ dst) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= vox * k) return;
    dst[i] = out32[(i / k) * 16 + i % k];
}

__global__ void f32_to_bf16_kernel(const float* __restrict__ a, bf16* __restrict__ b, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = __float2bfloat16_rn(a[i]);
}

// ---------------------------------------------------------------------------
// Network inputs of a pore geometry: the exact Euclidean distance transform,
// computed separably (the squared distance to the nearest feature voxel is
// min over the line of (squared distance so far + offset^2), one axis after
// the other; Saito & Toriwaki 1994).  Two transforms at once: .x the squared
// distance to the nearest solid voxel (0 on solids), .y to the nearest fluid
// voxel (0 on fluid).  A periodic axis measures offsets by the minimum image.
// One thread per voxel scans its whole line; lines are at most a few hundred
// voxels, so the scan costs a few hundred L1-resident loads per voxel.
// ---------------------------------------------------------------------------
constexpr int kEdtInf = 1 << 29;   // above any squared distance of a lattice of < 2^13 voxels per axis

__global__ void edt_axis_kernel(const int32_t* __restrict__ walls, const int2* __restrict__ src,
                                int2* __restrict__ dst, Dims d, int axis, int periodic) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)d.vox()) return;
    const int x = (int)(i % d.W), y = (int)((i / d.W) % d.H), z = (int)(i / ((size_t)d.W * d.H));
    const int n = axis == 0 ? d.W : axis == 1 ? d.H : d.D;
    const int p = axis == 0 ? x : axis == 1 ? y : z;
    const size_t stride = axis == 0 ? 1 : axis == 1 ? (size_t)d.W : (size_t)d.W * d.H;
    const size_t base = i - (size_t)p * stride;
    int bs = kEdtInf, bf = kEdtInf;
    for (int q = 0; q < n; ++q) {
        int o = p > q ? p - q : q - p;
        if (periodic && n - o < o) o = n - o;
        const int o2 = o * o;
        int vs, vf;
        if (src == nullptr) {   // first axis: features are the voxels of the line
            const bool solid = walls[base + (size_t)q * stride] != 0;
            vs = solid ? 0 : kEdtInf;
            vf = solid ? kEdtInf : 0;
        } else {
            const int2 v = src[base + (size_t)q * stride];
            vs = v.x; vf = v.y;
        }
        bs = min(bs, vs + o2);
        bf = min(bf, vf + o2);
    }
    dst[i] = make_int2(min(bs, kEdtInf), min(bf, kEdtInf));
}

// x[2 i] = solid mask, x[2 i + 1] = signed distance (positive in the fluid)
// times scale, rounded once from FP64.
__global__ void edt_features_kernel(const int32_t* __restrict__ walls, const int2* __restrict__ sq, size_t vox,
                                    double scale, float* __restrict__ x) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= vox) return;
    const int2 v = sq[i];
    x[2 * i] = walls[i] != 0 ? 1.0f : 0.0f;
    x[2 * i + 1] = (float)((sqrt((double)v.x) - sqrt((double)v.y)) * scale);
}

}  // namespace unet
}  // namespace mflbm
