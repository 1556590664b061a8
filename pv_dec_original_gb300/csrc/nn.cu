// Kernels of the learned warm start: a small 3D convolutional
// encoder-decoder that maps a signed-distance field plus inlet parameters to
// an initial rho / u field.  The reference has no counterpart (it always
// starts from rest, Node.cpp:30-37).
//
// Activations are BF16, channels-last (voxel-major, channel counts padded to
// multiples of 16); weights are BF16 [co][tap][ci] with an FP32 master copy
// for Adam; every product accumulates in FP32 on the tensor cores.  The
// 3x3x3 forward convolutions, stride-1 input gradients and weight
// gradients run on tcgen05 where the grid tiles (conv_tc.cu); the kernels
// here (mma.sync m16n8k16 BF16) take the rest and the comparison engine
// (lbm_nn_set_conv_engine).  A convolution is an implicit GEMM:
//   forward      rows = output voxels, cols = output channels, K = taps x ci
//   input grad   rows = input voxels,  cols = input channels,  K = taps x co
//                (the same kernel with the transposed weights [ci][tap][co])
//   weight grad  rows = output channels, cols = input channels of one tap,
//                K = output voxels (split over blocks, FP32 atomics)
// Kernel size 3 (padding 1, stride 1 or 2) or 1 (stride 1).
#include <cuda_bf16.h>

#include <atomic>
#include <cstdint>
#include <cstdio>

#include "lbm_internal.cuh"
#include "lbm_nn.h"

namespace {

using bf16 = __nv_bfloat16;

struct Conv {
    int D, H, W;     // input dims
    int Do, Ho, Wo;  // output dims
    int ci, co;      // padded channels
    int ks, stride, pad;
};

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int kRows = 64;   // GEMM rows per block (4 warps x 16)
constexpr int kPadK = 24;   // shared row stride in BF16 (16 + 8: no bank conflicts on fragment loads)

// Source voxel of GEMM row r for tap t, or -1.  MODE 0: r is an output
// voxel, the source an input voxel; MODE 1: r is an input voxel, the source
// the output voxel whose window covers r at tap t.
template <int MODE>
__device__ __forceinline__ int64_t source_voxel(const Conv& g, int64_t r, int t) {
    const int tz = t / (g.ks * g.ks), ty = (t / g.ks) % g.ks, tx = t % g.ks;
    if (MODE == 0) {
        const int ox = (int)(r % g.Wo), oy = (int)((r / g.Wo) % g.Ho), oz = (int)(r / ((int64_t)g.Wo * g.Ho));
        const int ix = ox * g.stride - g.pad + tx, iy = oy * g.stride - g.pad + ty, iz = oz * g.stride - g.pad + tz;
        if (ix < 0 || iy < 0 || iz < 0 || ix >= g.W || iy >= g.H || iz >= g.D) return -1;
        return ((int64_t)iz * g.H + iy) * g.W + ix;
    } else {
        const int ix = (int)(r % g.W), iy = (int)((r / g.W) % g.H), iz = (int)(r / ((int64_t)g.W * g.H));
        const int nx = ix + g.pad - tx, ny = iy + g.pad - ty, nz = iz + g.pad - tz;
        if (nx < 0 || ny < 0 || nz < 0) return -1;
        if (nx % g.stride || ny % g.stride || nz % g.stride) return -1;
        const int ox = nx / g.stride, oy = ny / g.stride, oz = nz / g.stride;
        if (ox >= g.Wo || oy >= g.Ho || oz >= g.Do) return -1;
        return ((int64_t)oz * g.Ho + oy) * g.Wo + ox;
    }
}

// out[r][n] = act(bias[n] + sum_{t,k} src[source(r,t)][k] * B[n][t][k]).
// BN = columns (padded channel count of the output, <= 64).
template <int MODE, int BN>
__global__ void __launch_bounds__(128) k_conv_gemm(const bf16* __restrict__ src, const bf16* __restrict__ B,
                                                   const float* __restrict__ bias, bf16* __restrict__ out,
                                                   float* __restrict__ out_f32, Conv g, int64_t rows, int kc,
                                                   int relu) {
    __shared__ __align__(16) bf16 As[kRows][kPadK];
    __shared__ __align__(16) bf16 Bs[BN][kPadK];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int gq = lane >> 2, tg = lane & 3;
    const int64_t r0 = (int64_t)blockIdx.x * kRows;
    const int taps = g.ks * g.ks * g.ks;
    float acc[BN / 8][4];
#pragma unroll
    for (int j = 0; j < BN / 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    // this thread's A row and half-row (8 channels)
    const int arow = tid >> 1, ahalf = tid & 1;
    const int64_t r = r0 + arow;
    for (int t = 0; t < taps; ++t) {
        const int64_t sv = r < rows ? source_voxel<MODE>(g, r, t) : -1;
        for (int c0 = 0; c0 < kc; c0 += 16) {
            uint4 av = make_uint4(0, 0, 0, 0);
            if (sv >= 0) av = *reinterpret_cast<const uint4*>(src + sv * kc + c0 + ahalf * 8);
            *reinterpret_cast<uint4*>(&As[arow][ahalf * 8]) = av;
            for (int e = tid; e < BN * 2; e += 128) {
                const int n = e >> 1, h = e & 1;
                *reinterpret_cast<uint4*>(&Bs[n][h * 8]) =
                    *reinterpret_cast<const uint4*>(B + ((int64_t)n * taps + t) * kc + c0 + h * 8);
            }
            __syncthreads();
            uint32_t a[4];
            const int ar = warp * 16 + gq;
            a[0] = *reinterpret_cast<const uint32_t*>(&As[ar][tg * 2]);
            a[1] = *reinterpret_cast<const uint32_t*>(&As[ar + 8][tg * 2]);
            a[2] = *reinterpret_cast<const uint32_t*>(&As[ar][tg * 2 + 8]);
            a[3] = *reinterpret_cast<const uint32_t*>(&As[ar + 8][tg * 2 + 8]);
#pragma unroll
            for (int j = 0; j < BN / 8; ++j) {
                const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&Bs[j * 8 + gq][tg * 2]);
                const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&Bs[j * 8 + gq][tg * 2 + 8]);
                mma_bf16(acc[j], a, b0, b1);
            }
            __syncthreads();
        }
    }
    // epilogue: bias, ReLU, BF16 (and optionally FP32) store
#pragma unroll
    for (int j = 0; j < BN / 8; ++j) {
        const int n = j * 8 + tg * 2;
        const float b0 = bias ? bias[n] : 0.f, b1 = bias ? bias[n + 1] : 0.f;
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            const int64_t rr = r0 + warp * 16 + gq + hh * 8;
            if (rr >= rows) continue;
            float v0 = acc[j][2 * hh] + b0, v1 = acc[j][2 * hh + 1] + b1;
            if (relu) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
            *reinterpret_cast<__nv_bfloat162*>(out + rr * BN + n) = __floats2bfloat162_rn(v0, v1);
            if (out_f32) { out_f32[rr * BN + n] = v0; out_f32[rr * BN + n + 1] = v1; }
        }
    }
}

// dW[co][t][ci] += sum over output voxels m of dY[m][co] * X[src(m,t)][ci]
// (FP32 atomics; one block per (tap, chunk of output voxels)).  CO, CI:
// padded channel counts (CO <= 64 rows in 16-row warp slices).
template <int CO, int CI>
__global__ void __launch_bounds__(128) k_conv_wgrad(const bf16* __restrict__ x, const bf16* __restrict__ dy,
                                                    float* __restrict__ dw, Conv g, int64_t rows, int chunk) {
    __shared__ __align__(16) bf16 As[CO][kPadK];  // [co][16 voxels]
    __shared__ __align__(16) bf16 Bs[CI][kPadK];  // [ci][16 voxels]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int gq = lane >> 2, tg = lane & 3;
    const int t = blockIdx.y;
    const int taps = g.ks * g.ks * g.ks;
    const int64_t m_begin = (int64_t)blockIdx.x * chunk;
    const int64_t m_end = m_begin + chunk < rows ? m_begin + chunk : rows;
    float acc[CI / 8][4];
#pragma unroll
    for (int j = 0; j < CI / 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    for (int64_t m0 = m_begin; m0 < m_end; m0 += 16) {
        // A: 16 voxels x CO channels, transposed into As[co][v]
        for (int e = tid; e < 16 * (CO / 8); e += 128) {
            const int v = e / (CO / 8), c8 = e % (CO / 8);
            const int64_t m = m0 + v;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (m < m_end) val = *reinterpret_cast<const uint4*>(dy + m * CO + c8 * 8);
            const bf16* pv = reinterpret_cast<const bf16*>(&val);
#pragma unroll
            for (int q = 0; q < 8; ++q) As[c8 * 8 + q][v] = pv[q];
        }
        // B: 16 voxels x CI channels of tap t, transposed into Bs[ci][v]
        for (int e = tid; e < 16 * (CI / 8); e += 128) {
            const int v = e / (CI / 8), c8 = e % (CI / 8);
            const int64_t m = m0 + v;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (m < m_end) {
                const int64_t sv = source_voxel<0>(g, m, t);
                if (sv >= 0) val = *reinterpret_cast<const uint4*>(x + sv * CI + c8 * 8);
            }
            const bf16* pv = reinterpret_cast<const bf16*>(&val);
#pragma unroll
            for (int q = 0; q < 8; ++q) Bs[c8 * 8 + q][v] = pv[q];
        }
        __syncthreads();
        if (warp * 16 < CO) {
            uint32_t a[4];
            const int ar = warp * 16 + gq;
            a[0] = *reinterpret_cast<const uint32_t*>(&As[ar][tg * 2]);
            a[1] = *reinterpret_cast<const uint32_t*>(&As[ar + 8][tg * 2]);
            a[2] = *reinterpret_cast<const uint32_t*>(&As[ar][tg * 2 + 8]);
            a[3] = *reinterpret_cast<const uint32_t*>(&As[ar + 8][tg * 2 + 8]);
#pragma unroll
            for (int j = 0; j < CI / 8; ++j) {
                const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&Bs[j * 8 + gq][tg * 2]);
                const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&Bs[j * 8 + gq][tg * 2 + 8]);
                mma_bf16(acc[j], a, b0, b1);
            }
        }
        __syncthreads();
    }
    if (warp * 16 < CO) {
#pragma unroll
        for (int j = 0; j < CI / 8; ++j) {
            const int n = j * 8 + tg * 2;
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int co = warp * 16 + gq + hh * 8;
                float* p = dw + ((int64_t)co * taps + t) * CI + n;
                atomicAdd(p, acc[j][2 * hh]);
                atomicAdd(p + 1, acc[j][2 * hh + 1]);
            }
        }
    }
}

// db[c] += sum_m dy[m][c]
__global__ void k_bias_grad(const bf16* __restrict__ dy, float* __restrict__ db, int64_t rows, int c) {
    const int ch = threadIdx.x % c;
    const int lanes = blockDim.x / c;
    float s = 0.f;
    for (int64_t m = (int64_t)blockIdx.x * lanes + threadIdx.x / c; m < rows; m += (int64_t)gridDim.x * lanes)
        s += __bfloat162float(dy[m * c + ch]);
    if (threadIdx.x / c < lanes) atomicAdd(db + ch, s);
}

// W [co][t][ci] -> Wt [ci][t][co]
__global__ void k_transpose_w(const bf16* __restrict__ w, bf16* __restrict__ wt, int co, int taps, int ci) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)co * taps * ci) return;
    const int c = (int)(e % ci), t = (int)((e / ci) % taps), o = (int)(e / ((int64_t)ci * taps));
    wt[((int64_t)c * taps + t) * co + o] = w[e];
}

// dy *= (y > 0): ReLU backward through the stored activation
__global__ void k_relu_bwd(const bf16* __restrict__ y, bf16* __restrict__ dy, int64_t n) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n && !(__bfloat162float(y[e]) > 0.f)) dy[e] = __float2bfloat16(0.f);
}

// nearest-neighbour x2 upsampling of [D][H][W][c] and its adjoint
__global__ void k_up2(const bf16* __restrict__ in, bf16* __restrict__ out, int D, int H, int W, int c) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)8 * D * H * W * c;
    if (e >= n) return;
    const int ch = (int)(e % c);
    const int64_t v = e / c;
    const int x = (int)(v % (2 * W)), y = (int)((v / (2 * W)) % (2 * H)), z = (int)(v / ((int64_t)4 * W * H));
    out[e] = in[(((int64_t)(z / 2) * H + y / 2) * W + x / 2) * c + ch];
}

__global__ void k_up2_bwd(const bf16* __restrict__ dout, bf16* __restrict__ din, int D, int H, int W, int c) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)D * H * W * c;
    if (e >= n) return;
    const int ch = (int)(e % c);
    const int64_t v = e / c;
    const int x = (int)(v % W), y = (int)((v / W) % H), z = (int)(v / ((int64_t)W * H));
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int zz = 2 * z + (k >> 2), yy = 2 * y + ((k >> 1) & 1), xx = 2 * x + (k & 1);
        s += __bfloat162float(dout[(((int64_t)zz * 2 * H + yy) * 2 * W + xx) * c + ch]);
    }
    din[e] = __float2bfloat16(s);
}

// The same element-wise kernels on 8 BF16 values (16 bytes) a thread, for
// 16-byte aligned tensors whose channel count (or length) is a multiple of
// 8: one index computation and one load / store instruction per 8 values
// (the one-value kernels spend their time on 64-bit index division).  The
// arithmetic per value is the one-value kernels', so results are identical.
union V8 {
    uint4 u;
    __nv_bfloat16 h[8];
};

__global__ void k_up2_v8(const uint4* __restrict__ in, uint4* __restrict__ out, int D, int H, int W, int c8) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)8 * D * H * W * c8;
    if (e >= n) return;
    const int ch = (int)(e % c8);
    const int64_t v = e / c8;
    const int x = (int)(v % (2 * W));
    const int64_t r = v / (2 * W);
    const int y = (int)(r % (2 * H)), z = (int)(r / (2 * H));
    out[e] = in[(((int64_t)(z >> 1) * H + (y >> 1)) * W + (x >> 1)) * c8 + ch];
}

__global__ void k_up2_bwd_v8(const uint4* __restrict__ dout, uint4* __restrict__ din, int D, int H, int W, int c8) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)D * H * W * c8;
    if (e >= n) return;
    const int ch = (int)(e % c8);
    const int64_t v = e / c8;
    const int x = (int)(v % W);
    const int64_t r = v / W;
    const int y = (int)(r % H), z = (int)(r / H);
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int zz = 2 * z + (k >> 2), yy = 2 * y + ((k >> 1) & 1), xx = 2 * x + (k & 1);
        V8 a;
        a.u = dout[(((int64_t)zz * 2 * H + yy) * 2 * W + xx) * c8 + ch];
#pragma unroll
        for (int j = 0; j < 8; ++j) s[j] += __bfloat162float(a.h[j]);
    }
    V8 o;
#pragma unroll
    for (int j = 0; j < 8; ++j) o.h[j] = __float2bfloat16(s[j]);
    din[e] = o.u;
}

__global__ void k_add_v8(const uint4* __restrict__ a, const uint4* __restrict__ b, uint4* __restrict__ out,
                         int64_t n8) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n8) return;
    V8 x, y, o;
    x.u = a[e];
    y.u = b[e];
#pragma unroll
    for (int j = 0; j < 8; ++j) o.h[j] = __float2bfloat16(__bfloat162float(x.h[j]) + __bfloat162float(y.h[j]));
    out[e] = o.u;
}

__global__ void k_relu_bwd_v8(const uint4* __restrict__ y, uint4* __restrict__ dy, int64_t n8) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n8) return;
    V8 a, g;
    a.u = y[e];
    g.u = dy[e];
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (!(__bfloat162float(a.h[j]) > 0.f)) g.h[j] = __float2bfloat16(0.f);
    dy[e] = g.u;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// out = a + b (BF16, FP32 add)
__global__ void k_add(const bf16* __restrict__ a, const bf16* __restrict__ b, bf16* __restrict__ out, int64_t n) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) out[e] = __float2bfloat16(__bfloat162float(a[e]) + __bfloat162float(b[e]));
}

// Masked mean squared error over the first nc channels of pred/target
// ([voxel][c], FP32): loss += sum / norm; dpred (BF16) = 2 (pred - target) / norm.
__global__ void k_mse(const float* __restrict__ pred, const float* __restrict__ target,
                      const uint8_t* __restrict__ mask, int64_t nvox, int c, int nc, float inv_norm,
                      bf16* __restrict__ dpred, float* __restrict__ loss) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (e < nvox * c) {
        const int ch = (int)(e % c);
        const int64_t v = e / c;
        float d = 0.f;
        if (ch < nc && mask[v]) d = pred[e] - target[v * nc + ch];
        l = d * d * inv_norm;
        dpred[e] = __float2bfloat16(2.f * d * inv_norm);
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// Adam on an FP32 master copy; the BF16 weights follow.
__global__ void k_adam(float* __restrict__ w, bf16* __restrict__ wb, const float* __restrict__ grad,
                       float* __restrict__ m, float* __restrict__ v, int64_t n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float gval = grad[e];
    const float mm = b1 * m[e] + (1.f - b1) * gval;
    const float vv = b2 * v[e] + (1.f - b2) * gval * gval;
    m[e] = mm;
    v[e] = vv;
    const float wn = w[e] - lr * (mm * c1) / (sqrtf(vv * c2) + eps);
    w[e] = wn;
    if (wb) wb[e] = __float2bfloat16(wn);
}

// --------------------------------------------------------------------------
// Signed distance field of a mask by jump flooding: seeds are the fluid
// voxels with a non-fluid 6-neighbour (or on the box face); every voxel
// keeps the nearest seed found at offsets k = N/2, N/4, ..., 1, then a final
// pass at offset 1.  sdf > 0 in fluid, < 0 outside, in lattice spacings.
// PLANAR: every z slice on its own (seeds from in-plane neighbours, search
// in the slice), for the in-slice distance to the wall.
template <bool PLANAR>
__global__ void k_jfa_seed(const uint8_t* __restrict__ mask, int D, int H, int W, int32_t* __restrict__ seed) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)D * H * W;
    if (v >= n) return;
    const int x = (int)(v % W), y = (int)((v / W) % H), z = (int)(v / ((int64_t)W * H));
    bool s = false;
    if (mask[v]) {
        const int d[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        for (int k = 0; k < (PLANAR ? 4 : 6) && !s; ++k) {
            const int xx = x + d[k][0], yy = y + d[k][1], zz = z + d[k][2];
            s = xx < 0 || yy < 0 || zz < 0 || xx >= W || yy >= H || zz >= D ||
                !mask[((int64_t)zz * H + yy) * W + xx];
        }
    }
    seed[v] = s ? (int32_t)v : -1;
}

template <bool PLANAR>
__global__ void k_jfa_step(const int32_t* __restrict__ in, int32_t* __restrict__ out, int D, int H, int W, int k) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)D * H * W;
    if (v >= n) return;
    const int x = (int)(v % W), y = (int)((v / W) % H), z = (int)(v / ((int64_t)W * H));
    int32_t best = in[v];
    float bd = 3.4e38f;
    if (best >= 0) {
        const float dx = (float)(x - (int)(best % W)), dy = (float)(y - (int)((best / W) % H)),
                    dz = (float)(z - (int)(best / ((int64_t)W * H)));
        bd = dx * dx + dy * dy + dz * dz;
    }
    for (int dz = (PLANAR ? 0 : -1); dz <= (PLANAR ? 0 : 1); ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int xx = x + dx * k, yy = y + dy * k, zz = z + dz * k;
                if (xx < 0 || yy < 0 || zz < 0 || xx >= W || yy >= H || zz >= D) continue;
                const int32_t s = in[((int64_t)zz * H + yy) * W + xx];
                if (s < 0) continue;
                const float ex = (float)(x - (int)(s % W)), ey = (float)(y - (int)((s / W) % H)),
                            ez = (float)(z - (int)(s / ((int64_t)W * H)));
                const float d = ex * ex + ey * ey + ez * ez;
                if (d < bd) { bd = d; best = s; }
            }
    out[v] = best;
}

// The same flooding with every seed stored as its packed coordinates
// x | y << 11 | z << 22 (grids up to 2048 x 2048 x 512: 31 bits, so an
// empty voxel's -1 stays the only negative value) and one thread per
// voxel on a (x blocks, y, z) grid: no 64-bit division per neighbour.  The
// squared distances are integers below 2^24, exact in FP32 and in int32
// alike, and neighbours are visited in the same order with the same strict
// comparison, so the nearest seed and the distances are those of the
// kernels above.
constexpr int kPackBitsXY = 11, kPackBitsZ = 9;
__host__ __device__ constexpr bool jfa_packs(int D, int H, int W) {
    return W <= (1 << kPackBitsXY) && H <= (1 << kPackBitsXY) && D <= (1 << kPackBitsZ);
}
__device__ __forceinline__ int32_t jfa_pack(int x, int y, int z) {
    return x | (y << kPackBitsXY) | (z << (2 * kPackBitsXY));
}
__device__ __forceinline__ int jfa_d2(int32_t s, int x, int y, int z) {
    const int ex = x - (s & ((1 << kPackBitsXY) - 1)), ey = y - ((s >> kPackBitsXY) & ((1 << kPackBitsXY) - 1)),
              ez = z - (s >> (2 * kPackBitsXY));
    return ex * ex + ey * ey + ez * ez;
}

template <bool PLANAR>
__global__ void k_jfa_seed_p(const uint8_t* __restrict__ mask, int D, int H, int W, int32_t* __restrict__ seed) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= W) return;
    const int64_t v = ((int64_t)z * H + y) * W + x;
    bool s = false;
    if (mask[v]) {
        const int d[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        for (int k = 0; k < (PLANAR ? 4 : 6) && !s; ++k) {
            const int xx = x + d[k][0], yy = y + d[k][1], zz = z + d[k][2];
            s = xx < 0 || yy < 0 || zz < 0 || xx >= W || yy >= H || zz >= D ||
                !mask[((int64_t)zz * H + yy) * W + xx];
        }
    }
    seed[v] = s ? jfa_pack(x, y, z) : -1;
}

template <bool PLANAR>
__global__ void k_jfa_step_p(const int32_t* __restrict__ in, int32_t* __restrict__ out, int D, int H, int W, int k) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= W) return;
    const int64_t v = ((int64_t)z * H + y) * W + x;
    int32_t best = in[v];
    int bd = best >= 0 ? jfa_d2(best, x, y, z) : 0x7fffffff;
    for (int dz = (PLANAR ? 0 : -1); dz <= (PLANAR ? 0 : 1); ++dz) {
        const int zz = z + dz * k;
        if (zz < 0 || zz >= D) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            const int yy = y + dy * k;
            if (yy < 0 || yy >= H) continue;
            const int32_t* row = in + ((int64_t)zz * H + yy) * W;
            for (int dx = -1; dx <= 1; ++dx) {
                const int xx = x + dx * k;
                if (xx < 0 || xx >= W) continue;
                const int32_t s = __ldg(row + xx);
                if (s < 0) continue;
                const int d = jfa_d2(s, x, y, z);
                if (d < bd) { bd = d; best = s; }
            }
        }
    }
    out[v] = best;
}

template <bool PLANAR>
__global__ void k_jfa_finish_p(const int32_t* __restrict__ seed, const uint8_t* __restrict__ mask, int D, int H,
                               int W, float* __restrict__ sdf) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= W) return;
    const int64_t v = ((int64_t)z * H + y) * W + x;
    const int32_t s = seed[v];
    const float d = s >= 0 ? sqrtf((float)jfa_d2(s, x, y, z)) : 0.f;
    sdf[v] = mask[v] ? d + 0.5f : (PLANAR ? 0.f : -(d + 0.5f));
}

template <bool PLANAR>
__global__ void k_jfa_finish(const int32_t* __restrict__ seed, const uint8_t* __restrict__ mask, int D, int H,
                             int W, float* __restrict__ sdf) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)D * H * W;
    if (v >= n) return;
    const int32_t s = seed[v];
    float d = 0.f;
    if (s >= 0) {
        const int x = (int)(v % W), y = (int)((v / W) % H), z = (int)(v / ((int64_t)W * H));
        const float ex = (float)(x - (int)(s % W)), ey = (float)(y - (int)((s / W) % H)),
                    ez = (float)(z - (int)(s / ((int64_t)W * H)));
        d = sqrtf(ex * ex + ey * ey + ez * ez);
    }
    // a seed voxel is half a spacing inside the wall
    sdf[v] = mask[v] ? d + 0.5f : (PLANAR ? 0.f : -(d + 0.5f));
}

// --------------------------------------------------------------------------
// Slice-wise Hagen-Poiseuille prior (flow along +z): with s the in-slice
// distance to the wall and R(z) its largest value in slice z,
// u_z = 2 Q / (pi R^2) (1 - (R - s)^2 / R^2) and rho - 1 from
// d rho / dz = -3 * 8 nu Q / (pi R^4), zero at the last slice;
// Q = pi R0^2 u_in / 2 on the first fluid slice.
__global__ void k_slice_max(const float* __restrict__ dist, int HW, float* __restrict__ R) {
    __shared__ float red[256];
    const int z = blockIdx.x;
    float m = 0.f;
    for (int i = threadIdx.x; i < HW; i += blockDim.x) m = fmaxf(m, dist[(int64_t)z * HW + i]);
    red[threadIdx.x] = m;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w /= 2) {
        if ((int)threadIdx.x < w) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) R[z] = red[0];
}

// one thread: per-slice peak velocity and density offset (suffix sums)
__global__ void k_prior_axis(const float* __restrict__ R, int D, double inlet, double nu, float* __restrict__ peak,
                             float* __restrict__ tail) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int z0 = -1;
    for (int z = 0; z < D && z0 < 0; ++z)
        if (R[z] > 0.f) z0 = z;
    const double pi = 3.14159265358979323846;
    const double Q = z0 < 0 ? 0.0 : pi * (double)R[z0] * (double)R[z0] * inlet / 2.0;
    double acc = 0.0;  // sum of drho over the slices downstream of z
    for (int z = D - 1; z >= 0; --z) {
        const double Rs = fmax((double)R[z], 1.0);
        peak[z] = (float)(2.0 * Q / (pi * Rs * Rs));
        tail[z] = (float)acc;
        if (R[z] > 0.f) acc += 3.0 * 8.0 * nu * Q / (pi * Rs * Rs * Rs * Rs);
    }
}

__global__ void k_prior_fill(const uint8_t* __restrict__ mask, const float* __restrict__ dist,
                             const float* __restrict__ R, const float* __restrict__ peak,
                             const float* __restrict__ tail, int64_t n, int HW, float* __restrict__ drho,
                             float* __restrict__ uz) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int z = (int)(v / HW);
    float u = 0.f, r = 0.f;
    if (mask[v]) {
        const float Rs = fmaxf(R[z], 1.f), e = Rs - dist[v];
        u = peak[z] * fminf(fmaxf(1.f - e * e / (Rs * Rs), 0.f), 1.f);
        r = tail[z];
    }
    uz[v] = u;
    drho[v] = r;
}

// Masked [1, 2, 1] / 4 filter along one axis (weights renormalised where a
// neighbour is solid or outside the box); zero on solid voxels.
__global__ void k_smooth_axis(const uint8_t* __restrict__ mask, const float* __restrict__ in,
                              float* __restrict__ out, int D, int H, int W, int axis) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)D * H * W;
    if (v >= n) return;
    if (!mask[v]) { out[v] = 0.f; return; }
    const int x = (int)(v % W), y = (int)((v / W) % H), z = (int)(v / ((int64_t)W * H));
    const int c = axis == 0 ? z : (axis == 1 ? y : x);
    const int len = axis == 0 ? D : (axis == 1 ? H : W);
    const int64_t st = axis == 0 ? (int64_t)W * H : (axis == 1 ? (int64_t)W : 1);
    float num = 2.f * in[v], den = 2.f;
    if (c + 1 < len && mask[v + st]) { num += in[v + st]; den += 1.f; }
    if (c - 1 >= 0 && mask[v - st]) { num += in[v - st]; den += 1.f; }
    out[v] = num / den;
}

// Network input [n][16] BF16, one voxel a thread (two 16-byte stores):
// channel 0 clamp(sdf sdf_scale, -3, 3), 1 the mask, 2 and 3 the scalar
// inlet mean and period (scaled), 4 z / D, 5 u_z prior / U, 6 (rho - 1)
// prior / U rho_scale, 7..15 zero; FP32 values rounded to BF16 once.
__global__ void k_ws_features(const float* __restrict__ sdf, const uint8_t* __restrict__ mask,
                              const float* __restrict__ uz_p, const float* __restrict__ drho_p, int64_t n, int64_t hw,
                              int D, float sdf_scale, float mean_in, float period_in, float inlet, float rho_scale,
                              uint4* __restrict__ x) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const float f[7] = {fminf(fmaxf(sdf[v] * sdf_scale, -3.f), 3.f), mask[v] ? 1.f : 0.f, mean_in, period_in,
                        (float)(int)(v / hw) / (float)D, uz_p[v] / inlet, drho_p[v] / inlet * rho_scale};
    V8 a, b;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        a.h[k] = __float2bfloat16(k < 7 ? f[k] : 0.f);
        b.h[k] = __float2bfloat16(0.f);
    }
    x[2 * v] = a.u;
    x[2 * v + 1] = b.u;
}

// Network output [n][c] (FP32) to fields [4][n]: rho - 1 = prior + y0 U /
// rho_scale, u = y1..3 U / u_scale (+ prior u_z); zero on solid voxels.
__global__ void k_ws_output(const float* __restrict__ y, int c, const uint8_t* __restrict__ mask,
                            const float* __restrict__ drho_p, const float* __restrict__ uz_p, int64_t n, float inlet,
                            float rho_scale, float u_scale, float* __restrict__ f) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const bool fl = mask[v] != 0;
    const float* yv = y + v * c;
    f[v] = fl ? drho_p[v] + yv[0] * inlet / rho_scale : 0.f;
    f[n + v] = fl ? yv[1] * inlet / u_scale : 0.f;
    f[2 * n + v] = fl ? yv[2] * inlet / u_scale : 0.f;
    f[3 * n + v] = fl ? yv[3] * inlet / u_scale + uz_p[v] : 0.f;
}

// Gather fluid voxels (index list) into per-node rho (1 + field 0) and
// interleaved u (3 per node).
__global__ void k_ws_gather(const float* __restrict__ f, int64_t n, const int64_t* __restrict__ idx, int64_t m,
                            float* __restrict__ rho, float* __restrict__ u) {
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= m) return;
    const int64_t v = idx[a];
    rho[a] = 1.f + f[v];
    u[3 * a] = f[n + v];
    u[3 * a + 1] = f[2 * n + v];
    u[3 * a + 2] = f[3 * n + v];
}

int report(const char* what, cudaError_t e) {
    char msg[256];
    std::snprintf(msg, sizeof(msg), "%s: %s", what, e == cudaSuccess ? "invalid argument" : cudaGetErrorString(e));
    lbm::set_last_global_error(msg);
    return e == cudaSuccess ? LBM_ERR_ARG : LBM_ERR_CUDA;
}

bool padded16(int c) { return c == 16 || c == 32 || c == 64; }  // the channel counts the kernels are built for

// Convolution engine (lbm_nn_set_conv_engine): tcgen05 where its shapes
// apply, or mma.sync everywhere.
std::atomic<int> g_engine{LBM_NN_ENGINE_AUTO};

// 3x3x3 on shapes the tensor-core kernels tile (conv_tc.cu): the forward
// convolution at stride 1 or 2, the input gradient at stride 1 (the weight
// gradient: conv3_wgrad_tc_applies).
bool use_tc(const Conv& g) {
    return g_engine.load() == LBM_NN_ENGINE_AUTO && g.ks == 3 &&
           lbm::conv3_tc_applies(g.D, g.H, g.W, g.ci, g.co, g.stride);
}
bool use_tc_dx(const Conv& g) { return g.stride == 1 && use_tc(g); }

Conv make_conv(const int dims_in[3], int ci, int co, int ks, int stride) {
    Conv g{};
    g.D = dims_in[0]; g.H = dims_in[1]; g.W = dims_in[2];
    g.ci = ci; g.co = co; g.ks = ks; g.stride = stride; g.pad = ks / 2;
    g.Do = (g.D + 2 * g.pad - ks) / stride + 1;
    g.Ho = (g.H + 2 * g.pad - ks) / stride + 1;
    g.Wo = (g.W + 2 * g.pad - ks) / stride + 1;
    return g;
}

template <int MODE>
cudaError_t launch_gemm(int bn, const bf16* src, const bf16* B, const float* bias, bf16* out, float* out_f32,
                        const Conv& g, int64_t rows, int kc, int relu, cudaStream_t st) {
    const unsigned blocks = (unsigned)lbm::ceil_div(rows, kRows);
    switch (bn) {
        case 16: k_conv_gemm<MODE, 16><<<blocks, 128, 0, st>>>(src, B, bias, out, out_f32, g, rows, kc, relu); break;
        case 32: k_conv_gemm<MODE, 32><<<blocks, 128, 0, st>>>(src, B, bias, out, out_f32, g, rows, kc, relu); break;
        default: k_conv_gemm<MODE, 64><<<blocks, 128, 0, st>>>(src, B, bias, out, out_f32, g, rows, kc, relu); break;
    }
    return cudaGetLastError();
}

template <int CO>
cudaError_t launch_wgrad_ci(int ci, const bf16* x, const bf16* dy, float* dw, const Conv& g, int64_t rows,
                            cudaStream_t st) {
    const int chunk = 2048;
    const dim3 grid((unsigned)lbm::ceil_div(rows, chunk), (unsigned)(g.ks * g.ks * g.ks));
    switch (ci) {
        case 16: k_conv_wgrad<CO, 16><<<grid, 128, 0, st>>>(x, dy, dw, g, rows, chunk); break;
        case 32: k_conv_wgrad<CO, 32><<<grid, 128, 0, st>>>(x, dy, dw, g, rows, chunk); break;
        default: k_conv_wgrad<CO, 64><<<grid, 128, 0, st>>>(x, dy, dw, g, rows, chunk); break;
    }
    return cudaGetLastError();
}

unsigned grid1(int64_t n) { return (unsigned)lbm::ceil_div(n > 0 ? n : 1, 256); }

// jump flooding into scratch (2 n int32), distances into out
template <bool PLANAR>
void jfa(const uint8_t* mask, int D, int H, int W, int32_t* scratch, float* out, cudaStream_t st) {
    const int64_t n = (int64_t)D * H * W;
    int32_t* a = scratch;
    int32_t* b = a + n;
    const int big = PLANAR ? (H > W ? H : W) : (D > H ? (D > W ? D : W) : (H > W ? H : W));
    int k = 1;
    while (k * 2 < big) k *= 2;
    if (jfa_packs(D, H, W) && H <= 65535 && D <= 65535) {
        const dim3 grid((unsigned)lbm::ceil_div(W, 128), (unsigned)H, (unsigned)D);
        k_jfa_seed_p<PLANAR><<<grid, 128, 0, st>>>(mask, D, H, W, a);
        for (; k >= 1; k /= 2) {
            k_jfa_step_p<PLANAR><<<grid, 128, 0, st>>>(a, b, D, H, W, k);
            int32_t* t = a; a = b; b = t;
        }
        k_jfa_step_p<PLANAR><<<grid, 128, 0, st>>>(a, b, D, H, W, 1);
        k_jfa_finish_p<PLANAR><<<grid, 128, 0, st>>>(b, mask, D, H, W, out);
        return;
    }
    k_jfa_seed<PLANAR><<<grid1(n), 256, 0, st>>>(mask, D, H, W, a);
    for (; k >= 1; k /= 2) {
        k_jfa_step<PLANAR><<<grid1(n), 256, 0, st>>>(a, b, D, H, W, k);
        int32_t* t = a; a = b; b = t;
    }
    k_jfa_step<PLANAR><<<grid1(n), 256, 0, st>>>(a, b, D, H, W, 1);
    k_jfa_finish<PLANAR><<<grid1(n), 256, 0, st>>>(b, mask, D, H, W, out);
}

}  // namespace

extern "C" {

lbm_status lbm_nn_conv3d_fwd(const void* x, const int dims_in[3], int ci, const void* w, const float* bias, int co,
                             int ksize, int stride, int relu, void* y, float* y_f32, void* stream) {
    if (!x || !dims_in || !w || !y || !padded16(ci) || !padded16(co) || (ksize != 1 && ksize != 3) ||
        (stride != 1 && stride != 2) || (ksize == 1 && stride != 1) || !aligned16(x) || !aligned16(w) ||
        !aligned16(y) || (y_f32 && !aligned16(y_f32)))
        return report("lbm_nn_conv3d_fwd", cudaSuccess);
    const Conv g = make_conv(dims_in, ci, co, ksize, stride);
    const int64_t rows = (int64_t)g.Do * g.Ho * g.Wo;
    cudaError_t e;
    if (use_tc(g) && aligned16(x))
        e = lbm::conv3_tc(x, g.D, g.H, g.W, ci, w, bias, co, relu, y, y_f32, g.stride,
                          static_cast<cudaStream_t>(stream));
    else
        e = launch_gemm<0>(co, static_cast<const bf16*>(x), static_cast<const bf16*>(w), bias, static_cast<bf16*>(y),
                           y_f32, g, rows, ci, relu, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? LBM_OK : report("lbm_nn_conv3d_fwd", e);
}

lbm_status lbm_nn_set_conv_engine(int engine) {
    if (engine != LBM_NN_ENGINE_AUTO && engine != LBM_NN_ENGINE_MMA_SYNC)
        return report("lbm_nn_set_conv_engine", cudaSuccess);
    g_engine.store(engine);
    return LBM_OK;
}

lbm_status lbm_nn_conv_status(void) {
    unsigned f = 0;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = lbm::conv_tc_status(&f);
    if (e != cudaSuccess) return report("lbm_nn_conv_status", e);
    if (f) {
        lbm::set_last_global_error("lbm_nn_conv_status: a tensor-core convolution's bounded wait gave up");
        return LBM_ERR_CUDA;
    }
    return LBM_OK;
}

lbm_status lbm_nn_conv3d_bwd(const void* x, const int dims_in[3], int ci, const void* w, void* w_t, int co,
                             int ksize, int stride, const void* dy, void* dx, float* dw, float* db, void* stream) {
    if (!x || !dims_in || !w || !dy || !padded16(ci) || !padded16(co) || (ksize != 1 && ksize != 3) ||
        (stride != 1 && stride != 2) || (ksize == 1 && stride != 1) || (dx && !w_t) || !aligned16(x) ||
        !aligned16(w) || !aligned16(dy) || (dx && (!aligned16(dx) || !aligned16(w_t))))
        return report("lbm_nn_conv3d_bwd", cudaSuccess);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const Conv g = make_conv(dims_in, ci, co, ksize, stride);
    const int taps = ksize * ksize * ksize;
    const int64_t rows_out = (int64_t)g.Do * g.Ho * g.Wo, rows_in = (int64_t)g.D * g.H * g.W;
    cudaError_t e = cudaSuccess;
    if (dx && use_tc_dx(g) && aligned16(dy)) {
        // stride 1: dx is the forward convolution of dy with the flipped, transposed weights
        e = lbm::conv3_flip_transpose(w, w_t, co, ci, st);
        if (e == cudaSuccess) e = lbm::conv3_tc(dy, g.Do, g.Ho, g.Wo, co, w_t, nullptr, ci, 0, dx, nullptr, 1, st);
    } else if (dx) {
        const int64_t nw = (int64_t)co * taps * ci;
        k_transpose_w<<<grid1(nw), 256, 0, st>>>(static_cast<const bf16*>(w), static_cast<bf16*>(w_t), co, taps, ci);
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = launch_gemm<1>(ci, static_cast<const bf16*>(dy), static_cast<const bf16*>(w_t), nullptr,
                               static_cast<bf16*>(dx), nullptr, g, rows_in, co, 0, st);
    }
    if (e == cudaSuccess && dw && g.ks == 3 && g_engine.load() == LBM_NN_ENGINE_AUTO && aligned16(x) &&
        aligned16(dy) && lbm::conv3_wgrad_tc_applies(g.D, g.H, g.W, ci, co, g.stride)) {
        e = lbm::conv3_wgrad_tc(x, g.D, g.H, g.W, ci, dy, co, g.stride, dw, st);
    } else if (e == cudaSuccess && dw) {
        const bf16* xb = static_cast<const bf16*>(x);
        const bf16* dyb = static_cast<const bf16*>(dy);
        switch (co) {
            case 16: e = launch_wgrad_ci<16>(ci, xb, dyb, dw, g, rows_out, st); break;
            case 32: e = launch_wgrad_ci<32>(ci, xb, dyb, dw, g, rows_out, st); break;
            default: e = launch_wgrad_ci<64>(ci, xb, dyb, dw, g, rows_out, st); break;
        }
    }
    if (e == cudaSuccess && db) {
        k_bias_grad<<<(unsigned)lbm::ceil_div(rows_out, 256), 256, 0, st>>>(static_cast<const bf16*>(dy), db,
                                                                            rows_out, co);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? LBM_OK : report("lbm_nn_conv3d_bwd", e);
}

lbm_status lbm_nn_relu_bwd(const void* y, void* dy, int64_t n, void* stream) {
    if (!y || !dy || n < 0) return report("lbm_nn_relu_bwd", cudaSuccess);
    if (n == 0) return LBM_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n % 8 == 0 && aligned16(y) && aligned16(dy))
        k_relu_bwd_v8<<<grid1(n / 8), 256, 0, st>>>(static_cast<const uint4*>(y), static_cast<uint4*>(dy), n / 8);
    else
        k_relu_bwd<<<grid1(n), 256, 0, st>>>(static_cast<const bf16*>(y), static_cast<bf16*>(dy), n);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : report("lbm_nn_relu_bwd", e);
}

lbm_status lbm_nn_upsample2(const void* x, const int dims_in[3], int c, void* y, int adjoint, void* stream) {
    if (!x || !dims_in || !y || c <= 0) return report("lbm_nn_upsample2", cudaSuccess);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n = (int64_t)dims_in[0] * dims_in[1] * dims_in[2] * c;
    if (c % 8 == 0 && aligned16(x) && aligned16(y)) {
        const int c8 = c / 8;
        if (!adjoint)
            k_up2_v8<<<grid1(n), 256, 0, st>>>(static_cast<const uint4*>(x), static_cast<uint4*>(y), dims_in[0],
                                               dims_in[1], dims_in[2], c8);
        else
            k_up2_bwd_v8<<<grid1(n / 8), 256, 0, st>>>(static_cast<const uint4*>(x), static_cast<uint4*>(y),
                                                       dims_in[0], dims_in[1], dims_in[2], c8);
    } else if (!adjoint)
        k_up2<<<grid1(8 * n), 256, 0, st>>>(static_cast<const bf16*>(x), static_cast<bf16*>(y), dims_in[0],
                                            dims_in[1], dims_in[2], c);
    else  // x = gradient of the upsampled tensor, y = gradient of the coarse one (dims_in)
        k_up2_bwd<<<grid1(n), 256, 0, st>>>(static_cast<const bf16*>(x), static_cast<bf16*>(y), dims_in[0],
                                            dims_in[1], dims_in[2], c);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : report("lbm_nn_upsample2", e);
}

lbm_status lbm_nn_add(const void* a, const void* b, void* out, int64_t n, void* stream) {
    if (!a || !b || !out || n < 0) return report("lbm_nn_add", cudaSuccess);
    if (n == 0) return LBM_OK;
    if (n % 8 == 0 && aligned16(a) && aligned16(b) && aligned16(out))
        k_add_v8<<<grid1(n / 8), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            static_cast<const uint4*>(a), static_cast<const uint4*>(b), static_cast<uint4*>(out), n / 8);
    else
        k_add<<<grid1(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const bf16*>(a),
                                                                       static_cast<const bf16*>(b),
                                                                       static_cast<bf16*>(out), n);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : report("lbm_nn_add", e);
}

lbm_status lbm_nn_mse(const float* pred, const float* target, const uint8_t* mask, int64_t nvox, int c, int nc,
                      float inv_norm, void* dpred, float* loss, void* stream) {
    if (!pred || !target || !mask || !dpred || !loss || nvox < 0 || nc > c) return report("lbm_nn_mse", cudaSuccess);
    k_mse<<<grid1(nvox * c), 256, 0, static_cast<cudaStream_t>(stream)>>>(pred, target, mask, nvox, c, nc, inv_norm,
                                                                           static_cast<bf16*>(dpred), loss);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : report("lbm_nn_mse", e);
}

lbm_status lbm_nn_adam(float* w, void* w_bf16, const float* grad, float* m, float* v, int64_t n, float lr,
                       float beta1, float beta2, float eps, int64_t step, void* stream) {
    if (!w || !grad || !m || !v || n < 0 || step < 1) return report("lbm_nn_adam", cudaSuccess);
    if (n == 0) return LBM_OK;
    const float c1 = 1.f / (1.f - powf(beta1, (float)step)), c2 = 1.f / (1.f - powf(beta2, (float)step));
    k_adam<<<grid1(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(w, static_cast<bf16*>(w_bf16), grad, m, v, n,
                                                                    lr, beta1, beta2, eps, c1, c2);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : report("lbm_nn_adam", e);
}

lbm_status lbm_sdf_from_mask(const uint8_t* mask, const int dims[3], float* sdf, void* scratch, void* stream) {
    if (!mask || !dims || !sdf || !scratch || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0)
        return report("lbm_sdf_from_mask", cudaSuccess);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int D = dims[0], H = dims[1], W = dims[2];
    jfa<false>(mask, D, H, W, static_cast<int32_t*>(scratch), sdf, st);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : report("lbm_sdf_from_mask", e);
}

lbm_status lbm_ws_prior(const uint8_t* mask, const int dims[3], double inlet, double nu, float* dist, float* drho,
                        float* uz, void* scratch, void* stream) {
    if (!mask || !dims || !dist || !drho || !uz || !scratch || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0)
        return report("lbm_ws_prior", cudaSuccess);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int D = dims[0], H = dims[1], W = dims[2];
    const int64_t n = (int64_t)D * H * W;
    int32_t* jf = static_cast<int32_t*>(scratch);
    float* R = reinterpret_cast<float*>(jf + 2 * n);
    float* peak = R + D;
    float* tail = peak + D;
    jfa<true>(mask, D, H, W, jf, dist, st);
    k_slice_max<<<D, 256, 0, st>>>(dist, H * W, R);
    k_prior_axis<<<1, 1, 0, st>>>(R, D, inlet, nu, peak, tail);
    k_prior_fill<<<grid1(n), 256, 0, st>>>(mask, dist, R, peak, tail, n, H * W, drho, uz);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : report("lbm_ws_prior", e);
}

lbm_status lbm_ws_smooth(const uint8_t* mask, const int dims[3], float* v, float* tmp, int rounds, void* stream) {
    if (!mask || !dims || !v || !tmp || rounds < 0 || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0)
        return report("lbm_ws_smooth", cudaSuccess);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int D = dims[0], H = dims[1], W = dims[2];
    const int64_t n = (int64_t)D * H * W;
    float* src = v;
    float* dst = tmp;
    for (int r = 0; r < rounds; ++r)
        for (int a = 0; a < 3; ++a) {  // z, y, x in turn
            k_smooth_axis<<<grid1(n), 256, 0, st>>>(mask, src, dst, D, H, W, a);
            float* t = src; src = dst; dst = t;
        }
    if (src != v) cudaMemcpyAsync(v, src, sizeof(float) * n, cudaMemcpyDeviceToDevice, st);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : report("lbm_ws_smooth", e);
}

lbm_status lbm_ws_features(const float* sdf, const uint8_t* mask, const float* uz_p, const float* drho_p,
                           const int dims[3], float sdf_scale, float mean_in, float period_in, float inlet,
                           float rho_scale, void* x, void* stream) {
    if (!sdf || !mask || !uz_p || !drho_p || !dims || !x || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0 ||
        !(inlet != 0.f) || !aligned16(x))
        return report("lbm_ws_features", cudaSuccess);
    const int64_t hw = (int64_t)dims[1] * dims[2], n = (int64_t)dims[0] * hw;
    k_ws_features<<<grid1(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        sdf, mask, uz_p, drho_p, n, hw, dims[0], sdf_scale, mean_in, period_in, inlet, rho_scale,
        static_cast<uint4*>(x));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : report("lbm_ws_features", e);
}

lbm_status lbm_ws_output(const float* y, int c, const uint8_t* mask, const float* drho_p, const float* uz_p,
                         int64_t nvox, float inlet, float rho_scale, float u_scale, float* fields, void* stream) {
    if (!y || c < 4 || !mask || !drho_p || !uz_p || nvox < 0 || !fields) return report("lbm_ws_output", cudaSuccess);
    if (nvox == 0) return LBM_OK;
    k_ws_output<<<grid1(nvox), 256, 0, static_cast<cudaStream_t>(stream)>>>(y, c, mask, drho_p, uz_p, nvox, inlet,
                                                                            rho_scale, u_scale, fields);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : report("lbm_ws_output", e);
}

lbm_status lbm_ws_gather(const float* fields, int64_t nvox, const int64_t* idx, int64_t nact, float* rho, float* u,
                         void* stream) {
    if (!fields || nvox < 0 || (nact > 0 && (!idx || !rho || !u)) || nact < 0) return report("lbm_ws_gather", cudaSuccess);
    if (nact == 0) return LBM_OK;
    k_ws_gather<<<grid1(nact), 256, 0, static_cast<cudaStream_t>(stream)>>>(fields, nvox, idx, nact, rho, u);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : report("lbm_ws_gather", e);
}

}  // extern "C"
