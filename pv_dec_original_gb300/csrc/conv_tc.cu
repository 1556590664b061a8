// 3x3x3 convolutions (stride 1, padding 1) of the warm-start network on the
// fifth-generation tensor cores: tcgen05.mma with the accumulators in tensor
// memory.  No reference counterpart (the reference always starts from rest).
//
// One CTA (4 warps) computes an output block of 8 (x) x 16 (y) x 4 (z)
// voxels and all co output channels.  Per 16-channel chunk of the input it
// stages, with cp.async, the input block plus its one-voxel halo (10 x 18 x
// 6 voxels) and the chunk of all 27 taps' weights in shared memory, in the
// canonical no-swizzle K-major layout of the MMA operands: core matrices of
// 8 rows x 16 bytes (8 channels), rows 16 bytes apart.
//   input block: [channel half k (2)][z][y][x][8 channels]
//   weights:     [tap][co / 8][channel half k][co % 8][8 channels]
// The 128 output voxels of one z plane (8 x by 16 y) are the M = 128 rows
// of one MMA: row m = 8 y + x, so rows m..m+7 are 8 consecutive x (one core
// matrix) and the 16 groups of 8 rows are 16 y rows, one input row (10
// voxels, 160 bytes) apart -- the stride-dimension offset.  The two channel
// halves of the K = 16 slice are one block plane apart -- the leading-
// dimension offset.  A tap (tx, ty, tz) is then just the descriptor's start
// address moved by tx + 10 (ty + 18 tz) voxels: the 27 taps reuse the staged
// block with no copies.  One elected thread issues the 4 planes x 27 taps
// MMAs of a chunk (M = 128, N = co, K = 16, BF16 x BF16 -> FP32) into four
// accumulators of co tensor-memory columns each and commits them to an
// mbarrier; every wait is bounded.  The epilogue reads the accumulators
// with tcgen05.ld (warp w owns tensor-memory lanes 32 w .. 32 w + 31, i.e.
// rows y = 4 w .. 4 w + 3), adds the bias, applies ReLU and stores BF16
// (and FP32 when asked) channels-last.
#include <cuda_bf16.h>

#include <cstdint>

#include "lbm_internal.cuh"

namespace {

using bf16 = __nv_bfloat16;

constexpr int TX = 8, TY = 16, TZ = 4;
constexpr int XB = TX + 2, YB = TY + 2, ZB = TZ + 2;
constexpr int BLOCK_VOX = XB * YB * ZB;          // 1080 staged voxels
constexpr int HALF_BYTES = BLOCK_VOX * 16;        // one channel half (8 channels) of the block
constexpr int TILE_BYTES = 2 * HALF_BYTES;        // 34,560
constexpr int kThreads = 128;
constexpr long kWaitLimit = 1L << 20;  // mbarrier polls (each bounded by the hardware's own time limit)

// Set when a bounded wait gave up (read and cleared by conv_tc_status).
__device__ unsigned g_conv_tc_flags;

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, no swizzle: start address, leading-
// dimension (K-direction core matrix) byte offset, stride-dimension (next 8
// rows) byte offset, descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (long k = 0; k < kWaitLimit; ++k) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

template <int CO>
__host__ __device__ constexpr int smem_bytes() {
    return TILE_BYTES + 27 * CO * 32 + 16;  // block, weights, mbarrier + tensor-memory address
}

template <int CO>
__host__ __device__ constexpr uint32_t tmem_cols() {
    return TZ * CO < 32 ? 32u : (uint32_t)(TZ * CO);  // a power of two for CO in {16, 32, 64}
}

// x [D][H][W][ci], w [co][27][ci], y [D][H][W][co]; D % 4 == 0, H % 16 == 0, W % 8 == 0.
template <int CO>
__global__ void __launch_bounds__(kThreads) k_conv3_tc(const bf16* __restrict__ x, const bf16* __restrict__ w,
                                                       const float* __restrict__ bias, bf16* __restrict__ y,
                                                       float* __restrict__ y32, int D, int H, int W, int ci,
                                                       int relu) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char* tile = smem;
    unsigned char* wsm = smem + TILE_BYTES;
    uint64_t* bar = reinterpret_cast<uint64_t*>(wsm + 27 * CO * 32);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nbx = W / TX, nby = H / TY;
    const int bx = blockIdx.x % nbx, by = (blockIdx.x / nbx) % nby, bz = blockIdx.x / (nbx * nby);
    const int x0 = bx * TX, y0 = by * TY, z0 = bz * TZ;
    constexpr uint32_t NCOL = tmem_cols<CO>();

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tslot)),
                     "r"(NCOL)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(saddr(bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    const uint32_t tile_a = saddr(tile), w_a = saddr(wsm);
    constexpr uint32_t IDESC = idesc_bf16(128, CO);
    bool ok = true;
    const int chunks = ci / 16;
    int c = 0;
    for (; c < chunks && ok; ++c) {
        // stage the input block (zero outside the grid: the padding) and the weights of this chunk
        for (int i = tid; i < 2 * BLOCK_VOX; i += kThreads) {
            const int v = i >> 1, k = i & 1;
            const int xx = v % XB, yy = (v / XB) % YB, zz = v / (XB * YB);
            const int gx = x0 - 1 + xx, gy = y0 - 1 + yy, gz = z0 - 1 + zz;
            const bool in = gx >= 0 && gy >= 0 && gz >= 0 && gx < W && gy < H && gz < D;
            const bf16* src = in ? x + (((int64_t)gz * H + gy) * W + gx) * ci + c * 16 + k * 8 : x;
            cp_async16(tile_a + k * HALF_BYTES + v * 16, src, in);
        }
        for (int i = tid; i < 27 * CO * 2; i += kThreads) {
            const int k = i & 1, n = (i >> 1) % CO, t = (i >> 1) / CO;
            cp_async16(w_a + t * (CO * 32) + (n >> 3) * 256 + k * 128 + (n & 7) * 16,
                       w + ((int64_t)n * 27 + t) * ci + c * 16 + k * 8, true);
        }
        asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int z = 0; z < TZ; ++z) {
                for (int t = 0; t < 27; ++t) {
                    const int tz = t / 9, ty = (t / 3) % 3, tx = t % 3;
                    const uint32_t a = tile_a + (((z + tz) * YB + ty) * XB + tx) * 16;
                    const uint64_t ad = smem_desc(a, HALF_BYTES, XB * 16);
                    const uint64_t bd = smem_desc(w_a + t * (CO * 32), 128, 256);
                    mma_bf16(tmem + (uint32_t)(z * CO), ad, bd, IDESC, (c > 0 || t > 0) ? 1u : 0u);
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             saddr(bar))
                         : "memory");
        }
        // every thread: the MMAs of this chunk are done (they read the staged block)
        ok = mbar_wait(saddr(bar), (uint32_t)(c & 1));
        ok = __syncthreads_and(ok);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        // epilogue: warp w reads lanes 32 w .. 32 w + 31 = rows y = 4 w + lane / 8, x = lane % 8
        const int m = 32 * warp + lane;
        const int gx = x0 + (m & 7), gy = y0 + (m >> 3);
        for (int z = 0; z < TZ; ++z) {
            const int64_t vox = ((int64_t)(z0 + z) * H + gy) * W + gx;
#pragma unroll
            for (int c16 = 0; c16 < CO / 16; ++c16) {
                float v[16];
                tc_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(z * CO + c16 * 16), v);
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                    v[k] += bias ? bias[c16 * 16 + k] : 0.f;
                    if (relu) v[k] = fmaxf(v[k], 0.f);
                }
                uint4 p[2];
                __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(p);
#pragma unroll
                for (int k = 0; k < 8; ++k) h[k] = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
                uint4* dst = reinterpret_cast<uint4*>(y + vox * CO + c16 * 16);
                dst[0] = p[0];
                dst[1] = p[1];
                if (y32) {
                    float4* d32 = reinterpret_cast<float4*>(y32 + vox * CO + c16 * 16);
#pragma unroll
                    for (int k = 0; k < 4; ++k) d32[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
                }
            }
        }
    } else {
        // the wait of chunk c - 1 gave up: record it, wait (bounded) once
        // more for that chunk's MMAs, then release the tensor memory
        if (tid == 0) atomicOr(&g_conv_tc_flags, 1u);
        mbar_wait(saddr(bar), (uint32_t)((c - 1) & 1));
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOL) : "memory");
}

// Wt [ci][t][co] = W [co][26 - t][ci]: the input gradient of a stride-1
// convolution is the forward convolution of dy with these weights.
__global__ void k_flip_transpose(const bf16* __restrict__ w, bf16* __restrict__ wt, int co, int ci) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)co * 27 * ci) return;
    const int c = (int)(e % ci), t = (int)((e / ci) % 27), o = (int)(e / ((int64_t)ci * 27));
    wt[((int64_t)c * 27 + (26 - t)) * co + o] = w[e];
}

template <int CO>
cudaError_t launch_co(const bf16* x, const bf16* w, const float* bias, bf16* y, float* y32, int D, int H, int W,
                      int ci, int relu, cudaStream_t st) {
    constexpr int bytes = smem_bytes<CO>();
    static_assert(bytes <= 227 * 1024, "shared memory");
    cudaError_t e = cudaFuncSetAttribute(k_conv3_tc<CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    const int64_t blocks = (int64_t)(W / TX) * (H / TY) * (D / TZ);
    k_conv3_tc<CO><<<(unsigned)blocks, kThreads, bytes, st>>>(x, w, bias, y, y32, D, H, W, ci, relu);
    return cudaGetLastError();
}

// Resident CTAs per SM times their tensor-memory columns must fit the 512
// columns of an SM (an allocation that cannot be met waits for another
// CTA's release): shared memory bounds the residency below that here --
// (co = 16) 4 x 64, (32) 3 x 128, (64) 2 x 256 columns.
static_assert((227 * 1024 / smem_bytes<16>()) * tmem_cols<16>() <= 512, "tensor memory (co 16)");
static_assert((227 * 1024 / smem_bytes<32>()) * tmem_cols<32>() <= 512, "tensor memory (co 32)");
static_assert((227 * 1024 / smem_bytes<64>()) * tmem_cols<64>() <= 512, "tensor memory (co 64)");

}  // namespace

namespace lbm {

bool conv3_tc_applies(int D, int H, int W, int ci, int co) {
    const bool ch = (ci == 16 || ci == 32 || ci == 64) && (co == 16 || co == 32 || co == 64);
    return ch && D > 0 && H > 0 && W > 0 && D % TZ == 0 && H % TY == 0 && W % TX == 0;
}

cudaError_t conv3_tc(const void* x, int D, int H, int W, int ci, const void* w, const float* bias, int co, int relu,
                     void* y, float* y32, cudaStream_t st) {
    const bf16* xb = static_cast<const bf16*>(x);
    const bf16* wb = static_cast<const bf16*>(w);
    bf16* yb = static_cast<bf16*>(y);
    switch (co) {
        case 16: return launch_co<16>(xb, wb, bias, yb, y32, D, H, W, ci, relu, st);
        case 32: return launch_co<32>(xb, wb, bias, yb, y32, D, H, W, ci, relu, st);
        default: return launch_co<64>(xb, wb, bias, yb, y32, D, H, W, ci, relu, st);
    }
}

cudaError_t conv3_flip_transpose(const void* w, void* wt, int co, int ci, cudaStream_t st) {
    const int64_t n = (int64_t)co * 27 * ci;
    k_flip_transpose<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(static_cast<const bf16*>(w), static_cast<bf16*>(wt),
                                                               co, ci);
    return cudaGetLastError();
}

cudaError_t conv_tc_status(unsigned* flags) {
    cudaError_t e = cudaMemcpyFromSymbol(flags, g_conv_tc_flags, sizeof(unsigned));
    if (e != cudaSuccess) return e;
    const unsigned zero = 0;
    return cudaMemcpyToSymbol(g_conv_tc_flags, &zero, sizeof(unsigned));
}

}  // namespace lbm
