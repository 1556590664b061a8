// 3x3x3 convolutions (padding 1, stride 1 or 2) of the warm-start network
// on the fifth-generation tensor cores: tcgen05.mma with the accumulators in
// tensor memory.  No reference counterpart (the reference always starts
// from rest).
//
// One CTA (4 warps) computes an output block of 8 (x) x 16 (y) x TZ (z)
// voxels (TZ = 4 at stride 1, 1 at stride 2) and all co output channels.
// Per 16-channel chunk of the input it stages the input voxels the block
// reads (the block plus its one-voxel halo, 10 x 18 x 6 at stride 1;
// 17 x 33 x 3 at stride 2) with tensor-memory-access copies
// (cp.async.bulk.tensor, one per channel half and x parity, zero-filled
// outside the grid: the padding; at stride 2 an element stride of 2 along x
// picks one parity) completing on an mbarrier, and the chunk of all 27
// taps' weights with cp.async, in the canonical no-swizzle K-major layout
// of the MMA operands: core matrices of 8 rows x 16 bytes (8 channels),
// rows 16 bytes apart.
//   input:   [channel half k (2)][x parity p (S)][z][y][x / S][8 channels]
//            (a parity plane padded to 128 bytes)
//   weights: [tap block][co / 8][channel half k][co % 8][8 channels]
//            (tap block: weight_block)
// The 128 output voxels of one z plane (8 x by 16 y) are the M = 128 rows
// of one MMA: row m = 8 y + x.  Output x reads input x = S x + tx - 1, so
// with the input's x split by parity (stride 2: even and odd columns in
// separate runs) rows m..m+7 are 8 consecutive staged voxels -- one core
// matrix -- and the 16 groups of 8 rows are 16 output rows, S input rows
// apart: the stride-dimension offset.  The two channel halves of the K = 16
// slice are one staged block apart: the leading-dimension offset.  A tap
// (tx, ty, tz) is just the descriptor's start address (parity tx mod S,
// column tx / S, row ty, plane S z + tz): the 27 taps reuse the staged block
// with no copies.  One elected thread issues the MMAs of a chunk (M = 128,
// K = 16, BF16 x BF16 -> FP32) into TZ accumulators of co tensor-memory
// columns each and commits them to an mbarrier; every wait is bounded.  At
// stride 2: TZ x 27 MMAs of N = co.  At stride 1 the accumulators of the
// TZ planes are adjacent column ranges and one staged plane feeds up to
// three output planes (through taps tz = 2, 1, 0), so each (ty, tx) takes
// one MMA per staged plane with N = 1-3 co: 9 x 6 = 54 MMAs instead of
// 4 x 27, each reading its A operand once.  The epilogue reads the
// accumulators with tcgen05.ld (warp w owns tensor-memory lanes 32 w ..
// 32 w + 31, i.e. rows y = 4 w .. 4 w + 3), adds the bias, applies ReLU and
// stores BF16 (and FP32 when asked) channels-last.
//
// Bound: the A operand (the staged input, 4 KB per MMA) is read from shared
// memory by every MMA; at co = 16 that operand traffic, not the tensor
// pipe, sets the rate (see the convolution profile).
#include <cuda.h>
#include <cuda_bf16.h>

#include <atomic>
#include <cstdint>

#include "lbm_internal.cuh"

namespace {

using bf16 = __nv_bfloat16;

constexpr int TX = 8, TY = 16;
constexpr int kThreads = 128;
constexpr long kWaitLimit = 1L << 20;  // mbarrier polls (each bounded by the hardware's own time limit)

// Staged geometry per stride: output planes per CTA, staged planes, rows,
// x parities and voxels per parity run.
template <int S>
struct Geo {
    static constexpr int TZ = S == 1 ? 4 : 1;
    static constexpr int ZB = S * (TZ - 1) + 3;
    static constexpr int YB = S * (TY - 1) + 3;
    static constexpr int PAR = S;
    static constexpr int XH = S == 1 ? TX + 2 : TX + 1;        // stride 2: input x = 2 xh + p, rows 0..16
    static constexpr int PLANE_RAW = ZB * YB * XH * 16;         // bytes one copy writes (17,280 / 14,256)
    static constexpr int PLANE = (PLANE_RAW + 127) / 128 * 128;  // copy destinations 128-byte aligned
    static constexpr int HALF = PAR * PLANE;                     // bytes of one channel half
    static constexpr int TILE = 2 * HALF;
    static constexpr int TX_BYTES = 2 * PAR * PLANE_RAW;         // bytes the copies of a chunk deliver
};

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

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// 4-D tiled tensor copy global -> shared completing on an mbarrier;
// coordinates innermost first (channel, x, y, z).
__device__ __forceinline__ void tma_load4(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                          uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
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

template <int S, int CO>
__host__ __device__ constexpr int smem_bytes() {
    return Geo<S>::TILE + 27 * CO * 32 + 32;  // input, weights, two mbarriers + tensor-memory address
}

template <int S, int CO>
__host__ __device__ constexpr uint32_t tmem_cols() {
    return Geo<S>::TZ * CO < 32 ? 32u : (uint32_t)(Geo<S>::TZ * CO);  // a power of two for CO in {16, 32, 64}
}

// Shared-memory block of tap t = 9 tz + 3 ty + tx in the staged weights.
// Stride 1 groups the three z taps of each (ty, tx) in the order tz = 2, 1,
// 0, so that one MMA of N = 3 co takes all three: staged plane zz feeds
// output planes zz - 2, zz - 1, zz through taps tz = 2, 1, 0, and the
// accumulators of those planes are the adjacent tensor-memory column
// ranges (z co .. z co + co - 1 for plane z).  Stride 2 keeps tap order.
template <int S>
__host__ __device__ constexpr int weight_block(int t) {
    return S == 1 ? ((t / 3) % 3 * 3 + t % 3) * 3 + (2 - t / 9) : t;
}

// x [Di][Hi][Wi][ci] (read through `map`: the 4-D tensor map of x, box
// 8 channels x (XH, or 2 XH with element stride 2) x YB x ZB), w [co][27][ci],
// y [Do][Ho][Wo][co] with Do = Di / S etc.; Do % TZ == 0, Ho % 16 == 0,
// Wo % 8 == 0 (the launcher checks).
template <int S, int CO>
__global__ void __launch_bounds__(kThreads) k_conv3_tc(const __grid_constant__ CUtensorMap map,
                                                       const bf16* __restrict__ w, const float* __restrict__ bias,
                                                       bf16* __restrict__ y, float* __restrict__ y32, int Do, int Ho,
                                                       int Wo, int ci, int relu) {
    using G = Geo<S>;
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char* tile = smem;
    unsigned char* wsm = smem + G::TILE;
    uint64_t* bar = reinterpret_cast<uint64_t*>(wsm + 27 * CO * 32);  // [0] MMAs done, [1] input copies done
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
    volatile int& copy_failed = *reinterpret_cast<volatile int*>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nbx = Wo / TX, nby = Ho / TY;
    const int bx = blockIdx.x % nbx, by = (blockIdx.x / nbx) % nby, bz = blockIdx.x / (nbx * nby);
    const int x0 = bx * TX, y0 = by * TY, z0 = bz * G::TZ;
    constexpr uint32_t NCOL = tmem_cols<S, CO>();

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tslot)),
                     "r"(NCOL)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(saddr(bar), 1);
        mbar_init(saddr(bar + 1), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        copy_failed = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    const uint32_t tile_a = saddr(tile), w_a = saddr(wsm);
    constexpr uint32_t IDESC = idesc_bf16(128, CO);
    constexpr uint32_t SBO = S * G::XH * 16;  // S input rows per output row
    bool ok = true;
    const int chunks = ci / 16;
    int c = 0;
    for (; c < chunks && ok; ++c) {
        // the input voxels of this chunk by tensor copies (zero outside the grid: the padding)
        if (tid == 0) {
            mbar_expect_tx(saddr(bar + 1), (uint32_t)G::TX_BYTES);
            for (int k = 0; k < 2; ++k)
                for (int p = 0; p < G::PAR; ++p)
                    tma_load4(tile_a + k * G::HALF + p * G::PLANE, &map, c * 16 + k * 8, S * x0 - 1 + p,
                              S * y0 - 1, S * z0 - 1, saddr(bar + 1));
        }
        // the weights of this chunk
        for (int i = tid; i < 27 * CO * 2; i += kThreads) {
            const int k = i & 1, n = (i >> 1) % CO, t = (i >> 1) / CO;
            cp_async16(w_a + weight_block<S>(t) * (CO * 32) + (n >> 3) * 256 + k * 128 + (n & 7) * 16,
                       w + ((int64_t)n * 27 + t) * ci + c * 16 + k * 8, true);
        }
        asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            if (mbar_wait(saddr(bar + 1), (uint32_t)(c & 1))) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                if constexpr (S == 1) {
                    // per (ty, tx): one MMA per staged plane zz, into output
                    // planes lo .. hi - 1 (N = (hi - lo) co) with the taps
                    // tz = zz - lo .. zz - hi + 1 (weight_block); 54 MMAs
                    // instead of 108, each reading its A operand once.  The
                    // first (ty, tx) of the first chunk starts with planes 2
                    // and 5, whose output ranges (0..2 and 3) cover every
                    // accumulator once: they initialise it.
                    static_assert(G::TZ == 4 && G::ZB == 6, "merged z taps: 4 output planes, 6 staged");
                    constexpr int kOrder[6] = {2, 5, 0, 1, 3, 4};
                    constexpr uint32_t ID1 = idesc_bf16(128, CO), ID2 = idesc_bf16(128, 2 * CO),
                                       ID3 = idesc_bf16(128, 3 * CO);
                    for (int u = 0; u < 9; ++u) {
                        const int ty = u / 3, tx = u % 3;
                        for (int j = 0; j < 6; ++j) {
                            const int zz = kOrder[j];
                            const int lo = zz > 2 ? zz - 2 : 0, hi = zz + 1 < G::TZ ? zz + 1 : G::TZ;
                            const int np = hi - lo, b0 = 2 - (zz - lo);
                            const uint32_t a = tile_a + ((zz * G::YB + ty) * G::XH + tx) * 16;
                            const uint64_t ad = smem_desc(a, G::HALF, SBO);
                            const uint64_t bd = smem_desc(w_a + (u * 3 + b0) * (CO * 32), 128, 256);
                            mma_bf16(tmem + (uint32_t)(lo * CO), ad, bd, np == 3 ? ID3 : (np == 2 ? ID2 : ID1),
                                     (c > 0 || u > 0 || j >= 2) ? 1u : 0u);
                        }
                    }
                } else {
                    for (int z = 0; z < G::TZ; ++z) {
                        for (int t = 0; t < 27; ++t) {
                            const int tz = t / 9, ty = (t / 3) % 3, tx = t % 3;
                            const int zz = S * z + tz, p = tx % S, xo = tx / S;
                            const uint32_t a = tile_a + p * G::PLANE + ((zz * G::YB + ty) * G::XH + xo) * 16;
                            const uint64_t ad = smem_desc(a, G::HALF, SBO);
                            const uint64_t bd = smem_desc(w_a + weight_block<S>(t) * (CO * 32), 128, 256);
                            mma_bf16(tmem + (uint32_t)(z * CO), ad, bd, IDESC, (c > 0 || t > 0) ? 1u : 0u);
                        }
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 saddr(bar))
                             : "memory");
            } else {
                copy_failed = 1;
            }
        }
        __syncthreads();
        if (copy_failed) {
            // the copies did not complete in time: record it and wait
            // (bounded) once more before the shared memory is released
            if (tid == 0) {
                atomicOr(&g_conv_tc_flags, 2u);
                mbar_wait(saddr(bar + 1), (uint32_t)(c & 1));
            }
            ok = false;
            c = -1;  // no MMAs of this chunk to wait for; those of earlier chunks are done
            break;
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
        for (int z = 0; z < G::TZ; ++z) {
            const int64_t vox = ((int64_t)(z0 + z) * Ho + gy) * Wo + gx;
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
    } else if (c > 0) {
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

// ---------------------------------------------------------------------------
// Weight gradient dW[o][t][c] += sum over output voxels m of
// dY[m][o] X[src(m, t)][c] (stride 1 or 2) on tcgen05.  GEMM rows are the
// 27 ci (tap, input channel) pairs R = t ci + c in tiles of 128 (M), the
// columns the co output channels (N), and K = 16 output voxels of one x-row
// an MMA (Wo % 16 == 0).  Per 16-voxel slice the CTA stages, with cp.async,
// the im2col rows of its tiles -- for every (tap, 8-channel group) the 16
// voxels' source values, zero where the tap falls outside the grid -- and
// dY of the 16 voxels, both MN-major: a core matrix is 8 voxels x 8
// channels, 128 contiguous bytes; the next 8 rows (channels) lie 256 bytes
// on, the next 8 voxels 128.  Two stages: the copies of slice k + 1 overlap
// the MMAs of slice k (an mbarrier per stage, every wait bounded).  The
// tiles of a CTA accumulate in tensor memory over its share of the slices
// (CTAs along y take different tiles); the epilogue adds them to dW with
// FP32 atomics.
constexpr int kTileBytes = 128 * 32;  // one 128-row x 16-voxel BF16 tile

__host__ __device__ constexpr uint32_t idesc_bf16_mn(int m, int n) {
    return idesc_bf16(m, n) | (1u << 15) | (1u << 16);  // A and B MN-major
}

template <int CO>
__global__ void __launch_bounds__(kThreads) k_conv3_wgrad_tc(const bf16* __restrict__ x, const bf16* __restrict__ dy,
                                                             float* __restrict__ dw, int Di, int Hi, int Wi, int Do,
                                                             int Ho, int Wo, int ci, int S, int tpg, int ncols,
                                                             int slices_per_cta, int nslices) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int RT = (27 * ci + 127) / 128;
    const int tile0 = blockIdx.y * tpg;
    const int ntiles = min(tpg, RT - tile0);
    const int stage_bytes = tpg * kTileBytes + CO * 32;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * stage_bytes);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int s_begin = blockIdx.x * slices_per_cta;
    const int s_end = min(nslices, s_begin + slices_per_cta);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tslot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(saddr(bar), 1);
        mbar_init(saddr(bar + 1), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;
    const uint32_t smem_a = saddr(smem);
    const int xs = Wo / 16;  // slices per output row

    // one slice's copies into stage b
    auto stage = [&](int sl, int b) {
        const uint32_t a_base = smem_a + b * stage_bytes, b_base = a_base + tpg * kTileBytes;
        const int row = sl / xs, ox0 = (sl - row * xs) * 16;
        const int oy = row % Ho, oz = row / Ho;
        const int64_t m0 = ((int64_t)oz * Ho + oy) * Wo + ox0;
        for (int i = tid; i < (CO / 8) * 16; i += kThreads) {
            const int og = i >> 4, v = i & 15;
            cp_async16(b_base + og * 256 + v * 16, dy + (m0 + v) * CO + og * 8, true);
        }
        for (int i = tid; i < ntiles * 256; i += kThreads) {
            const int lg = i >> 4, v = i & 15;
            const int R = (tile0 * 16 + lg) * 8;  // first row of this 8-row group
            const int t = R / ci, cg = (R - t * ci) >> 3;
            const int tz = t / 9, ty = (t / 3) % 3, tx = t % 3;
            const int ix = S * (ox0 + v) + tx - 1, iy = S * oy + ty - 1, iz = S * oz + tz - 1;
            const bool in = t < 27 && ix >= 0 && iy >= 0 && iz >= 0 && ix < Wi && iy < Hi && iz < Di;
            const bf16* src = in ? x + (((int64_t)iz * Hi + iy) * Wi + ix) * ci + cg * 8 : x;
            cp_async16(a_base + lg * 256 + v * 16, src, in);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };

    constexpr uint32_t IDESC = idesc_bf16_mn(128, CO);
    bool ok = true;
    uint32_t uses[2] = {0u, 0u};
    if (s_begin < s_end) stage(s_begin, 0);
    int sl = s_begin;
    for (; sl < s_end && ok; ++sl) {
        const int b = (sl - s_begin) & 1;
        if (sl + 1 < s_end) {
            // the other stage is free once the MMAs of the previous slice are done
            if (sl > s_begin) ok = mbar_wait(saddr(bar + (b ^ 1)), (uses[b ^ 1] - 1) & 1);
            ok = __syncthreads_and(ok);
            if (!ok) break;
            stage(sl + 1, b ^ 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a_base = smem_a + b * stage_bytes, b_base = a_base + tpg * kTileBytes;
            const uint64_t bd = smem_desc(b_base, 128, 256);
            for (int j = 0; j < ntiles; ++j)
                mma_bf16(tmem + (uint32_t)(j * CO), smem_desc(a_base + j * kTileBytes, 128, 256), bd, IDESC,
                         sl > s_begin ? 1u : 0u);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             saddr(bar + b))
                         : "memory");
        }
        ++uses[b];
    }
    // the MMAs of the last slice (each stage's last use) are done
    if (ok && s_end > s_begin) {
        const int bl = (s_end - 1 - s_begin) & 1;
        ok = mbar_wait(saddr(bar + bl), (uses[bl] - 1) & 1);
    }
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok && s_end > s_begin) {
        for (int j = 0; j < ntiles; ++j) {
            const int R = (tile0 + j) * 128 + 32 * warp + lane;
            const int t = R / ci, c = R - t * ci;
#pragma unroll
            for (int c16 = 0; c16 < CO / 16; ++c16) {
                float v[16];
                tc_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(j * CO + c16 * 16), v);
                if (t < 27) {
#pragma unroll
                    for (int k = 0; k < 16; ++k) atomicAdd(dw + ((int64_t)(c16 * 16 + k) * 27 + t) * ci + c, v[k]);
                }
            }
        }
    } else if (!ok) {
        // a wait gave up: record it, wait (bounded) for both stages' MMAs, release the tensor memory
        if (tid == 0) atomicOr(&g_conv_tc_flags, 1u);
        for (int b = 0; b < 2; ++b)
            if (uses[b]) mbar_wait(saddr(bar + b), (uses[b] - 1) & 1);
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

template <int CO>
cudaError_t launch_wgrad_co(const bf16* x, const bf16* dy, float* dw, int Di, int Hi, int Wi, int ci, int S,
                            cudaStream_t st) {
    const int Do = (Di - 1) / S + 1, Ho = (Hi - 1) / S + 1, Wo = (Wi - 1) / S + 1;
    const int RT = (27 * ci + 127) / 128;
    const int tpg_max = 256 / CO;  // tensor-memory columns of a CTA <= 256
    const int groups = (RT + tpg_max - 1) / tpg_max;
    const int tpg = (RT + groups - 1) / groups;
    int ncols = 32;
    while (ncols < tpg * CO) ncols *= 2;
    const int nslices = (int)((int64_t)Do * Ho * Wo / 16);
    const int want = 4 * 152 / groups > 1 ? 4 * 152 / groups : 1;
    const int spc = (nslices + want - 1) / want;
    const int nx = (nslices + spc - 1) / spc;
    // shared memory: two stages, two mbarriers and the tensor-memory slot,
    // padded so that at most 512 / ncols CTAs reside on an SM (their
    // tensor memory then always fits)
    const int actual = 2 * (tpg * kTileBytes + CO * 32) + 32;
    const int per_sm = 512 / ncols;
    int bytes = 233472 / (per_sm + 1) + 1024;
    if (bytes < actual) bytes = actual;
    cudaError_t e =
        cudaFuncSetAttribute(k_conv3_wgrad_tc<CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    k_conv3_wgrad_tc<CO><<<dim3((unsigned)nx, (unsigned)groups), kThreads, bytes, st>>>(
        x, dy, dw, Di, Hi, Wi, Do, Ho, Wo, ci, S, tpg, ncols, spc, nslices);
    return cudaGetLastError();
}

// Wt [ci][t][co] = W [co][26 - t][ci]: the input gradient of a stride-1
// convolution is the forward convolution of dy with these weights.
__global__ void k_flip_transpose(const bf16* __restrict__ w, bf16* __restrict__ wt, int co, int ci) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)co * 27 * ci) return;
    const int c = (int)(e % ci), t = (int)((e / ci) % 27), o = (int)(e / ((int64_t)ci * 27));
    wt[((int64_t)c * 27 + (26 - t)) * co + o] = w[e];
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library), looked up once.
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_tiled() {
    static std::atomic<EncodeTiled> fn{nullptr};
    EncodeTiled f = fn.load(std::memory_order_acquire);
    if (!f) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        f = reinterpret_cast<EncodeTiled>(p);
        fn.store(f, std::memory_order_release);
    }
    return f;
}

// The tensor map of x [Di][Hi][Wi][ci] BF16 for stride S: box 8 channels x
// XH voxels along x (stride 2: 2 XH with element stride 2, one parity) x YB
// x ZB, zero fill outside the tensor.
template <int S>
cudaError_t input_map(CUtensorMap* map, const bf16* x, int Di, int Hi, int Wi, int ci) {
    using G = Geo<S>;
    EncodeTiled f = encode_tiled();
    if (!f) return cudaErrorNotSupported;
    const cuuint64_t dims[4] = {(cuuint64_t)ci, (cuuint64_t)Wi, (cuuint64_t)Hi, (cuuint64_t)Di};
    const cuuint64_t strides[3] = {(cuuint64_t)ci * 2, (cuuint64_t)Wi * ci * 2, (cuuint64_t)Hi * Wi * ci * 2};
    const cuuint32_t box[4] = {8, (cuuint32_t)(S * G::XH), (cuuint32_t)G::YB, (cuuint32_t)G::ZB};
    const cuuint32_t estride[4] = {1, (cuuint32_t)S, 1, 1};
    const CUresult r = f(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(x), dims, strides, box, estride,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int S, int CO>
cudaError_t launch_co(const bf16* x, const bf16* w, const float* bias, bf16* y, float* y32, int Di, int Hi, int Wi,
                      int ci, int relu, cudaStream_t st) {
    constexpr int bytes = smem_bytes<S, CO>();
    static_assert(bytes <= 227 * 1024, "shared memory");
    CUtensorMap map;
    cudaError_t e = input_map<S>(&map, x, Di, Hi, Wi, ci);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_conv3_tc<S, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    const int Do = Di / S, Ho = Hi / S, Wo = Wi / S;
    const int64_t blocks = (int64_t)(Wo / TX) * (Ho / TY) * (Do / Geo<S>::TZ);
    k_conv3_tc<S, CO><<<(unsigned)blocks, kThreads, bytes, st>>>(map, w, bias, y, y32, Do, Ho, Wo, ci, relu);
    return cudaGetLastError();
}

// Resident CTAs per SM times their tensor-memory columns must fit the 512
// columns of an SM (an allocation that cannot be met waits for another
// CTA's release): shared memory bounds the residency below that here --
// stride 1: (co = 16) 4 x 64, (32) 3 x 128, (64) 2 x 256 columns; stride 2:
// at most 3 x 32, 2 x 32, 2 x 64.
template <int S, int CO>
constexpr bool tmem_fits() {
    return (227 * 1024 / smem_bytes<S, CO>()) * tmem_cols<S, CO>() <= 512;
}
static_assert(tmem_fits<1, 16>() && tmem_fits<1, 32>() && tmem_fits<1, 64>(), "tensor memory (stride 1)");
static_assert(tmem_fits<2, 16>() && tmem_fits<2, 32>() && tmem_fits<2, 64>(), "tensor memory (stride 2)");

template <int S>
cudaError_t launch_s(const void* x, int Di, int Hi, int Wi, int ci, const void* w, const float* bias, int co,
                     int relu, void* y, float* y32, cudaStream_t st) {
    const bf16* xb = static_cast<const bf16*>(x);
    const bf16* wb = static_cast<const bf16*>(w);
    bf16* yb = static_cast<bf16*>(y);
    switch (co) {
        case 16: return launch_co<S, 16>(xb, wb, bias, yb, y32, Di, Hi, Wi, ci, relu, st);
        case 32: return launch_co<S, 32>(xb, wb, bias, yb, y32, Di, Hi, Wi, ci, relu, st);
        default: return launch_co<S, 64>(xb, wb, bias, yb, y32, Di, Hi, Wi, ci, relu, st);
    }
}

}  // namespace

namespace lbm {

bool conv3_tc_applies(int D, int H, int W, int ci, int co, int stride) {
    const bool ch = (ci == 16 || ci == 32 || ci == 64) && (co == 16 || co == 32 || co == 64);
    if (!ch || D <= 0 || H <= 0 || W <= 0) return false;
    if (stride == 1) return D % Geo<1>::TZ == 0 && H % TY == 0 && W % TX == 0;
    if (stride == 2)
        return D % 2 == 0 && H % 2 == 0 && W % 2 == 0 && (D / 2) % Geo<2>::TZ == 0 && (H / 2) % TY == 0 &&
               (W / 2) % TX == 0;
    return false;
}

cudaError_t conv3_tc(const void* x, int D, int H, int W, int ci, const void* w, const float* bias, int co, int relu,
                     void* y, float* y32, int stride, cudaStream_t st) {
    return stride == 2 ? launch_s<2>(x, D, H, W, ci, w, bias, co, relu, y, y32, st)
                       : launch_s<1>(x, D, H, W, ci, w, bias, co, relu, y, y32, st);
}

bool conv3_wgrad_tc_applies(int D, int H, int W, int ci, int co, int stride) {
    const bool ch = (ci == 16 || ci == 32 || ci == 64) && (co == 16 || co == 32 || co == 64);
    if (!ch || D <= 0 || H <= 0 || W <= 0 || (stride != 1 && stride != 2)) return false;
    const int64_t Wo = (W - 1) / stride + 1;
    const int64_t vox = (int64_t)((D - 1) / stride + 1) * ((H - 1) / stride + 1) * Wo;
    return Wo % 16 == 0 && vox / 16 < ((int64_t)1 << 31);
}

cudaError_t conv3_wgrad_tc(const void* x, int D, int H, int W, int ci, const void* dy, int co, int stride, float* dw,
                           cudaStream_t st) {
    const bf16* xb = static_cast<const bf16*>(x);
    const bf16* db = static_cast<const bf16*>(dy);
    switch (co) {
        case 16: return launch_wgrad_co<16>(xb, db, dw, D, H, W, ci, stride, st);
        case 32: return launch_wgrad_co<32>(xb, db, dw, D, H, W, ci, stride, st);
        default: return launch_wgrad_co<64>(xb, db, dw, D, H, W, ci, stride, st);
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
