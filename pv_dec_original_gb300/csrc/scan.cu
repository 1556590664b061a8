// Exclusive prefix sum of int64 counts: one pass per level (block-local scan
// of 2048 items, scan of the block totals, offset add).  Used by the set-up
// compactions (boundary lists, segments, voxelizer column lists).
#include "lbm_internal.cuh"

namespace lbm {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kChunk = kThreads * kItems;

__global__ void scan_blocks(const int64_t* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                            int64_t* __restrict__ block_sums) {
    __shared__ int64_t warp_tot[kThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kChunk + (int64_t)threadIdx.x * kItems;
    int64_t v[kItems];
    int64_t run = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        int64_t x = (base + i < n) ? in[base + i] : 0;
        v[i] = run;
        run += x;
    }
    // inclusive scan of per-thread totals within the warp
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t incl = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int64_t t = lane < kThreads / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, t, d);
            if (lane >= d) t += y;
        }
        if (lane < kThreads / 32) warp_tot[lane] = t;  // inclusive warp prefix
    }
    __syncthreads();
    int64_t offset = (incl - run) + (warp > 0 ? warp_tot[warp - 1] : 0);
#pragma unroll
    for (int i = 0; i < kItems; ++i)
        if (base + i < n) out[base + i] = v[i] + offset;
    if (threadIdx.x == kThreads - 1) block_sums[blockIdx.x] = offset + run;
}

__global__ void add_offsets(int64_t* __restrict__ out, int64_t n, const int64_t* __restrict__ block_off) {
    const int64_t base = (int64_t)blockIdx.x * kChunk;
    const int64_t add = block_off[blockIdx.x];
    for (int i = threadIdx.x; i < kChunk; i += kThreads)
        if (base + i < n) out[base + i] += add;
}

cudaError_t scan_rec(const int64_t* in, int64_t* out, int64_t n, int64_t* d_total, cudaStream_t s) {
    const int64_t nb = ceil_div(n, kChunk);
    int64_t* sums = nullptr;
    int64_t* sums_scan = nullptr;
    cudaError_t e = cudaMallocAsync(&sums, sizeof(int64_t) * (nb + 1), s);
    if (e != cudaSuccess) return e;
    e = cudaMallocAsync(&sums_scan, sizeof(int64_t) * (nb + 1), s);
    if (e != cudaSuccess) { cudaFreeAsync(sums, s); return e; }
    scan_blocks<<<(unsigned)nb, kThreads, 0, s>>>(in, out, n, sums);
    if (nb == 1) {
        e = cudaMemcpyAsync(d_total, sums, sizeof(int64_t), cudaMemcpyDeviceToDevice, s);
    } else {
        e = scan_rec(sums, sums_scan, nb, d_total, s);
        if (e == cudaSuccess) add_offsets<<<(unsigned)nb, kThreads, 0, s>>>(out, n, sums_scan);
    }
    cudaFreeAsync(sums, s);
    cudaFreeAsync(sums_scan, s);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace

cudaError_t exclusive_scan_i64(const int64_t* d_in, int64_t* d_out, int64_t n, int64_t* total, cudaStream_t s) {
    if (n <= 0) {
        if (total) *total = 0;
        return cudaSuccess;
    }
    int64_t* d_total = nullptr;
    cudaError_t e = cudaMallocAsync(&d_total, sizeof(int64_t), s);
    if (e != cudaSuccess) return e;
    e = scan_rec(d_in, d_out, n, d_total, s);
    if (e == cudaSuccess && total) {
        e = cudaMemcpyAsync(total, d_total, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    cudaFreeAsync(d_total, s);
    return e;
}

}  // namespace lbm
