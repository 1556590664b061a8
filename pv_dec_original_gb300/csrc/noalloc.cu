// Moment sums without any allocation, for callers that cannot allocate.
//
// Some callers of this library cannot call cudaMalloc: code that runs while
// a CUDA graph is being captured, real-time loops whose memory is fixed
// up-front, and host frameworks whose pool allocator owns all device memory.
// lbm_moment_sums_noalloc serves them.  It is the read-out reduction of the
// step kernel (per-block partial sums, then one fixed-order final sum)
// applied to a caller-owned device array of FP64 distributions, with the
// per-block partials kept in a file-scope device array instead of memory
// from cudaMalloc.
//
// Limits and rules:
//   - At most kNoAllocMaxNodes = 4,194,304 nodes per call (16,384 blocks of
//     256 threads; the scratch array is 16,384 x 4 doubles = 512 KiB, held
//     by every GPU that loads the library until the process exits).  Larger
//     inputs are rejected with LBM_ERR_ARG.
//   - The first call on a device looks up the scratch array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture.
//   - Every call shares the one scratch array.  Each block overwrites its own
//     partials before the final sum reads them, so nothing has to start at
//     zero, but calls that overlap on the GPU (different streams, or graphs
//     replayed concurrently) race on it: serialise them.
//   - The scratch address is kept per device ordinal for the life of the
//     process; a device reset (cudaDeviceReset) between calls is not
//     supported.
//   - A CUDA error left pending by earlier, unrelated work is not reported
//     as this call's: the call takes it from the runtime first, returns
//     LBM_ERR_CUDA naming it as earlier, and launches nothing.
//   - No cudaMalloc, cudaFree or allocating library routine is called.
#include <cstdio>
#include <mutex>

#include "lbm_internal.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int64_t kNoAllocMaxBlocks = 16384;
constexpr int64_t kNoAllocMaxNodes = kNoAllocMaxBlocks * kThreads;
constexpr int kSums = 4;  // sum(rho - 1), momentum x, y, z

}  // namespace

// The per-block partials of every call.  Host code must not use this name as
// a pointer (it is a host-side stand-in): the device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxBlocks * kSums];

namespace {

template <int Q>
__global__ void __launch_bounds__(kThreads) k_partials(const double* __restrict__ f, int64_t nact,
                                                     double* __restrict__ partials) {
    __shared__ double red[kThreads / 32][kSums];
    const int64_t a = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    double v[kSums] = {0.0, 0.0, 0.0, 0.0};
    if (a < nact) {
        double r = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const double x = f[a * Q + q];
            r += x;
            jx += x * lbm::Lat<Q>::cx(q);
            jy += x * lbm::Lat<Q>::cy(q);
            jz += x * lbm::Lat<Q>::cz(q);
        }
        v[0] = r - 1.0; v[1] = jx; v[2] = jy; v[3] = jz;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kSums; ++k) {
        double x = v[k];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) x += __shfl_down_sync(0xffffffffu, x, d);
        if (lane == 0) red[warp][k] = x;
    }
    __syncthreads();
    if (threadIdx.x < kSums) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += red[w][threadIdx.x];
        partials[(int64_t)blockIdx.x * kSums + threadIdx.x] = s;
    }
}

// One block, fixed order: deterministic for a given node count.
__global__ void __launch_bounds__(kThreads) k_final(const double* __restrict__ partials, int64_t nblocks,
                                                  int64_t nact, double* __restrict__ out) {
    __shared__ double red[kThreads][kSums];
    double acc[kSums] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t b = threadIdx.x; b < nblocks; b += kThreads)
#pragma unroll
        for (int k = 0; k < kSums; ++k) acc[k] += partials[b * kSums + k];
#pragma unroll
    for (int k = 0; k < kSums; ++k) red[threadIdx.x][k] = acc[k];
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
#pragma unroll
            for (int k = 0; k < kSums; ++k) red[threadIdx.x][k] += red[threadIdx.x + w][k];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = (double)nact + red[0][0];  // mass
        out[1] = red[0][1];
        out[2] = red[0][2];
        out[3] = red[0][3];
    }
}

// Device address of the scratch array, looked up once per device.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch[kMaxDevices] = {};

// Errors are reported through lbm_last_global_error().
int report(int code, const char* what) {
    char msg[256];
    std::snprintf(msg, sizeof(msg), "lbm_moment_sums_noalloc: %s", what);
    lbm::set_last_global_error(msg);
    return code;
}

}  // namespace

extern "C" {

lbm_status lbm_moment_sums_noalloc(const double* d_f, int64_t nact, int Q, double* d_out, void* stream) {
    if (Q != 19 && Q != 27) return report(LBM_ERR_ARG, "Q must be 19 or 27");
    if (nact < 0 || (nact > 0 && !d_f) || !d_out) return report(LBM_ERR_ARG, "null buffer or negative size");
    if (nact > kNoAllocMaxNodes)
        return report(LBM_ERR_ARG, "more than 4194304 nodes: exceeds the fixed scratch array of this entry point");
    {
        // an error of earlier work must not be read below as a failure of these launches
        const cudaError_t earlier = cudaGetLastError();
        if (earlier != cudaSuccess) {
            char msg[200];
            std::snprintf(msg, sizeof(msg), "a CUDA error from earlier work was pending (%s); nothing launched",
                          cudaGetErrorName(earlier));
            return report(LBM_ERR_CUDA, msg);
        }
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return report(LBM_ERR_CUDA, "cudaGetDevice failed");
    if (dev < 0 || dev >= kMaxDevices) return report(LBM_ERR_ARG, "device ordinal beyond 63");
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_scratch[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return report(LBM_ERR_CUDA, cudaGetErrorString(e));
            g_scratch[dev] = static_cast<double*>(p);
        }
        scratch = g_scratch[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t nblocks = nact > 0 ? lbm::ceil_div(nact, kThreads) : 0;
    if (nblocks > 0) {
        if (Q == 19) k_partials<19><<<(unsigned)nblocks, kThreads, 0, st>>>(d_f, nact, scratch);
        else k_partials<27><<<(unsigned)nblocks, kThreads, 0, st>>>(d_f, nact, scratch);
    }
    k_final<<<1, kThreads, 0, st>>>(scratch, nblocks, nact, d_out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return report(LBM_ERR_CUDA, cudaGetErrorString(e));
    return LBM_OK;
}

}  // extern "C"
