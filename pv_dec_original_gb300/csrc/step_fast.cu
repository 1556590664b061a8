// Storage-typed initialisation for the FP32-arithmetic formats.
#include "step_kernels.cuh"

namespace lbm {

cudaError_t init_state_fast(int precision, int Q, int what, void* f, int64_t stride, const double* fa,
                            int64_t nact, cudaStream_t st) {
    switch (precision) {
        case P_F32: return init_typed<float>(Q, what, f, stride, fa, nact, st);
        case P_F16: return init_typed<__half>(Q, what, f, stride, fa, nact, st);
        case P_BF16: return init_typed<__nv_bfloat16>(Q, what, f, stride, fa, nact, st);
        default: return cudaErrorInvalidValue;
    }
}

namespace {

// Next-to-wall read-out of the FP32 formats, as doubles: out[0] = |tau| of
// the last step, out[1..3] = sum tau, out[4] = sum |tau| (each [nnw]); the
// sums are the folded accumulators plus the pending ring slots first ..
// first + pending - 1 (float4 [slot][nnw]).
__global__ void k_nw_readout(const float2* __restrict__ accf, const float4* __restrict__ ring, int64_t nnw,
                             int first, int pending, int last, const float* __restrict__ wss_ckpt,
                             double* __restrict__ out) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nnw) return;
    out[p] = last < 0 ? 0.0 : wss_ckpt ? (double)wss_ckpt[p] : (double)ring[(int64_t)last * nnw + p].w;
    double v[4];
    for (int k = 0; k < 4; ++k) {
        const float2 a = accf[k * nnw + p];
        v[k] = (double)a.x + (double)a.y;
    }
    for (int j = 0; j < pending; ++j) {
        const float4 r = ring[(int64_t)(first + j) * nnw + p];
        v[0] += (double)r.x; v[1] += (double)r.y; v[2] += (double)r.z; v[3] += (double)r.w;
    }
    for (int k = 0; k < 4; ++k) out[(1 + k) * nnw + p] = v[k];
}

}  // namespace

cudaError_t nw_readout_f32(const float2* accf, const float* ring, int64_t nnw, int first, int pending, int last,
                           const float* wss_ckpt, double* out, cudaStream_t st) {
    if (nnw <= 0) return cudaSuccess;
    k_nw_readout<<<(unsigned)ceil_div(nnw, 256), 256, 0, st>>>(accf, reinterpret_cast<const float4*>(ring), nnw,
                                                              first, pending, last, wss_ckpt, out);
    return cudaGetLastError();
}

}  // namespace lbm
