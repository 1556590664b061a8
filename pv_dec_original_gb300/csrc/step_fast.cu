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

// Warp blocks of the compact step kernel (layout in step_kernels.cuh), one
// warp of this kernel per warp of 32 active nodes: lane masks by ballot,
// first entries by shuffle from the lowest lane of each mask.
__global__ void k_warp_block(const uint64_t* __restrict__ act_word, const int32_t* __restrict__ sp_of_act,
                             int64_t nact, int64_t nnw, uint32_t* __restrict__ out) {
    constexpr int WB = kWarpBlockWords;
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool in = a < nact;
    const uint64_t w = in ? act_word[a] : 0ull;
    const int32_t e = in ? sp_of_act[a] : -1;
    const uint32_t seg = (uint32_t)word_segment(w);
    const uint32_t prev = __shfl_up_sync(0xffffffffu, seg, 1);
    const uint32_t segmask = __ballot_sync(0xffffffffu, in && lane > 0 && seg != prev);
    const uint32_t nwm = __ballot_sync(0xffffffffu, in && word_nw(w));
    const uint32_t otm = __ballot_sync(0xffffffffu, in && e >= nnw);
    const uint32_t bcm = __ballot_sync(0xffffffffu, in && word_class(w) >= CLS_BC0);
    const uint32_t nw0 = __shfl_sync(0xffffffffu, (uint32_t)e, nwm ? __ffs(nwm) - 1 : 0);
    const uint32_t ot0 = __shfl_sync(0xffffffffu, (uint32_t)(e - (int32_t)nnw), otm ? __ffs(otm) - 1 : 0);
    const uint32_t seg0 = __shfl_sync(0xffffffffu, seg, 0);
    if (lane == 0 && in) {
        uint32_t* b = out + (size_t)WB * (a >> 5);
        b[0] = seg0; b[1] = segmask; b[2] = nwm; b[3] = otm;
        b[4] = bcm; b[5] = nwm ? nw0 : 0u; b[6] = otm ? ot0 : 0u; b[7] = 0u;
    }
}

// Rows of q * stride + delta_q (padding entries 0).
template <int Q>
__global__ void k_seg_abs(const int32_t* __restrict__ delta, int64_t nseg, int64_t stride, int32_t* __restrict__ out) {
    constexpr int DR = kDeltaRow<Q>;
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nseg * DR) return;
    const int q = (int)(k % DR);
    out[k] = q < Q ? (int32_t)(q * stride + delta[k]) : 0;
}

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

cudaError_t build_compact_meta(int Q, const uint64_t* act_word, const int32_t* sp_of_act, int64_t nact, int64_t nnw,
                               const int32_t* seg_delta, int64_t nseg, int64_t stride, uint32_t* warp_block,
                               int32_t* seg_abs, cudaStream_t st) {
    if ((int64_t)Q * stride >= ((int64_t)1 << 31)) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(warp_block, 0, sizeof(uint32_t) * kWarpBlockWords * block_warps(nact), st);
    if (e != cudaSuccess) return e;
    const int64_t n = nseg * (Q == 19 ? kDeltaRow<19> : kDeltaRow<27>);
    if (n > 0) {
        if (Q == 19) k_seg_abs<19><<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(seg_delta, nseg, stride, seg_abs);
        else k_seg_abs<27><<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(seg_delta, nseg, stride, seg_abs);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (nact > 0) {
        k_warp_block<<<(unsigned)ceil_div(nact, 256), 256, 0, st>>>(act_word, sp_of_act, nact, nnw, warp_block);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t nw_readout_f32(const float2* accf, const float* ring, int64_t nnw, int first, int pending, int last,
                           const float* wss_ckpt, double* out, cudaStream_t st) {
    if (nnw <= 0) return cudaSuccess;
    k_nw_readout<<<(unsigned)ceil_div(nnw, 256), 256, 0, st>>>(accf, reinterpret_cast<const float4*>(ring), nnw,
                                                              first, pending, last, wss_ckpt, out);
    return cudaGetLastError();
}

}  // namespace lbm
