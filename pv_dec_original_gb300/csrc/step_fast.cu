// FP32-arithmetic step kernels for FP32, FP16-offset and BF16-offset storage
// (compiled with FMA contraction on).
#include "step_kernels.cuh"

namespace lbm {

cudaError_t launch_step_fast(int Q, int precision, int mode, int kind, const StepParams& p, cudaStream_t st) {
    switch (precision) {
        case P_F32: return launch_typed<float>(Q, mode, kind, p, st);
        case P_F16: return launch_typed<__half>(Q, mode, kind, p, st);
        case P_BF16: return launch_typed<__nv_bfloat16>(Q, mode, kind, p, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t init_state_fast(int precision, int Q, int what, void* f, int64_t stride, int64_t npts,
                            const double* fa, const int64_t* act_pt, int64_t nact, cudaStream_t st) {
    switch (precision) {
        case P_F32: return init_typed<float>(Q, what, f, stride, npts, fa, act_pt, nact, st);
        case P_F16: return init_typed<__half>(Q, what, f, stride, npts, fa, act_pt, nact, st);
        case P_BF16: return init_typed<__nv_bfloat16>(Q, what, f, stride, npts, fa, act_pt, nact, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace lbm
