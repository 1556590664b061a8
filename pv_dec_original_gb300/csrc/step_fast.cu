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

}  // namespace lbm
