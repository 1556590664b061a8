// FP32 storage (offsets d = f - w), FP32 arithmetic, FMA contraction on.
#include "step_kernels.cuh"

namespace lbm {

cudaError_t launch_step_f32(int Q, int mode, int kind, int variant, const StepParams& p, cudaStream_t st) {
    return launch_typed<float>(Q, mode, kind, variant, p, st);
}

}  // namespace lbm
