// FP32 storage (offsets d = f - w), FP32 arithmetic, FMA contraction on.
#include "step_kernels.cuh"

namespace lbm {

cudaError_t launch_step_f32(int Q, int mode, int kind, int variant, const StepParams& p, cudaStream_t st) {
    return launch_typed<float>(Q, mode, kind, variant, p, st);
}

cudaError_t launch_multi_f32(int Q, int mode, const StepParams& even, const StepParams& odd, int nsteps,
                              unsigned* bar, cudaStream_t st) {
    return launch_multi_typed<float>(Q, mode, even, odd, nsteps, bar, st);
}

}  // namespace lbm
