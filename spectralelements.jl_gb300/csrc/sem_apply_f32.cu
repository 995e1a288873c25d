// Fused element-operator kernels, FP32 arithmetic, n = 2..9.
#include "sem_apply_launch.cuh"

namespace sem {
int launch_apply_f32_lo(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s,
                        int* tile) {
  return launch_apply_range<PF32, 2, 9>(g, ops, c, s, tile);
}
}  // namespace sem
