// Fused element-operator kernels, FP32 arithmetic, n = 10..17.
#include "sem_apply_launch.cuh"

namespace sem {
int launch_apply_f32_hi(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s,
                        int* tile) {
  return launch_apply_range<PF32, 10, 17>(g, ops, c, s, tile);
}
}  // namespace sem
