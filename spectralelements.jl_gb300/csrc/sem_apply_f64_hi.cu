// Fused element-operator kernels, native FP64 arithmetic, n = 10..17.
#include "sem_apply_launch.cuh"

namespace sem {
int launch_apply_f64_hi(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s,
                        int* tile) {
  return launch_apply_range<PF64, 10, 17>(g, ops, c, s, tile);
}
}  // namespace sem
