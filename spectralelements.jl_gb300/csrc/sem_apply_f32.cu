// Fused element-operator kernels, PF32 arithmetic (all n from 2 to 17).
#include "sem_apply_launch.cuh"

namespace sem {
int launch_apply_f32(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s) {
  return launch_apply_p<PF32>(g, ops, c, s);
}
}  // namespace sem
