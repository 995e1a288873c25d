// Fused element-operator kernels, PF64 arithmetic (all n from 2 to 17).
#include "sem_apply_launch.cuh"

namespace sem {
int launch_apply_f64(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s) {
  return launch_apply_p<PF64>(g, ops, c, s);
}
}  // namespace sem
