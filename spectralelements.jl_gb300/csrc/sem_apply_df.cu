// Fused element-operator kernels, PDF arithmetic (all n from 2 to 17).
#include "sem_apply_launch.cuh"

namespace sem {
int launch_apply_df(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s) {
  return launch_apply_p<PDF>(g, ops, c, s);
}
}  // namespace sem
