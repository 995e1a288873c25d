// Fused element-operator kernels, PDF (double-float) arithmetic, n = 10..17.
#include "sem_apply_launch.cuh"

namespace sem {
int launch_apply_df_hi(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s,
                        int* tile) {
  return launch_apply_range<PDF, 10, 17>(g, ops, c, s, tile);
}
}  // namespace sem
