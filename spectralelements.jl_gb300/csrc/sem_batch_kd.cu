// Persistent batched-PCG kernels for n = 2, 3, 4, 5, 6, one resident CTA per SM (up to 255 registers a thread).
#include "sem_batch_kernel.cuh"

namespace sem {
int launch_batch_kd(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  return launch_batch_range<2, 6, 1>(n, c, ops, s);
}
int max_clusters_kd(int n, int csize) { return max_clusters_range<2, 6, 1>(n, csize); }
}  // namespace sem
