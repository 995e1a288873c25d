// Persistent batched-PCG kernels for n = 10, 11, one resident CTA per SM (up to 255 registers a thread).
#include "sem_batch_kernel.cuh"

namespace sem {
int launch_batch_kf(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  return launch_batch_range<10, 11, 1>(n, c, ops, s);
}
int max_clusters_kf(int n, int csize) { return max_clusters_range<10, 11, 1>(n, csize); }
}  // namespace sem
