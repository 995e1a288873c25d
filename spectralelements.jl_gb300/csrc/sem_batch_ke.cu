// Persistent batched-PCG kernels for n = 7, 8, 9, one resident CTA per SM (up to 255 registers a thread).
#include "sem_batch_kernel.cuh"

namespace sem {
int launch_batch_ke(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  return launch_batch_range<7, 9, 1>(n, c, ops, s);
}
int max_clusters_ke(int n, int csize) { return max_clusters_range<7, 9, 1>(n, csize); }
}  // namespace sem
