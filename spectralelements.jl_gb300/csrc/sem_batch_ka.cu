// Persistent batched-PCG kernels for n = 2, 3, 4, 5, 6, two resident CTAs per SM (up to 128 registers a thread).
#include "sem_batch_kernel.cuh"

namespace sem {
int launch_batch_ka(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  return launch_batch_range<2, 6, 2>(n, c, ops, s);
}
int max_clusters_ka(int n, int csize) { return max_clusters_range<2, 6, 2>(n, csize); }
}  // namespace sem
