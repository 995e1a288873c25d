// Persistent batched-PCG kernels for n = 10, 11, two resident CTAs per SM (up to 128 registers a thread).
#include "sem_batch_kernel.cuh"

namespace sem {
int launch_batch_kc(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  return launch_batch_range<10, 11, 2>(n, c, ops, s);
}
int max_clusters_kc(int n, int csize) { return max_clusters_range<10, 11, 2>(n, csize); }
}  // namespace sem
