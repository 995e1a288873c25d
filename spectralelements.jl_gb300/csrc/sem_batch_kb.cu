// Persistent batched-PCG kernels for n = 7, 8, 9, two resident CTAs per SM (up to 128 registers a thread).
#include "sem_batch_kernel.cuh"

namespace sem {
int launch_batch_kb(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  return launch_batch_range<7, 9, 2>(n, c, ops, s);
}
int max_clusters_kb(int n, int csize) { return max_clusters_range<7, 9, 2>(n, csize); }
}  // namespace sem
