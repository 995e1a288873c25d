// Persistent batched-PCG kernels for n = 10, 11 (one template instance per order).
#include "sem_batch_kernel.cuh"

namespace sem {
int launch_batch_group_c(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  switch (n) {
    case 10: return launch_batch_order<10>(c, ops, s);
    case 11: return launch_batch_order<11>(c, ops, s);
    default: return set_error(SEM_ERR_UNSUPPORTED, "batch order %d not in this group", n);
  }
}
}  // namespace sem
