// Persistent batched-PCG kernels for n = 7, 8, 9 (one template instance per order).
#include "sem_batch_kernel.cuh"

namespace sem {
int launch_batch_group_b(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  switch (n) {
    case 7: return launch_batch_order<7>(c, ops, s);
    case 8: return launch_batch_order<8>(c, ops, s);
    case 9: return launch_batch_order<9>(c, ops, s);
    default: return set_error(SEM_ERR_UNSUPPORTED, "batch order %d not in this group", n);
  }
}
}  // namespace sem
