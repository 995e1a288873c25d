// Persistent batched-PCG kernels for n = 2, 3, 4, 5, 6 (one template instance per order).
#include "sem_batch_kernel.cuh"

namespace sem {
int launch_batch_group_a(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  switch (n) {
    case 2: return launch_batch_order<2>(c, ops, s);
    case 3: return launch_batch_order<3>(c, ops, s);
    case 4: return launch_batch_order<4>(c, ops, s);
    case 5: return launch_batch_order<5>(c, ops, s);
    case 6: return launch_batch_order<6>(c, ops, s);
    default: return set_error(SEM_ERR_UNSUPPORTED, "batch order %d not in this group", n);
  }
}
}  // namespace sem
