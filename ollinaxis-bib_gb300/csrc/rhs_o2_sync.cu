// Order two: the first stage of a grid after a ``syncboxes`` copy onto it
// (the sync variant of rhs_sync.cu).
#include "rhs_kernel.cuh"

namespace ollin {

void launch_rhs_o2_sync(const StageArgs& a, cudaStream_t s) { launch_rhs_family<false, true, 2>(a, s); }

}  // namespace ollin
