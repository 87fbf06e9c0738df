// Order two: the first stage of a grid after both a maximal-slicing solve and
// a ``syncboxes`` copy onto it (the variant of rhs_stale_sync.cu).
#include "rhs_kernel.cuh"

namespace ollin {

void launch_rhs_o2_stale_sync(const StageArgs& a, cudaStream_t s) { launch_rhs_family<true, true, 2>(a, s); }

}  // namespace ollin
