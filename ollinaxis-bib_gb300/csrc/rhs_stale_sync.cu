// The first stage of a grid after both a maximal-slicing solve and a
// ``syncboxes`` copy onto it (src/geometry/maximalslicing.f90,
// src/base/syncboxes.f90): the derivatives of the other fields, and the
// lapse quantities of the last ``auxiliary`` call, come from the state kept
// from before the copy (the partner box's at a copied point), while the
// lapse and its first and second derivatives are those ``maximalslicing``
// computed on this grid from the solved lapse.  A separate translation unit,
// so that these six instantiations compile beside the others.
#include "rhs_kernel.cuh"

namespace ollin {

void launch_rhs_stale_sync(const StageArgs& a, cudaStream_t s) { launch_rhs_family<true, true, 4>(a, s); }

}  // namespace ollin
