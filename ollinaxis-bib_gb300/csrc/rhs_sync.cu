// The first stage of a grid after ``syncboxes`` (src/base/syncboxes.f90)
// copied another refinement box's data onto it.  syncboxes copies the
// auxiliary arrays (derivatives, curvature) along with the evolved ones, and
// the next ``onestep`` computes its first sources before any ``auxiliary``
// call.  So at a copied point those quantities are the partner box's, and at
// the other points they are this grid's from before the copy, while the
// dissipation reads the current state (StageArgs::smap, xa, xb).  A separate
// translation unit, so that these six instantiations compile beside the
// ordinary ones.
#include "rhs_kernel.cuh"

namespace ollin {

void launch_rhs_sync(const StageArgs& a, cudaStream_t s) { launch_rhs_family<false, true, 4>(a, s); }

}  // namespace ollin
