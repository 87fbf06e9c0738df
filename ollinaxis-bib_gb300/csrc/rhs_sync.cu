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

void launch_rhs_sync(const StageArgs& a, cudaStream_t s) {
    dim3 blk(32, OLLIN_RHS_THREADS / 32);
    const int nj = a.G.nz - a.G.jlo + 1;
    dim3 grd((a.G.nr + blk.x - 1) / blk.x, (nj + blk.y - 1) / blk.y);
    const bool sh = a.P.shift != 0, sc = a.P.scalar != 0, ad = a.P.shiftadvect != 0;
    if (!sh && !sc) launch_chained(rhs_kernel<false, false, false, false, true>, grd, blk, s, a);
    else if (!sh && sc) launch_chained(rhs_kernel<false, true, false, false, true>, grd, blk, s, a);
    else if (!sc && ad) launch_chained(rhs_kernel<true, false, true, false, true>, grd, blk, s, a);
    else if (!sc) launch_chained(rhs_kernel<true, false, false, false, true>, grd, blk, s, a);
    else if (ad) launch_chained(rhs_kernel<true, true, true, false, true>, grd, blk, s, a);
    else launch_chained(rhs_kernel<true, true, false, false, true>, grd, blk, s, a);
}

}  // namespace ollin
