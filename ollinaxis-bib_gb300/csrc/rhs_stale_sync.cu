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

void launch_rhs_stale_sync(const StageArgs& a, cudaStream_t s) {
    dim3 blk(32, OLLIN_RHS_THREADS / 32);
    const int nj = a.G.nz - a.G.jlo + 1;
    dim3 grd((a.G.nr + blk.x - 1) / blk.x, (nj + blk.y - 1) / blk.y);
    const bool sh = a.P.shift != 0, sc = a.P.scalar != 0, ad = a.P.shiftadvect != 0;
    if (!sh && !sc) launch_chained(rhs_kernel<false, false, false, true, true>, grd, blk, s, a);
    else if (!sh && sc) launch_chained(rhs_kernel<false, true, false, true, true>, grd, blk, s, a);
    else if (!sc && ad) launch_chained(rhs_kernel<true, false, true, true, true>, grd, blk, s, a);
    else if (!sc) launch_chained(rhs_kernel<true, false, false, true, true>, grd, blk, s, a);
    else if (ad) launch_chained(rhs_kernel<true, true, true, true, true>, grd, blk, s, a);
    else launch_chained(rhs_kernel<true, true, false, true, true>, grd, blk, s, a);
}

}  // namespace ollin
