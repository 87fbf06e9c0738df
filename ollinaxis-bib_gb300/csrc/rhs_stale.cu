// The first stage of a level after a maximal-slicing solve
// (src/geometry/maximalslicing.f90).  ``maximalslicing`` replaces the lapse
// and recomputes its first and second derivatives, but the next ``onestep``
// computes its first sources before any ``auxiliary`` call, so the
// covariant second derivatives of the lapse, its Laplacian, falpha and its
// advective derivatives are still those of the lapse before the solve
// (StageArgs::alpha_aux).  A separate translation unit, so that these six
// instantiations compile beside the ordinary ones.
#include "rhs_kernel.cuh"

namespace ollin {

void launch_rhs_stale(const StageArgs& a, cudaStream_t s) {
    dim3 blk(32, OLLIN_RHS_THREADS / 32);
    const int nj = a.G.nz - a.G.jlo + 1;
    dim3 grd((a.G.nr + blk.x - 1) / blk.x, (nj + blk.y - 1) / blk.y);
    const bool sh = a.P.shift != 0, sc = a.P.scalar != 0, ad = a.P.shiftadvect != 0;
    if (!sh && !sc) launch_chained(rhs_kernel<false, false, false, true>, grd, blk, s, a);
    else if (!sh && sc) launch_chained(rhs_kernel<false, true, false, true>, grd, blk, s, a);
    else if (!sc && ad) launch_chained(rhs_kernel<true, false, true, true>, grd, blk, s, a);
    else if (!sc) launch_chained(rhs_kernel<true, false, false, true>, grd, blk, s, a);
    else if (ad) launch_chained(rhs_kernel<true, true, true, true>, grd, blk, s, a);
    else launch_chained(rhs_kernel<true, true, false, true>, grd, blk, s, a);
}

namespace {
// the fused multi-instance twins of the six instantiations above
struct MultiRegs {
    MultiRegs() {
        register_rhs_multi<false, false, false, true>();
        register_rhs_multi<false, true, false, true>();
        register_rhs_multi<true, false, true, true>();
        register_rhs_multi<true, false, false, true>();
        register_rhs_multi<true, true, true, true>();
        register_rhs_multi<true, true, false, true>();
    }
};
const MultiRegs multi_regs;
}  // namespace

}  // namespace ollin
