// The fused right-hand-side + Runge-Kutta stage kernel (rhs_kernel.cuh):
// the launcher of the ordinary stages.  The first stage of a level after a
// maximal-slicing solve is launched from rhs_stale.cu.
#include "rhs_kernel.cuh"

namespace ollin {

void launch_rhs(const StageArgs& a, cudaStream_t s) {
    dim3 blk(32, OLLIN_RHS_THREADS / 32);
    const int nj = a.G.nz - a.G.jlo + 1;
    dim3 grd((a.G.nr + blk.x - 1) / blk.x, (nj + blk.y - 1) / blk.y);
    const bool sh = a.P.shift != 0, sc = a.P.scalar != 0, ad = a.P.shiftadvect != 0;
    if (!sh && !sc) launch_chained(rhs_kernel<false, false, false, false>, grd, blk, s, a);
    else if (!sh && sc) launch_chained(rhs_kernel<false, true, false, false>, grd, blk, s, a);
    else if (!sc && ad) launch_chained(rhs_kernel<true, false, true, false>, grd, blk, s, a);
    else if (!sc) launch_chained(rhs_kernel<true, false, false, false>, grd, blk, s, a);
    else if (ad) launch_chained(rhs_kernel<true, true, true, false>, grd, blk, s, a);
    else launch_chained(rhs_kernel<true, true, false, false>, grd, blk, s, a);
}

namespace {
// the fused multi-instance twins of the six instantiations above
struct MultiRegs {
    MultiRegs() {
        register_rhs_multi<false, false, false, false>();
        register_rhs_multi<false, true, false, false>();
        register_rhs_multi<true, false, true, false>();
        register_rhs_multi<true, false, false, false>();
        register_rhs_multi<true, true, true, false>();
        register_rhs_multi<true, true, false, false>();
    }
};
const MultiRegs multi_regs;
}  // namespace

}  // namespace ollin
