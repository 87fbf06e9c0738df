// The fused right-hand-side + Runge-Kutta stage kernel (rhs_kernel.cuh):
// the launcher of the ordinary stages.  The first stage of a level after a
// maximal-slicing solve is launched from rhs_stale.cu.
#include "rhs_kernel.cuh"

namespace ollin {

void launch_rhs(const StageArgs& a, cudaStream_t s) { launch_rhs_family<false, false, 4>(a, s); }

namespace {
// the fused multi-instance twins of the six instantiations above
struct MultiRegs {
    MultiRegs() { register_rhs_family<false, false, 4>(); }
};
const MultiRegs multi_regs;
}  // namespace

}  // namespace ollin
