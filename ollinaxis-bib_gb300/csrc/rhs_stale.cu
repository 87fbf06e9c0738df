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

void launch_rhs_stale(const StageArgs& a, cudaStream_t s) { launch_rhs_family<true, false, 4>(a, s); }

namespace {
// the fused multi-instance twins of the six instantiations above
struct MultiRegs {
    MultiRegs() { register_rhs_family<true, false, 4>(); }
};
const MultiRegs multi_regs;
}  // namespace

}  // namespace ollin
