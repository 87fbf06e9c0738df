// The fused right-hand-side + Runge-Kutta stage kernel in order two
// (derivatives.f90, derivadvect.f90 and dissipation.f90 order-two branches,
// two ghost zones): the ordinary stages and their fused multi-instance twins.
#include "rhs_kernel.cuh"

namespace ollin {

void launch_rhs_o2(const StageArgs& a, cudaStream_t s) { launch_rhs_family<false, false, 2>(a, s); }

namespace {
struct MultiRegs {
    MultiRegs() { register_rhs_family<false, false, 2>(); }
};
const MultiRegs multi_regs;
}  // namespace

}  // namespace ollin
