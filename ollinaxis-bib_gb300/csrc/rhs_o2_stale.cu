// Order two: the first stage of a level after a maximal-slicing solve (the
// stale lapse of rhs_stale.cu) and its fused multi-instance twins.
#include "rhs_kernel.cuh"

namespace ollin {

void launch_rhs_o2_stale(const StageArgs& a, cudaStream_t s) { launch_rhs_family<true, false, 2>(a, s); }

namespace {
struct MultiRegs {
    MultiRegs() { register_rhs_family<true, false, 2>(); }
};
const MultiRegs multi_regs;
}  // namespace

}  // namespace ollin
