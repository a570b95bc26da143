// k_r32cr.cu -- realize(Acceleration) kernel instantiations, FP32 recursions
// with double-float residual refinement (the mixed form), chain driver, and
// its FP64 recomputation pass.
#include "r32c_launch.cuh"

namespace sbg {

void realize32ChainRefined(const KArgs& a, cudaStream_t s) {
    r32ChainPick<true>(a, s);
    realizeFallback(a, false, s);
}

}  // namespace sbg
