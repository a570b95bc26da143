// k_rk32cr.cu -- fixed-step RK-Merson persistent kernel instantiations, FP32
// recursions with double-float residual refinement (the mixed form), chain
// driver.
#include "rk32c_launch.cuh"

namespace sbg {

void rk32ChainRefined(const KArgs& a, cudaStream_t s) { rk32ChainPick<true>(a, s); }

}  // namespace sbg
