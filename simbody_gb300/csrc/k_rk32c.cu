// k_rk32c.cu -- fixed-step RK-Merson persistent kernel instantiations, FP32
// recursions with FP64 state accumulation, chain driver: the dispatch and the
// unrefined form (the refined form is in k_rk32cr.cu).
#include "rk32c_launch.cuh"

namespace sbg {

void rk32Chain(const KArgs& a, bool refine, cudaStream_t s) {
    if (refine) rk32ChainRefined(a, s);
    else rk32ChainPick<false>(a, s);
}

}  // namespace sbg
