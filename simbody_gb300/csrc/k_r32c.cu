// k_r32c.cu -- realize(Acceleration) kernel instantiations, FP32 recursions,
// chain driver: the dispatch and the unrefined form (the refined form, with
// its FP64 recomputation pass, is in k_r32cr.cu; variant 8, the staged chain
// driver of one shared chain topology, in k_r32s.cu).
#include "r32c_launch.cuh"

namespace sbg {

void realize32Chain(const KArgs& a, bool refine, cudaStream_t s) {
    if (a.P->variant == 8) realize32ChainStaged(a, refine, s);  // k_r32s.cu
    else if (refine) realize32ChainRefined(a, s);
    else r32ChainPick<false>(a, s);
}

}  // namespace sbg
