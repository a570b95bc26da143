// k_r32c.cu -- realize(Acceleration) kernel instantiations, FP32 recursions,
// chain driver (refine = double-float residual refinement; variant 4 = at
// most 128 registers).
#include "abi_device.cuh"

namespace sbg {

template <bool REF, int MINB> static void go(const KArgs& a, cudaStream_t s) {
    const int nb = (a.P->nChain + 127) / 128;
    float* sc = static_cast<float*>(a.scratch);
    if (a.P->nm == 1) realizeKernel<float, 1, REF, false, MINB><<<nb, 128, 0, s>>>(*a.T, 0, a.P->nChain, a.y, a.ydot, sc, a.status);
    else realizeKernel<float, 3, REF, false, MINB><<<nb, 128, 0, s>>>(*a.T, 0, a.P->nChain, a.y, a.ydot, sc, a.status);
}

void realize32Chain(const KArgs& a, bool refine, cudaStream_t s) {
    if (refine) { if (a.P->variant == 4) go<true, 4>(a, s); else go<true, 1>(a, s); }
    else { if (a.P->variant == 4) go<false, 4>(a, s); else go<false, 1>(a, s); }
}

}  // namespace sbg
