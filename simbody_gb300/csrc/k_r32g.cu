// k_r32g.cu -- realize(Acceleration) kernel instantiations, FP32 recursions,
// level-parallel driver; and the FP32 M^-1 f kernels.
#include "abi_device.cuh"

namespace sbg {

template <bool REF, int MINB> static void go(const KArgs& a, cudaStream_t s) {
    realizeKernel<float, 3, REF, true, MINB><<<a.P->nGroupBlocks, 128, 0, s>>>(*a.T, a.P->groupFirst, 0, a.y, a.ydot,
                                                                                  static_cast<float*>(a.scratch), a.status);
}

void realize32Group(const KArgs& a, bool refine, cudaStream_t s) {
    if (refine) {
        if (a.P->variant >= 4) go<true, 4>(a, s); else go<true, 1>(a, s);
        realizeFallback(a, true, s);
    }
    else { if (a.P->variant >= 4) go<false, 4>(a, s); else go<false, 1>(a, s); }
}

void minv32Chain(const KArgs& a, cudaStream_t s) {
    const Launch1D L = spread(a.P->nChain, 128);
    float* sc = static_cast<float*>(a.scratch);
    if (a.P->nm == 1) minvKernel<float, 1, false><<<L.grid, L.block, 0, s>>>(*a.T, 0, a.P->nChain, a.y, a.f, a.ydot, sc, a.status);
    else minvKernel<float, 3, false><<<L.grid, L.block, 0, s>>>(*a.T, 0, a.P->nChain, a.y, a.f, a.ydot, sc, a.status);
}
void minv32Group(const KArgs& a, cudaStream_t s) {
    minvKernel<float, 3, true><<<a.P->nGroupBlocks, 128, 0, s>>>(*a.T, a.P->groupFirst, 0, a.y, a.f, a.ydot,
                                                                   static_cast<float*>(a.scratch), a.status);
}

}  // namespace sbg
