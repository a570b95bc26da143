// k_r64.cu -- realize(Acceleration) and M^-1 f kernel instantiations, FP64.
#include "abi_device.cuh"

namespace sbg {


void realize64Chain(const KArgs& a, cudaStream_t s) {
    const Launch1D L = spread(a.P->nChain, 128);
    double* sc = static_cast<double*>(a.scratch);
    if (a.P->nm == 1) realizeKernel<double, 1, false, false><<<L.grid, L.block, 0, s>>>(*a.T, a.P->chainFirst, a.P->nChain, a.y, a.ydot, sc, a.status);
    else realizeKernel<double, 3, false, false><<<L.grid, L.block, 0, s>>>(*a.T, a.P->chainFirst, a.P->nChain, a.y, a.ydot, sc, a.status);
}
void realize64Group(const KArgs& a, cudaStream_t s) {
    realizeKernel<double, 3, false, true><<<a.P->nGroupBlocks, 128, 0, s>>>(*a.T, a.P->groupFirst, 0, a.y, a.ydot,
                                                                              static_cast<double*>(a.scratch), a.status);
}
void minv64Chain(const KArgs& a, cudaStream_t s) {
    const Launch1D L = spread(a.P->nChain, 128);
    double* sc = static_cast<double*>(a.scratch);
    if (a.P->nm == 1) minvKernel<double, 1, false><<<L.grid, L.block, 0, s>>>(*a.T, 0, a.P->nChain, a.y, a.f, a.ydot, sc, a.status);
    else minvKernel<double, 3, false><<<L.grid, L.block, 0, s>>>(*a.T, 0, a.P->nChain, a.y, a.f, a.ydot, sc, a.status);
}
void minv64Group(const KArgs& a, cudaStream_t s) {
    minvKernel<double, 3, true><<<a.P->nGroupBlocks, 128, 0, s>>>(*a.T, a.P->groupFirst, 0, a.y, a.f, a.ydot,
                                                                    static_cast<double*>(a.scratch), a.status);
}

}  // namespace sbg
