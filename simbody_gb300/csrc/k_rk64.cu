// k_rk64.cu -- fixed-step RK-Merson persistent kernel instantiations, FP64.
#include "abi_device.cuh"

namespace sbg {

void rk64Chain(const KArgs& a, cudaStream_t s) {
    const Launch1D L = spread(a.P->nChain, 128);
    double* fb = static_cast<double*>(a.fbuf);
    double* sc = static_cast<double*>(a.scratch);
    if (a.P->nm == 1)
        rkMersonKernel<double, 1, false, false><<<L.grid, L.block, 0, s>>>(*a.T, 0, a.P->nChain, a.ystate, a.time, fb, a.fplane, sc,
                                                                   a.status, a.h, a.step, a.accuracy, a.consTol, a.projectEveryStep);
    else
        rkMersonKernel<double, 3, false, false><<<L.grid, L.block, 0, s>>>(*a.T, 0, a.P->nChain, a.ystate, a.time, fb, a.fplane, sc,
                                                                   a.status, a.h, a.step, a.accuracy, a.consTol, a.projectEveryStep);
}
void rk64Group(const KArgs& a, cudaStream_t s) {
    rkMersonKernel<double, 3, false, true><<<a.P->nGroupBlocks, 128, 0, s>>>(
        *a.T, a.P->groupFirst, 0, a.ystate, a.time, static_cast<double*>(a.fbuf), a.fplane, static_cast<double*>(a.scratch), a.status,
        a.h, a.step, a.accuracy, a.consTol, a.projectEveryStep);
}

}  // namespace sbg
