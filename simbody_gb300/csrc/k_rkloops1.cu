// k_rkloops1.cu -- RK-Merson with Constraint::Ball loop closures (FP64, the
// one-thread driver) for batches of width 1 (every non-Free body has one
// mobility); the width-3 form is in k_rkloops.cu.
#include "abi_device.cuh"

namespace sbg {

void rkLoopWidth1(const KArgs& a, cudaStream_t s) {
    double* sc = static_cast<double*>(a.scratchLoop);
    double* fb = static_cast<double*>(a.fbufLoop);
    const int first = a.P->nChain;
    const Launch1D L = spread(a.P->nLoop, 128);
    rkMersonKernel<double, 1, false, false, 1, true><<<L.grid, L.block, 0, s>>>(
        *a.T, first, a.P->nLoop, a.ystate, a.time, fb, a.fplane, sc, a.status, a.h, a.step, a.accuracy, a.consTol,
        a.projectEveryStep);
}

}  // namespace sbg
