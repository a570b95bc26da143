// k_rkloops.cu -- RK-Merson with Constraint::Ball loop closures (FP64, the
// one-thread driver): multipliers, projections and quaternion normalisation
// inside the persistent kernel.
#include "abi_device.cuh"

namespace sbg {

// Batch width 3 here; width 1 (every non-Free body one mobility) in
// k_rkloops1.cu, so that the two compile in parallel.
void rkLoop(const KArgs& a, cudaStream_t s) {
    if (a.P->nm == 1) {
        rkLoopWidth1(a, s);
        return;
    }
    double* sc = static_cast<double*>(a.scratchLoop);
    double* fb = static_cast<double*>(a.fbufLoop);
    const int first = a.P->nChain;
    const Launch1D L = spread(a.P->nLoop, 128);
    rkMersonKernel<double, 3, false, false, 1, true><<<L.grid, L.block, 0, s>>>(
        *a.T, first, a.P->nLoop, a.ystate, a.time, fb, a.fplane, sc, a.status, a.h, a.step, a.accuracy, a.consTol,
        a.projectEveryStep);
}

}  // namespace sbg
