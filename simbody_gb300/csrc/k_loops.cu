// k_loops.cu -- kernels of the loop-closure segments (FP64): realize with
// Constraint::Ball multipliers and the tree M^-1 of those instances on the
// one-thread driver, and the level-parallel driver's realize and RK-Merson
// (the one-thread RK-Merson is in k_rkloops.cu).
#include "abi_device.cuh"

namespace sbg {


void realizeLoop(const KArgs& a, cudaStream_t s) {
    double* sc = static_cast<double*>(a.scratchLoop);
    const int first = a.P->nChain;
    const Launch1D L = spread(a.P->nLoop, 128);
    if (a.P->nm == 1)
        realizeKernel<double, 1, false, false, 1, true><<<L.grid, L.block, 0, s>>>(*a.T, first, a.P->nLoop, a.y, a.ydot, sc, a.status);
    else
        realizeKernel<double, 3, false, false, 1, true><<<L.grid, L.block, 0, s>>>(*a.T, first, a.P->nLoop, a.y, a.ydot, sc, a.status);
}

void minvLoop(const KArgs& a, cudaStream_t s) {
    double* sc = static_cast<double*>(a.scratchLoop);
    const int first = a.P->nChain;
    const Launch1D L = spread(a.P->nLoop, 128);
    if (a.P->nm == 1)
        minvKernel<double, 1, false><<<L.grid, L.block, 0, s>>>(*a.T, first, a.P->nLoop, a.y, a.f, a.ydot, sc, a.status);
    else
        minvKernel<double, 3, false><<<L.grid, L.block, 0, s>>>(*a.T, first, a.P->nLoop, a.y, a.f, a.ydot, sc, a.status);
}

// Loop-closure instances on the level-parallel driver (FP64): tree passes on
// the lanes of each instance's group, the multiplier solve and projections on
// its first lane. Blocks [loopGroupFirst, +nLoopGroupBlocks) of the block
// table; FP64 scratch and stage planes, records record-major (width in
// T.sstride).
void rkLoopGroup(const KArgs& a, cudaStream_t s) {
    if (a.P->nLoopGroupBlocks <= 0) return;
    rkMersonKernel<double, 3, false, true, 1, true><<<a.P->nLoopGroupBlocks, 128, 0, s>>>(
        *a.T, a.P->loopGroupFirst, 0, a.ystate, a.time, static_cast<double*>(a.fbufLoop), a.fplane,
        static_cast<double*>(a.scratchLoop), a.status, a.h, a.step, a.accuracy, a.consTol, a.projectEveryStep);
}
void realizeLoopGroup(const KArgs& a, cudaStream_t s) {
    if (a.P->nLoopGroupBlocks <= 0) return;
    realizeKernel<double, 3, false, true, 1, true><<<a.P->nLoopGroupBlocks, 128, 0, s>>>(
        *a.T, a.P->loopGroupFirst, 0, a.y, a.ydot, static_cast<double*>(a.scratchLoop), a.status);
}

}  // namespace sbg
