// k_ops.cu -- launchers of the tree operators (ops_device.cuh), FP64.
#include "abi_device.cuh"
#include "ops_device.cuh"

namespace sbg {

// The chain segment, the loop-closure segment and the level-parallel segment
// in turn on one stream (a tree operator is one short pass over the batch).
cudaError_t launchTreeOp(const DevTables& T, const LaunchPlan& P, const OpIO& io, const double* y, double* scratch,
                         double* scratchLoop, int32_t* status, cudaStream_t s) {
    if (P.nChain > 0) {
        const Launch1D L = spread(P.nChain, 128);
        if (P.nm == 1) treeOpKernel<1, 0><<<L.grid, L.block, 0, s>>>(T, 0, P.nChain, y, scratch, io, status);
        else treeOpKernel<3, 0><<<L.grid, L.block, 0, s>>>(T, 0, P.nChain, y, scratch, io, status);
    }
    if (P.nLoop > 0) {
        const Launch1D L = spread(P.nLoop, 128);
        if (P.nm == 1) treeOpKernel<1, 1><<<L.grid, L.block, 0, s>>>(T, P.nChain, P.nLoop, y, scratchLoop, io, status);
        else treeOpKernel<3, 1><<<L.grid, L.block, 0, s>>>(T, P.nChain, P.nLoop, y, scratchLoop, io, status);
    }
    if (P.nGroupBlocks > 0)
        treeOpKernel<3, 2><<<P.nGroupBlocks, 128, 0, s>>>(T, P.groupFirst, 0, y, scratch, io, status);
    return cudaGetLastError();
}

}  // namespace sbg
