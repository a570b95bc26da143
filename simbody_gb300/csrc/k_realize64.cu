// k_realize64.cu -- realize(Acceleration) and M^-1 f kernel instantiations,
// FP64 recursions.
#include "abi_device.cuh"

namespace sbg {

cudaError_t launchRealize64(const DevTables& T, int nm, const double* y, double* ydot, void* scratch,
                            int32_t* status, cudaStream_t s) {
    const int threads = 128, blocks = (T.ninst + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    double* sc = static_cast<double*>(scratch);
    if (nm == 1) realizeKernel<double, 1, kTile, false><<<blocks, threads, 0, s>>>(T, y, ydot, sc, status);
    else realizeKernel<double, 3, kTile, false><<<blocks, threads, 0, s>>>(T, y, ydot, sc, status);
    return cudaGetLastError();
}

cudaError_t launchMInv64(const DevTables& T, int nm, const double* y, const double* f, double* out,
                         void* scratch, int32_t* status, cudaStream_t s) {
    const int threads = 128, blocks = (T.ninst + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    double* sc = static_cast<double*>(scratch);
    if (nm == 1) minvKernel<double, 1, kTile><<<blocks, threads, 0, s>>>(T, y, f, out, sc, status);
    else minvKernel<double, 3, kTile><<<blocks, threads, 0, s>>>(T, y, f, out, sc, status);
    return cudaGetLastError();
}

}  // namespace sbg
