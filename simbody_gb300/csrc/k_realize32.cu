// k_realize32.cu -- realize(Acceleration) kernel instantiations, float recursions.
#include "abi_device.cuh"

namespace sbg {

cudaError_t launchRealize32(const DevTables& T, int nm, const double* y, double* ydot, void* scratch,
                            int32_t* status, cudaStream_t s) {
    const int threads = 128, blocks = (T.ninst + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    float* sc = static_cast<float*>(scratch);
    if (nm == 1) realizeKernel<float, 1><<<blocks, threads, 0, s>>>(T, y, ydot, sc, status);
    else realizeKernel<float, 3><<<blocks, threads, 0, s>>>(T, y, ydot, sc, status);
    return cudaGetLastError();
}

cudaError_t launchMInv32(const DevTables& T, int nm, const double* y, const double* f, double* out, void* scratch,
                         int32_t* status, cudaStream_t s) {
    const int threads = 128, blocks = (T.ninst + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    float* sc = static_cast<float*>(scratch);
    if (nm == 1) minvKernel<float, 1><<<blocks, threads, 0, s>>>(T, y, f, out, sc, status);
    else minvKernel<float, 3><<<blocks, threads, 0, s>>>(T, y, f, out, sc, status);
    return cudaGetLastError();
}

}  // namespace sbg
