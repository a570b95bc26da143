// k_realize32.cu -- realize(Acceleration) and M^-1 f kernel instantiations,
// FP32 recursions (refine = the double-float residual refinement step).
#include "abi_device.cuh"

namespace sbg {

template <bool REF>
static void realize32(const DevTables& T, int nm, bool tiled, int blocks, const double* y, double* ydot, float* sc,
                      int32_t* status, cudaStream_t s) {
    if (!tiled) realizeKernel<float, 3, 1, REF><<<blocks, 128, 0, s>>>(T, y, ydot, sc, status);
    else if (nm == 1) realizeKernel<float, 1, kTile, REF><<<blocks, 128, 0, s>>>(T, y, ydot, sc, status);
    else realizeKernel<float, 3, kTile, REF><<<blocks, 128, 0, s>>>(T, y, ydot, sc, status);
}

cudaError_t launchRealize32(const DevTables& T, int nm, bool tiled, bool refine, const double* y, double* ydot,
                            void* scratch, int32_t* status, cudaStream_t s) {
    const int blocks = (T.ninst + 127) / 128;
    if (blocks == 0) return cudaSuccess;
    float* sc = static_cast<float*>(scratch);
    if (refine) realize32<true>(T, nm, tiled, blocks, y, ydot, sc, status, s);
    else realize32<false>(T, nm, tiled, blocks, y, ydot, sc, status, s);
    return cudaGetLastError();
}

cudaError_t launchMInv32(const DevTables& T, int nm, bool tiled, const double* y, const double* f, double* out,
                         void* scratch, int32_t* status, cudaStream_t s) {
    const int threads = 128, blocks = (T.ninst + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    float* sc = static_cast<float*>(scratch);
    if (!tiled) minvKernel<float, 3, 1><<<blocks, threads, 0, s>>>(T, y, f, out, sc, status);
    else if (nm == 1) minvKernel<float, 1, kTile><<<blocks, threads, 0, s>>>(T, y, f, out, sc, status);
    else minvKernel<float, 3, kTile><<<blocks, threads, 0, s>>>(T, y, f, out, sc, status);
    return cudaGetLastError();
}

}  // namespace sbg
