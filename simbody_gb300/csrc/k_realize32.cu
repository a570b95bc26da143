// k_realize32.cu -- realize(Acceleration) and M^-1 f kernel instantiations,
// FP32 recursions (refine = the double-float residual refinement step).
#include "abi_device.cuh"

namespace sbg {

// occupancy variant: 1 = registers as needed (2 blocks of 128 per SM),
// 4 = at most 128 registers (4 blocks per SM, a few spills)
template <bool REF>
static void realize32(const DevTables& T, int nm, int variant, int blocks, const double* y,
                      double* ydot, float* sc, int32_t* status, cudaStream_t s) {
    if (variant == 4) {
    if (nm == 1) realizeKernel<float, 1, kTile, REF, 4><<<blocks, 128, 0, s>>>(T, y, ydot, sc, status);
        else realizeKernel<float, 3, kTile, REF, 4><<<blocks, 128, 0, s>>>(T, y, ydot, sc, status);
        return;
    }
    if (nm == 1) realizeKernel<float, 1, kTile, REF><<<blocks, 128, 0, s>>>(T, y, ydot, sc, status);
    else realizeKernel<float, 3, kTile, REF><<<blocks, 128, 0, s>>>(T, y, ydot, sc, status);
}

cudaError_t launchRealize32(const DevTables& T, int nm, bool refine, int variant, const double* y,
                            double* ydot, void* scratch, int32_t* status, cudaStream_t s) {
    const int blocks = (T.ninst + 127) / 128;
    if (blocks == 0) return cudaSuccess;
    float* sc = static_cast<float*>(scratch);
    if (refine) realize32<true>(T, nm, variant, blocks, y, ydot, sc, status, s);
    else realize32<false>(T, nm, variant, blocks, y, ydot, sc, status, s);
    return cudaGetLastError();
}

cudaError_t launchMInv32(const DevTables& T, int nm, const double* y, const double* f, double* out,
                         void* scratch, int32_t* status, cudaStream_t s) {
    const int threads = 128, blocks = (T.ninst + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    float* sc = static_cast<float*>(scratch);
    if (nm == 1) minvKernel<float, 1, kTile><<<blocks, threads, 0, s>>>(T, y, f, out, sc, status);
    else minvKernel<float, 3, kTile><<<blocks, threads, 0, s>>>(T, y, f, out, sc, status);
    return cudaGetLastError();
}

}  // namespace sbg
