// k_rk32.cu -- fixed-step RK-Merson persistent kernel instantiations, FP32
// recursions with FP64 state accumulation (refine = the double-float residual
// refinement step in every stage).
#include "abi_device.cuh"

namespace sbg {

template <bool REF>
static void rk32(const DevTables& T, int nm, bool tiled, int blocks, double* y, double* time, float* fb,
                 int64_t fplane, float* sc, int32_t* status, double h, int nsteps, double acc, double ctol, int pes,
                 cudaStream_t s) {
    if (!tiled)
        rkMersonKernel<float, 3, 1, REF><<<blocks, 128, 0, s>>>(T, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes);
    else if (nm == 1)
        rkMersonKernel<float, 1, kTile, REF><<<blocks, 128, 0, s>>>(T, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes);
    else
        rkMersonKernel<float, 3, kTile, REF><<<blocks, 128, 0, s>>>(T, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes);
}

cudaError_t launchRK32(const DevTables& T, int nm, bool tiled, bool refine, double* y, double* time, void* fbuf,
                       int64_t fplane, void* scratch, int32_t* status, double h, int nsteps, double acc, double ctol,
                       int pes, cudaStream_t s) {
    const int blocks = (T.ninst + 127) / 128;
    if (blocks == 0) return cudaSuccess;
    float* fb = static_cast<float*>(fbuf);
    float* sc = static_cast<float*>(scratch);
    if (refine) rk32<true>(T, nm, tiled, blocks, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes, s);
    else rk32<false>(T, nm, tiled, blocks, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes, s);
    return cudaGetLastError();
}

}  // namespace sbg
