// k_rk32.cu -- fixed-step RK-Merson persistent kernel instantiations, FP32
// recursions with FP64 state accumulation (refine = the double-float residual
// refinement step in every stage; variant 4 = at most 128 registers).
#include "abi_device.cuh"

namespace sbg {

template <bool REF, int MINB>
static void rk32(const DevTables& T, int nm, int blocks, double* y, double* time, float* fb, int64_t fplane,
                 float* sc, int32_t* status, double h, int nsteps, double acc, double ctol, int pes, cudaStream_t s) {
    if (nm == 1)
        rkMersonKernel<float, 1, kTile, REF, MINB><<<blocks, 128, 0, s>>>(T, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes);
    else
        rkMersonKernel<float, 3, kTile, REF, MINB><<<blocks, 128, 0, s>>>(T, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes);
}

cudaError_t launchRK32(const DevTables& T, int nm, bool refine, int variant, double* y, double* time, void* fbuf,
                       int64_t fplane, void* scratch, int32_t* status, double h, int nsteps, double acc, double ctol,
                       int pes, cudaStream_t s) {
    const int blocks = (T.ninst + 127) / 128;
    if (blocks == 0) return cudaSuccess;
    float* fb = static_cast<float*>(fbuf);
    float* sc = static_cast<float*>(scratch);
    if (refine) {
        if (variant == 4) rk32<true, 4>(T, nm, blocks, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes, s);
        else rk32<true, 1>(T, nm, blocks, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes, s);
    } else {
        if (variant == 4) rk32<false, 4>(T, nm, blocks, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes, s);
        else rk32<false, 1>(T, nm, blocks, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes, s);
    }
    return cudaGetLastError();
}

}  // namespace sbg
