// k_rk32.cu -- fixed-step RK-Merson persistent kernel instantiations, float recursions.
#include "abi_device.cuh"

namespace sbg {

cudaError_t launchRK32(const DevTables& T, int nm, double* y, double* time, void* fbuf, int64_t fplane,
                       void* scratch, int32_t* status, double h, int nsteps, double acc, double ctol, int pes,
                       cudaStream_t s) {
    const int threads = 128, blocks = (T.ninst + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    float* fb = static_cast<float*>(fbuf);
    float* sc = static_cast<float*>(scratch);
    if (nm == 1) rkMersonKernel<float, 1><<<blocks, threads, 0, s>>>(T, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes);
    else rkMersonKernel<float, 3><<<blocks, threads, 0, s>>>(T, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes);
    return cudaGetLastError();
}

}  // namespace sbg
