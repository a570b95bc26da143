// k_rk64.cu -- fixed-step RK-Merson persistent kernel instantiations, FP64 recursions.
#include "abi_device.cuh"

namespace sbg {

cudaError_t launchRK64(const DevTables& T, int nm, double* y, double* time, void* fbuf, int64_t fplane,
                       void* scratch, int32_t* status, double h, int nsteps, double acc, double ctol, int pes,
                       cudaStream_t s) {
    const int threads = 128, blocks = (T.ninst + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    double* fb = static_cast<double*>(fbuf);
    double* sc = static_cast<double*>(scratch);
    if (nm == 1)
        rkMersonKernel<double, 1, kTile, false><<<blocks, threads, 0, s>>>(T, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes);
    else
        rkMersonKernel<double, 3, kTile, false><<<blocks, threads, 0, s>>>(T, y, time, fb, fplane, sc, status, h, nsteps, acc, ctol, pes);
    return cudaGetLastError();
}

}  // namespace sbg
