// k_util.cu -- state packing kernels, quaternion normalization and the
// precision dispatch of the launchers.
#include "abi_device.cuh"

namespace sbg {

// Integrator::initialize forces a projection: quaternions are normalized
// (Integrator.cpp:376-377, RigidBodyNodeSpec_Ball.h:417-434).
__global__ void normalizeQuatKernel(DevTables T, double* __restrict__ y) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T.ninst) return;
    const int inst = T.order[t];
    const int64_t base = T.ybase[inst], stride = T.ystride[inst];
    const int body0 = T.ibody[inst], nb = T.inb[inst];
    for (int lb = 0; lb < nb; ++lb) {
        const int row = body0 + lb;
        const int type = T.info[row] & 15;
        if (type != T_BALL && type != T_FREE) continue;
        const int qo = T.qoff[row];
        double qq[4];
        for (int j = 0; j < 4; ++j) qq[j] = y[base + (int64_t)(qo + j) * stride];
        const double len = sqrt(qq[0] * qq[0] + qq[1] * qq[1] + qq[2] * qq[2] + qq[3] * qq[3]);
        for (int j = 0; j < 4; ++j) y[base + (int64_t)(qo + j) * stride] = qq[j] / len;
    }
}

// Pack/unpack between the host's per-instance packing and the columns.
// part 0: all of [q,u]; part 1: the u slots only (nu values per instance).
__global__ void scatterKernel(DevTables T, const int64_t* __restrict__ hostOff, const double* __restrict__ packed,
                              double* __restrict__ cols, int part) {
    const int inst = blockIdx.x;
    const int nq = T.inq[inst];
    const int cnt = part == 0 ? nq + T.inu[inst] : T.inu[inst];
    const int c0 = part == 0 ? 0 : nq;
    const int64_t base = T.ybase[inst], stride = T.ystride[inst], off = hostOff[inst];
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) cols[base + (int64_t)(c0 + k) * stride] = packed[off + k];
}
__global__ void gatherKernel(DevTables T, const int64_t* __restrict__ hostOff, const double* __restrict__ cols,
                             double* __restrict__ packed, int part) {
    const int inst = blockIdx.x;
    const int nq = T.inq[inst];
    const int cnt = part == 0 ? nq + T.inu[inst] : T.inu[inst];
    const int c0 = part == 0 ? 0 : nq;
    const int64_t base = T.ybase[inst], stride = T.ystride[inst], off = hostOff[inst];
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) packed[off + k] = cols[base + (int64_t)(c0 + k) * stride];
}

cudaError_t launchRealize64(const DevTables& T, int nm, const double* y, double* ydot, void* scratch,
                            int32_t* status, cudaStream_t s);
cudaError_t launchRealize32(const DevTables& T, int nm, bool refine, int variant, const double* y,
                            double* ydot, void* scratch, int32_t* status, cudaStream_t s);
cudaError_t launchMInv64(const DevTables& T, int nm, const double* y, const double* f, double* out,
                         void* scratch, int32_t* status, cudaStream_t s);
cudaError_t launchMInv32(const DevTables& T, int nm, const double* y, const double* f, double* out,
                         void* scratch, int32_t* status, cudaStream_t s);
cudaError_t launchRK64(const DevTables& T, int nm, double* y, double* time, void* fbuf, int64_t fplane,
                       void* scratch, int32_t* status, double h, int nsteps, double acc, double ctol, int pes,
                       cudaStream_t s);
cudaError_t launchRK32(const DevTables& T, int nm, bool refine, int variant, double* y, double* time, void* fbuf,
                       int64_t fplane, void* scratch, int32_t* status, double h, int nsteps, double acc, double ctol,
                       int pes, cudaStream_t s);

cudaError_t launchRealize(const DevTables& T, int precision, int nm, int variant, const double* y,
                          double* ydot, void* scratch, int32_t* status, cudaStream_t s) {
    if (precision == SBG_PRECISION_FP64) return launchRealize64(T, nm, y, ydot, scratch, status, s);
    return launchRealize32(T, nm, precision == SBG_PRECISION_MIXED, variant, y, ydot, scratch, status, s);
}

cudaError_t launchMInv(const DevTables& T, int precision, int nm, const double* y, const double* f,
                       double* out, void* scratch, int32_t* status, cudaStream_t s) {
    return precision == SBG_PRECISION_FP64 ? launchMInv64(T, nm, y, f, out, scratch, status, s)
                                           : launchMInv32(T, nm, y, f, out, scratch, status, s);
}

cudaError_t launchRKMerson(const DevTables& T, int precision, int nm, int variant, double* y, double* time,
                           void* fbuf, int64_t fplane, void* scratch, int32_t* status, double h, int nsteps,
                           double accuracy, double consTol, int projectEveryStep, cudaStream_t s) {
    if (precision == SBG_PRECISION_FP64)
        return launchRK64(T, nm, y, time, fbuf, fplane, scratch, status, h, nsteps, accuracy, consTol,
                          projectEveryStep, s);
    return launchRK32(T, nm, precision == SBG_PRECISION_MIXED, variant, y, time, fbuf, fplane, scratch, status, h,
                      nsteps, accuracy, consTol, projectEveryStep, s);
}

cudaError_t launchNormalizeQuat(const DevTables& T, double* y, cudaStream_t s) {
    const int threads = 128, blocks = (T.ninst + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    normalizeQuatKernel<<<blocks, threads, 0, s>>>(T, y);
    return cudaGetLastError();
}

cudaError_t launchScatter(const DevTables& T, const int64_t* hostOff, const double* packed, double* cols, int part,
                          cudaStream_t s) {
    if (T.ninst == 0) return cudaSuccess;
    scatterKernel<<<T.ninst, 128, 0, s>>>(T, hostOff, packed, cols, part);
    return cudaGetLastError();
}

cudaError_t launchGather(const DevTables& T, const int64_t* hostOff, const double* cols, double* packed, int part,
                         cudaStream_t s) {
    if (T.ninst == 0) return cudaSuccess;
    gatherKernel<<<T.ninst, 128, 0, s>>>(T, hostOff, cols, packed, part);
    return cudaGetLastError();
}

}  // namespace sbg
