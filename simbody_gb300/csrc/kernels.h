// kernels.h -- host-callable launchers of the CUDA kernels (abi_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "engine.h"
#include "../../include/simbody_gb300.h"

namespace sbg {

// precision: 0 = FP64, 1 = mixed (FP32 recursions). nm = largest non-Free
// mobility count in the batch (1, 2 or 3), a compile-time width.
cudaError_t launchRealize(const DevTables& T, int precision, int nm, const double* y, double* ydot, void* scratch,
                          int32_t* status, cudaStream_t s);
cudaError_t launchRKMerson(const DevTables& T, int precision, int nm, double* y, double* time, void* fbuf,
                           int64_t fplane, void* scratch, int32_t* status, double h, int nsteps, double accuracy,
                           double consTol, int projectEveryStep, cudaStream_t s);
cudaError_t launchNormalizeQuat(const DevTables& T, double* y, cudaStream_t s);
// part 0 moves whole [q,u] records, part 1 only the u slots.
cudaError_t launchScatter(const DevTables& T, const int64_t* hostOff, const double* packed, double* cols, int part,
                          cudaStream_t s);
cudaError_t launchGather(const DevTables& T, const int64_t* hostOff, const double* cols, double* packed, int part,
                         cudaStream_t s);
cudaError_t launchMInv(const DevTables& T, int precision, int nm, const double* y, const double* f, double* out,
                       void* scratch, int32_t* status, cudaStream_t s);

}  // namespace sbg
