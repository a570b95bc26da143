// kernels.h -- host-callable launchers of the CUDA kernels (abi_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "engine.h"
#include "../../include/simbody_gb300.h"

namespace sbg {

// precision: SBG_PRECISION_FP64, _MIXED (FP32 recursions + double-float
// residual refinement) or _MIXED_FAST (FP32 recursions only). nm = largest
// non-Free mobility count (1 or 3), a compile-time width. Every batch uses
// warp-tiled state columns and scratch records.
// variant: kernel occupancy variant (1 or 4), chosen by the batch's tuner.
cudaError_t launchRealize(const DevTables& T, int precision, int nm, int variant, const double* y,
                          double* ydot, void* scratch, int32_t* status, cudaStream_t s);
cudaError_t launchRKMerson(const DevTables& T, int precision, int nm, int variant, double* y, double* time,
                           void* fbuf, int64_t fplane, void* scratch, int32_t* status, double h, int nsteps,
                           double accuracy, double consTol, int projectEveryStep, cudaStream_t s);
cudaError_t launchNormalizeQuat(const DevTables& T, double* y, cudaStream_t s);
// part 0 moves whole [q,u] records, part 1 only the u slots.
cudaError_t launchScatter(const DevTables& T, const int64_t* hostOff, const double* packed, double* cols, int part,
                          cudaStream_t s);
cudaError_t launchGather(const DevTables& T, const int64_t* hostOff, const double* cols, double* packed, int part,
                         cudaStream_t s);
cudaError_t launchMInv(const DevTables& T, int precision, int nm, const double* y, const double* f,
                       double* out, void* scratch, int32_t* status, cudaStream_t s);

}  // namespace sbg
