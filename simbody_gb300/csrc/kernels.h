// kernels.h -- host-callable launchers of the CUDA kernels (k_*.cu, serve.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "engine.h"
#include "../../include/simbody_gb300.h"

namespace sbg {

// Streams of a batch: the chain segment runs on `main`, the level-parallel
// segment on `side` (forked from and joined back into `main` with events),
// so the two overlap on the GPU.
struct Streams {
    cudaStream_t main, side;
    cudaEvent_t fork, join;
};

// How far one RK-Merson call steps (RungeKuttaMersonIntegrator with a fixed
// step size, AbstractIntegratorRep.cpp:341-577):
//   nsteps >= 0  exactly nsteps steps of h (t1 = t0 + h; tMax = infinity)
//   nsteps <  0  Integrator::stepTo(tStop) with interpolation off
//                (setAllowInterpolation(false): tMax = tStop). Each step picks
//                t1 by takeOneStep's rule (:536-544): tStop when it lies within
//                0.95 h, t0 + h when it lies beyond 1.001 h, else tStop; the
//                call ends once t reaches tStop.
//   init         Integrator::initialize first: quaternions normalised (the
//                caller's launch) and, with loop closures, the forced
//                position and velocity projections; 0 continues the
//                integration where the previous call left it.
//   maxSteps     > 0: at most this many steps in this launch (the one-step
//                launches of a mixed batch integration)
//   launch       index of this one-step launch (only its parity is used)
struct StepCtl {
    int nsteps;
    int init;
    double tStop;
    int maxSteps;
    int launch;
};
constexpr int kMaxStepsPerCall = 1 << 30;

// precision: SBG_PRECISION_FP64, _MIXED (FP32 recursions + double-float
// residual refinement) or _MIXED_FAST (FP32 recursions only).
// Buffers of a batch the launchers need besides the tables.
struct BatchBufs {
    void* scratch;       // scratch of the chain and group segments (R)
    void* scratchLoop;   // FP64 scratch of the loop-closure segment
    void* fbuf;          // RK stage derivatives (R), 4 planes of fplane elements
    void* fbufLoop;      // FP64 stage derivatives of the loop-closure segment, 4 planes
    int64_t fplane;
};
cudaError_t launchRealize(const DevTables& T, const LaunchPlan& P, int precision, const double* y, double* ydot,
                          const BatchBufs& B, int32_t* status, const Streams& s);
cudaError_t launchMInv(const DevTables& T, const LaunchPlan& P, int precision, const double* y, const double* f,
                       double* out, const BatchBufs& B, int32_t* status, const Streams& s);
cudaError_t launchRKMerson(const DevTables& T, const LaunchPlan& P, int precision, double* y, double* time,
                           const BatchBufs& B, int32_t* status, double h, StepCtl step, double accuracy,
                           double consTol, int projectEveryStep, const Streams& s);
// Tree operators (k_ops.cu, ops_device.cuh). Operands in the host packing:
// u-like arrays nu values per instance at uoff[inst]; body arrays one entry
// per mobilized body, in descriptor body order, from boff[inst] (6 values per
// SpatialVec, 10 per spatial inertia). scratch is FP64 scratch laid out like
// the batch's own (its element offsets), scratchLoop the loop segment's.
enum : int { OP_RESIDUAL = 0, OP_MV = 1, OP_JV = 2, OP_JTF = 3, OP_COMPOSITE = 4 };
struct OpIO {
    int kind;
    const double* x;      // udot / a / u-like vector (null = zero)
    const double* fmob;   // applied mobility forces (null = zero)
    const double* fbody;  // applied body forces in Ground (null = zero)
    double* out;
    const int64_t* uoff;
    const int64_t* boff;
};
cudaError_t launchTreeOp(const DevTables& T, const LaunchPlan& P, const OpIO& io, const double* y, double* scratch,
                         double* scratchLoop, int32_t* status, cudaStream_t s);
cudaError_t launchNormalizeQuat(const DevTables& T, double* y, cudaStream_t s);
// qdotdot of every instance from the resident y and ydot, nq values per
// instance at qHost[inst] of out.
cudaError_t launchQDotDot(const DevTables& T, const int64_t* qHost, const double* y, const double* ydot, double* out,
                          cudaStream_t s);
// part 0 moves whole [q,u] records, part 1 only the u slots; instances
// [inst0, inst0 + count) (count < 0: to the end).
cudaError_t launchScatter(const DevTables& T, const int64_t* hostOff, const double* packed, double* cols, int part,
                          cudaStream_t s, int inst0 = 0, int count = -1);
cudaError_t launchGather(const DevTables& T, const int64_t* hostOff, const double* cols, double* packed, int part,
                         cudaStream_t s, int inst0 = 0, int count = -1);


// Grid of a one-thread-per-instance launch of n threads with at most bs per
// block: blocks shrink (to no fewer than 8 threads) until there are at least
// two per SM, so that a small batch spreads over every SM (an FP64-bound
// kernel otherwise leaves most SMs' FP64 units idle).
struct Launch1D {
    int grid, block;
};
inline Launch1D spread(int64_t n, int bs) {
    static int sms = 0;
    if (!sms) {
        int d = 0, c = 0;
        if (cudaGetDevice(&d) == cudaSuccess && cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, d) == cudaSuccess)
            sms = c > 0 ? c : 1;
        else
            sms = 1;
    }
    while (bs > 8 && (n + bs - 1) / bs < 2 * sms) bs >>= 1;
    return Launch1D{(int)((n + bs - 1) / bs), bs};
}

// Error-controlled RK-Merson (k_rkadapt.cu): Integrator::setFinalTime(tFinal),
// initialize, stepTo(tFinal) with the given initial, minimum and maximum step
// sizes (<= 0: the reference's defaults: initial 0.01, no limits) and at most
// maxSteps accepted steps per instance. stats: accepted and rejected steps per
// instance (2 values each; null = not wanted).
struct AdaptCtl {
    double tFinal, hInit, hMin, hMax, accuracy, consTol;
    int projectEveryStep, maxSteps;
    long long* stats;
};

// Per-segment launchers (k_r64.cu, k_r32c.cu, k_r32g.cu, k_rk64.cu,
// k_rk32c.cu, k_rk32g.cu).
struct KArgs {
    const DevTables* T;
    const LaunchPlan* P;
    const double* y;     // realize / M^-1 input state
    double* ydot;        // realize / M^-1 output
    const double* f;     // M^-1 input forces
    double* ystate;      // RK state (in place)
    double* time;
    void* fbuf;
    int64_t fplane;
    void* scratch;
    void* scratchLoop;   // FP64 scratch of the loop-closure segment
    void* fbufLoop;      // FP64 stage derivatives of the loop-closure segment
    int32_t* status;
    double h, accuracy, consTol;
    StepCtl step;
    int projectEveryStep;
};
void realize64Chain(const KArgs& a, cudaStream_t s);
void realize64Group(const KArgs& a, cudaStream_t s);
void minv64Chain(const KArgs& a, cudaStream_t s);
void minv64Group(const KArgs& a, cudaStream_t s);
void realize32Chain(const KArgs& a, bool refine, cudaStream_t s);
// Variant 8: the chain driver with record fields staged through shared
// memory (one shared chain topology, no Free bodies, segment start a
// multiple of 32).
void realize32ChainStaged(const KArgs& a, bool refine, cudaStream_t s);
void realize32Group(const KArgs& a, bool refine, cudaStream_t s);
void minv32Chain(const KArgs& a, cudaStream_t s);
void minv32Group(const KArgs& a, cudaStream_t s);
void rk64Chain(const KArgs& a, cudaStream_t s);
void rk64Group(const KArgs& a, cudaStream_t s);
void rk32Chain(const KArgs& a, bool refine, cudaStream_t s);
void rk32Group(const KArgs& a, bool refine, cudaStream_t s);
// FP64 recomputation of the instances the mixed realize flagged
// SBG_INST_ILL_CONDITIONED (k_fallback.cu); a no-op without T.scratch64.
void realizeFallback(const KArgs& a, bool group, cudaStream_t s);
void realizeLoop(const KArgs& a, cudaStream_t s);  // k_loops.cu
void minvLoop(const KArgs& a, cudaStream_t s);
void rkLoop(const KArgs& a, cudaStream_t s);
void rkLoopWidth1(const KArgs& a, cudaStream_t s);  // k_rkloops1.cu: rkLoop for batch width 1
void rkLoopGroup(const KArgs& a, cudaStream_t s);      // loop closures, level-parallel driver
void rkAdaptiveChain(const KArgs& a, const AdaptCtl& ac, cudaStream_t s);  // k_rkadapt.cu (FP64)
void rkAdaptiveGroup(const KArgs& a, const AdaptCtl& ac, cudaStream_t s);
// One FP64 RK-Merson step for each instance in FP64 mode at this launch
// (T.fbList[launch & 1]) on FP64 records at rowsBase: one thread (lanes 1) or
// kFbLanes lanes of the level-parallel driver per instance (k_fallback.cu).
void rkFp64List(const KArgs& a, const int64_t* rowsBase, double* rows, int lanes, cudaStream_t s);
cudaError_t launchRKFp64List(const DevTables& T, const LaunchPlan& P, double* y, double* time, int32_t* status,
                             double h, StepCtl step, double accuracy, double consTol, int projectEveryStep,
                             int64_t fplane, const int64_t* rowsBase, double* rows, int lanes, cudaStream_t s);
cudaError_t launchFillInt(int32_t* p, int n, int v, cudaStream_t s);
// *out = instances with steps left in a one-step integration call
cudaError_t launchCountUnfinished(int n, const int32_t* stepsLeft, const double* time, const int32_t* status,
                                  double tStop, int32_t* out, cudaStream_t s);
void realizeLoopGroup(const KArgs& a, cudaStream_t s);

}  // namespace sbg
