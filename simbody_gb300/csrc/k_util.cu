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
    if (T.incons[inst] > 0) return;  // loop closures: the RK kernel's initialization projects and normalizes
    const int64_t base = T.ybase[inst], stride = T.ystride[inst];
    const int body0 = T.ibody[inst], nb = T.inb[inst];
    for (int lb = 0; lb < nb; ++lb) {
        const int row = body0 + lb;
        if (T.info[row] & F_QUAT) normalizeQuatAt(y, base, stride, T.qoff[row]);
    }
}

// State::getQDotDot() at Stage::Acceleration from the resident state and the
// last realize's udot, into the host packing (nq values per instance from
// qHost[inst]): qdotdot = udot for Pin/Slider/Universal; for the quaternion
// of a Ball or Free body N(q) udot_w - |w|^2/4 q with the unnormalized q
// (Rotation.h:1006-1013: convertAngVelDotToQuaternionDotDot), then the Free
// body's translational udot (RigidBodyNodeSpec_Ball.h:355-390,
// RigidBodyNodeSpec_Free.h:418-455). One thread per instance.
__global__ void qdotdotKernel(DevTables T, const int64_t* __restrict__ qHost, const double* __restrict__ y,
                              const double* __restrict__ ydot, double* __restrict__ out) {
    const int inst = blockIdx.x * blockDim.x + threadIdx.x;
    if (inst >= T.ninst) return;
    const int64_t base = T.ybase[inst], stride = T.ystride[inst];
    const int nq = T.inq[inst], body0 = T.ibody[inst], nb = T.inb[inst];
    double* o = out + qHost[inst];
    auto Y = [&](int k) { return y[base + (int64_t)k * stride]; };
    auto UD = [&](int k) { return ydot[base + (int64_t)(nq + k) * stride]; };
    for (int lb = 0; lb < nb; ++lb) {
        const int row = body0 + lb;
        const int type = T.info[row] & 15, n = (T.info[row] >> 4) & 15;
        const int qo = T.qoff[row], uo = T.uoff[row];
        if (type == T_BALL || type == T_FREE) {
            if (!(T.info[row] & F_QUAT)) {
                // body-fixed X-Y-Z angles: Rotation::convertAngAccInParentToBodyXYZDotDot
                // (Rotation.h:1041-1060) with qdot = N_P(q) w (Rotation.h:395-406)
                double c0, s0, c1, s1;
                sincos(Y(qo), &s0, &c0);
                sincos(Y(qo + 1), &s1, &c1);
                const double ooc1 = 1.0 / c1;
                const double w0 = Y(nq + uo), w1 = Y(nq + uo + 1), w2 = Y(nq + uo + 2);
                const double b0 = UD(uo), b1 = UD(uo + 1), b2 = UD(uo + 2);
                const double tw = (s0 * w1 - c0 * w2) * ooc1, tb = (s0 * b1 - c0 * b2) * ooc1;
                const double qd0 = w0 + tw * s1, qd2 = -tw;
                const double qd1 = c0 * w1 + s0 * w2;
                const double q1oc1 = qd1 * ooc1;
                o[qo + 0] = (b0 + tb * s1) + (qd0 * s1 - qd2) * q1oc1;
                o[qo + 1] = (c0 * b1 + s0 * b2) + qd0 * qd2 * c1;
                o[qo + 2] = -tb + (qd2 * s1 - qd0) * q1oc1;
                if (type == T_FREE) {
                    for (int k = 0; k < 3; ++k) o[qo + 3 + k] = UD(uo + 3 + k);
                    o[qo + 6] = 0.0;
                } else {
                    o[qo + 3] = 0.0;  // the unused slot
                }
                continue;
            }
        } else {  // u = qdot
            for (int k = 0; k < n; ++k) o[qo + k] = UD(uo + k);
            continue;
        }
        const double q0 = Y(qo), q1 = Y(qo + 1), q2 = Y(qo + 2), q3 = Y(qo + 3);
        const double w0 = Y(nq + uo), w1 = Y(nq + uo + 1), w2 = Y(nq + uo + 2);
        const double b0 = UD(uo), b1 = UD(uo + 1), b2 = UD(uo + 2);
        const double e0 = 0.5 * q0, e1 = 0.5 * q1, e2 = 0.5 * q2, e3 = 0.5 * q3;
        const double s = -0.25 * (w0 * w0 + w1 * w1 + w2 * w2);
        o[qo + 0] = (-e1 * b0 + -e2 * b1 + -e3 * b2) + s * q0;
        o[qo + 1] = (e0 * b0 + e3 * b1 + -e2 * b2) + s * q1;
        o[qo + 2] = (-e3 * b0 + e0 * b1 + e1 * b2) + s * q2;
        o[qo + 3] = (e2 * b0 + -e1 * b1 + e0 * b2) + s * q3;
        if (type == T_FREE)
            for (int k = 0; k < 3; ++k) o[qo + 4 + k] = UD(uo + 3 + k);
    }
}

cudaError_t launchQDotDot(const DevTables& T, const int64_t* qHost, const double* y, const double* ydot, double* out,
                          cudaStream_t s) {
    const int threads = 128, blocks = (T.ninst + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    qdotdotKernel<<<blocks, threads, 0, s>>>(T, qHost, y, ydot, out);
    return cudaGetLastError();
}

// Pack/unpack between the host's per-instance packing and the columns.
// part 0: all of [q,u]; part 1: the u slots only (nu values per instance).
__global__ void scatterKernel(DevTables T, const int64_t* __restrict__ hostOff, const double* __restrict__ packed,
                              double* __restrict__ cols, int part, int inst0) {
    const int inst = inst0 + blockIdx.x;
    const int nq = T.inq[inst];
    const int cnt = part == 0 ? nq + T.inu[inst] : T.inu[inst];
    const int c0 = part == 0 ? 0 : nq;
    const int64_t base = T.ybase[inst], stride = T.ystride[inst], off = hostOff[inst];
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) cols[base + (int64_t)(c0 + k) * stride] = packed[off + k];
}
__global__ void gatherKernel(DevTables T, const int64_t* __restrict__ hostOff, const double* __restrict__ cols,
                             double* __restrict__ packed, int part, int inst0) {
    const int inst = inst0 + blockIdx.x;
    const int nq = T.inq[inst];
    const int cnt = part == 0 ? nq + T.inu[inst] : T.inu[inst];
    const int c0 = part == 0 ? 0 : nq;
    const int64_t base = T.ybase[inst], stride = T.ystride[inst], off = hostOff[inst];
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) packed[off + k] = cols[base + (int64_t)(c0 + k) * stride];
}

// Run the chain segment, then the loop-closure segment, on the main stream
// and the level-parallel segment on the side stream, forked from and joined
// back into the main stream.
template <class FC, class FL, class FG>
static cudaError_t forkJoin(const LaunchPlan& P, const Streams& s, FC chain, FL loops, FG group) {
    const bool c = P.nChain > 0 || P.nLoop > 0, g = P.nGroupBlocks > 0;
    auto mainWork = [&](cudaStream_t st) {
        if (P.nChain > 0) chain(st);
        if (P.nLoop > 0) loops(st);
    };
    if (c && g) {
        cudaError_t e = cudaEventRecord(s.fork, s.main);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s.side, s.fork, 0);
        if (e != cudaSuccess) return e;
        group(s.side);
        mainWork(s.main);
        e = cudaEventRecord(s.join, s.side);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s.main, s.join, 0);
        if (e != cudaSuccess) return e;
    } else if (c) {
        mainWork(s.main);
    } else if (g) {
        group(s.main);
    }
    return cudaGetLastError();
}

static KArgs baseArgs(const DevTables& T, const LaunchPlan& P, const BatchBufs& B, int32_t* status) {
    KArgs a{};
    a.T = &T; a.P = &P; a.scratch = B.scratch; a.scratchLoop = B.scratchLoop; a.fbuf = B.fbuf;
    a.fbufLoop = B.fbufLoop; a.fplane = B.fplane; a.status = status;
    return a;
}

cudaError_t launchRealize(const DevTables& T, const LaunchPlan& P, int precision, const double* y, double* ydot,
                          const BatchBufs& B, int32_t* status, const Streams& s) {
    KArgs a = baseArgs(T, P, B, status);
    a.y = y; a.ydot = ydot;
    auto loops = [&](cudaStream_t st) { realizeLoop(a, st); };
    if (precision == SBG_PRECISION_FP64)
        return forkJoin(P, s, [&](cudaStream_t st) { realize64Chain(a, st); }, loops,
                        [&](cudaStream_t st) { realize64Group(a, st); });
    const bool ref = precision == SBG_PRECISION_MIXED;
    return forkJoin(P, s, [&](cudaStream_t st) { realize32Chain(a, ref, st); }, loops,
                    [&](cudaStream_t st) { realize32Group(a, ref, st); });
}

cudaError_t launchMInv(const DevTables& T, const LaunchPlan& P, int precision, const double* y, const double* f,
                       double* out, const BatchBufs& B, int32_t* status, const Streams& s) {
    KArgs a = baseArgs(T, P, B, status);
    a.y = y; a.f = f; a.ydot = out;
    auto loops = [&](cudaStream_t st) { minvLoop(a, st); };
    if (precision == SBG_PRECISION_FP64)
        return forkJoin(P, s, [&](cudaStream_t st) { minv64Chain(a, st); }, loops,
                        [&](cudaStream_t st) { minv64Group(a, st); });
    return forkJoin(P, s, [&](cudaStream_t st) { minv32Chain(a, st); }, loops,
                    [&](cudaStream_t st) { minv32Group(a, st); });
}

cudaError_t launchRKMerson(const DevTables& T, const LaunchPlan& P, int precision, double* y, double* time,
                           const BatchBufs& B, int32_t* status, double h, StepCtl step, double accuracy,
                           double consTol, int projectEveryStep, const Streams& s) {
    KArgs a = baseArgs(T, P, B, status);
    a.ystate = y; a.time = time; a.h = h; a.step = step; a.accuracy = accuracy; a.consTol = consTol;
    a.projectEveryStep = projectEveryStep;
    auto loops = [&](cudaStream_t st) { rkLoop(a, st); };
    if (precision == SBG_PRECISION_FP64)
        return forkJoin(P, s, [&](cudaStream_t st) { rk64Chain(a, st); }, loops,
                        [&](cudaStream_t st) { rk64Group(a, st); });
    const bool ref = precision == SBG_PRECISION_MIXED;
    return forkJoin(P, s, [&](cudaStream_t st) { rk32Chain(a, ref, st); }, loops,
                    [&](cudaStream_t st) { rk32Group(a, ref, st); });
}

cudaError_t launchRKFp64List(const DevTables& T, const LaunchPlan& P, double* y, double* time, int32_t* status,
                             double h, StepCtl step, double accuracy, double consTol, int projectEveryStep,
                             int64_t fplane, const int64_t* rowsBase, double* rows, int lanes, cudaStream_t s) {
    KArgs a{};
    a.T = &T; a.P = &P; a.ystate = y; a.time = time; a.status = status; a.h = h; a.step = step;
    a.accuracy = accuracy; a.consTol = consTol; a.projectEveryStep = projectEveryStep; a.fplane = fplane;
    rkFp64List(a, rowsBase, rows, lanes, s);
    return cudaGetLastError();
}

__global__ void fillIntKernel(int32_t* __restrict__ p, int n, int v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}
cudaError_t launchFillInt(int32_t* p, int n, int v, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    fillIntKernel<<<(n + 255) / 256, 256, 0, s>>>(p, n, v);
    return cudaGetLastError();
}

// Instances of a one-step integration call that have steps left (stepsLeft
// > 0; with stepsLeft null: time < tStop and no TIMEOUT status).
__global__ void countUnfinishedKernel(int n, const int32_t* __restrict__ stepsLeft, const double* __restrict__ time,
                                      const int32_t* __restrict__ status, double tStop, int32_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool left = false;
    if (i < n) left = stepsLeft ? stepsLeft[i] > 0 : (time[i] < tStop && !(status[i] & SBG_INST_TIMEOUT));
    const unsigned b = __ballot_sync(0xffffffffu, left);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(out, __popc(b));
}
cudaError_t launchCountUnfinished(int n, const int32_t* stepsLeft, const double* time, const int32_t* status,
                                  double tStop, int32_t* out, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(int32_t), s);
    if (e != cudaSuccess || n <= 0) return e;
    countUnfinishedKernel<<<(n + 255) / 256, 256, 0, s>>>(n, stepsLeft, time, status, tStop, out);
    return cudaGetLastError();
}

cudaError_t launchNormalizeQuat(const DevTables& T, double* y, cudaStream_t s) {
    const int threads = 128, blocks = (T.ninst + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    normalizeQuatKernel<<<blocks, threads, 0, s>>>(T, y);
    return cudaGetLastError();
}

cudaError_t launchScatter(const DevTables& T, const int64_t* hostOff, const double* packed, double* cols, int part,
                          cudaStream_t s, int inst0, int count) {
    if (count < 0) count = T.ninst - inst0;
    if (count <= 0) return cudaSuccess;
    scatterKernel<<<count, 128, 0, s>>>(T, hostOff, packed, cols, part, inst0);
    return cudaGetLastError();
}

cudaError_t launchGather(const DevTables& T, const int64_t* hostOff, const double* cols, double* packed, int part,
                         cudaStream_t s, int inst0, int count) {
    if (count < 0) count = T.ninst - inst0;
    if (count <= 0) return cudaSuccess;
    gatherKernel<<<count, 128, 0, s>>>(T, hostOff, cols, packed, part, inst0);
    return cudaGetLastError();
}

}  // namespace sbg
