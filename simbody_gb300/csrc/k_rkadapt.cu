// k_rkadapt.cu -- error-controlled (variable-step) Runge-Kutta-Merson over a
// batch, FP64: Integrator::setFinalTime(tFinal), initialize(state) and
// stepTo(tFinal) of a RungeKuttaMersonIntegrator with error control
// (AbstractIntegratorRep.cpp:341-577), every instance with its own step size,
// accept/reject decisions and time, inside one persistent kernel per segment.
//
// Each attempt takes the five stages of the fixed-step kernel
// (RungeKuttaMersonIntegrator.cpp:86-140; f0 is kept across rejected
// attempts, as the reference keeps the derivatives saved at the start of the
// step), then, without touching y:
//   - the error norm of 0.2 |y1 - ysave| (IntegratorRep.h:454-523), with the
//     scaling of u frozen at the start of the step;
//   - the projection test of attemptDAEStep (AbstractIntegratorRep.cpp:158-199):
//     when the norm is within 2^4 accuracy, quaternions whose RMS error passes
//     max(2 consTol, sqrt(consTol)) fail the attempt (norm = infinity), and
//     quaternions are normalized when it passes consTol (or every step), the
//     radial part of their error estimate removed and the norm recomputed
//     (RigidBodyNodeSpec_Ball.h:417-434);
//   - adjustStepSize (:448-502) picks the next step size and accepts the
//     step when it did not shrink.
// An accepted step writes y1 (with its normalized quaternions); a rejected one
// leaves y and retries with the smaller step. Each step's t1 follows
// takeOneStep's rule against tMax = tFinal (:536-544), which marks a step
// shortened to reach tFinal as artificially limited.
#include "abi_device.cuh"

namespace sbg {

// AbstractIntegratorRep::adjustStepSize (AbstractIntegratorRep.cpp:448-502):
// returns whether the step succeeded (the new size is not smaller); hMin /
// hMax <= 0: no user limit.
__device__ __forceinline__ bool adjustStepSizeDev(double err, int errOrder, bool limited, double accuracy, double hMin,
                                                  double hMax, double& h) {
    const double Safety = 0.9, MinShrink = 0.1, MaxGrow = 5, HysteresisLow = 0.9, HysteresisHigh = 1.2;
    double hNew;
    if (!isfinite(err)) hNew = MinShrink * h;
    else if (err == 0) hNew = MaxGrow * h;
    else hNew = Safety * h * pow(accuracy / err, 1.0 / double(errOrder));
    if (hNew > h && (limited || hNew < HysteresisHigh * h)) hNew = h;
    if (hNew < h) {
        if (err <= accuracy) hNew = h;
        else hNew = fmin(hNew, HysteresisLow * h);
    }
    hNew = fmin(hNew, MaxGrow * h);
    hNew = fmax(hNew, MinShrink * h);
    if (hMin > 0) hNew = fmax(hNew, hMin);
    if (hMax > 0) hNew = fmin(hNew, hMax);
    const bool success = hNew >= h;
    h = hNew;
    return success;
}

// The q part of the error norm for one quaternion q with error estimate dq:
// N Wu NInv dq with unit weights (IntegratorRep.h:500-523, Rotation.h:712-748).
__device__ __forceinline__ double quatErrSq(const double* q, const double* dq) {
    const double e0 = 2 * q[0], e1 = 2 * q[1], e2 = 2 * q[2], e3 = 2 * q[3];
    const double du0 = -e1 * dq[0] + e0 * dq[1] - e3 * dq[2] + e2 * dq[3];
    const double du1 = -e2 * dq[0] + e3 * dq[1] + e0 * dq[2] - e1 * dq[3];
    const double du2 = -e3 * dq[0] - e2 * dq[1] + e1 * dq[2] + e0 * dq[3];
    const double g0 = q[0] / 2, g1 = q[1] / 2, g2 = q[2] / 2, g3 = q[3] / 2;
    const double o0 = -g1 * du0 + -g2 * du1 + -g3 * du2;
    const double o1 = g0 * du0 + g3 * du1 + -g2 * du2;
    const double o2 = -g3 * du0 + g0 * du1 + g1 * du2;
    const double o3 = g2 * du0 + -g1 * du1 + g0 * du2;
    return o0 * o0 + o1 * o1 + o2 * o2 + o3 * o3;
}

template <int NM, bool GROUP>
__global__ void __launch_bounds__(128) rkMersonAdaptiveKernel(DevTables T, int first, int count, double* __restrict__ y,
                                                              double* __restrict__ time, double* __restrict__ fbuf,
                                                              int64_t fplane, double* __restrict__ scratch,
                                                              int32_t* __restrict__ status, AdaptCtl ac) {
    const Slot s = GROUP ? groupSlot(T, first) : chainSlot(T, first, count);
    if (s.inst < 0) return;
    const int inst = s.inst;
    const int64_t base = T.ybase[inst], stride = T.ystride[inst];
    const int nq = T.inq[inst], nu = T.inu[inst];
    const int body0 = T.ibody[inst], nb = T.inb[inst];
    double* f0 = fbuf;
    double* fA = fbuf + fplane;
    double* fB = fbuf + 2 * fplane;
    double* fC = fbuf + 3 * fplane;
    int st = 0;
    double tc = time[inst];
    const double tFinal = ac.tFinal;
    double h = ac.hInit > 0 ? ac.hInit : 0.01;  // the system timescale / 10 (AbstractIntegratorRep.cpp:41-49)
    if (ac.hMin > 0) h = fmax(h, ac.hMin);
    if (ac.hMax > 0) h = fmin(h, ac.hMax);
    const double acc = ac.accuracy, consTol = ac.consTol;
    const double projLimit = fmax(2 * consTol, sqrt(consTol));
    auto stage = [&](int stg, double c, const double* a, const double* b, double* dst) {
        StageSrc<double> src{y, f0, a, b, base, stride, nq, stg, c};
        FOut<double> o{dst, base, stride, nq};
        st |= rhs<double, NM, false, GROUP>(T, s, scratch, src, o);
        if (!groupAll<GROUP>(o.finite, s)) st |= SBG_INST_NONFINITE;
        if constexpr (GROUP) __syncwarp(s.mask);  // the next stage reads what other lanes wrote
    };
    auto sum = [&](double v) {
        if constexpr (GROUP) return groupSum(v, s);
        else return v;
    };
    long long nAcc = 0, nRej = 0;
    bool haveF0 = false;
    while (tc < tFinal) {
        if (nAcc >= ac.maxSteps) { st |= SBG_INST_TIMEOUT; break; }
        if (!haveF0) {
            stage(0, 0.0, fA, fB, f0);  // f0 = f(y0), kept across rejected attempts
            haveF0 = true;
        }
        bool limited = false;
        double t1;
        if (tFinal < tc + 0.95 * h) { limited = true; t1 = tFinal; }
        else if (tFinal > tc + 1.001 * h) t1 = tc + h;
        else t1 = tFinal;
        if (!(t1 > tc)) { st |= SBG_INST_TIMEOUT; break; }
        const double hs = t1 - tc;
        stage(1, hs / 3, fA, fB, fA);   // f1 -> fA
        stage(2, hs / 6, fA, fB, fB);   // f2 -> fB
        stage(3, hs / 8, fB, fB, fC);   // f3 -> fC
        stage(4, hs / 2, fB, fC, fA);   // f4 -> fA
        const double h6 = hs / 6, h2 = hs / 2;
        auto y1At = [&](int64_t e, double* ysv) {
            const double y0 = y[e];
            const double a0 = f0[e], aB = fB[e], aC = fC[e], aA = fA[e];
            *ysv = y0 + h2 * ((a0 - 3.0 * aB) + 4.0 * aC);
            return y0 + h6 * ((a0 + 4.0 * aC) + aA);
        };
        // error norm and quaternion errors of y1, y untouched
        double sq = 0, sqP = 0, su = 0, squat = 0, nquat = 0;
        for (int lb = s.gl; lb < nb; lb += s.G) {
            const int row = body0 + lb;
            const int type = T.info[row] & 15, n = (T.info[row] >> 4) & 15;
            const int qo = T.qoff[row], uo = T.uoff[row];
            const int nqb = type == T_BALL ? 4 : (type == T_FREE ? 7 : n);
            double q1[7], dq[7];
            for (int j = 0; j < nqb; ++j) {
                double ysv;
                q1[j] = y1At(base + (int64_t)(qo + j) * stride, &ysv);
                dq[j] = 0.2 * fabs(q1[j] - ysv);
            }
            if (T.info[row] & F_QUAT) {
                sq += quatErrSq(q1, dq);
                const double len = sqrt(q1[0] * q1[0] + q1[1] * q1[1] + q1[2] * q1[2] + q1[3] * q1[3]);
                squat += (len - 1) * (len - 1);
                nquat += 1;
                // the same after normalization, the radial part of dq removed
                double qn[4], dqn[4];
                for (int k = 0; k < 4; ++k) qn[k] = q1[k] / len;
                const double d = dq[0] * qn[0] + dq[1] * qn[1] + dq[2] * qn[2] + dq[3] * qn[3];
                for (int k = 0; k < 4; ++k) dqn[k] = dq[k] - d * qn[k];
                sqP += quatErrSq(qn, dqn);
                for (int j = 4; j < nqb; ++j) { sq += dq[j] * dq[j]; sqP += dq[j] * dq[j]; }
            } else {
                for (int j = 0; j < nqb; ++j) { sq += dq[j] * dq[j]; sqP += dq[j] * dq[j]; }
            }
            for (int j = 0; j < n; ++j) {
                const int64_t e = base + (int64_t)(nq + uo + j) * stride;
                double ysv;
                const double y1v = y1At(e, &ysv);
                const double vi = fabs(y[e]);
                const double us = vi > 1 ? 1 / vi : 1.0;  // calcRelativeScaling, frozen at step start
                const double d = us * (0.2 * fabs(y1v - ysv));
                su += d * d;
            }
        }
        sq = sum(sq); sqP = sum(sqP); su = sum(su); squat = sum(squat); nquat = sum(nquat);
        const double un = nu ? sqrt(su / nu) : 0.0;
        double qnorm = nq ? sqrt(sq / nq) : 0.0;
        double errNorm = qnorm >= un ? qnorm : un;
        bool proj = false;
        if (errNorm <= 16 * acc) {  // attemptDAEStep's projection (AbstractIntegratorRep.cpp:158-199)
            const double quatNorm = nquat > 0 ? sqrt(squat / nquat) : 0.0;
            if (quatNorm > projLimit) {
                errNorm = INFINITY;  // the step did not converge
            } else if (quatNorm > consTol || ac.projectEveryStep) {
                proj = true;
                qnorm = nq ? sqrt(sqP / nq) : 0.0;
                errNorm = qnorm >= un ? qnorm : un;
            }
        }
        if (adjustStepSizeDev(errNorm, 4, limited, acc, ac.hMin, ac.hMax, h)) {
            bool fin = true;
            for (int lb = s.gl; lb < nb; lb += s.G) {
                const int row = body0 + lb;
                const int type = T.info[row] & 15, n = (T.info[row] >> 4) & 15;
                const int qo = T.qoff[row], uo = T.uoff[row];
                const int nqb = type == T_BALL ? 4 : (type == T_FREE ? 7 : n);
                double q1[7];
                for (int j = 0; j < nqb; ++j) {
                    double ysv;
                    q1[j] = y1At(base + (int64_t)(qo + j) * stride, &ysv);
                }
                if (proj && (T.info[row] & F_QUAT)) {
                    const double len = sqrt(q1[0] * q1[0] + q1[1] * q1[1] + q1[2] * q1[2] + q1[3] * q1[3]);
                    for (int k = 0; k < 4; ++k) q1[k] = q1[k] / len;
                }
                double u1[6];
                for (int j = 0; j < n; ++j) {
                    double ysv;
                    u1[j] = y1At(base + (int64_t)(nq + uo + j) * stride, &ysv);
                }
                // all of this body's y1 is formed from y0 before any of it is written
                for (int j = 0; j < nqb; ++j) { y[base + (int64_t)(qo + j) * stride] = q1[j]; fin &= isfinite(q1[j]); }
                for (int j = 0; j < n; ++j) { y[base + (int64_t)(nq + uo + j) * stride] = u1[j]; fin &= isfinite(u1[j]); }
            }
            if (!groupAll<GROUP>(fin, s)) st |= SBG_INST_NONFINITE;
            tc = t1;
            ++nAcc;
            haveF0 = false;
        } else {
            ++nRej;
            if (nRej > 64LL * ac.maxSteps) { st |= SBG_INST_TIMEOUT; break; }
        }
        if constexpr (GROUP) __syncwarp(s.mask);
    }
    if (s.gl == 0) {
        time[inst] = tc;
        status[inst] = st;
        if (ac.stats) {
            ac.stats[2 * (int64_t)inst] = nAcc;
            ac.stats[2 * (int64_t)inst + 1] = nRej;
        }
    }
}

void rkAdaptiveChain(const KArgs& a, const AdaptCtl& ac, cudaStream_t s) {
    if (a.P->nChain <= 0) return;
    const Launch1D L = spread(a.P->nChain, 128);
    double* fb = static_cast<double*>(a.fbuf);
    double* sc = static_cast<double*>(a.scratch);
    if (a.P->nm == 1)
        rkMersonAdaptiveKernel<1, false><<<L.grid, L.block, 0, s>>>(*a.T, 0, a.P->nChain, a.ystate, a.time, fb, a.fplane,
                                                                    sc, a.status, ac);
    else
        rkMersonAdaptiveKernel<3, false><<<L.grid, L.block, 0, s>>>(*a.T, 0, a.P->nChain, a.ystate, a.time, fb, a.fplane,
                                                                    sc, a.status, ac);
}

void rkAdaptiveGroup(const KArgs& a, const AdaptCtl& ac, cudaStream_t s) {
    if (a.P->nGroupBlocks <= 0) return;
    rkMersonAdaptiveKernel<3, true><<<a.P->nGroupBlocks, 128, 0, s>>>(
        *a.T, a.P->groupFirst, 0, a.ystate, a.time, static_cast<double*>(a.fbuf), a.fplane,
        static_cast<double*>(a.scratch), a.status, ac);
}

}  // namespace sbg
