// ops_device.cuh -- the O(n) tree operators of SimbodyMatterSubsystem for a
// batch, in FP64 (the reference's Real) whatever the batch's precision:
//   residual   calcResidualForceIgnoringConstraints (SimbodyMatterSubsystem.h:2234,
//              SimbodyMatterSubsystemRep.cpp:5532-5617): M x + C(q,u) - f - ~J F
//   mv         multiplyByM (SimbodyMatterSubsystemRep.cpp:5411-5447): M x
//   jv         multiplyBySystemJacobian (:6293-6313): J x, one SpatialVec per body
//   jtf        multiplyBySystemJacobianTranspose (:6326-6350): ~J F
//   composite  calcCompositeBodyInertias (:5196-5205): one SpatialInertia per body
//
// One sweep base to tip (position kinematics through body1, with velocity
// kinematics for the residual, and the body accelerations
// A = ~Phi A_parent + H x [+ a]), then one tip to base (body forces
// F = own + sum Phi_c F_c, tau = ~H F - f; or the composite inertias). The
// bodies of a level are spread over the G lanes of the instance's group
// (G = 1 for the one-thread layouts); a parent pulls its children's results
// after a level barrier. Each body's record holds its kinematics [0,18), the
// body1 fields [18,42), H at kRecH, and the operator's A [42,48) and F
// [48,54) (composite inertias: [42,52)).
#pragma once
#include "kernels.h"

namespace sbg {

constexpr int kOpA = 42, kOpF = 48, kOpC = 42;

// q from the state columns; u only for the residual (Stage::Velocity); no
// force elements (body1 then leaves bF and f zero).
struct OpSrc {
    static constexpr bool kMInv = true;
    const double* y;
    int64_t base, stride;
    int nq;
    bool withU;
    __device__ __forceinline__ double q(int k) const { return y[base + (int64_t)k * stride]; }
    __device__ __forceinline__ double u(int k) const { return withU ? y[base + (int64_t)(nq + k) * stride] : 0.0; }
    __device__ __forceinline__ double fext(int) const { return 0.0; }
};
struct OpSink {
    template <class R> __device__ __forceinline__ void qdot(int, R) {}
    template <class R> __device__ __forceinline__ void udot(int, R) {}
};

// Unit inertia of a unit point mass at p (MassProperties.h:458-466, 866-867).
__device__ __forceinline__ S3<double> pointMassUnit(V3<double> p) {
    const double xx = p.x * p.x, yy = p.y * p.y, zz = p.z * p.z;
    return S3<double>{yy + zz, xx + zz, xx + yy, -p.x * p.y, -p.x * p.z, -p.y * p.z};
}
__device__ __forceinline__ S3<double> operator+(const S3<double>& a, const S3<double>& b) {
    return S3<double>{a.xx + b.xx, a.yy + b.yy, a.zz + b.zz, a.xy + b.xy, a.xz + b.xz, a.yz + b.yz};
}
__device__ __forceinline__ S3<double> operator-(const S3<double>& a, const S3<double>& b) {
    return S3<double>{a.xx - b.xx, a.yy - b.yy, a.zz - b.zz, a.xy - b.xy, a.xz - b.xz, a.yz - b.yz};
}
__device__ __forceinline__ S3<double> operator*(double s, const S3<double>& a) {
    return S3<double>{s * a.xx, s * a.yy, s * a.zz, s * a.xy, s * a.xz, s * a.yz};
}

// rec(lb): record of local row lb in the instance's scratch.
template <int NM, class SC, class RecOf>
__device__ __forceinline__ int treeOp(const DevTables& T, int inst, const SC& S, RecOf rec, const double* y,
                                      const OpIO& io, int gl, int G, unsigned mask) {
    const int kind = io.kind;
    const int body0 = T.ibody[inst];
    const int* ls = T.levStart + T.ilev[inst];
    const int nlev = T.inlev[inst];
    const int64_t u0 = io.uoff[inst], b0 = io.boff[inst];
    const OpSrc src{y, T.ybase[inst], T.ystride[inst], T.inq[inst], kind == OP_RESIDUAL};
    OpSink sink;
    const double* PT = T.par64;
    bool finite = true;
    const bool accel = kind == OP_RESIDUAL || kind == OP_MV || kind == OP_JV;

    for (int L = 0; L < nlev; ++L) {  // base to tip
        for (int lb = ls[L] + gl; lb < ls[L + 1]; lb += G) {
            const int row = body0 + lb, r = rec(lb);
            const int parent = T.parent[row];
            const Kin<double> P = parent < 0 ? groundKin<double>() : loadKin<double>(S, rec(parent));
            const Kin<double> K = body1<double, NM>(T, row, r, S, src, sink, z3<double>(), P);
            storeKin(S, r, K);
            if (!accel) continue;
            // A = ~Phi A_parent + H x (+ a) (RigidBodyNodeSpec.cpp:566-582, 658-669, 762-775)
            V3<double> Aw = z3<double>(), Av = z3<double>();
            if (parent >= 0) {
                const int rp = rec(parent);
                Aw = ld3<double>(S, rp, kOpA);
                Av = ld3<double>(S, rp, kOpA + 3) + cross(Aw, ld3<double>(S, r, kRecL));
            }
            const int n = (T.info[row] >> 4) & 15, uo = T.uoff[row];
            if (io.x)
                for (int j = 0; j < n; ++j) {
                    const double xj = io.x[u0 + uo + j];
                    Aw = axpy(Aw, xj, ld3<double>(S, r, kRecH + 6 * j));
                    Av = axpy(Av, xj, ld3<double>(S, r, kRecH + 6 * j + 3));
                }
            if (kind == OP_RESIDUAL) {
                Aw = Aw + ld3<double>(S, r, kRecA);
                Av = Av + ld3<double>(S, r, kRecA + 3);
            }
            st3<double>(S, r, kOpA, Aw);
            st3<double>(S, r, kOpA + 3, Av);
            if (kind == OP_JV) {
                double* o = io.out + 6 * (b0 + T.bidx[row]);
                o[0] = Aw.x; o[1] = Aw.y; o[2] = Aw.z; o[3] = Av.x; o[4] = Av.y; o[5] = Av.z;
                finite &= isfinite(Aw.x + Aw.y + Aw.z + Av.x + Av.y + Av.z);
            }
        }
        if (G > 1) __syncwarp(mask);
    }
    if (kind == OP_JV) return finite ? 0 : SBG_INST_NONFINITE;

    for (int L = nlev - 1; L >= 0; --L) {  // tip to base
        for (int lb = ls[L] + gl; lb < ls[L + 1]; lb += G) {
            const int row = body0 + lb, r = rec(lb);
            const double m = PT[(int64_t)row * kParamStride];
            const V3<double> pc = ld3<double>(S, r, kRecPc);
            const S3<double> Gi{S(r, kRecGi), S(r, kRecGi + 1), S(r, kRecGi + 2), S(r, kRecGi + 3),
                                S(r, kRecGi + 4), S(r, kRecGi + 5)};
            const int cb = T.cbeg[row], cn = T.ccnt[row];
            if (kind == OP_COMPOSITE) {
                // R = Mk + sum R_c.shift(-l_c) (RigidBodyNode.cpp:232-243,
                // MassProperties.h:1037-1044, 1110-1116)
                double Rm = m;
                V3<double> Rp = pc;
                S3<double> RG = Gi;
                for (int k = 0; k < cn; ++k) {
                    const int rc = rec(T.clist[cb + k]);
                    const double cm = S(rc, kOpC);
                    const V3<double> cp = ld3<double>(S, rc, kOpC + 1);
                    const S3<double> cG{S(rc, kOpC + 4), S(rc, kOpC + 5), S(rc, kOpC + 6), S(rc, kOpC + 7),
                                        S(rc, kOpC + 8), S(rc, kOpC + 9)};
                    const V3<double> pNew = cp + ld3<double>(S, rc, kRecL);
                    const S3<double> sG = (cG - pointMassUnit(cp)) + pointMassUnit(pNew);
                    const double mt = Rm + cm, oom = 1.0 / mt;
                    Rp = oom * (Rm * Rp + cm * pNew);
                    RG = oom * (Rm * RG + cm * sG);
                    Rm = mt;
                }
                // the children have been read: this body's record takes R
                S(r, kOpC) = Rm;
                st3<double>(S, r, kOpC + 1, Rp);
                S(r, kOpC + 4) = RG.xx; S(r, kOpC + 5) = RG.yy; S(r, kOpC + 6) = RG.zz;
                S(r, kOpC + 7) = RG.xy; S(r, kOpC + 8) = RG.xz; S(r, kOpC + 9) = RG.yz;
                double* o = io.out + 10 * (b0 + T.bidx[row]);
                o[0] = Rm; o[1] = Rp.x; o[2] = Rp.y; o[3] = Rp.z;
                o[4] = RG.xx; o[5] = RG.yy; o[6] = RG.zz; o[7] = RG.xy; o[8] = RG.xz; o[9] = RG.yz;
                finite &= isfinite(Rm + Rp.x + Rp.y + Rp.z + RG.xx + RG.yy + RG.zz + RG.xy + RG.xz + RG.yz);
                continue;
            }
            // own force (RigidBodyNodeSpec.cpp:624-627, 685-686, 806), Mk A =
            // m (G A_w + p x A_v, A_v - p x A_w) (MassProperties.h:1071-1072)
            V3<double> Fw = z3<double>(), Fv = z3<double>();
            if (kind != OP_JTF) {
                const V3<double> Aw = ld3<double>(S, r, kOpA), Av = ld3<double>(S, r, kOpA + 3);
                Fw = m * (mul(Gi, Aw) + cross(pc, Av));
                Fv = m * (Av - cross(pc, Aw));
                if (kind == OP_RESIDUAL) {  // gyroscopic force (RigidBodyNode.cpp:98-174)
                    const V3<double> w = ld3<double>(S, r, 12);
                    Fw = Fw + m * cross(w, mul(Gi, w));
                    Fv = Fv + m * cross(w, cross(w, pc));
                }
            }
            if (io.fbody && kind != OP_MV) {
                const double* fb = io.fbody + 6 * (b0 + T.bidx[row]);
                const V3<double> aw = mk3(fb[0], fb[1], fb[2]), av = mk3(fb[3], fb[4], fb[5]);
                if (kind == OP_JTF) { Fw = Fw + aw; Fv = Fv + av; }
                else { Fw = Fw - aw; Fv = Fv - av; }
            }
            for (int k = 0; k < cn; ++k) {  // Phi F = (F_w + l x F_v, F_v)
                const int rc = rec(T.clist[cb + k]);
                const V3<double> cw = ld3<double>(S, rc, kOpF), cv = ld3<double>(S, rc, kOpF + 3);
                Fw = Fw + (cw + cross(ld3<double>(S, rc, kRecL), cv));
                Fv = Fv + cv;
            }
            st3<double>(S, r, kOpF, Fw);
            st3<double>(S, r, kOpF + 3, Fv);
            const int n = (T.info[row] >> 4) & 15, uo = T.uoff[row];
            for (int j = 0; j < n; ++j) {
                double t = dot(ld3<double>(S, r, kRecH + 6 * j), Fw) + dot(ld3<double>(S, r, kRecH + 6 * j + 3), Fv);
                if (kind == OP_RESIDUAL && io.fmob) t = t - io.fmob[u0 + uo + j];
                io.out[u0 + uo + j] = t;
                finite &= isfinite(t);
            }
        }
        if (G > 1) __syncwarp(mask);
    }
    return finite ? 0 : SBG_INST_NONFINITE;
}

// SEG 0: one-thread instances in 32-wide interleaved tiles; 1: the loop-closure
// segment (one thread, records at stride sstride); 2: the level-parallel
// segment (field-major rows).
template <int NM, int SEG>
__global__ void __launch_bounds__(128) treeOpKernel(DevTables T, int first, int count, const double* __restrict__ y,
                                                   double* __restrict__ scratch, OpIO io,
                                                   int32_t* __restrict__ status) {
    const Slot s = SEG == 2 ? groupSlot(T, first) : chainSlot(T, first, count);
    if (s.inst < 0) return;
    const int body0 = T.ibody[s.inst];
    int st;
    if constexpr (SEG == 0) {
        const ScrTiled<double> S{scratch + T.sbase[s.inst]};
        st = treeOp<NM>(T, s.inst, S, [&](int lb) { return (int)T.srec[body0 + lb]; }, y, io, 0, 1, 0u);
    } else if constexpr (SEG == 1) {
        const ScrStrided<double> S{scratch + T.sbase[s.inst], (int)T.sstride[s.inst]};
        st = treeOp<NM>(T, s.inst, S, [&](int lb) { return (int)T.srec[body0 + lb]; }, y, io, 0, 1, 0u);
    } else {
        const ScrRows<double> S{scratch + T.sbase[s.inst], T.inb[s.inst]};
        st = treeOp<NM>(T, s.inst, S, [](int lb) { return lb; }, y, io, s.gl, s.G, s.mask);
        st = (int)__reduce_or_sync(s.mask, (unsigned)st);
    }
    if (s.gl == 0) status[s.inst] = st;
}

}  // namespace sbg
