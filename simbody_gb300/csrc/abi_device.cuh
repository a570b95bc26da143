// abi_device.cuh -- articulated-body forward dynamics and fixed-step
// Runge-Kutta-Merson integration for a batch of multibody instances.
//
// The RHS of one instance is a set of sweeps over its level-ordered body
// table (the reference's rbNodeLevels):
//   pass 1 (base to tip)  position + velocity kinematics, gravity and mobility
//                         forces (RigidBodyNodeSpec.h:229-333,
//                         RigidBodyNode.cpp:54-174, Force_Gravity.cpp:531-556,
//                         Force.cpp:339-443)
//   pass 2 (tip to base)  articulated body inertias fused with the first udot
//                         pass (RigidBodyNodeSpec.cpp:249-400)
//   pass 3 (base to tip)  second udot pass (RigidBodyNodeSpec.cpp:408-446)
// The mixed form (R = float) adds one step of iterative refinement: pass 3
// also runs the outward half of inverse dynamics in double-float (hi+lo FP32
// pairs with error-free transformations), pass 4 (tip to base) finishes the
// residual r = f - tau(udot0) and runs the first M^-1 pass on it, pass 5 (base
// to tip) applies udot = udot0 + M^-1 r with the FP32 factorization. This
// takes the relative udot error of an FP32 recursion (up to ~1e-4 on random
// trees) to the few-1e-6 level set by the FP32 kinematics, as long as M is
// well conditioned. Where the correction exceeds 1e-4 of udot (an
// ill-conditioned M, the FP32 factorisation too poor for the refinement to
// converge) the instance is flagged SBG_INST_ILL_CONDITIONED and, in a
// realize or the server's mixed lane, recomputed in FP64 on an FP64 mirror
// of its records.
//
// Two mappings drive the same per-body code:
//   chain driver  one thread per instance walks its rows in order; along a
//                 chain (parent = previous row) the parent's values travel in
//                 registers; scratch records of 32 instances interleave lane
//                 by lane (element f of record rec at (rec + f) * 32).
//   group driver  G lanes share one instance and take the bodies of a level
//                 in parallel (trees with wide levels); a parent pulls its
//                 children's contributions after a group barrier; records are
//                 field-major within the instance (element f of row r at
//                 r + f * nbodies), so lanes on one level read contiguously.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "engine.h"
#include "spatial.cuh"
#include "kernels.h"

namespace sbg {

enum { T_PIN = 0, T_SLIDER = 1, T_UNIV = 2, T_BALL = 3, T_FREE = 4, T_GIMBAL = 5, T_TRANSL = 6, T_CYL = 7,
       T_PLANAR = 8, T_BUSHING = 9, T_WELD = 10, T_SCREW = 11 };

// Scratch accessors: S(rec, f) is element f of the record at rec.
template <class R> struct ScrTiled {
    R* p;
    __device__ __forceinline__ R& operator()(int rec, int f) const { return p[(rec + f) * kTile]; }
};
// Loop-closure records: element f of record rec at (rec + f) * s, with the
// stride of the instance (32 inside a batch's interleaved tiles, 1 for an
// instance whose record is its own).
template <class R> struct ScrStrided {
    R* p;
    int s;
    __device__ __forceinline__ R& operator()(int rec, int f) const { return p[(rec + f) * s]; }
};
template <class R> struct ScrRows {
    R* p;
    int P;  // rows of the instance
    __device__ __forceinline__ R& operator()(int rec, int f) const { return p[rec + f * P]; }
};

template <class R> __device__ __forceinline__ const R* paramTable(const DevTables& T) {
    if constexpr (std::is_same<R, double>::value) return T.par64; else return T.par32;
}
template <class R> __device__ __forceinline__ const R* coefTable(const DevTables& T) {
    if constexpr (std::is_same<R, double>::value) return T.fcoef64; else return T.fcoef32;
}
template <class R> __device__ __forceinline__ const R* q0Table(const DevTables& T) {
    if constexpr (std::is_same<R, double>::value) return T.fq064; else return T.fq032;
}

template <class R, class SC> __device__ __forceinline__ void st3(const SC& S, int rec, int f, V3<R> v) {
    S(rec, f) = v.x; S(rec, f + 1) = v.y; S(rec, f + 2) = v.z;
}
template <class R, class SC> __device__ __forceinline__ V3<R> ld3(const SC& S, int rec, int f) {
    return V3<R>{S(rec, f), S(rec, f + 1), S(rec, f + 2)};
}

template <class R> __device__ __forceinline__ void sincosR(R x, R* s, R* c) {
    if constexpr (std::is_same<R, double>::value) sincos(x, s, c); else sincosf(x, s, c);
}
template <class R> __device__ __forceinline__ R sqrtR(R x) {
    if constexpr (std::is_same<R, double>::value) return sqrt(x); else return sqrtf(x);
}
template <class R> __device__ __forceinline__ R powR(R x, R y) {
    if constexpr (std::is_same<R, double>::value) return pow(x, y); else return powf(x, y);
}
template <class R> __device__ __forceinline__ R tanhR(R x) {
    if constexpr (std::is_same<R, double>::value) return tanh(x); else return tanhf(x);
}

// ------------------------------------------------------------- double-float
// hi + lo pairs of FP32 with error-free transformations (Dekker/Knuth two-sum,
// FMA-based two-product); the intrinsics keep the compiler from contracting
// or reassociating them.
struct DF { float hi, lo; };
__device__ __forceinline__ DF dfq(float a) { return DF{a, 0.f}; }
__device__ __forceinline__ DF twoSum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return DF{s, e};
}
__device__ __forceinline__ DF quickTwoSum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF operator+(DF a, DF b) {
    DF s = twoSum(a.hi, b.hi);
    const DF t = twoSum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = quickTwoSum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return quickTwoSum(s.hi, s.lo);
}
__device__ __forceinline__ DF operator+(DF a, float b) {
    DF s = twoSum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return quickTwoSum(s.hi, s.lo);
}
__device__ __forceinline__ DF operator-(DF a) { return DF{-a.hi, -a.lo}; }
__device__ __forceinline__ DF operator-(DF a, DF b) { return a + (-b); }
__device__ __forceinline__ DF operator*(DF a, float b) {
    const float p = __fmul_rn(a.hi, b);
    const float e = __fmaf_rn(a.hi, b, -p);
    return quickTwoSum(p, __fmaf_rn(a.lo, b, e));
}
struct DF3 { DF x, y, z; };
__device__ __forceinline__ DF3 zdf3() { return DF3{dfq(0.f), dfq(0.f), dfq(0.f)}; }
__device__ __forceinline__ DF3 operator+(DF3 a, DF3 b) { return DF3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ DF3 operator+(DF3 a, V3<float> b) { return DF3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ DF3 operator-(DF3 a, DF3 b) { return DF3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ DF3 scale(DF3 a, float s) { return DF3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ DF exactProd(float s, float v) { const float p = __fmul_rn(s, v); return DF{p, __fmaf_rn(s, v, -p)}; }
// a + s*v, s and v exact floats
__device__ __forceinline__ DF3 axpyDF(DF3 a, float s, V3<float> v) {
    return DF3{a.x + exactProd(s, v.x), a.y + exactProd(s, v.y), a.z + exactProd(s, v.z)};
}
// float vector x df vector
__device__ __forceinline__ DF3 crossFD(V3<float> a, DF3 b) {
    return DF3{b.z * a.y - b.y * a.z, b.x * a.z - b.z * a.x, b.y * a.x - b.x * a.y};
}
__device__ __forceinline__ DF dotFD(V3<float> a, DF3 b) { return (b.x * a.x + b.y * a.y) + b.z * a.z; }
__device__ __forceinline__ DF3 symMulDF(const S3<float>& S, DF3 v) {
    return DF3{(v.x * S.xx + v.y * S.xy) + v.z * S.xz, (v.x * S.xy + v.y * S.yy) + v.z * S.yz,
               (v.x * S.xz + v.y * S.yz) + v.z * S.zz};
}
template <class SC> __device__ __forceinline__ DF3 ldDF3(const SC& S, int rec, int f) {
    return DF3{DF{float(S(rec, f)), float(S(rec, f + 1))}, DF{float(S(rec, f + 2)), float(S(rec, f + 3))},
               DF{float(S(rec, f + 4)), float(S(rec, f + 5))}};
}
template <class SC> __device__ __forceinline__ void stDF3(const SC& S, int rec, int f, DF3 v) {
    S(rec, f) = v.x.hi; S(rec, f + 1) = v.x.lo; S(rec, f + 2) = v.y.hi; S(rec, f + 3) = v.y.lo;
    S(rec, f + 4) = v.z.hi; S(rec, f + 5) = v.z.lo;
}

// Body-fixed X-Y-Z angles q[0..2]: cos and sin of each and R_FM
// (Rotation::setRotationToBodyFixedXYZ(c, s), Rotation.h:342-349).
template <class R> struct XYZ {
    R c0, c1, s0, s1, ooc1;
};
template <class R> __device__ __forceinline__ XYZ<R> bodyXYZ(const R* q, M3<R>& Rm) {
    R c[3], sn[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) sincosR(q[k], &sn[k], &c[k]);
    const R s0s1 = sn[0] * sn[1], s2c0 = sn[2] * c[0], c0c2 = c[0] * c[2], nc1 = -c[1];
    Rm.a[0] = c[1] * c[2];              Rm.a[1] = sn[2] * nc1;               Rm.a[2] = sn[1];
    Rm.a[3] = s2c0 + s0s1 * c[2];       Rm.a[4] = c0c2 - s0s1 * sn[2];       Rm.a[5] = sn[0] * nc1;
    Rm.a[6] = sn[0] * sn[2] - sn[1] * c0c2; Rm.a[7] = sn[0] * c[2] + sn[1] * s2c0; Rm.a[8] = c[0] * c[1];
    return XYZ<R>{c[0], c[1], sn[0], sn[1], R(1) / c[1]};
}

// ------------------------------------------------------------------ kinematics
template <class R> struct Kin {
    M3<R> R_;
    V3<R> p, w, v;
};
// SmoothSphereHalfSpaceForceImpl::calcForce (SmoothSphereHalfSpaceForce.cpp:
// 252-336) for the spheres of one body against half-spaces fixed in Ground:
// adds to (Mw, Fv) the moment about Bo and the force of -force applied at the
// contact point, which lies midway through the indentation. K is the body's
// position and velocity (Ground's velocity is zero, so the contact point's
// velocity is the sphere body's).
// Out of line, with everything passed by value, so that the rows without
// contacts do not pay for its registers.
template <class R> struct Wrench { V3<R> w, v; };
template <class R>
__device__ __noinline__ Wrench<R> contactForces(const R* KP, int kb, int kc, Kin<R> K, Wrench<R> F) {
    V3<R> Mw = F.w, Fv = F.v;
    for (int k = 0; k < kc; ++k) {
        const R* c = KP + (int64_t)kb + (int64_t)k * kContactStride;
        const V3<R> n = mk3(c[4], c[5], c[6]);
        const V3<R> centre = mul(K.R_, mk3(c[0], c[1], c[2])) + K.p;
        const R indentation = -(dot(centre - mk3(c[7], c[8], c[9]), -n) - c[3]);
        const V3<R> r = ((centre + c[3] * n) - (R(0.5) * indentation) * n) - K.p;
        const V3<R> v = K.v + cross(K.w, r);
        const R vn = dot(v, n);
        const V3<R> vt = v - vn * n;
        // Hertz, smoothed about zero indentation, then Hunt-Crossley
        const R fh = c[10] * powR(sqrtR(indentation * indentation + c[16]), R(1.5)) *
                     (R(0.5) + R(0.5) * tanhR(c[17] * indentation));
        const R fhc = fh * (R(1) + R(1.5) * c[11] * vn) * (R(0.5) + R(0.5) * tanhR(c[18] * (vn + c[19])));
        // smoothed static / dynamic / viscous friction along the slip
        const R vslip = sqrtR(dot(vt, vt) + c[16]);
        const R vrel = vslip / c[15];
        const R ff = fhc * ((vrel < R(1) ? vrel : R(1)) * (c[13] + R(2) * (c[12] - c[13]) / (R(1) + vrel * vrel)) +
                            c[14] * vslip);
        const V3<R> force = fhc * n + (ff / vslip) * vt;
        Mw = Mw - cross(r, force);
        Fv = Fv - force;
    }
    return Wrench<R>{Mw, Fv};
}

template <class R> __device__ __forceinline__ Kin<R> groundKin() { return Kin<R>{ident3<R>(), z3<R>(), z3<R>(), z3<R>()}; }
template <class R, class SC> __device__ __forceinline__ Kin<R> loadKin(const SC& S, int rec) {
    Kin<R> k;
#pragma unroll
    for (int i = 0; i < 9; ++i) k.R_.a[i] = S(rec, i);
    k.p = ld3<R>(S, rec, 9); k.w = ld3<R>(S, rec, 12); k.v = ld3<R>(S, rec, 15);
    return k;
}
template <class R, class SC> __device__ __forceinline__ void storeKin(const SC& S, int rec, const Kin<R>& k) {
#pragma unroll
    for (int i = 0; i < 9; ++i) S(rec, i) = k.R_.a[i];
    st3<R>(S, rec, 9, k.p); st3<R>(S, rec, 12, k.w); st3<R>(S, rec, 15, k.v);
}

// Pass 1 for one body: parent kinematics in, own kinematics out; writes qdot
// and the record fields pc, Gi, l, a, bF, H, f (NM = padded record width).
// Src::q(k), Src::u(k) give the (double) state.
template <class R, int NM, class SC, class Src, class Out>
__device__ __forceinline__ Kin<R> body1(const DevTables& T, int row, int rec, const SC& S, const Src& src, Out& out,
                                        V3<R> g, const Kin<R>& P) {
    const R* PT = paramTable<R>(T);
    const R* FC = coefTable<R>(T);
    const R* FQ = q0Table<R>(T);
    const int info = T.info[row];
    const int type = info & 15, n = (info >> 4) & 15;
    const int nw = n == 6 ? 6 : NM;
    const int qo = T.qoff[row], uo = T.uoff[row];
    const R* pr = PT + (int64_t)row * kParamStride;
    const R m = pr[0];
    const V3<R> com = mk3(pr[1], pr[2], pr[3]);
    const S3<R> Gb{pr[4], pr[5], pr[6], pr[7], pr[8], pr[9]};

    // state of this mobilizer
    R q[7], u[6];
    const int nq = type == T_BALL ? 4 : (type == T_FREE ? 7 : n);
#pragma unroll
    for (int j = 0; j < 7; ++j) q[j] = j < nq ? R(src.q(qo + j)) : R(0);
#pragma unroll
    for (int j = 0; j < 6; ++j) u[j] = j < n ? R(src.u(uo + j)) : R(0);

    // X_FM (mobilizer specific) and qdot = N(q) u
    M3<R> RFM = ident3<R>();
    V3<R> pFM = z3<R>();
    V3<R> y1 = z3<R>();  // Universal: second H_FM column
    XYZ<R> ea{R(1), R(1), R(0), R(0), R(1)};  // body-fixed X-Y-Z angles
    const bool quat = (info & F_QUAT) != 0;
    switch (type) {
    case T_WELD:  // RigidBodyNode_Weld.cpp:389-396: X_FM = identity, no q
        break;
    case T_GIMBAL:   // RigidBodyNodeSpec_Gimbal.h: calcX_FM, u = qdot
    case T_BUSHING:  // RigidBodyNodeSpec_Bushing.h: angles then p_FM, u = qdot
        ea = bodyXYZ<R>(q, RFM);
        for (int j = 0; j < n; ++j) out.qdot(qo + j, u[j]);
        if (type == T_BUSHING) pFM = mk3(q[3], q[4], q[5]);
        break;
    case T_TRANSL:  // RigidBodyNodeSpec_Translation.h
        pFM = mk3(q[0], q[1], q[2]);
        for (int j = 0; j < 3; ++j) out.qdot(qo + j, u[j]);
        break;
    case T_CYL:       // RigidBodyNodeSpec_Cylinder.h: about and along Fz
    case T_PLANAR: {  // RigidBodyNodeSpec_Planar.h: about Fz, along Fx and Fy
        R s, c;
        sincosR(q[0], &s, &c);
        RFM.a[0] = c; RFM.a[1] = -s; RFM.a[3] = s; RFM.a[4] = c;
        pFM = type == T_CYL ? mk3(R(0), R(0), q[1]) : mk3(q[1], q[2], R(0));
        for (int j = 0; j < n; ++j) out.qdot(qo + j, u[j]);
        break;
    }
    case T_PIN:      // RigidBodyNodeSpec_Pin.h:103-122
    case T_SCREW: {  // RigidBodyNodeSpec_Screw.h:121-132: about Fz, p_FM = (0, 0, q pitch)
        R s, c;
        sincosR(q[0], &s, &c);
        RFM.a[0] = c; RFM.a[1] = -s; RFM.a[3] = s; RFM.a[4] = c;
        if (type == T_SCREW) pFM = mk3(R(0), R(0), q[0] * pr[34]);
        out.qdot(qo, u[0]);
        break;
    }
    case T_SLIDER:  // RigidBodyNodeSpec_Slider.h:100-119
        pFM.x = q[0];
        out.qdot(qo, u[0]);
        break;
    case T_UNIV: {  // RigidBodyNodeSpec_Universal.h:124-166
        R s1, c1, s2, c2;
        sincosR(q[0], &s1, &c1);
        sincosR(q[1], &s2, &c2);
        RFM.a[0] = c2;       RFM.a[1] = R(0); RFM.a[2] = s2;
        RFM.a[3] = s2 * s1;  RFM.a[4] = c1;   RFM.a[5] = -s1 * c2;
        RFM.a[6] = -s2 * c1; RFM.a[7] = s1;   RFM.a[8] = c1 * c2;
        y1 = mk3(R(0), c1, s1);
        out.qdot(qo, u[0]);
        out.qdot(qo + 1, u[1]);
        break;
    }
    default: {  // Ball / Free
        if (!quat) {
            // body-fixed X-Y-Z angles (RigidBodyNodeSpec_Ball.h:118-127, 198-209):
            // qdot = N_P(q) w_FM (Rotation.h:395-406); the last q slot is unused
            ea = bodyXYZ<R>(q, RFM);
            const R t = (ea.s0 * u[1] - ea.c0 * u[2]) * ea.ooc1;
            out.qdot(qo + 0, u[0] + t * ea.s1);
            out.qdot(qo + 1, ea.c0 * u[1] + ea.s0 * u[2]);
            out.qdot(qo + 2, -t);
            if (type == T_FREE) {
                pFM = mk3(q[3], q[4], q[5]);
                for (int j = 0; j < 3; ++j) out.qdot(qo + 3 + j, u[3 + j]);
                out.qdot(qo + 6, R(0));
            } else {
                out.qdot(qo + 3, R(0));
            }
            break;
        }
        // quaternion (RigidBodyNodeSpec_Ball.h:134-214)
        const R len = sqrtR(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
        const R oo = R(1) / len;
        const R e0 = q[0] * oo, e1 = q[1] * oo, e2 = q[2] * oo, e3 = q[3] * oo;
        const R q00 = e0 * e0, q11 = e1 * e1, q22 = e2 * e2, q33 = e3 * e3;
        const R q01 = e0 * e1, q02 = e0 * e2, q03 = e0 * e3, q12 = e1 * e2, q13 = e1 * e3, q23 = e2 * e3;
        const R a = q00 - q11, b = q22 - q33;
        RFM.a[0] = q00 + q11 - q22 - q33; RFM.a[1] = R(2) * (q12 - q03); RFM.a[2] = R(2) * (q13 + q02);
        RFM.a[3] = R(2) * (q12 + q03);    RFM.a[4] = a + b;              RFM.a[5] = R(2) * (q23 - q01);
        RFM.a[6] = R(2) * (q13 - q02);    RFM.a[7] = R(2) * (q23 + q01); RFM.a[8] = a - b;
        // qdot = N(q) w with e = q/2 (Rotation.h:712-719, 990-992)
        const R h0 = q[0] * R(0.5), h1 = q[1] * R(0.5), h2 = q[2] * R(0.5), h3 = q[3] * R(0.5);
        out.qdot(qo + 0, -h1 * u[0] - h2 * u[1] - h3 * u[2]);
        out.qdot(qo + 1, h0 * u[0] + h3 * u[1] - h2 * u[2]);
        out.qdot(qo + 2, -h3 * u[0] + h0 * u[1] + h1 * u[2]);
        out.qdot(qo + 3, h2 * u[0] - h1 * u[1] + h0 * u[2]);
        if (type == T_FREE) {
            pFM = mk3(q[4], q[5], q[6]);
            out.qdot(qo + 4, u[3]);
            out.qdot(qo + 5, u[4]);
            out.qdot(qo + 6, u[5]);
        }
        break;
    }
    }

    // body transforms (RigidBodyNodeSpec.h:554-569)
    M3<R> RPF, RMB;
#pragma unroll
    for (int i = 0; i < 9; ++i) { RPF.a[i] = pr[10 + i]; RMB.a[i] = pr[22 + i]; }
    const V3<R> pPF = mk3(pr[19], pr[20], pr[21]);
    const V3<R> pMB = mk3(pr[31], pr[32], pr[33]);
    const M3<R> RFB = (info & F_RMB_I) ? RFM : mul(RFM, RMB);
    const V3<R> r = (info & F_PMB_0) ? z3<R>() : mul(RFM, pMB);  // r_MB_F
    const V3<R> pFB = r + pFM;
    const M3<R> RPB = (info & F_RPF_I) ? RFB : mul(RPF, RFB);
    const V3<R> pPB = ((info & F_RPF_I) ? pFB : mul(RPF, pFB)) + pPF;
    Kin<R> K;
    K.R_ = mul(P.R_, RPB);
    const V3<R> l = mul(P.R_, pPB);  // Phi (RigidBodyNode.cpp:63)
    K.p = l + P.p;
    const M3<R> RGF = (info & F_RPF_I) ? P.R_ : mul(P.R_, RPF);

    // H_PB_G columns (RigidBodyNodeSpec.cpp:44-74), stored; V_PB_G = H u
    V3<R> VPw = z3<R>(), VPv = z3<R>();
    V3<R> wFM = z3<R>();
    auto putH = [&](int j, V3<R> hw, V3<R> hv) {
        st3<R>(S, rec, kRecH + 6 * j, hw);
        st3<R>(S, rec, kRecH + 6 * j + 3, hv);
        VPw = axpy(VPw, u[j], hw);
        VPv = axpy(VPv, u[j], hv);
    };
    // -(r x e_j) for the unit axes
    const V3<R> nrx = mk3(R(0), -r.z, r.y), nry = mk3(r.z, R(0), -r.x), nrz = mk3(-r.y, r.x, R(0));
    V3<R> hdw = z3<R>();  // sum_j u_j HDot_FM_w_j
    switch (type) {
    case T_PIN:
    case T_CYL:
    case T_PLANAR:
        putH(0, col(RGF, 2), mul(RGF, nrz));
        wFM = mk3(R(0), R(0), u[0]);
        if (type == T_CYL) putH(1, z3<R>(), col(RGF, 2));
        if (type == T_PLANAR) { putH(1, z3<R>(), col(RGF, 0)); putH(2, z3<R>(), col(RGF, 1)); }
        break;
    case T_TRANSL:
        for (int j = 0; j < 3; ++j) putH(j, z3<R>(), col(RGF, j));
        break;
    case T_GIMBAL:
    case T_BUSHING: {
        // H_FM_w columns (1,0,0), (0,c0,s0), (s1,-s0 c1,c0 c1) and their time
        // derivatives with qdot = u (RigidBodyNodeSpec_Gimbal.h)
        const V3<R> h1 = mk3(R(0), ea.c0, ea.s0), h2 = mk3(ea.s1, -ea.s0 * ea.c1, ea.c0 * ea.c1);
        putH(0, col(RGF, 0), mul(RGF, nrx));
        putH(1, mul(RGF, h1), mul(RGF, -cross(r, h1)));
        putH(2, mul(RGF, h2), mul(RGF, -cross(r, h2)));
        wFM = axpy(axpy(mk3(u[0], R(0), R(0)), u[1], h1), u[2], h2);
        const R dc0 = -ea.s0 * u[0], dc1 = -ea.s1 * u[1], ds0 = ea.c0 * u[0], ds1 = ea.c1 * u[1];
        hdw = axpy(u[1] * mk3(R(0), dc0, ds0), u[2],
                   mk3(ds1, -ds0 * ea.c1 - ea.s0 * dc1, dc0 * ea.c1 + ea.c0 * dc1));
        if (type == T_BUSHING)
            for (int j = 0; j < 3; ++j) putH(3 + j, z3<R>(), col(RGF, j));
        break;
    }
    case T_SLIDER:
        putH(0, z3<R>(), col(RGF, 0));
        break;
    case T_UNIV:
        putH(0, col(RGF, 0), mul(RGF, nrx));
        putH(1, mul(RGF, y1), mul(RGF, -cross(r, y1)));
        wFM = axpy(mk3(u[0], R(0), R(0)), u[1], y1);
        hdw = u[1] * cross(wFM, y1);
        break;
    case T_WELD:  // no mobilities: V_PB_G = VD_PB_G = 0 (RigidBodyNode_Weld.cpp:378-386)
        break;
    case T_SCREW:  // H_FM = [(0,0,1); (0,0,pitch)] (RigidBodyNodeSpec_Screw.h:134-140), constant in F
        putH(0, col(RGF, 2), mul(RGF, mk3(R(0), R(0), pr[34]) + nrz));
        wFM = mk3(R(0), R(0), u[0]);
        break;
    default:
        putH(0, col(RGF, 0), mul(RGF, nrx));
        putH(1, col(RGF, 1), mul(RGF, nry));
        putH(2, col(RGF, 2), mul(RGF, nrz));
        wFM = mk3(u[0], u[1], u[2]);
        if (type == T_FREE) {
            putH(3, z3<R>(), col(RGF, 0));
            putH(4, z3<R>(), col(RGF, 1));
            putH(5, z3<R>(), col(RGF, 2));
        }
        break;
    }
    // HDot*u (RigidBodyNodeSpec.cpp:82-129) without forming HDot:
    //   VD_w = R_GF hdw + w_GF x V_w,
    //   VD_v = R_GF(-(r x hdw) - (w_FM x r) x w_FM) + w_GF x V_v
    // with hdw = sum_j u_j HDot_FM_w_j (non-zero for the Universal only).
    const V3<R> VDw = mul(RGF, hdw) + cross(P.w, VPw);
    const V3<R> VDv = mul(RGF, -cross(r, hdw) - cross(cross(wFM, r), wFM)) + cross(P.w, VPv);

    // RigidBodyNode.cpp:54-84, 98-174
    const S3<R> Gi = reexpress(K.R_, Gb);
    const V3<R> pc = mul(K.R_, com);
    K.w = P.w + VPw;
    K.v = (P.v + cross(P.w, l)) + VPv;
    const V3<R> bw = m * cross(K.w, mul(Gi, K.w));
    const V3<R> bv = m * cross(K.w, cross(K.w, pc));
    const V3<R> aw = VDw;
    const V3<R> av = VDv + cross(P.w, K.v - P.v);
    // gravity (Force_Gravity.cpp:549-551)
    V3<R> Fv = m * g;
    V3<R> Fw = cross(pc, Fv);
    if constexpr (!Src::kMInv)
        if (info & F_CONTACT) {
            const R* KP;
            if constexpr (std::is_same<R, double>::value) KP = T.kpar64; else KP = T.kpar32;
            const Wrench<R> W = contactForces<R>(KP, T.kbeg[row], T.kcnt[row], K, Wrench<R>{Fw, Fv});
            Fw = W.w;
            Fv = W.v;
        }

    // mobility forces, in element order (Force.cpp:339-351, 434-443);
    // M^-1 f takes the given f and no body forces instead.
    R f[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) f[j] = R(0);
    const int fb = T.fbeg[row], fc = Src::kMInv ? 0 : T.fcnt[row];
    if constexpr (Src::kMInv)
        for (int j = 0; j < n; ++j) f[j] = R(src.fext(uo + j));
    for (int k = 0; k < fc; ++k) {
        const int kw = T.fkind_which[fb + k];
        const int which = kw & 255;
        const R coef = FC[fb + k];
        R v;
        if ((kw >> 8) == 0) v = -coef * (R(src.q(qo + which)) - FQ[fb + k]);
        else v = -coef * u[which];
#pragma unroll
        for (int j = 0; j < 6; ++j)
            if (j == which) f[j] = f[j] + v;
    }

    st3<R>(S, rec, kRecPc, pc);
    S(rec, kRecGi + 0) = Gi.xx; S(rec, kRecGi + 1) = Gi.yy; S(rec, kRecGi + 2) = Gi.zz;
    S(rec, kRecGi + 3) = Gi.xy; S(rec, kRecGi + 4) = Gi.xz; S(rec, kRecGi + 5) = Gi.yz;
    st3<R>(S, rec, kRecL, l);
    st3<R>(S, rec, kRecA, aw); st3<R>(S, rec, kRecA + 3, av);
    if constexpr (Src::kMInv) { st3<R>(S, rec, kRecBF, z3<R>()); st3<R>(S, rec, kRecBF + 3, z3<R>()); }
    else { st3<R>(S, rec, kRecBF, bw - Fw); st3<R>(S, rec, kRecBF + 3, bv - Fv); }
    const int ef = kRecH + 6 * nw;
    for (int j = 0; j < n; ++j) S(rec, ef + j) = f[j];
    return K;
}

// ------------------------------------------------------------------ pass 2
// D^-1: closed forms for 1..3 columns (SmallMatrixMixed.h:841-960), LU with
// partial pivoting for 6 (LAPACK getrf/getri semantics, :859-894).
template <class R, int N> __device__ __forceinline__ bool invertSmall(const R* D, R* DI) {
    bool ok = true;
    if constexpr (N == 1) {
        DI[0] = R(1) / D[0];
        ok = D[0] != R(0);
    } else if constexpr (N == 2) {
        const R d = D[0] * D[3] - D[1] * D[2];
        const R ood = R(1) / d;
        DI[0] = ood * D[3]; DI[1] = -ood * D[1]; DI[2] = -ood * D[2]; DI[3] = ood * D[0];
        ok = d != R(0);
    } else if constexpr (N == 3) {
#define MM(i, j) D[3 * (i) + (j)]
        const R d00 = MM(1, 1) * MM(2, 2) - MM(1, 2) * MM(2, 1), nd01 = MM(1, 2) * MM(2, 0) - MM(1, 0) * MM(2, 2),
                d02 = MM(1, 0) * MM(2, 1) - MM(1, 1) * MM(2, 0);
        const R d = MM(0, 0) * d00 + MM(0, 1) * nd01 + MM(0, 2) * d02;
        const R ood = R(1) / d;
        const R nd10 = MM(0, 2) * MM(2, 1) - MM(0, 1) * MM(2, 2), d11 = MM(0, 0) * MM(2, 2) - MM(0, 2) * MM(2, 0),
                nd12 = MM(0, 1) * MM(2, 0) - MM(0, 0) * MM(2, 1), d20 = MM(0, 1) * MM(1, 2) - MM(0, 2) * MM(1, 1),
                nd21 = MM(0, 2) * MM(1, 0) - MM(0, 0) * MM(1, 2), d22 = MM(0, 0) * MM(1, 1) - MM(0, 1) * MM(1, 0);
#undef MM
        DI[0] = ood * d00;  DI[1] = ood * nd10; DI[2] = ood * d20;
        DI[3] = ood * nd01; DI[4] = ood * d11;  DI[5] = ood * nd21;
        DI[6] = ood * d02;  DI[7] = ood * nd12; DI[8] = ood * d22;
        ok = d != R(0);
    } else {
        R A[N * N];
        int piv[N];
#pragma unroll
        for (int i = 0; i < N * N; ++i) A[i] = D[i];
#pragma unroll
        for (int j = 0; j < N; ++j) {
            int p = j;
            R best = fabs(A[j * N + j]);
#pragma unroll
            for (int i = j + 1; i < N; ++i) {
                const R v = fabs(A[i * N + j]);
                if (v > best) { best = v; p = i; }
            }
            piv[j] = p;
#pragma unroll
            for (int k = 0; k < N; ++k) {  // swap rows j and p
                const R tj = A[j * N + k];
                R tp = tj;
#pragma unroll
                for (int i = j + 1; i < N; ++i) if (i == p) tp = A[i * N + k];
#pragma unroll
                for (int i = j + 1; i < N; ++i) if (i == p) A[i * N + k] = tj;
                A[j * N + k] = tp;
            }
            if (A[j * N + j] == R(0)) ok = false;
            const R rcp = R(1) / A[j * N + j];
#pragma unroll
            for (int i = j + 1; i < N; ++i) A[i * N + j] = A[i * N + j] * rcp;
#pragma unroll
            for (int i = j + 1; i < N; ++i)
#pragma unroll
                for (int k = j + 1; k < N; ++k) A[i * N + k] = A[i * N + k] - A[i * N + j] * A[j * N + k];
        }
#pragma unroll
        for (int c = 0; c < N; ++c) {
            R x[N];
#pragma unroll
            for (int i = 0; i < N; ++i) x[i] = R(i == c ? 1 : 0);
#pragma unroll
            for (int j = 0; j < N; ++j) {  // row interchanges in order
                const R xj = x[j];
                R xp = xj;
#pragma unroll
                for (int i = j + 1; i < N; ++i) if (i == piv[j]) xp = x[i];
#pragma unroll
                for (int i = j + 1; i < N; ++i) if (i == piv[j]) x[i] = xj;
                x[j] = xp;
            }
#pragma unroll
            for (int i = 0; i < N; ++i)
#pragma unroll
                for (int k = 0; k < i; ++k) x[i] = x[i] - A[i * N + k] * x[k];
#pragma unroll
            for (int i = N - 1; i >= 0; --i) {
#pragma unroll
                for (int k = i + 1; k < N; ++k) x[i] = x[i] - A[i * N + k] * x[k];
                x[i] = x[i] / A[i * N + i];
            }
#pragma unroll
            for (int i = 0; i < N; ++i) DI[i * N + c] = x[i];
        }
    }
    return ok;
}

// What a child hands its parent in pass 2: P+ shifted by -l and Phi z+.
template <class R> struct C2 {
    AB<R> P;
    V3<R> zw, zv;
};
template <class R> __device__ __forceinline__ C2<R> zeroC2() {
    C2<R> c;
    c.P.M = S3<R>{R(0), R(0), R(0), R(0), R(0), R(0)};
    c.P.J = c.P.M;
#pragma unroll
    for (int i = 0; i < 9; ++i) c.P.F.a[i] = R(0);
    c.zw = z3<R>();
    c.zv = z3<R>();
    return c;
}
template <class R> __device__ __forceinline__ void addC2(C2<R>& a, const C2<R>& b) {
    a.P.M.xx += b.P.M.xx; a.P.M.yy += b.P.M.yy; a.P.M.zz += b.P.M.zz;
    a.P.M.xy += b.P.M.xy; a.P.M.xz += b.P.M.xz; a.P.M.yz += b.P.M.yz;
    a.P.J.xx += b.P.J.xx; a.P.J.yy += b.P.J.yy; a.P.J.zz += b.P.J.zz;
    a.P.J.xy += b.P.J.xy; a.P.J.xz += b.P.J.xz; a.P.J.yz += b.P.J.yz;
#pragma unroll
    for (int i = 0; i < 9; ++i) a.P.F.a[i] += b.P.F.a[i];
    a.zw = a.zw + b.zw;
    a.zv = a.zv + b.zv;
}
template <class R, class SC> __device__ __forceinline__ C2<R> loadC2(const SC& S, int rec) {
    C2<R> c;
    const int e = kRecPacc;
    c.P.M = S3<R>{S(rec, e + 0), S(rec, e + 1), S(rec, e + 2), S(rec, e + 3), S(rec, e + 4), S(rec, e + 5)};
    c.P.J = S3<R>{S(rec, e + 6), S(rec, e + 7), S(rec, e + 8), S(rec, e + 9), S(rec, e + 10), S(rec, e + 11)};
#pragma unroll
    for (int i = 0; i < 9; ++i) c.P.F.a[i] = S(rec, e + 12 + i);
    c.zw = ld3<R>(S, rec, e + 21);
    c.zv = ld3<R>(S, rec, e + 24);
    return c;
}
template <class R, class SC> __device__ __forceinline__ void storeC2(const SC& S, int rec, const C2<R>& c) {
    const int e = kRecPacc;
    S(rec, e + 0) = c.P.M.xx; S(rec, e + 1) = c.P.M.yy; S(rec, e + 2) = c.P.M.zz;
    S(rec, e + 3) = c.P.M.xy; S(rec, e + 4) = c.P.M.xz; S(rec, e + 5) = c.P.M.yz;
    S(rec, e + 6) = c.P.J.xx; S(rec, e + 7) = c.P.J.yy; S(rec, e + 8) = c.P.J.zz;
    S(rec, e + 9) = c.P.J.xy; S(rec, e + 10) = c.P.J.xz; S(rec, e + 11) = c.P.J.yz;
#pragma unroll
    for (int i = 0; i < 9; ++i) S(rec, e + 12 + i) = c.P.F.a[i];
    st3<R>(S, rec, e + 21, c.zw);
    st3<R>(S, rec, e + 24, c.zv);
}
template <class R, class SC> __device__ __forceinline__ void pushC2(const SC& S, int rec, const C2<R>& c) {
    C2<R> a = loadC2<R>(S, rec);
    addC2(a, c);
    storeC2(S, rec, a);
}

// Pass 2 for one body with N columns (N = 6 for Free, else the batch width
// with unused columns zero and an identity block in D). `in` holds the
// children's contributions. Returns whether D was invertible and the
// contribution for the parent. Order chosen for short live ranges: P, z, PH,
// eps, D, DI, then G one column at a time folded into P+ and z+.
template <class R, int N, class SC>
__device__ __forceinline__ bool body2(const DevTables& T, int row, int rec, int n, const SC& S, R m, const C2<R>& in,
                                      C2<R>& outC) {
    const int ef = kRecH + 6 * N, eDI = ef + N, eG = eDI + N * N, eEps = eG + 6 * N;
    // P = ArticulatedInertia(Mk) + children (RigidBodyNodeSpec.cpp:259-279)
    AB<R> P;
    {
        const V3<R> pc = ld3<R>(S, rec, kRecPc);
        P.M = S3<R>{m + in.P.M.xx, m + in.P.M.yy, m + in.P.M.zz, in.P.M.xy, in.P.M.xz, in.P.M.yz};
        P.J = S3<R>{m * S(rec, kRecGi) + in.P.J.xx, m * S(rec, kRecGi + 1) + in.P.J.yy,
                    m * S(rec, kRecGi + 2) + in.P.J.zz, m * S(rec, kRecGi + 3) + in.P.J.xy,
                    m * S(rec, kRecGi + 4) + in.P.J.xz, m * S(rec, kRecGi + 5) + in.P.J.yz};
        const V3<R> mp = m * pc;
        P.F.a[0] = in.P.F.a[0];         P.F.a[1] = -mp.z + in.P.F.a[1]; P.F.a[2] = mp.y + in.P.F.a[2];
        P.F.a[3] = mp.z + in.P.F.a[3];  P.F.a[4] = in.P.F.a[4];         P.F.a[5] = -mp.x + in.P.F.a[5];
        P.F.a[6] = -mp.y + in.P.F.a[6]; P.F.a[7] = mp.x + in.P.F.a[7];  P.F.a[8] = in.P.F.a[8];
    }
    // z = (P a + b) - F + sum_children Phi z+ (RigidBodyNodeSpec.cpp:380-392)
    V3<R> zw, zv;
    {
        V3<R> cw, cv;
        abmul(P, ld3<R>(S, rec, kRecA), ld3<R>(S, rec, kRecA + 3), cw, cv);
        zw = (cw + ld3<R>(S, rec, kRecBF)) + in.zw;
        zv = (cv + ld3<R>(S, rec, kRecBF + 3)) + in.zv;
    }
    // PH = P H; D = ~H PH; eps = f - ~H z (:294-296, :394)
    V3<R> PHw[N], PHv[N];
    R D[N * N], eps[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
        V3<R> hw = z3<R>(), hv = z3<R>();
        if (j < n) { hw = ld3<R>(S, rec, kRecH + 6 * j); hv = ld3<R>(S, rec, kRecH + 6 * j + 3); }
        abmul(P, hw, hv, PHw[j], PHv[j]);
        eps[j] = j < n ? S(rec, ef + j) - (dot(hw, zw) + dot(hv, zv)) : R(0);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
        V3<R> hw = z3<R>(), hv = z3<R>();
        if (i < n) { hw = ld3<R>(S, rec, kRecH + 6 * i); hv = ld3<R>(S, rec, kRecH + 6 * i + 3); }
#pragma unroll
        for (int j = 0; j < N; ++j)
            D[i * N + j] = (i < n && j < n) ? dot(hw, PHw[j]) + dot(hv, PHv[j]) : R(i == j ? 1 : 0);
    }
    R DI[N * N];
    const bool ok = invertSmall<R, N>(D, DI);
    // G = PH DI one column at a time; P+ = P - G ~PH with the mass and
    // inertia blocks symmetrized (:297-324); z+ = z + G eps.
    R mm[9], ms[9], in9[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) { mm[i] = R(0); ms[i] = R(0); in9[i] = R(0); }
    V3<R> zpw = zw, zpv = zv;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        V3<R> gw = z3<R>(), gv = z3<R>();
#pragma unroll
        for (int k = 0; k < N; ++k) { gw = axpy(gw, DI[k * N + j], PHw[k]); gv = axpy(gv, DI[k * N + j], PHv[k]); }
        const R g3w[3] = {gw.x, gw.y, gw.z}, g3v[3] = {gv.x, gv.y, gv.z};
        const R hw3[3] = {PHw[j].x, PHw[j].y, PHw[j].z}, hv3[3] = {PHv[j].x, PHv[j].y, PHv[j].z};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                mm[3 * a + b] = mm[3 * a + b] + g3w[a] * hv3[b];
                ms[3 * a + b] = ms[3 * a + b] + g3v[a] * hv3[b];
                in9[3 * a + b] = in9[3 * a + b] + g3w[a] * hw3[b];
            }
        if (j < n) {
            st3<R>(S, rec, eG + 6 * j, gw);
            st3<R>(S, rec, eG + 6 * j + 3, gv);
            S(rec, eEps + j) = eps[j];
            zpw = axpy(zpw, eps[j], gw);
            zpv = axpy(zpv, eps[j], gv);
        }
    }
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j)
            if (i < n && j < n) S(rec, eDI + i * N + j) = DI[i * N + j];
    AB<R> PP;
    PP.M = S3<R>{P.M.xx - ms[0], P.M.yy - ms[4], P.M.zz - ms[8], P.M.xy - (ms[3] + ms[1]) / R(2),
                 P.M.xz - (ms[6] + ms[2]) / R(2), P.M.yz - (ms[7] + ms[5]) / R(2)};
    PP.J = S3<R>{P.J.xx - in9[0], P.J.yy - in9[4], P.J.zz - in9[8], P.J.xy - (in9[3] + in9[1]) / R(2),
                 P.J.xz - (in9[6] + in9[2]) / R(2), P.J.yz - (in9[7] + in9[5]) / R(2)};
#pragma unroll
    for (int i = 0; i < 9; ++i) PP.F.a[i] = P.F.a[i] - mm[i];
    // contribution to the parent: P+ shifted by -l, Phi z+
    const V3<R> l = ld3<R>(S, rec, kRecL);
    outC.P = abshift(PP, l);
    outC.zw = zpw + cross(l, zpv);
    outC.zv = zpv;
    return ok;
}

// Free (6 columns): inlined like the other mobilizers. An out-of-line call
// would take the addresses of its in/out structs and of the state source and
// sink, which puts them in local memory on every path.
template <class R, class SC>
__device__ __forceinline__ bool body2Free(const DevTables& T, int row, int rec, const SC& S, R m, const C2<R>& in,
                                       C2<R>& outC) {
    return body2<R, 6, SC>(T, row, rec, 6, S, m, in, outC);
}

// ------------------------------------------------------------------ pass 3
// udot = DI eps - ~G A+, A = A+ + H udot + a (RigidBodyNodeSpec.cpp:408-446).
// With REF (mixed form) udot0 goes to the record and the outward half of the
// double-float inverse dynamics runs alongside: A_df, then the body's own
// force term F_df = Mk A_df + b - F_gravity (stored at kRecFdf).
template <class R> struct A3 {
    V3<R> w, v;
    DF3 dw, dv;  // double-float copy (mixed form only)
};

template <class R, int N, bool REF, class SC, class Out>
__device__ __forceinline__ A3<R> body3(const DevTables& T, int row, int rec, int n, const SC& S, Out& out,
                                       const A3<R>& Ap, bool hasParent) {
    const int ef = kRecH + 6 * N, eDI = ef + N, eG = eDI + N * N, eEps = eG + 6 * N, eU0 = eEps + N;
    const V3<R> l = ld3<R>(S, rec, kRecL);
    V3<R> Apw = z3<R>(), Apv = z3<R>();
    DF3 Dw{}, Dv{};
    if constexpr (REF) { Dw = zdf3(); Dv = zdf3(); }
    if (hasParent) {
        Apw = Ap.w;
        Apv = Ap.v + cross(Ap.w, l);
        if constexpr (REF) { Dw = Ap.dw; Dv = Ap.dv - crossFD(l, Ap.dw); }  // A_v + A_w x l
    }
    R eps[N];
#pragma unroll
    for (int j = 0; j < N; ++j) eps[j] = j < n ? S(rec, eEps + j) : R(0);
    A3<R> A;
    A.w = Apw;
    A.v = Apv;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        if (i < n) {
            R s = R(0);
#pragma unroll
            for (int k = 0; k < N; ++k)
                if (k < n) s = s + S(rec, eDI + i * N + k) * eps[k];
            const R ud = s - (dot(ld3<R>(S, rec, eG + 6 * i), Apw) + dot(ld3<R>(S, rec, eG + 6 * i + 3), Apv));
            const V3<R> hw = ld3<R>(S, rec, kRecH + 6 * i), hv = ld3<R>(S, rec, kRecH + 6 * i + 3);
            if constexpr (REF) {
                S(rec, eU0 + i) = ud;
                Dw = axpyDF(Dw, ud, hw);
                Dv = axpyDF(Dv, ud, hv);
            } else {
                out.udot(T.uoff[row] + i, ud);
            }
            A.w = axpy(A.w, ud, hw);
            A.v = axpy(A.v, ud, hv);
        }
    }
    const V3<R> aw = ld3<R>(S, rec, kRecA), av = ld3<R>(S, rec, kRecA + 3);
    A.w = A.w + aw;
    A.v = A.v + av;
    if constexpr (REF) {
        A.dw = Dw + aw;
        A.dv = Dv + av;
        // own inverse-dynamics force: Mk A + b - F (MassProperties.h:1071-1072)
        const R m = paramTable<R>(T)[(int64_t)row * kParamStride];
        const V3<R> pc = ld3<R>(S, rec, kRecPc);
        const S3<R> Gi{S(rec, kRecGi), S(rec, kRecGi + 1), S(rec, kRecGi + 2), S(rec, kRecGi + 3),
                       S(rec, kRecGi + 4), S(rec, kRecGi + 5)};
        const DF3 Fw = scale(symMulDF(Gi, A.dw) + crossFD(pc, A.dv), m) + ld3<R>(S, rec, kRecBF);
        const DF3 Fv = scale(A.dv - crossFD(pc, A.dw), m) + ld3<R>(S, rec, kRecBF + 3);
        stDF3(S, rec, kRecFdf, Fw);
        stDF3(S, rec, kRecFdf + 6, Fv);
    }
    return A;
}

template <class R, bool REF, class SC, class Out>
__device__ __forceinline__ void body3Free(const DevTables& T, int row, int rec, const SC& S, Out& out, const A3<R>& Ap,
                                       bool hasParent, A3<R>& A) {
    A = body3<R, 6, REF>(T, row, rec, 6, S, out, Ap, hasParent);
}

template <class R, class SC> __device__ __forceinline__ void storeA3(const SC& S, int rec, const A3<R>& A, bool df) {
    st3<R>(S, rec, 0, A.w);
    st3<R>(S, rec, 3, A.v);
    if constexpr (std::is_same<R, float>::value)
        if (df) { stDF3(S, rec, 6, A.dw); stDF3(S, rec, 12, A.dv); }
}
template <class R, class SC> __device__ __forceinline__ A3<R> loadA3(const SC& S, int rec, bool df) {
    A3<R> A;
    A.w = ld3<R>(S, rec, 0);
    A.v = ld3<R>(S, rec, 3);
    if constexpr (std::is_same<R, float>::value)
        if (df) { A.dw = ldDF3(S, rec, 6); A.dv = ldDF3(S, rec, 12); }
    return A;
}

// ------------------------------------------------------- passes 4 and 5 (REF)
// Pass 4 (tip to base): F_df = own + children (Phi F), r = f - ~H F_df, then
// the first M^-1 pass on r: z2 = children Phi z2+, eps2 = r - ~H z2,
// z2+ = z2 + G eps2 (RigidBodyNodeSpec.cpp:483-515).
struct C4 { DF3 Fw, Fv; V3<float> zw, zv; };
__device__ __forceinline__ C4 zeroC4() { return C4{zdf3(), zdf3(), z3<float>(), z3<float>()}; }
__device__ __forceinline__ void addC4(C4& a, const C4& b) {
    a.Fw = a.Fw + b.Fw; a.Fv = a.Fv + b.Fv; a.zw = a.zw + b.zw; a.zv = a.zv + b.zv;
}
template <class SC> __device__ __forceinline__ C4 loadC4(const SC& S, int rec) {
    return C4{ldDF3(S, rec, kRecFdf), ldDF3(S, rec, kRecFdf + 6), ld3<float>(S, rec, kRecZ2acc),
              ld3<float>(S, rec, kRecZ2acc + 3)};
}
template <class SC> __device__ __forceinline__ void storeC4(const SC& S, int rec, const C4& c) {
    stDF3(S, rec, kRecFdf, c.Fw);
    stDF3(S, rec, kRecFdf + 6, c.Fv);
    st3<float>(S, rec, kRecZ2acc, c.zw);
    st3<float>(S, rec, kRecZ2acc + 3, c.zv);
}

// `in` = children's contributions; `own` = the body's own F_df (plus, in the
// chain driver, what children pushed into it) and z2 accumulator.
template <int N, class SC>
__device__ __forceinline__ C4 body4(const DevTables& T, int row, int rec, int n, const SC& S, const C4& own,
                                    const C4& in) {
    const int ef = kRecH + 6 * N, eDI = ef + N, eG = eDI + N * N, eEps = eG + 6 * N;
    const DF3 Fw = own.Fw + in.Fw, Fv = own.Fv + in.Fv;
    const V3<float> zw = own.zw + in.zw, zv = own.zv + in.zv;
    V3<float> zpw = zw, zpv = zv;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        if (j < n) {
            const V3<float> hw = ld3<float>(S, rec, kRecH + 6 * j), hv = ld3<float>(S, rec, kRecH + 6 * j + 3);
            const DF tau = dotFD(hw, Fw) + dotFD(hv, Fv);
            const DF rr = dfq(S(rec, ef + j)) - tau;
            const float r = __fadd_rn(rr.hi, rr.lo);
            const float e2 = r - (dot(hw, zw) + dot(hv, zv));
            S(rec, eEps + j) = e2;
            zpw = axpy(zpw, e2, ld3<float>(S, rec, eG + 6 * j));
            zpv = axpy(zpv, e2, ld3<float>(S, rec, eG + 6 * j + 3));
        }
    }
    const V3<float> l = ld3<float>(S, rec, kRecL);
    return C4{Fw + crossFD(l, Fv), Fv, zpw + cross(l, zpv), zpv};
}

template <class SC>
__device__ __forceinline__ void body4Free(const DevTables& T, int row, int rec, const SC& S, const C4& own,
                                       const C4& in, C4& outC) {
    outC = body4<6>(T, row, rec, 6, S, own, in);
}

// Pass 5 (base to tip): delta = DI eps2 - ~G A+, A = A+ + H delta; the result
// udot = udot0 + delta (RigidBodyNodeSpec.cpp:521-552).
template <int N, class SC, class Out>
__device__ __forceinline__ A3<float> body5(const DevTables& T, int row, int rec, int n, const SC& S, Out& out,
                                           const A3<float>& Ap, bool hasParent) {
    const int ef = kRecH + 6 * N, eDI = ef + N, eG = eDI + N * N, eEps = eG + 6 * N, eU0 = eEps + N;
    V3<float> Apw = z3<float>(), Apv = z3<float>();
    if (hasParent) {
        const V3<float> l = ld3<float>(S, rec, kRecL);
        Apw = Ap.w;
        Apv = Ap.v + cross(Ap.w, l);
    }
    float eps[N];
#pragma unroll
    for (int j = 0; j < N; ++j) eps[j] = j < n ? S(rec, eEps + j) : 0.f;
    A3<float> A;
    A.w = Apw;
    A.v = Apv;
    const int uo = T.uoff[row];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        if (i < n) {
            float s = 0.f;
#pragma unroll
            for (int k = 0; k < N; ++k)
                if (k < n) s = s + S(rec, eDI + i * N + k) * eps[k];
            const float d = s - (dot(ld3<float>(S, rec, eG + 6 * i), Apw) + dot(ld3<float>(S, rec, eG + 6 * i + 3), Apv));
            out.udot(uo + i, S(rec, eU0 + i) + d);
            out.note(S(rec, eU0 + i), d);
            A.w = axpy(A.w, d, ld3<float>(S, rec, kRecH + 6 * i));
            A.v = axpy(A.v, d, ld3<float>(S, rec, kRecH + 6 * i + 3));
        }
    }
    return A;
}

template <class SC, class Out>
__device__ __forceinline__ void body5Free(const DevTables& T, int row, int rec, const SC& S, Out& out,
                                       const A3<float>& Ap, bool hasParent, A3<float>& A) {
    A = body5<6>(T, row, rec, 6, S, out, Ap, hasParent);
}

// ---------------------------------------------------------------- drivers
// Chain driver: one thread, rows in order; carries along chains, pushes into
// the parent's record otherwise. Returns SBG_INST_* bits.
template <class R, int NM, bool REF, bool LOOPS = false, class SC, class Src, class Out>
__device__ __forceinline__ int rhsChain(const DevTables& T, int inst, const SC& S, const Src& src, Out& out) {
    static_assert(!REF || std::is_same<R, float>::value, "refinement is for the FP32 recursion");
    const int body0 = T.ibody[inst], nb = T.inb[inst];
    const V3<R> g = mk3(R(T.grav[3 * inst]), R(T.grav[3 * inst + 1]), R(T.grav[3 * inst + 2]));
    const R* PT = paramTable<R>(T);
    {   // pass 1
        Kin<R> carry = groundKin<R>();
        for (int lb = 0; lb < nb; ++lb) {
            const int row = body0 + lb;
            const int info = T.info[row];
            const int parent = T.parent[row];
            const int rec = T.srec[row];
            const Kin<R> P = parent < 0 ? groundKin<R>()
                             : (info & F_CARRY) ? carry : loadKin<R>(S, T.srec[body0 + parent]);
            carry = body1<R, NM>(T, row, rec, S, src, out, g, P);
            if (info & F_MEMCHILD) {
                storeKin(S, rec, carry);
                storeC2(S, rec, zeroC2<R>());
            }
            if constexpr (LOOPS)
                if (info & F_LOOPBODY) storeKin(S, T.lrec[row], carry);
        }
    }
    bool ok = true;
    {   // pass 2
        C2<R> carry = zeroC2<R>();
        bool have = false;
        for (int lb = nb - 1; lb >= 0; --lb) {
            const int row = body0 + lb;
            const int info = T.info[row];
            const int n = (info >> 4) & 15;
            const int rec = T.srec[row];
            const R m = PT[(int64_t)row * kParamStride];
            C2<R> in = (info & F_MEMCHILD) ? loadC2<R>(S, rec) : zeroC2<R>();
            if (have) addC2(in, carry);
            C2<R> outC;
            if (n == 6) ok &= body2Free<R>(T, row, rec, S, m, in, outC);
            else ok &= body2<R, NM>(T, row, rec, n, S, m, in, outC);
            const int parent = T.parent[row];
            have = (info & F_CARRY) != 0;
            if (have) carry = outC;
            else if (parent >= 0) pushC2(S, T.srec[body0 + parent], outC);
        }
    }
    {   // pass 3
        A3<R> carry{};
        for (int lb = 0; lb < nb; ++lb) {
            const int row = body0 + lb;
            const int info = T.info[row];
            const int n = (info >> 4) & 15;
            const int rec = T.srec[row];
            const int parent = T.parent[row];
            const A3<R> Ap = parent < 0 ? A3<R>{} : (info & F_CARRY) ? carry : loadA3<R>(S, T.srec[body0 + parent], REF);
            if (n == 6) body3Free<R, REF>(T, row, rec, S, out, Ap, parent >= 0, carry);
            else carry = body3<R, NM, REF>(T, row, rec, n, S, out, Ap, parent >= 0);
            if constexpr (LOOPS)
                if (info & F_LOOPBODY) {
                    st3<R>(S, T.lrec[row], kSlotA, carry.w);
                    st3<R>(S, T.lrec[row], kSlotA + 3, carry.v);
                }
            if (info & F_MEMCHILD) {
                storeA3(S, rec, carry, REF);
                if constexpr (REF)
                    for (int i = 0; i < 6; ++i) S(rec, kRecZ2acc + i) = R(0);
            }
        }
    }
    if constexpr (REF) {
        {   // pass 4
            C4 carry = zeroC4();
            bool have = false;
            for (int lb = nb - 1; lb >= 0; --lb) {
                const int row = body0 + lb;
                const int info = T.info[row];
                const int n = (info >> 4) & 15;
                const int rec = T.srec[row];
                C4 own{ldDF3(S, rec, kRecFdf), ldDF3(S, rec, kRecFdf + 6), z3<float>(), z3<float>()};
                if (info & F_MEMCHILD) { own.zw = ld3<float>(S, rec, kRecZ2acc); own.zv = ld3<float>(S, rec, kRecZ2acc + 3); }
                const C4 in = have ? carry : zeroC4();
                C4 outC;
                if (n == 6) body4Free(T, row, rec, S, own, in, outC);
                else outC = body4<NM>(T, row, rec, n, S, own, in);
                const int parent = T.parent[row];
                have = (info & F_CARRY) != 0;
                if (have) carry = outC;
                else if (parent >= 0) {
                    const int pr = T.srec[body0 + parent];
                    C4 a = loadC4(S, pr);
                    addC4(a, outC);
                    storeC4(S, pr, a);
                }
            }
        }
        {   // pass 5
            A3<float> carry{};
            for (int lb = 0; lb < nb; ++lb) {
                const int row = body0 + lb;
                const int info = T.info[row];
                const int n = (info >> 4) & 15;
                const int rec = T.srec[row];
                const int parent = T.parent[row];
                const A3<float> Ap = parent < 0 ? A3<float>{} : (info & F_CARRY) ? carry : loadA3<float>(S, T.srec[body0 + parent], false);
                if (n == 6) body5Free(T, row, rec, S, out, Ap, parent >= 0, carry);
                else carry = body5<NM>(T, row, rec, n, S, out, Ap, parent >= 0);
                if (info & F_MEMCHILD) storeA3(S, rec, carry, false);
            }
        }
    }
    return ok ? 0 : SBG_INST_SINGULAR_D;
}

// Group driver: G lanes (gl = lane within the group, mask = the group's
// lanes) share one instance; the bodies of a level are spread over the lanes;
// a barrier separates levels; parents pull their children's contributions.
// Returns SBG_INST_* bits (identical on every lane of the group).
// LOOPS also writes the slot records of the loop bodies (rows nb + slot of S):
// kinematics in pass 1, A_GB in pass 3.
template <class R, int NM, bool REF, bool LOOPS = false, class SC, class Src, class Out>
__device__ __noinline__ int rhsGroup(const DevTables& T, int inst, const SC& S, const Src& src, Out& out,
                                     int gl, int G, unsigned mask) {
    static_assert(!REF || std::is_same<R, float>::value, "refinement is for the FP32 recursion");
    const int body0 = T.ibody[inst];
    const int nbI = T.inb[inst];
    const int* ls = T.levStart + T.ilev[inst];  // local row where each level starts (nlev + 1 entries)
    const int nlev = T.inlev[inst];
    const V3<R> g = mk3(R(T.grav[3 * inst]), R(T.grav[3 * inst + 1]), R(T.grav[3 * inst + 2]));
    const R* PT = paramTable<R>(T);
    for (int L = 0; L < nlev; ++L) {  // pass 1
        for (int lb = ls[L] + gl; lb < ls[L + 1]; lb += G) {
            const int row = body0 + lb;
            const int parent = T.parent[row];
            const Kin<R> P = parent < 0 ? groundKin<R>() : loadKin<R>(S, parent);
            const Kin<R> K = body1<R, NM>(T, row, lb, S, src, out, g, P);
            storeKin(S, lb, K);
            if constexpr (LOOPS)
                if (T.info[row] & F_LOOPBODY) storeKin(S, nbI + T.lslot[row], K);
        }
        __syncwarp(mask);
    }
    bool ok = true;
    for (int L = nlev - 1; L >= 0; --L) {  // pass 2
        for (int lb = ls[L] + gl; lb < ls[L + 1]; lb += G) {
            const int row = body0 + lb;
            const int n = (T.info[row] >> 4) & 15;
            const R m = PT[(int64_t)row * kParamStride];
            C2<R> in = zeroC2<R>();
            const int cb = T.cbeg[row], cn = T.ccnt[row];
            for (int k = 0; k < cn; ++k) addC2(in, loadC2<R>(S, T.clist[cb + k]));
            C2<R> outC;
            if (n == 6) ok &= body2Free<R>(T, row, lb, S, m, in, outC);
            else ok &= body2<R, NM>(T, row, lb, n, S, m, in, outC);
            storeC2(S, lb, outC);
        }
        __syncwarp(mask);
    }
    for (int L = 0; L < nlev; ++L) {  // pass 3
        for (int lb = ls[L] + gl; lb < ls[L + 1]; lb += G) {
            const int row = body0 + lb;
            const int n = (T.info[row] >> 4) & 15;
            const int parent = T.parent[row];
            const A3<R> Ap = parent < 0 ? A3<R>{} : loadA3<R>(S, parent, REF);
            A3<R> A;
            if (n == 6) body3Free<R, REF>(T, row, lb, S, out, Ap, parent >= 0, A);
            else A = body3<R, NM, REF>(T, row, lb, n, S, out, Ap, parent >= 0);
            storeA3(S, lb, A, REF);
            if constexpr (LOOPS)
                if (T.info[row] & F_LOOPBODY) {
                    st3<R>(S, nbI + T.lslot[row], kSlotA, A.w);
                    st3<R>(S, nbI + T.lslot[row], kSlotA + 3, A.v);
                }
        }
        __syncwarp(mask);
    }
    if constexpr (REF) {
        for (int L = nlev - 1; L >= 0; --L) {  // pass 4
            for (int lb = ls[L] + gl; lb < ls[L + 1]; lb += G) {
                const int row = body0 + lb;
                const int n = (T.info[row] >> 4) & 15;
                const C4 own{ldDF3(S, lb, kRecFdf), ldDF3(S, lb, kRecFdf + 6), z3<float>(), z3<float>()};
                C4 in = zeroC4();
                const int cb = T.cbeg[row], cn = T.ccnt[row];
                for (int k = 0; k < cn; ++k) addC4(in, loadC4(S, T.clist[cb + k]));
                C4 outC;
                if (n == 6) body4Free(T, row, lb, S, own, in, outC);
                else outC = body4<NM>(T, row, lb, n, S, own, in);
                storeC4(S, lb, outC);
            }
            __syncwarp(mask);
        }
        for (int L = 0; L < nlev; ++L) {  // pass 5
            for (int lb = ls[L] + gl; lb < ls[L + 1]; lb += G) {
                const int row = body0 + lb;
                const int n = (T.info[row] >> 4) & 15;
                const int parent = T.parent[row];
                const A3<float> Ap = parent < 0 ? A3<float>{} : loadA3<float>(S, parent, false);
                A3<float> A;
                if (n == 6) body5Free(T, row, lb, S, out, Ap, parent >= 0, A);
                else A = body5<NM>(T, row, lb, n, S, out, Ap, parent >= 0);
                storeA3(S, lb, A, false);
            }
            __syncwarp(mask);
        }
    }
    const int st = ok ? 0 : SBG_INST_SINGULAR_D;
    return (int)__reduce_or_sync(mask, (unsigned)st);
}

// ----------------------------------------------------------------- sources
struct YSrc {
    static constexpr bool kMInv = false;
    const double* y;
    int64_t base, stride;
    int nq;
    __device__ __forceinline__ double q(int k) const { return y[base + (int64_t)k * stride]; }
    __device__ __forceinline__ double u(int k) const { return y[base + (int64_t)(nq + k) * stride]; }
};
// umax / dmax: largest |udot0| and |refinement correction| seen by body5
// (mixed form), for the ill-conditioning test.
struct YdOut {
    double* yd;
    int64_t base, stride;
    int nq;
    bool finite = true;
    float umax = 0.f, dmax = 0.f;
    __device__ __forceinline__ void note(float u0, float d) { umax = fmaxf(umax, fabsf(u0)); dmax = fmaxf(dmax, fabsf(d)); }
    template <class R> __device__ __forceinline__ void qdot(int k, R v) {
        yd[base + (int64_t)k * stride] = double(v);
        finite &= isfinite(v);
    }
    template <class R> __device__ __forceinline__ void udot(int k, R v) {
        yd[base + (int64_t)(nq + k) * stride] = double(v);
        finite &= isfinite(v);
    }
    __device__ __forceinline__ double udotGet(int k) const { return yd[base + (int64_t)(nq + k) * stride]; }
};
// M^-1 f: q from the state columns, u = 0, f from fcol (u slots); the result
// goes to the u slots of out (SimbodyMatterSubsystemRep.cpp:5357-5400).
struct MInvSrc {
    static constexpr bool kMInv = true;
    const double* y;
    const double* f;
    int64_t base, stride;
    int nq;
    __device__ __forceinline__ double q(int k) const { return y[base + (int64_t)k * stride]; }
    __device__ __forceinline__ double u(int) const { return 0.0; }
    __device__ __forceinline__ double fext(int k) const { return f[base + (int64_t)(nq + k) * stride]; }
};
struct MInvOut {
    double* o;
    int64_t base, stride;
    int nq;
    bool finite = true;
    template <class R> __device__ __forceinline__ void qdot(int, R) {}
    template <class R> __device__ __forceinline__ void udot(int k, R v) {
        o[base + (int64_t)(nq + k) * stride] = double(v);
        finite &= isfinite(v);
    }
};
// Stage input y0 + c * combo(f) of RK-Merson formed on the fly while pass 1
// loads q/u (RungeKuttaMersonIntegrator.cpp:108-126).
template <class F> struct StageSrc {
    static constexpr bool kMInv = false;
    const double* y;
    const F* f0; const F* fa; const F* fb;
    int64_t base, stride;
    int nq, stage;
    double c;
    __device__ __forceinline__ double at(int k) const {
        const int64_t e = base + (int64_t)k * stride;
        const double y0 = y[e];
        switch (stage) {
        case 0: return y0;
        case 1: return y0 + c * double(f0[e]);                                              // h/3 f0
        case 2: return y0 + c * (double(f0[e]) + double(fa[e]));                            // h/6 (f0+f1)
        case 3: return y0 + c * (double(f0[e]) + 3.0 * double(fa[e]));                      // h/8 (f0+3f2)
        default: return y0 + c * ((double(f0[e]) - 3.0 * double(fa[e])) + 4.0 * double(fb[e]));  // h/2 (f0-3f2+4f3)
        }
    }
    __device__ __forceinline__ double q(int k) const { return at(k); }
    __device__ __forceinline__ double u(int k) const { return at(nq + k); }
};
template <class F> struct FOut {
    F* f;
    int64_t base, stride;
    int nq;
    bool finite = true;
    float umax = 0.f, dmax = 0.f;
    __device__ __forceinline__ void note(float u0, float d) { umax = fmaxf(umax, fabsf(u0)); dmax = fmaxf(dmax, fabsf(d)); }
    template <class R> __device__ __forceinline__ void qdot(int k, R v) { f[base + (int64_t)k * stride] = F(v); finite &= isfinite(v); }
    template <class R> __device__ __forceinline__ void udot(int k, R v) { f[base + (int64_t)(nq + k) * stride] = F(v); finite &= isfinite(v); }
    __device__ __forceinline__ double udotGet(int k) const { return double(f[base + (int64_t)(nq + k) * stride]); }
};

// Thread/group -> instance mapping. Chain kernels: thread t of the launch
// takes order[first + t], t < count. Group kernels: block b covers order
// positions [blkFirst[b], blkFirst[b+1]) with G = blkG[b] lanes per instance.
struct Slot {
    int inst;   // -1: idle
    int gl, G;
    unsigned mask;
};
__device__ __forceinline__ Slot chainSlot(const DevTables& T, int first, int count) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    return Slot{t < count ? T.order[first + t] : -1, 0, 1, 0u};
}
__device__ __forceinline__ Slot groupSlot(const DevTables& T, int blk0) {
    const int b = blk0 + blockIdx.x;
    const int G = T.blkG[b];
    const int pos = T.blkFirst[b] + (int)threadIdx.x / G;
    const int lane = threadIdx.x & 31;
    const unsigned mask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
    return Slot{pos < T.blkFirst[b + 1] ? T.order[pos] : -1, (int)threadIdx.x % G, G, mask};
}

#include "loops_device.cuh"

// Mixed form: SBG_INST_ILL_CONDITIONED when the refinement correction exceeds
// kIllConditioned of udot0 (max-norms over the instance, i.e. over the lanes
// of its group). The correction is about cond(M) times the FP32 rounding, so
// a large one means the FP32 factorisation is too poor for the mixed form's
// accuracy bar. Non-negative floats order like their bit patterns.
template <bool GROUP, class Out>
__device__ __forceinline__ int illConditioned(const DevTables& T, const Out& out, const Slot& s) {
    float um = out.umax, dm = out.dmax;
    if constexpr (GROUP) {
        um = __uint_as_float(__reduce_max_sync(s.mask, __float_as_uint(um)));
        dm = __uint_as_float(__reduce_max_sync(s.mask, __float_as_uint(dm)));
    }
    const float tol = (T.fbList || T.ictl) ? kIllConditionedStep : kIllConditioned;
    if (T.kcnt) {
        // Contact spheres: the indentation is a small difference of body
        // positions, which FP32 kinematics resolve to about 1e-5 of it, so
        // these instances take the FP64 path of the mixed form.
        const int b0 = T.ibody[s.inst], nb = T.inb[s.inst];
        for (int r = 0; r < nb; ++r)
            if (T.info[b0 + r] & F_CONTACT) return SBG_INST_ILL_CONDITIONED;
    }
    return dm > tol * um ? SBG_INST_ILL_CONDITIONED : 0;
}

// One RHS of the instance owned by slot s, through either driver; LOOPS adds
// the Ball loop-closure multipliers (FP64; one-thread or level-parallel driver).
template <class R, int NM, bool REF, bool GROUP, bool LOOPS = false, class Src, class Out>
__device__ __forceinline__ int rhs(const DevTables& T, const Slot& s, R* scratch, const Src& src, Out& out) {
    if constexpr (LOOPS) {
        static_assert(std::is_same<R, double>::value && !REF, "loop closures run in FP64");
        double* rec0 = scratch + T.sbase[s.inst];
        if constexpr (GROUP) {
            // tree passes on the group's lanes; the multiplier solve and the
            // constraint sweeps (loop paths only) on its first lane, the
            // Gram columns on its first three
            // record-major rows (the first lane's serial loop work touches a
            // few records many times: they stay in L1)
            const ScrGen S{rec0, (int)T.sstride[s.inst], 1};
            int st = rhsGroup<double, NM, false, true>(T, s.inst, S, src, out, s.gl, s.G, s.mask);
            if (T.incons[s.inst] > 0) {
                const LoopState L = loopStateRows(T, s.inst, rec0, nullptr, nullptr, nullptr, 0, 0);
                int lst = 0;
                if (s.G >= 3) lst = loopForwardDynamicsLanes<NM>(L, out, s.gl, s.mask);
                else if (s.gl == 0) lst = loopForwardDynamics<NM, true>(L, out);
                __syncwarp(s.mask);
                lst = (int)__reduce_or_sync(s.mask, (unsigned)lst);
                if (!(lst & SBG_INST_CHOLESKY_FAIL)) loopCorrectionOutRows<NM>(L, out, s.gl, s.G, s.mask);
                st |= lst;
            }
            return st;
        } else {
            const int sst = (int)T.sstride[s.inst];
            const ScrStrided<double> S{rec0, sst};
            int st = rhsChain<double, NM, false, true>(T, s.inst, S, src, out);
            if (T.incons[s.inst] > 0)
                st |= loopForwardDynamics<NM>(loopStateChain(T, s.inst, rec0, sst, nullptr, nullptr, nullptr, 0, 0), out);
            return st;
        }
    } else if constexpr (GROUP) {
        const ScrRows<R> S{scratch + T.sbase[s.inst], T.inb[s.inst]};
        int st = rhsGroup<R, NM, REF>(T, s.inst, S, src, out, s.gl, s.G, s.mask);
        if constexpr (REF) st |= illConditioned<true>(T, out, s);
        return st;
    } else {
        const ScrTiled<R> S{scratch + T.sbase[s.inst]};
        int st = rhsChain<R, NM, REF>(T, s.inst, S, src, out);
        if constexpr (REF) st |= illConditioned<false>(T, out, s);
        return st;
    }
}

template <bool GROUP> __device__ __forceinline__ bool groupAll(bool v, const Slot& s) {
    if constexpr (GROUP) return __all_sync(s.mask, v); else return v;
}

// ------------------------------------------------------------ realize kernel
template <class R, int NM, bool REF, bool GROUP, int MINB = 1, bool LOOPS = false, int BS = 128>
__global__ void __launch_bounds__(BS, MINB) realizeKernel(DevTables T, int first, int count, const double* __restrict__ y,
                                                           double* __restrict__ ydot, R* __restrict__ scratch,
                                                           int32_t* __restrict__ status) {
    const Slot s = GROUP ? groupSlot(T, first) : chainSlot(T, first, count);
    if (s.inst < 0) return;
    YSrc src{y, T.ybase[s.inst], T.ystride[s.inst], T.inq[s.inst]};
    YdOut out{ydot, T.ybase[s.inst], T.ystride[s.inst], T.inq[s.inst]};
    int st = rhs<R, NM, REF, GROUP, LOOPS>(T, s, scratch, src, out);
    if (!groupAll<GROUP>(out.finite, s)) st |= SBG_INST_NONFINITE;
    if (s.gl == 0) status[s.inst] = st;
}

// Mixed form: the instances of a segment (order positions [first, first +
// count)) whose refinement reported an ill-conditioned M are recomputed in
// FP64 on the FP64 mirror of their records, one thread per instance (the
// level-parallel layout with a single lane). The other threads return at
// once. T.fallbacks counts the recomputed instances.
template <int NM, bool GROUP>
__global__ void __launch_bounds__(128) realizeFallbackKernel(DevTables T, int first, int count,
                                                             const double* __restrict__ y, double* __restrict__ ydot,
                                                             int32_t* __restrict__ status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int inst = T.order[first + t];
    if (!(status[inst] & SBG_INST_ILL_CONDITIONED)) return;
    YSrc src{y, T.ybase[inst], T.ystride[inst], T.inq[inst]};
    YdOut out{ydot, T.ybase[inst], T.ystride[inst], T.inq[inst]};
    int st;
    if constexpr (GROUP) {
        const ScrRows<double> S{T.scratch64 + T.sbase[inst], T.inb[inst]};
        st = rhsGroup<double, NM, false>(T, inst, S, src, out, 0, 1, 1u << (threadIdx.x & 31));
    } else {
        const ScrTiled<double> S{T.scratch64 + T.sbase[inst]};
        st = rhsChain<double, NM, false>(T, inst, S, src, out);
    }
    if (!out.finite) st |= SBG_INST_NONFINITE;
    status[inst] = st;
    atomicAdd(T.fallbacks, 1ULL);
}

template <class R, int NM, bool GROUP>
__global__ void __launch_bounds__(128) minvKernel(DevTables T, int first, int count, const double* __restrict__ y,
                                                  const double* __restrict__ f, double* __restrict__ out,
                                                  R* __restrict__ scratch, int32_t* __restrict__ status) {
    const Slot s = GROUP ? groupSlot(T, first) : chainSlot(T, first, count);
    if (s.inst < 0) return;
    MInvSrc src{y, f, T.ybase[s.inst], T.ystride[s.inst], T.inq[s.inst]};
    MInvOut o{out, T.ybase[s.inst], T.ystride[s.inst], T.inq[s.inst]};
    int st = rhs<R, NM, false, GROUP>(T, s, scratch, src, o);
    if (!groupAll<GROUP>(o.finite, s)) st |= SBG_INST_NONFINITE;
    if (s.gl == 0) status[s.inst] = st;
}

// q /= |q| for the quaternion at q slot qo (RigidBodyNodeSpec_Ball.h:417-434).
__device__ __forceinline__ void normalizeQuatAt(double* y, int64_t base, int64_t stride, int qo) {
    double qq[4];
    for (int j = 0; j < 4; ++j) qq[j] = y[base + (int64_t)(qo + j) * stride];
    const double len = sqrt(qq[0] * qq[0] + qq[1] * qq[1] + qq[2] * qq[2] + qq[3] * qq[3]);
    for (int j = 0; j < 4; ++j) y[base + (int64_t)(qo + j) * stride] = qq[j] / len;
}

// ---------------------------------------------------- RK Merson persistent
// Sum over the lanes of a group (butterfly within the group's lanes).
__device__ __forceinline__ double groupSum(double v, const Slot& s) {
    for (int off = s.G >> 1; off > 0; off >>= 1) v += __shfl_xor_sync(s.mask, v, off);
    return v;
}

// One RK-Merson stage RHS of a level-parallel instance of the mixed form,
// out of line (the kernel keeps a single call site): the mixed RHS, then,
// once the refinement reports an ill-conditioned M and `fallback` allows it,
// the FP64 RHS on the FP64 mirror of the records from then on (*rhs64).
// Returns the status bits (kStFp64 when it switched); *finite reports the
// derivatives.
template <int NM, class R>
__device__ __noinline__ int stageRhsMixedGroup(const DevTables& T, const Slot& s, R* scratch, bool fallback,
                                               bool* rhs64, const double* y, const R* f0, const R* a, const R* b,
                                               int64_t base, int64_t stride, int nq, int stg, double c, R* dst,
                                               bool* finite) {
    StageSrc<R> src{y, f0, a, b, base, stride, nq, stg, c};
    FOut<R> o{dst, base, stride, nq};
    int r = 0;
    if (!*rhs64) {
        r = rhs<R, NM, true, true>(T, s, scratch, src, o);
        if (!(fallback && (r & SBG_INST_ILL_CONDITIONED))) {
            *finite = o.finite;
            return r;
        }
        *rhs64 = true;
        o.finite = true;
        r = kStFp64;
    }
    r |= rhs<double, NM, false, true>(T, s, T.scratch64, src, o);
    *finite = o.finite;
    return r;
}

// Group g of G lanes of the FP64 list kernel: the g-th instance in FP64
// mode at this launch.
template <int G> __device__ __forceinline__ Slot listSlot(const DevTables& T, int launch) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int g = t / G, lane = threadIdx.x & 31;
    const int* list = T.fbList + (int64_t)(launch & 1) * T.ninst;
    const unsigned mask = G == 32 ? 0xffffffffu : ((1u << G) - 1u) << (lane & ~(G - 1));
    return Slot{g < T.fbCount[launch & 1] ? list[g] : -1, t % G, G, mask};
}

// One-step launches of a mixed batch integration: the instance's mode at the
// next launch (written by this launch's owner of the instance only); FP64
// puts it on the next list.
__device__ __forceinline__ void fbNext(const DevTables& T, int launch, int inst, bool fp64) {
    const int k = (launch + 1) & 1;
    T.fbMode[(int64_t)k * T.ninst + inst] = fp64 ? 1 : 0;
    if (fp64) T.fbList[(int64_t)k * T.ninst + atomicAdd(T.fbCount + k, 1)] = inst;
}

// LIST: the FP64 steps of the instances in FP64 mode during the one-step
// launches of a mixed batch integration (R = double, fbuf = the FP64 stage
// planes, scratch = FP64 records at T.sbase per instance). With GROUP,
// kFbLanes lanes per instance through the level-parallel driver on the
// field-major layout; without, one thread per instance through the one-thread
// driver on contiguous records.
template <class R, int NM, bool REF, bool GROUP, int MINB = 1, bool LOOPS = false, int BS = 128, bool LIST = false>
__global__ void __launch_bounds__(BS, MINB) rkMersonKernel(DevTables T, int first, int count, double* __restrict__ y,
                                                            double* __restrict__ time, R* __restrict__ fbuf,
                                                            int64_t fplane, R* __restrict__ scratch,
                                                            int32_t* __restrict__ status, double h, StepCtl sc,
                                                            double accuracy, double consTol, int projectEveryStep) {
    static_assert(!LIST || (std::is_same<R, double>::value && !REF && !LOOPS), "the FP64 list is FP64");
    const Slot s = LIST ? (GROUP ? listSlot<kFbLanes>(T, sc.launch) : listSlot<1>(T, sc.launch))
                        : GROUP ? groupSlot(T, first) : chainSlot(T, first, count);
    if (s.inst < 0) return;
    const int inst = s.inst;
    // One-step launches of a mixed batch integration: an instance in FP64 mode
    // is the list kernel's at this launch.
    const bool split = !LIST && REF && T.fbList != nullptr;
    if (split && T.fbMode[(int64_t)(sc.launch & 1) * T.ninst + inst]) return;
    bool toFp64 = false;  // split: this launch's mixed step met an ill-conditioned M
    const int64_t base = T.ybase[inst], stride = T.ystride[inst];
    const int nq = T.inq[inst], nu = T.inu[inst];
    const int body0 = T.ibody[inst], nb = T.inb[inst];
    R* f0 = fbuf;
    R* fA = fbuf + fplane;
    R* fB = fbuf + 2 * fplane;
    R* fC = fbuf + 3 * fplane;
    int st = status[inst];
    double tc = time[inst];
    // Per-instance control (serving): this launch's steps, whether it starts
    // the integration, the instance's own step size and tolerances.
    int nst = sc.nsteps;
    const double tStop = sc.tStop;
    const int maxSteps = sc.maxSteps > 0 ? sc.maxSteps : kMaxStepsPerCall;
    // steps this instance still has to take in a fixed-count call of one-step
    // launches (read before any lane of the group can change it)
    int left = T.stepsLeft ? T.stepsLeft[inst] : kMaxStepsPerCall;
    bool init = sc.init != 0, pes = projectEveryStep != 0;
    if (T.ictl) {
        const int c = T.ictl[inst];
        nst = c & kCtlSteps;
        init = (c & kCtlInit) != 0;
        pes = (c & kCtlProjectEveryStep) != 0;
        h = T.iparam[3 * inst];
        accuracy = T.iparam[3 * inst + 1];
        consTol = T.iparam[3 * inst + 2];
        // Integrator::initialize normalizes quaternions (Integrator.cpp:376-377);
        // instances with loop closures project in loopInitialize instead.
        if (init && !(LOOPS && T.incons[inst] > 0)) {
            for (int lb = s.gl; lb < nb; lb += s.G) {
                if (T.info[body0 + lb] & F_QUAT) normalizeQuatAt(y, base, stride, T.qoff[body0 + lb]);
            }
            if constexpr (GROUP) __syncwarp(s.mask);
        }
    }
    const double projLimit = fmax(2 * consTol, sqrt(consTol));
    // Mixed form in the server's lane: once the refinement reports an
    // ill-conditioned M, the instance's RHS runs in FP64 on the FP64 mirror of
    // its records (that stage's RHS included) for kFp64Steps steps, then the
    // mixed form is tried again (kStFp64 and the step count in its status
    // word keep that across launches).
    const bool fallback = REF && GROUP && T.ictl && T.scratch64;
    bool rhs64 = fallback && (st & kStFp64);
    auto stage = [&](int stg, double c, const R* a, const R* b, R* dst) {
        StageSrc<R> src{y, f0, a, b, base, stride, nq, stg, c};
        FOut<R> o{dst, base, stride, nq};
        if constexpr (LIST && !GROUP) {
            st |= rhsChain<R, NM, false>(T, inst, ScrStrided<R>{scratch + T.sbase[inst], 1}, src, o);
        } else if constexpr (REF && GROUP) {
            bool fin = true;
            const bool was64 = rhs64;
            st |= stageRhsMixedGroup<NM, R>(T, s, scratch, fallback, &rhs64, y, f0, a, b, base, stride, nq, stg, c,
                                            dst, &fin);
            if (rhs64 && !was64)  // switched at this stage: this step and the next kFp64Steps - 1
                st = (st & ~kStFp64LeftMask) | kStWasFp64 | (kFp64Steps << kStFp64LeftShift);
            o.finite = fin;
        } else {
            st |= rhs<R, NM, REF, GROUP, LOOPS>(T, s, scratch, src, o);
        }
        if (!groupAll<GROUP>(o.finite, s)) st |= SBG_INST_NONFINITE;
        if constexpr (GROUP) __syncwarp(s.mask);  // the next stage reads what other lanes wrote
    };
    // The loop-closure state of this instance (either driver's layout; only
    // instantiated with R = double); its projections run on the first lane
    // of a group. The stage planes fB/fC are free outside a step.
    auto loopState = [&]() {
        double* rec0 = reinterpret_cast<double*>(scratch) + T.sbase[inst];
        double* sv = reinterpret_cast<double*>(fB);
        double* dl = reinterpret_cast<double*>(fC);
        if constexpr (GROUP) return loopStateRows(T, inst, rec0, y, sv, dl, base, stride);
        else return loopStateChain(T, inst, rec0, (int)T.sstride[inst], y, sv, dl, base, stride);
    };
    // Integrator::initialize with loop closures: forced position and
    // velocity projection (IntegratorRep.h:856-895).
    auto loopLeaderOr = [&](int bits) {
        if constexpr (GROUP) {
            __syncwarp(s.mask);
            return (int)__reduce_or_sync(s.mask, (unsigned)bits);
        } else {
            return bits;
        }
    };
    if constexpr (LOOPS)
        if (init && T.incons[inst] > 0) {
            int lst = 0;
            if (s.gl == 0) lst = loopInitialize<NM>(loopState(), consTol);
            st |= loopLeaderOr(lst);
        }
    for (int step = 0;; ++step) {
        // t1 of this step (StepCtl): a fixed count of full steps, or
        // takeOneStep's choice against tMax = tStop (AbstractIntegratorRep.cpp:536-544)
        double t1;
        if (step >= maxSteps) break;
        if (left <= 0) break;  // this instance has taken its steps
        if (nst >= 0) {
            if (step >= nst) break;
            t1 = tc + h;
        } else {
            if (!(tc < tStop)) break;
            if (tStop < tc + 0.95 * h) t1 = tStop;
            else if (tStop > tc + 1.001 * h) t1 = tc + h;
            else t1 = tStop;
            if (!(t1 > tc) || step >= kMaxStepsPerCall) {  // time no longer advances
                st |= SBG_INST_TIMEOUT;
                break;
            }
        }
        const double hs = t1 - tc;
        stage(0, 0.0, fA, fB, f0);      // f0 = f(y0)
        stage(1, hs / 3, fA, fB, fA);   // f1 -> fA
        stage(2, hs / 6, fA, fB, fB);   // f2 -> fB (input uses f1 in fA)
        stage(3, hs / 8, fB, fB, fC);   // f3 -> fC (input uses f2 in fB)
        stage(4, hs / 2, fB, fC, fA);   // f4 -> fA (ysave input uses f2, f3)
        if (split && (st & SBG_INST_ILL_CONDITIONED)) {
            // The step met an ill-conditioned M: leave y and t as they were;
            // the FP64 list kernel takes this step at the next launch, and
            // the next few.
            st &= ~SBG_INST_ILL_CONDITIONED;
            toFp64 = true;
            if (s.gl == 0) T.fbLeft[inst] = kFp64Steps;
            break;
        }
        // y1 = y0 + h/6 (f0 + 4 f3 + f4); yerr = 0.2 |y1 - ysave|; error norm
        // (RungeKuttaMersonIntegrator.cpp:124-139, IntegratorRep.h:454-523).
        // Each lane of a group takes every G-th body.
        const double h6 = hs / 6, h2 = hs / 2;
        double sq = 0, su = 0, squat = 0, nquat = 0;
        bool fin = true;
        for (int lb = s.gl; lb < nb; lb += s.G) {
            const int row = body0 + lb;
            const int type = T.info[row] & 15;
            const int n = (T.info[row] >> 4) & 15;
            const int qo = T.qoff[row], uo = T.uoff[row];
            const int nqb = type == T_BALL ? 4 : (type == T_FREE ? 7 : n);
            double q1[7], dq[7];
            for (int j = 0; j < nqb; ++j) {
                const int64_t e = base + (int64_t)(qo + j) * stride;
                const double y0 = y[e];
                const double a0 = double(f0[e]), aB = double(fB[e]), aC = double(fC[e]), aA = double(fA[e]);
                const double ys = y0 + h2 * ((a0 - 3.0 * aB) + 4.0 * aC);
                const double y1v = y0 + h6 * ((a0 + 4.0 * aC) + aA);
                q1[j] = y1v;
                dq[j] = 0.2 * fabs(y1v - ys);
                y[e] = y1v;
                fin &= isfinite(y1v);
            }
            if (T.info[row] & F_QUAT) {
                // N * NInv * dq with unnormalized q1 (Rotation.h:712-748)
                const double e0 = 2 * q1[0], e1 = 2 * q1[1], e2 = 2 * q1[2], e3 = 2 * q1[3];
                const double du0 = -e1 * dq[0] + e0 * dq[1] - e3 * dq[2] + e2 * dq[3];
                const double du1 = -e2 * dq[0] + e3 * dq[1] + e0 * dq[2] - e1 * dq[3];
                const double du2 = -e3 * dq[0] - e2 * dq[1] + e1 * dq[2] + e0 * dq[3];
                const double g0 = q1[0] / 2, g1 = q1[1] / 2, g2 = q1[2] / 2, g3 = q1[3] / 2;
                const double o0 = -g1 * du0 + -g2 * du1 + -g3 * du2;
                const double o1 = g0 * du0 + g3 * du1 + -g2 * du2;
                const double o2 = -g3 * du0 + g0 * du1 + g1 * du2;
                const double o3 = g2 * du0 + -g1 * du1 + g0 * du2;
                sq += o0 * o0 + o1 * o1 + o2 * o2 + o3 * o3;
                for (int j = 4; j < nqb; ++j) sq += dq[j] * dq[j];
                const double len = sqrt(q1[0] * q1[0] + q1[1] * q1[1] + q1[2] * q1[2] + q1[3] * q1[3]);
                squat += (len - 1) * (len - 1);
                nquat += 1;
            } else {
                for (int j = 0; j < nqb; ++j) sq += dq[j] * dq[j];
            }
            for (int j = 0; j < n; ++j) {
                const int64_t e = base + (int64_t)(nq + uo + j) * stride;
                const double y0 = y[e];
                const double a0 = double(f0[e]), aB = double(fB[e]), aC = double(fC[e]), aA = double(fA[e]);
                const double ys = y0 + h2 * ((a0 - 3.0 * aB) + 4.0 * aC);
                const double y1v = y0 + h6 * ((a0 + 4.0 * aC) + aA);
                const double vi = fabs(y0);
                const double us = vi > 1 ? 1 / vi : 1.0;  // calcRelativeScaling, frozen at step start
                const double d = us * (0.2 * fabs(y1v - ys));
                su += d * d;
                y[e] = y1v;
                fin &= isfinite(y1v);
            }
        }
        if constexpr (GROUP) {
            sq = groupSum(sq, s);
            su = groupSum(su, s);
            squat = groupSum(squat, s);
            nquat = groupSum(nquat, s);
            fin = __all_sync(s.mask, fin);
        }
        if (!fin) st |= SBG_INST_NONFINITE;
        const double qn = nq ? sqrt(sq / nq) : 0.0, un = nu ? sqrt(su / nu) : 0.0;
        const double errNorm = qn >= un ? qn : un;
        // projection gate and quaternion normalization
        // (AbstractIntegratorRep.cpp:158-190, SimbodyMatterSubsystemRep.cpp:4096-4183)
        bool loopsDone = false;
        if constexpr (LOOPS)
            if (T.incons[inst] > 0) {
                loopsDone = true;
                if (errNorm <= 16 * accuracy) {
                    const double quatNorm = nquat > 0 ? sqrt(squat / nquat) : 0.0;
                    int lst = 0;
                    if (GROUP && s.G >= 3)
                        lst = loopProjectStepLanes<NM>(loopState(), quatNorm, consTol, projLimit, pes, s.gl, s.mask);
                    else if (s.gl == 0)
                        lst = loopProjectStep<NM>(loopState(), quatNorm, consTol, projLimit, pes);
                    st |= loopLeaderOr(lst);
                }
            }
        if (!loopsDone && errNorm <= 16 * accuracy && nquat > 0) {
            const double quatNorm = sqrt(squat / nquat);
            if (quatNorm > projLimit) st |= SBG_INST_PROJECTION_FAILED;
            else if (quatNorm > consTol || pes) {
                for (int lb = s.gl; lb < nb; lb += s.G) {
                    const int row = body0 + lb;
                    if (T.info[row] & F_QUAT) normalizeQuatAt(y, base, stride, T.qoff[row]);
                }
            }
        }
        if constexpr (GROUP) __syncwarp(s.mask);
        if (fallback && rhs64) {  // one FP64 step taken: back to the mixed form after kFp64Steps
            const int n64 = ((st & kStFp64LeftMask) >> kStFp64LeftShift) - 1;
            st &= ~kStFp64LeftMask;
            if (n64 > 0) {
                st |= n64 << kStFp64LeftShift;
            } else {
                rhs64 = false;
                st &= ~kStFp64;
            }
        }
        tc = t1;
        --left;
        if (s.gl == 0) {
            if (T.stepsLeft) T.stepsLeft[inst] = left;
            if constexpr (LIST) {
                --T.fbLeft[inst];
                atomicAdd(T.fbSteps, 1ULL);
            }
        }
    }
    if (s.gl == 0) {
        if constexpr (LIST) fbNext(T, sc.launch, inst, T.fbLeft[inst] > 0);
        else if (split) fbNext(T, sc.launch, inst, toFp64);
    }
    if (s.gl == 0) {
        time[inst] = tc;
        status[inst] = st;
    }
}

}  // namespace sbg
