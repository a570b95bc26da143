// abi_device.cuh -- articulated-body forward dynamics and fixed-step
// Runge-Kutta-Merson integration for a batch of multibody instances.
//
// One thread owns one instance (a System state). The RHS is a set of sweeps
// over the instance's level-ordered body table:
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
// trees) to the few-1e-6 level set by the FP32 kinematics.
//
// Per-body intermediates live in a scratch record (engine.h); its element e
// is at p[e*SS]: SS = 32 for warp-tiled records of instances sharing one
// topology (a warp's accesses coalesce), SS = 1 for per-instance contiguous
// records. Along a chain (parent = previous row) the parent's values travel
// in registers instead of through the record.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "engine.h"
#include "spatial.cuh"
#include "kernels.h"

namespace sbg {

enum { T_PIN = 0, T_SLIDER = 1, T_UNIV = 2, T_BALL = 3, T_FREE = 4 };

template <class R, int SS> struct Scr {
    R* p;
    __device__ __forceinline__ R& operator()(int e) const { return p[e * SS]; }
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

template <class R, int SS> __device__ __forceinline__ void st3(const Scr<R, SS>& S, int e, V3<R> v) {
    S(e) = v.x; S(e + 1) = v.y; S(e + 2) = v.z;
}
template <class R, int SS> __device__ __forceinline__ V3<R> ld3(const Scr<R, SS>& S, int e) {
    return V3<R>{S(e), S(e + 1), S(e + 2)};
}

template <class R> __device__ __forceinline__ void sincosR(R x, R* s, R* c) {
    if constexpr (std::is_same<R, double>::value) sincos(x, s, c); else sincosf(x, s, c);
}
template <class R> __device__ __forceinline__ R sqrtR(R x) {
    if constexpr (std::is_same<R, double>::value) return sqrt(x); else return sqrtf(x);
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
__device__ __forceinline__ DF3 dfq3(V3<float> v) { return DF3{dfq(v.x), dfq(v.y), dfq(v.z)}; }
__device__ __forceinline__ DF3 operator+(DF3 a, DF3 b) { return DF3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ DF3 operator+(DF3 a, V3<float> b) { return DF3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ DF3 operator-(DF3 a, DF3 b) { return DF3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ DF3 scale(DF3 a, float s) { return DF3{a.x * s, a.y * s, a.z * s}; }
// a + s*v with s a df scalar's hi part times float vector (s exact float)
__device__ __forceinline__ DF3 axpyDF(DF3 a, float s, V3<float> v) {
    return DF3{a.x + DF{__fmul_rn(s, v.x), __fmaf_rn(s, v.x, -__fmul_rn(s, v.x))},
               a.y + DF{__fmul_rn(s, v.y), __fmaf_rn(s, v.y, -__fmul_rn(s, v.y))},
               a.z + DF{__fmul_rn(s, v.z), __fmaf_rn(s, v.z, -__fmul_rn(s, v.z))}};
}
// float vector x df vector (exact-float left operand)
__device__ __forceinline__ DF3 crossFD(V3<float> a, DF3 b) {
    return DF3{b.z * a.y - b.y * a.z, b.x * a.z - b.z * a.x, b.y * a.x - b.x * a.y};
}
__device__ __forceinline__ DF dotFD(V3<float> a, DF3 b) { return (b.x * a.x + b.y * a.y) + b.z * a.z; }
__device__ __forceinline__ DF3 symMulDF(const S3<float>& S, DF3 v) {
    return DF3{(v.x * S.xx + v.y * S.xy) + v.z * S.xz, (v.x * S.xy + v.y * S.yy) + v.z * S.yz,
               (v.x * S.xz + v.y * S.yz) + v.z * S.zz};
}

// ------------------------------------------------------------------ pass 1
// Src::q(k), Src::u(k) give the (double) state; Out::qdot(k, v) receives qdot.
template <class R, int NM, int SS, class Src, class Out>
__device__ __forceinline__ void pass1(const DevTables& T, int body0, int nb, const Scr<R, SS>& S, const Src& src,
                                      Out& out, V3<R> g) {
    const R* PT = paramTable<R>(T);
    const R* FC = coefTable<R>(T);
    const R* FQ = q0Table<R>(T);
    M3<R> cR = ident3<R>();
    V3<R> cp = z3<R>(), cw = z3<R>(), cv = z3<R>();  // previous row's kinematics
    for (int lb = 0; lb < nb; ++lb) {
        const int row = body0 + lb;
        const int info = T.info[row];
        const int type = info & 15, n = (info >> 4) & 15;
        const int nw = n == 6 ? 6 : NM;  // padded record width of this row
        const int parent = T.parent[row];
        const int qo = T.qoff[row], uo = T.uoff[row];
        const int rec = T.srec[row];
        const R* pr = PT + (int64_t)row * kParamStride;
        const R m = pr[0];
        const V3<R> com = mk3(pr[1], pr[2], pr[3]);
        const S3<R> Gb{pr[4], pr[5], pr[6], pr[7], pr[8], pr[9]};

        // parent kinematics
        M3<R> RGP;
        V3<R> pGP, wGP, vGP;
        if (parent < 0) {
            RGP = ident3<R>(); pGP = z3<R>(); wGP = z3<R>(); vGP = z3<R>();
        } else if (info & F_CARRY) {
            RGP = cR; pGP = cp; wGP = cw; vGP = cv;
        } else {
            const int pe = T.srec[body0 + parent];
#pragma unroll
            for (int i = 0; i < 9; ++i) RGP.a[i] = S(pe + i);
            pGP = ld3(S, pe + 9); wGP = ld3(S, pe + 12); vGP = ld3(S, pe + 15);
        }

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
        switch (type) {
        case T_PIN: {  // RigidBodyNodeSpec_Pin.h:103-122
            R s, c;
            sincosR(q[0], &s, &c);
            RFM.a[0] = c; RFM.a[1] = -s; RFM.a[3] = s; RFM.a[4] = c;
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
        default: {  // Ball / Free quaternion (RigidBodyNodeSpec_Ball.h:134-214)
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
        const M3<R> RGB = mul(RGP, RPB);
        const V3<R> l = mul(RGP, pPB);  // Phi (RigidBodyNode.cpp:63)
        const V3<R> pGB = l + pGP;
        const M3<R> RGF = (info & F_RPF_I) ? RGP : mul(RGP, RPF);

        // H_PB_G columns (RigidBodyNodeSpec.cpp:44-74), stored; V_PB_G = H u
        V3<R> VPw = z3<R>(), VPv = z3<R>();
        V3<R> wFM = z3<R>();
        const int eH = rec + kRecH;
        auto putH = [&](int j, V3<R> hw, V3<R> hv) {
            st3(S, eH + 6 * j, hw);
            st3(S, eH + 6 * j + 3, hv);
            VPw = axpy(VPw, u[j], hw);
            VPv = axpy(VPv, u[j], hv);
        };
        // -(r x e_j) for the unit axes
        const V3<R> nrx = mk3(R(0), -r.z, r.y), nry = mk3(r.z, R(0), -r.x), nrz = mk3(-r.y, r.x, R(0));
        switch (type) {
        case T_PIN:
            putH(0, col(RGF, 2), mul(RGF, nrz));
            wFM = mk3(R(0), R(0), u[0]);
            break;
        case T_SLIDER:
            putH(0, z3<R>(), col(RGF, 0));
            break;
        case T_UNIV:
            putH(0, col(RGF, 0), mul(RGF, nrx));
            putH(1, mul(RGF, y1), mul(RGF, -cross(r, y1)));
            wFM = axpy(mk3(u[0], R(0), R(0)), u[1], y1);
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
        const V3<R> hdw = (type == T_UNIV) ? u[1] * cross(wFM, y1) : z3<R>();
        const V3<R> VDw = mul(RGF, hdw) + cross(wGP, VPw);
        const V3<R> VDv = mul(RGF, -cross(r, hdw) - cross(cross(wFM, r), wFM)) + cross(wGP, VPv);

        // RigidBodyNode.cpp:54-84, 98-174
        const S3<R> Gi = reexpress(RGB, Gb);
        const V3<R> pc = mul(RGB, com);
        const V3<R> wGB = wGP + VPw;
        const V3<R> vGB = (vGP + cross(wGP, l)) + VPv;
        const V3<R> bw = m * cross(wGB, mul(Gi, wGB));
        const V3<R> bv = m * cross(wGB, cross(wGB, pc));
        const V3<R> aw = VDw;
        const V3<R> av = VDv + cross(wGP, vGB - vGP);
        // gravity (Force_Gravity.cpp:549-551)
        const V3<R> Fv = m * g;
        const V3<R> Fw = cross(pc, Fv);

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

        // store
        if (info & F_MEMCHILD) {
#pragma unroll
            for (int i = 0; i < 9; ++i) S(rec + i) = RGB.a[i];
            st3(S, rec + 9, pGB); st3(S, rec + 12, wGB); st3(S, rec + 15, vGB);
        }
        cR = RGB; cp = pGB; cw = wGB; cv = vGB;
        st3(S, rec + kRecPc, pc);
        S(rec + kRecGi + 0) = Gi.xx; S(rec + kRecGi + 1) = Gi.yy; S(rec + kRecGi + 2) = Gi.zz;
        S(rec + kRecGi + 3) = Gi.xy; S(rec + kRecGi + 4) = Gi.xz; S(rec + kRecGi + 5) = Gi.yz;
        st3(S, rec + kRecL, l);
        st3(S, rec + kRecA, aw); st3(S, rec + kRecA + 3, av);
        if constexpr (Src::kMInv) { st3(S, rec + kRecBF, z3<R>()); st3(S, rec + kRecBF + 3, z3<R>()); }
        else { st3(S, rec + kRecBF, bw - Fw); st3(S, rec + kRecBF + 3, bv - Fv); }
        if (info & F_MEMACC)
            for (int i = 0; i < 27; ++i) S(rec + kRecPacc + i) = R(0);
        const int ef = eH + 6 * nw;
        for (int j = 0; j < n; ++j) S(ef + j) = f[j];
    }
}

// ------------------------------------------------------------------ pass 2
// Articulated body inertia fused with the first udot pass for one body with
// N columns (N = 6 for Free, else the batch width NM with unused columns
// zero and an identity block in D). Returns false on a singular D.
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
        // cofactor inverse (SmallMatrixMixed.h:921-960)
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
        // LU with partial pivoting, then A X = I (LAPACK getrf/getri semantics,
        // SmallMatrixMixed.h:859-894).
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

// Values a child hands to its parent in the inward sweeps.
template <class R> struct Carry2 {
    AB<R> P;        // shifted P+
    V3<R> zw, zv;   // Phi z+
};

// Order chosen for short live ranges: P, c = P a, z, PH, eps, D, DI, then G
// one column at a time folded into P+ and z+.
template <class R, int N, int SS>
__device__ __forceinline__ bool pass2BodyImpl(const DevTables& T, int body0, int row, int n, const Scr<R, SS>& S,
                                              R m, bool haveCarry, Carry2<R>& cy) {
    const int info = T.info[row];
    const int rec = T.srec[row];
    const int eH = rec + kRecH;
    const int ef = eH + 6 * N, eDI = ef + N, eG = eDI + N * N, eEps = eG + 6 * N;
    // P = ArticulatedInertia(Mk) + children (RigidBodyNodeSpec.cpp:259-279)
    AB<R> P;
    V3<R> zaw = z3<R>(), zav = z3<R>();
    {
        const V3<R> pc = ld3(S, rec + kRecPc);
        P.M = S3<R>{m, m, m, R(0), R(0), R(0)};
        P.J = S3<R>{m * S(rec + kRecGi), m * S(rec + kRecGi + 1), m * S(rec + kRecGi + 2),
                    m * S(rec + kRecGi + 3), m * S(rec + kRecGi + 4), m * S(rec + kRecGi + 5)};
        const V3<R> mp = m * pc;
        P.F.a[0] = R(0);  P.F.a[1] = -mp.z; P.F.a[2] = mp.y;
        P.F.a[3] = mp.z;  P.F.a[4] = R(0);  P.F.a[5] = -mp.x;
        P.F.a[6] = -mp.y; P.F.a[7] = mp.x;  P.F.a[8] = R(0);
        if (info & F_MEMACC) {
            const int ea = rec + kRecPacc;
            P.M.xx += S(ea + 0); P.M.yy += S(ea + 1); P.M.zz += S(ea + 2);
            P.M.xy += S(ea + 3); P.M.xz += S(ea + 4); P.M.yz += S(ea + 5);
            P.J.xx += S(ea + 6); P.J.yy += S(ea + 7); P.J.zz += S(ea + 8);
            P.J.xy += S(ea + 9); P.J.xz += S(ea + 10); P.J.yz += S(ea + 11);
#pragma unroll
            for (int i = 0; i < 9; ++i) P.F.a[i] += S(ea + 12 + i);
            zaw = ld3(S, rec + kRecZacc);
            zav = ld3(S, rec + kRecZacc + 3);
        }
        if (haveCarry) {
            P.M.xx += cy.P.M.xx; P.M.yy += cy.P.M.yy; P.M.zz += cy.P.M.zz;
            P.M.xy += cy.P.M.xy; P.M.xz += cy.P.M.xz; P.M.yz += cy.P.M.yz;
            P.J.xx += cy.P.J.xx; P.J.yy += cy.P.J.yy; P.J.zz += cy.P.J.zz;
            P.J.xy += cy.P.J.xy; P.J.xz += cy.P.J.xz; P.J.yz += cy.P.J.yz;
#pragma unroll
            for (int i = 0; i < 9; ++i) P.F.a[i] += cy.P.F.a[i];
            zaw = zaw + cy.zw;
            zav = zav + cy.zv;
        }
    }
    // z = (P a + b) - F + sum_children Phi z+ (RigidBodyNodeSpec.cpp:380-392)
    V3<R> zw, zv;
    {
        V3<R> cw, cv;
        abmul(P, ld3(S, rec + kRecA), ld3(S, rec + kRecA + 3), cw, cv);
        zw = (cw + ld3(S, rec + kRecBF)) + zaw;
        zv = (cv + ld3(S, rec + kRecBF + 3)) + zav;
    }
    // PH = P H; D = ~H PH; eps = f - ~H z (:294-296, :394)
    V3<R> PHw[N], PHv[N];
    R D[N * N], eps[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
        V3<R> hw = z3<R>(), hv = z3<R>();
        if (j < n) { hw = ld3(S, eH + 6 * j); hv = ld3(S, eH + 6 * j + 3); }
        abmul(P, hw, hv, PHw[j], PHv[j]);
        eps[j] = j < n ? S(ef + j) - (dot(hw, zw) + dot(hv, zv)) : R(0);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
        V3<R> hw = z3<R>(), hv = z3<R>();
        if (i < n) { hw = ld3(S, eH + 6 * i); hv = ld3(S, eH + 6 * i + 3); }
#pragma unroll
        for (int j = 0; j < N; ++j)
            D[i * N + j] = (i < n && j < n) ? dot(hw, PHw[j]) + dot(hv, PHv[j]) : R(i == j ? 1 : 0);
    }
    R DI[N * N];
    const bool ok = invertSmall<R, N>(D, DI);
    // G = PH DI one column at a time; P+ = P - G ~PH with the mass and
    // inertia blocks symmetrized (:297-324); z+ = z + G eps.
    R mm[9], ms[9], in[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) { mm[i] = R(0); ms[i] = R(0); in[i] = R(0); }
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
                in[3 * a + b] = in[3 * a + b] + g3w[a] * hw3[b];
            }
        if (j < n) {
            st3(S, eG + 6 * j, gw);
            st3(S, eG + 6 * j + 3, gv);
            S(eEps + j) = eps[j];
            zpw = axpy(zpw, eps[j], gw);
            zpv = axpy(zpv, eps[j], gv);
        }
    }
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j)
            if (i < n && j < n) S(eDI + i * N + j) = DI[i * N + j];
    AB<R> PP;
    PP.M = S3<R>{P.M.xx - ms[0], P.M.yy - ms[4], P.M.zz - ms[8], P.M.xy - (ms[3] + ms[1]) / R(2),
                 P.M.xz - (ms[6] + ms[2]) / R(2), P.M.yz - (ms[7] + ms[5]) / R(2)};
    PP.J = S3<R>{P.J.xx - in[0], P.J.yy - in[4], P.J.zz - in[8], P.J.xy - (in[3] + in[1]) / R(2),
                 P.J.xz - (in[6] + in[2]) / R(2), P.J.yz - (in[7] + in[5]) / R(2)};
#pragma unroll
    for (int i = 0; i < 9; ++i) PP.F.a[i] = P.F.a[i] - mm[i];

    // hand P+ (shifted by -l) and Phi z+ to the parent
    const int parent = T.parent[row];
    if (parent >= 0) {
        const V3<R> l = ld3(S, rec + kRecL);
        cy.P = abshift(PP, l);
        cy.zw = zpw + cross(l, zpv);
        cy.zv = zpv;
        if (!(info & F_CARRY)) {
            const int pa = T.srec[body0 + parent] + kRecPacc;
            S(pa + 0) += cy.P.M.xx; S(pa + 1) += cy.P.M.yy; S(pa + 2) += cy.P.M.zz;
            S(pa + 3) += cy.P.M.xy; S(pa + 4) += cy.P.M.xz; S(pa + 5) += cy.P.M.yz;
            S(pa + 6) += cy.P.J.xx; S(pa + 7) += cy.P.J.yy; S(pa + 8) += cy.P.J.zz;
            S(pa + 9) += cy.P.J.xy; S(pa + 10) += cy.P.J.xz; S(pa + 11) += cy.P.J.yz;
#pragma unroll
            for (int i = 0; i < 9; ++i) S(pa + 12 + i) += cy.P.F.a[i];
            S(pa + 21) += cy.zw.x; S(pa + 22) += cy.zw.y; S(pa + 23) += cy.zw.z;
            S(pa + 24) += cy.zv.x; S(pa + 25) += cy.zv.y; S(pa + 26) += cy.zv.z;
        }
    }
    return ok;
}

// Free (6 columns) runs once per tree; kept out of line so its register
// demand does not spill the common path.
template <class R, int SS>
__device__ __noinline__ bool pass2Free(const DevTables& T, int body0, int row, const Scr<R, SS>& S, R m,
                                       bool haveCarry, Carry2<R>& cy) {
    return pass2BodyImpl<R, 6, SS>(T, body0, row, 6, S, m, haveCarry, cy);
}

// ------------------------------------------------------------------ pass 3
// udot = DI eps - ~G A+, A = A+ + H udot + a (RigidBodyNodeSpec.cpp:408-446).
// With REF (mixed form) udot0 goes to the record and the outward half of the
// double-float inverse dynamics runs alongside: A_df, then the body's own
// force term F_df = Mk A_df + b - F_gravity.
struct Carry3 {
    V3<float> Aw, Av;
    DF3 Dw, Dv;
};
template <class R> struct Carry3T { V3<R> Aw, Av; };

template <class R, int N, int SS, bool REF, class Out>
__device__ __forceinline__ void pass3BodyImpl(const DevTables& T, int body0, int row, int n, const Scr<R, SS>& S,
                                              Out& out, Carry3T<R>& cy, DF3& cDw, DF3& cDv) {
    const int info = T.info[row];
    const int rec = T.srec[row];
    const int eH = rec + kRecH;
    const int ef = eH + 6 * N, eDI = ef + N, eG = eDI + N * N, eEps = eG + 6 * N, eU0 = eEps + N;
    const int parent = T.parent[row];
    const V3<R> l = ld3(S, rec + kRecL);
    V3<R> Apw = z3<R>(), Apv = z3<R>();
    DF3 Dpw{}, Dpv{};
    if constexpr (REF) { Dpw = DF3{dfq(0.f), dfq(0.f), dfq(0.f)}; Dpv = Dpw; }
    if (parent >= 0) {
        V3<R> w, v;
        if (info & F_CARRY) {
            w = cy.Aw; v = cy.Av;
            if constexpr (REF) { Dpw = cDw; Dpv = cDv; }
        } else {
            const int pe = T.srec[body0 + parent];
            w = ld3(S, pe); v = ld3(S, pe + 3);
            if constexpr (REF) {
                Dpw = DF3{DF{S(pe + 6), S(pe + 7)}, DF{S(pe + 8), S(pe + 9)}, DF{S(pe + 10), S(pe + 11)}};
                Dpv = DF3{DF{S(pe + 12), S(pe + 13)}, DF{S(pe + 14), S(pe + 15)}, DF{S(pe + 16), S(pe + 17)}};
            }
        }
        Apw = w;
        Apv = v + cross(w, l);
        if constexpr (REF) Dpv = Dpv - crossFD(l, Dpw);  // A_v + A_w x l = A_v - l x A_w, in df
    }
    R eps[N];
#pragma unroll
    for (int j = 0; j < N; ++j) eps[j] = j < n ? S(eEps + j) : R(0);
    V3<R> Aw = Apw, Av = Apv;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        if (i < n) {
            R s = R(0);
#pragma unroll
            for (int k = 0; k < N; ++k)
                if (k < n) s = s + S(eDI + i * N + k) * eps[k];
            const R ud = s - (dot(ld3(S, eG + 6 * i), Apw) + dot(ld3(S, eG + 6 * i + 3), Apv));
            const V3<R> hw = ld3(S, eH + 6 * i), hv = ld3(S, eH + 6 * i + 3);
            if constexpr (REF) {
                S(eU0 + i) = ud;
                Dpw = axpyDF(Dpw, ud, hw);
                Dpv = axpyDF(Dpv, ud, hv);
            } else {
                out.udot(T.uoff[row] + i, ud);
            }
            Aw = axpy(Aw, ud, hw);
            Av = axpy(Av, ud, hv);
        }
    }
    const V3<R> aw = ld3(S, rec + kRecA), av = ld3(S, rec + kRecA + 3);
    Aw = Aw + aw;
    Av = Av + av;
    cy.Aw = Aw;
    cy.Av = Av;
    if (info & F_MEMCHILD) { st3(S, rec, Aw); st3(S, rec + 3, Av); }
    if constexpr (REF) {
        Dpw = Dpw + aw;
        Dpv = Dpv + av;
        cDw = Dpw;
        cDv = Dpv;
        if (info & F_MEMCHILD) {
            S(rec + 6) = Dpw.x.hi; S(rec + 7) = Dpw.x.lo; S(rec + 8) = Dpw.y.hi; S(rec + 9) = Dpw.y.lo;
            S(rec + 10) = Dpw.z.hi; S(rec + 11) = Dpw.z.lo;
            S(rec + 12) = Dpv.x.hi; S(rec + 13) = Dpv.x.lo; S(rec + 14) = Dpv.y.hi; S(rec + 15) = Dpv.y.lo;
            S(rec + 16) = Dpv.z.hi; S(rec + 17) = Dpv.z.lo;
        }
        // own inverse-dynamics force: Mk A + b - F (SpatialInertia*SpatialVec,
        // MassProperties.h:1071-1072)
        const R m = paramTable<R>(T)[(int64_t)row * kParamStride];
        const V3<R> pc = ld3(S, rec + kRecPc);
        const S3<R> Gi{S(rec + kRecGi), S(rec + kRecGi + 1), S(rec + kRecGi + 2), S(rec + kRecGi + 3),
                       S(rec + kRecGi + 4), S(rec + kRecGi + 5)};
        const DF3 Fw = scale(symMulDF(Gi, Dpw) + crossFD(pc, Dpv), m) + ld3(S, rec + kRecBF);
        const DF3 Fv = scale(Dpv - crossFD(pc, Dpw), m) + ld3(S, rec + kRecBF + 3);
        const int eF = rec + kRecFdf;
        S(eF + 0) = Fw.x.hi; S(eF + 1) = Fw.x.lo; S(eF + 2) = Fw.y.hi; S(eF + 3) = Fw.y.lo;
        S(eF + 4) = Fw.z.hi; S(eF + 5) = Fw.z.lo;
        S(eF + 6) = Fv.x.hi; S(eF + 7) = Fv.x.lo; S(eF + 8) = Fv.y.hi; S(eF + 9) = Fv.y.lo;
        S(eF + 10) = Fv.z.hi; S(eF + 11) = Fv.z.lo;
        if (info & F_MEMACC)
            for (int i = 0; i < 6; ++i) S(rec + kRecZ2acc + i) = R(0);
    }
}

template <class R, int SS, bool REF, class Out>
__device__ __noinline__ void pass3Free(const DevTables& T, int body0, int row, const Scr<R, SS>& S, Out& out,
                                       Carry3T<R>& cy, DF3& cDw, DF3& cDv) {
    pass3BodyImpl<R, 6, SS, REF>(T, body0, row, 6, S, out, cy, cDw, cDv);
}

// ------------------------------------------------------- passes 4 and 5 (REF)
// Pass 4 (tip to base): F_df = own + children (Phi F), r = f - ~H F_df, then
// the first M^-1 pass on r: z2 = children Phi z2+, eps2 = r - ~H z2,
// z2+ = z2 + G eps2 (RigidBodyNodeSpec.cpp:483-515).
struct Carry4 { DF3 Fw, Fv; V3<float> zw, zv; };

template <int N, int SS>
__device__ __forceinline__ void pass4BodyImpl(const DevTables& T, int body0, int row, int n,
                                              const Scr<float, SS>& S, bool haveCarry, Carry4& cy) {
    const int info = T.info[row];
    const int rec = T.srec[row];
    const int eH = rec + kRecH;
    const int ef = eH + 6 * N, eDI = ef + N, eG = eDI + N * N, eEps = eG + 6 * N;
    const int eF = rec + kRecFdf;
    DF3 Fw{DF{S(eF + 0), S(eF + 1)}, DF{S(eF + 2), S(eF + 3)}, DF{S(eF + 4), S(eF + 5)}};
    DF3 Fv{DF{S(eF + 6), S(eF + 7)}, DF{S(eF + 8), S(eF + 9)}, DF{S(eF + 10), S(eF + 11)}};
    V3<float> zw = z3<float>(), zv = z3<float>();
    if (info & F_MEMACC) { zw = ld3(S, rec + kRecZ2acc); zv = ld3(S, rec + kRecZ2acc + 3); }
    if (haveCarry) {
        Fw = Fw + cy.Fw; Fv = Fv + cy.Fv;
        zw = zw + cy.zw; zv = zv + cy.zv;
    }
    V3<float> zpw = zw, zpv = zv;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        if (j < n) {
            const V3<float> hw = ld3(S, eH + 6 * j), hv = ld3(S, eH + 6 * j + 3);
            const DF tau = dotFD(hw, Fw) + dotFD(hv, Fv);
            const DF rr = dfq(S(ef + j)) - tau;
            const float r = __fadd_rn(rr.hi, rr.lo);
            const float e2 = r - (dot(hw, zw) + dot(hv, zv));
            S(eEps + j) = e2;
            zpw = axpy(zpw, e2, ld3(S, eG + 6 * j));
            zpv = axpy(zpv, e2, ld3(S, eG + 6 * j + 3));
        }
    }
    const int parent = T.parent[row];
    if (parent >= 0) {
        const V3<float> l = ld3(S, rec + kRecL);
        cy.Fw = Fw + crossFD(l, Fv);
        cy.Fv = Fv;
        cy.zw = zpw + cross(l, zpv);
        cy.zv = zpv;
        if (!(info & F_CARRY)) {
            const int pr = T.srec[body0 + parent];
            const int pF = pr + kRecFdf;
            DF3 a{DF{S(pF + 0), S(pF + 1)}, DF{S(pF + 2), S(pF + 3)}, DF{S(pF + 4), S(pF + 5)}};
            DF3 b{DF{S(pF + 6), S(pF + 7)}, DF{S(pF + 8), S(pF + 9)}, DF{S(pF + 10), S(pF + 11)}};
            a = a + cy.Fw;
            b = b + cy.Fv;
            S(pF + 0) = a.x.hi; S(pF + 1) = a.x.lo; S(pF + 2) = a.y.hi; S(pF + 3) = a.y.lo;
            S(pF + 4) = a.z.hi; S(pF + 5) = a.z.lo;
            S(pF + 6) = b.x.hi; S(pF + 7) = b.x.lo; S(pF + 8) = b.y.hi; S(pF + 9) = b.y.lo;
            S(pF + 10) = b.z.hi; S(pF + 11) = b.z.lo;
            const int pz = pr + kRecZ2acc;
            S(pz + 0) += cy.zw.x; S(pz + 1) += cy.zw.y; S(pz + 2) += cy.zw.z;
            S(pz + 3) += cy.zv.x; S(pz + 4) += cy.zv.y; S(pz + 5) += cy.zv.z;
        }
    }
}

template <int SS>
__device__ __noinline__ void pass4Free(const DevTables& T, int body0, int row, const Scr<float, SS>& S,
                                       bool haveCarry, Carry4& cy) {
    pass4BodyImpl<6, SS>(T, body0, row, 6, S, haveCarry, cy);
}

// Pass 5 (base to tip): delta = DI eps2 - ~G A+, A = A+ + H delta; the result
// udot = udot0 + delta (RigidBodyNodeSpec.cpp:521-552).
template <int N, int SS, class Out>
__device__ __forceinline__ void pass5BodyImpl(const DevTables& T, int body0, int row, int n,
                                              const Scr<float, SS>& S, Out& out, Carry3T<float>& cy) {
    const int info = T.info[row];
    const int rec = T.srec[row];
    const int eH = rec + kRecH;
    const int ef = eH + 6 * N, eDI = ef + N, eG = eDI + N * N, eEps = eG + 6 * N, eU0 = eEps + N;
    const int parent = T.parent[row];
    V3<float> Apw = z3<float>(), Apv = z3<float>();
    if (parent >= 0) {
        V3<float> w, v;
        if (info & F_CARRY) { w = cy.Aw; v = cy.Av; }
        else {
            const int pe = T.srec[body0 + parent];
            w = ld3(S, pe); v = ld3(S, pe + 3);
        }
        const V3<float> l = ld3(S, rec + kRecL);
        Apw = w;
        Apv = v + cross(w, l);
    }
    float eps[N];
#pragma unroll
    for (int j = 0; j < N; ++j) eps[j] = j < n ? S(eEps + j) : 0.f;
    V3<float> Aw = Apw, Av = Apv;
    const int uo = T.uoff[row];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        if (i < n) {
            float s = 0.f;
#pragma unroll
            for (int k = 0; k < N; ++k)
                if (k < n) s = s + S(eDI + i * N + k) * eps[k];
            const float d = s - (dot(ld3(S, eG + 6 * i), Apw) + dot(ld3(S, eG + 6 * i + 3), Apv));
            out.udot(uo + i, S(eU0 + i) + d);
            Aw = axpy(Aw, d, ld3(S, eH + 6 * i));
            Av = axpy(Av, d, ld3(S, eH + 6 * i + 3));
        }
    }
    cy.Aw = Aw;
    cy.Av = Av;
    if (info & F_MEMCHILD) { st3(S, rec, Aw); st3(S, rec + 3, Av); }
}

template <int SS, class Out>
__device__ __noinline__ void pass5Free(const DevTables& T, int body0, int row, const Scr<float, SS>& S, Out& out,
                                       Carry3T<float>& cy) {
    pass5BodyImpl<6, SS>(T, body0, row, 6, S, out, cy);
}

// One RHS evaluation of one instance. Returns SBG_INST_* bits. REF turns on
// the refinement step of the mixed form (R = float only).
template <class R, int NM, int SS, bool REF, class Src, class Out>
__device__ __noinline__ int rhsInstance(const DevTables& T, int inst, const Scr<R, SS>& S, const Src& src,
                                        Out& out) {
    static_assert(!REF || std::is_same<R, float>::value, "refinement is for the FP32 recursion");
    const int body0 = T.ibody[inst], nb = T.inb[inst];
    const V3<R> g = mk3(R(T.grav[3 * inst]), R(T.grav[3 * inst + 1]), R(T.grav[3 * inst + 2]));
    const R* PT = paramTable<R>(T);
    pass1<R, NM, SS>(T, body0, nb, S, src, out, g);
    bool ok = true;
    {
        Carry2<R> cy;
        bool have = false;
        for (int lb = nb - 1; lb >= 0; --lb) {
            const int row = body0 + lb;
            const int info = T.info[row];
            const int n = (info >> 4) & 15;
            const R m = PT[(int64_t)row * kParamStride];
            if (n == 6) ok &= pass2Free<R, SS>(T, body0, row, S, m, have, cy);
            else ok &= pass2BodyImpl<R, NM, SS>(T, body0, row, n, S, m, have, cy);
            have = (info & F_CARRY) != 0;
        }
    }
    {
        Carry3T<R> cy{z3<R>(), z3<R>()};
        DF3 cDw{}, cDv{};
        for (int lb = 0; lb < nb; ++lb) {
            const int row = body0 + lb;
            const int n = (T.info[row] >> 4) & 15;
            if (n == 6) pass3Free<R, SS, REF>(T, body0, row, S, out, cy, cDw, cDv);
            else pass3BodyImpl<R, NM, SS, REF>(T, body0, row, n, S, out, cy, cDw, cDv);
        }
    }
    if constexpr (REF) {
        {
            Carry4 cy;
            bool have = false;
            for (int lb = nb - 1; lb >= 0; --lb) {
                const int row = body0 + lb;
                const int info = T.info[row];
                const int n = (info >> 4) & 15;
                if (n == 6) pass4Free<SS>(T, body0, row, S, have, cy);
                else pass4BodyImpl<NM, SS>(T, body0, row, n, S, have, cy);
                have = (info & F_CARRY) != 0;
            }
        }
        {
            Carry3T<float> cy{z3<float>(), z3<float>()};
            for (int lb = 0; lb < nb; ++lb) {
                const int row = body0 + lb;
                const int n = (T.info[row] >> 4) & 15;
                if (n == 6) pass5Free<SS>(T, body0, row, S, out, cy);
                else pass5BodyImpl<NM, SS>(T, body0, row, n, S, out, cy);
            }
        }
    }
    return ok ? 0 : SBG_INST_SINGULAR_D;
}

template <class R, int SS> __device__ __forceinline__ Scr<R, SS> scratchOf(const DevTables& T, R* scratch, int inst) {
    return Scr<R, SS>{scratch + T.sbase[inst]};
}

// ------------------------------------------------------------ realize kernel
struct YSrc {
    static constexpr bool kMInv = false;
    const double* y;
    int64_t base, stride;
    int nq;
    __device__ __forceinline__ double q(int k) const { return y[base + (int64_t)k * stride]; }
    __device__ __forceinline__ double u(int k) const { return y[base + (int64_t)(nq + k) * stride]; }
};
struct YdOut {
    double* yd;
    int64_t base, stride;
    int nq;
    bool finite = true;
    template <class R> __device__ __forceinline__ void qdot(int k, R v) {
        yd[base + (int64_t)k * stride] = double(v);
        finite &= isfinite(v);
    }
    template <class R> __device__ __forceinline__ void udot(int k, R v) {
        yd[base + (int64_t)(nq + k) * stride] = double(v);
        finite &= isfinite(v);
    }
};

template <class R, int NM, int SS, bool REF, int MINB = 1>
__global__ void __launch_bounds__(128, MINB) realizeKernel(DevTables T, const double* __restrict__ y,
                                                     double* __restrict__ ydot, R* __restrict__ scratch,
                                                     int32_t* __restrict__ status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T.ninst) return;
    const int inst = T.order[t];
    const Scr<R, SS> S = scratchOf<R, SS>(T, scratch, inst);
    YSrc src{y, T.ybase[inst], T.ystride[inst], T.inq[inst]};
    YdOut out{ydot, T.ybase[inst], T.ystride[inst], T.inq[inst]};
    int st = rhsInstance<R, NM, SS, REF>(T, inst, S, src, out);
    if (!out.finite) st |= SBG_INST_NONFINITE;
    status[inst] = st;
}

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

template <class R, int NM, int SS>
__global__ void __launch_bounds__(128) minvKernel(DevTables T, const double* __restrict__ y,
                                                  const double* __restrict__ f, double* __restrict__ out,
                                                  R* __restrict__ scratch, int32_t* __restrict__ status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T.ninst) return;
    const int inst = T.order[t];
    const Scr<R, SS> S = scratchOf<R, SS>(T, scratch, inst);
    MInvSrc src{y, f, T.ybase[inst], T.ystride[inst], T.inq[inst]};
    MInvOut o{out, T.ybase[inst], T.ystride[inst], T.inq[inst]};
    int st = rhsInstance<R, NM, SS, false>(T, inst, S, src, o);
    if (!o.finite) st |= SBG_INST_NONFINITE;
    status[inst] = st;
}

// ---------------------------------------------------- RK Merson persistent
// Stage input y0 + c * combo(f) formed on the fly while pass 1 loads q/u.
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
    template <class R> __device__ __forceinline__ void qdot(int k, R v) { f[base + (int64_t)k * stride] = F(v); finite &= isfinite(v); }
    template <class R> __device__ __forceinline__ void udot(int k, R v) { f[base + (int64_t)(nq + k) * stride] = F(v); finite &= isfinite(v); }
};

template <class R, int NM, int SS, bool REF, int MINB = 1>
__global__ void __launch_bounds__(128, MINB) rkMersonKernel(DevTables T, double* __restrict__ y, double* __restrict__ time,
                                                      R* __restrict__ fbuf, int64_t fplane, R* __restrict__ scratch,
                                                      int32_t* __restrict__ status, double h, int nsteps,
                                                      double accuracy, double consTol, int projectEveryStep) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T.ninst) return;
    const int inst = T.order[t];
    const Scr<R, SS> S = scratchOf<R, SS>(T, scratch, inst);
    const int64_t base = T.ybase[inst], stride = T.ystride[inst];
    const int nq = T.inq[inst], nu = T.inu[inst];
    const int body0 = T.ibody[inst], nb = T.inb[inst];
    R* f0 = fbuf;
    R* fA = fbuf + fplane;
    R* fB = fbuf + 2 * fplane;
    R* fC = fbuf + 3 * fplane;
    int st = status[inst];
    double tc = time[inst];
    const double projLimit = fmax(2 * consTol, sqrt(consTol));
    for (int step = 0; step < nsteps; ++step) {
        const double t1 = tc + h;
        const double hs = t1 - tc;
        // f0 = f(y0)
        {
            StageSrc<R> src{y, f0, fA, fB, base, stride, nq, 0, 0.0};
            FOut<R> o{f0, base, stride, nq};
            st |= rhsInstance<R, NM, SS, REF>(T, inst, S, src, o);
            if (!o.finite) st |= SBG_INST_NONFINITE;
        }
        {   // f1 -> fA
            StageSrc<R> src{y, f0, fA, fB, base, stride, nq, 1, hs / 3};
            FOut<R> o{fA, base, stride, nq};
            st |= rhsInstance<R, NM, SS, REF>(T, inst, S, src, o);
        }
        {   // f2 -> fB   (input uses f1 in fA)
            StageSrc<R> src{y, f0, fA, fB, base, stride, nq, 2, hs / 6};
            FOut<R> o{fB, base, stride, nq};
            st |= rhsInstance<R, NM, SS, REF>(T, inst, S, src, o);
        }
        {   // f3 -> fC   (input uses f2 in fB)
            StageSrc<R> src{y, f0, fB, fB, base, stride, nq, 3, hs / 8};
            FOut<R> o{fC, base, stride, nq};
            st |= rhsInstance<R, NM, SS, REF>(T, inst, S, src, o);
        }
        {   // f4 -> fA   (ysave input uses f2 in fB, f3 in fC)
            StageSrc<R> src{y, f0, fB, fC, base, stride, nq, 4, hs / 2};
            FOut<R> o{fA, base, stride, nq};
            st |= rhsInstance<R, NM, SS, REF>(T, inst, S, src, o);
        }
        // y1 = y0 + h/6 (f0 + 4 f3 + f4); yerr = 0.2 |y1 - ysave|; error norm
        // (RungeKuttaMersonIntegrator.cpp:124-139, IntegratorRep.h:454-523).
        const double h6 = hs / 6, h2 = hs / 2;
        double sq = 0, su = 0, squat = 0;
        int nquat = 0;
        bool fin = true;
        for (int lb = 0; lb < nb; ++lb) {
            const int row = body0 + lb;
            const int type = T.info[row] & 15;
            const int qo = T.qoff[row];
            const int nqb = type == T_BALL ? 4 : (type == T_FREE ? 7 : ((T.info[row] >> 4) & 15));
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
            if (type == T_BALL || type == T_FREE) {
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
                ++nquat;
            } else {
                for (int j = 0; j < nqb; ++j) sq += dq[j] * dq[j];
            }
        }
        for (int k = 0; k < nu; ++k) {
            const int64_t e = base + (int64_t)(nq + k) * stride;
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
        if (!fin) st |= SBG_INST_NONFINITE;
        const double qn = nq ? sqrt(sq / nq) : 0.0, un = nu ? sqrt(su / nu) : 0.0;
        const double errNorm = qn >= un ? qn : un;
        // projection gate and quaternion normalization
        // (AbstractIntegratorRep.cpp:158-190, SimbodyMatterSubsystemRep.cpp:4096-4183)
        if (errNorm <= 16 * accuracy && nquat > 0) {
            const double quatNorm = sqrt(squat / nquat);
            if (quatNorm > projLimit) st |= SBG_INST_PROJECTION_FAILED;
            else if (quatNorm > consTol || projectEveryStep) {
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
        }
        tc = t1;
    }
    time[inst] = tc;
    status[inst] = st;
}

}  // namespace sbg
