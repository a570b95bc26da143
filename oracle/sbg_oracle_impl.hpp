// sbg_oracle_impl.hpp -- templated bodies of the oracle recursions.
// TEST INFRASTRUCTURE ONLY (see sbg_oracle.hpp).
#pragma once
#include "sbg_oracle.hpp"

namespace sbgo {

template <class R> inline M33<R> loadR(const double* r) {
    M33<R> A;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) A(i, j) = R(r[3 * i + j]);
    return A;
}
template <class R> inline V3<R> loadV(const double* p) { return v3<R>(R(p[0]), R(p[1]), R(p[2])); }

// ------------------------------------------------------------- D inverse
// Mat<n,n>::invert(): closed forms for n<=3 (SmallMatrixMixed.h:897-960), LU
// with partial pivoting (LAPACK getrf/getri, :859-894) for larger n.
template <class R> inline bool invertD(int n, const R* D, R* DI) {
    if (n == 1) { DI[0] = R(1) / D[0]; return true; }
    if (n == 2) {
        const R d = D[0] * D[3] - D[1] * D[2];
        const R ood = R(1) / d;
        DI[0] = ood * D[3]; DI[1] = -ood * D[1]; DI[2] = -ood * D[2]; DI[3] = ood * D[0];
        return true;
    }
    if (n == 3) {
        auto m = [&](int i, int j) { return D[3 * i + j]; };
        const R d00 = m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1), nd01 = m(1, 2) * m(2, 0) - m(1, 0) * m(2, 2),
                d02 = m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0);
        const R d = m(0, 0) * d00 + m(0, 1) * nd01 + m(0, 2) * d02;
        const R ood = R(1) / d;
        const R nd10 = m(0, 2) * m(2, 1) - m(0, 1) * m(2, 2), d11 = m(0, 0) * m(2, 2) - m(0, 2) * m(2, 0),
                nd12 = m(0, 1) * m(2, 0) - m(0, 0) * m(2, 1), d20 = m(0, 1) * m(1, 2) - m(0, 2) * m(1, 1),
                nd21 = m(0, 2) * m(1, 0) - m(0, 0) * m(1, 2), d22 = m(0, 0) * m(1, 1) - m(0, 1) * m(1, 0);
        DI[0] = ood * d00;  DI[1] = ood * nd10; DI[2] = ood * d20;
        DI[3] = ood * nd01; DI[4] = ood * d11;  DI[5] = ood * nd21;
        DI[6] = ood * d02;  DI[7] = ood * nd12; DI[8] = ood * d22;
        return true;
    }
    // General n: LU with partial pivoting, then solve A X = I column by column.
    R A[36];
    int piv[6];
    for (int i = 0; i < n * n; ++i) A[i] = D[i];
    for (int j = 0; j < n; ++j) {
        int p = j;
        R best = abs(A[j * n + j]);
        for (int i = j + 1; i < n; ++i) {
            const R v = abs(A[i * n + j]);
            if (v > best) { best = v; p = i; }
        }
        piv[j] = p;
        if (A[p * n + j] == R(0)) return false;  // getrf info > 0: singular
        if (p != j)
            for (int k = 0; k < n; ++k) std::swap(A[j * n + k], A[p * n + k]);
        const R r = R(1) / A[j * n + j];
        for (int i = j + 1; i < n; ++i) A[i * n + j] = A[i * n + j] * r;
        for (int i = j + 1; i < n; ++i)
            for (int k = j + 1; k < n; ++k) A[i * n + k] = A[i * n + k] - A[i * n + j] * A[j * n + k];
    }
    for (int c = 0; c < n; ++c) {
        R x[6];
        for (int i = 0; i < n; ++i) x[i] = R(i == c ? 1 : 0);
        for (int j = 0; j < n; ++j)
            if (piv[j] != j) std::swap(x[j], x[piv[j]]);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < i; ++k) x[i] = x[i] - A[i * n + k] * x[k];
        for (int i = n - 1; i >= 0; --i) {
            for (int k = i + 1; k < n; ++k) x[i] = x[i] - A[i * n + k] * x[k];
            x[i] = x[i] / A[i * n + i];
        }
        for (int i = 0; i < n; ++i) DI[i * n + c] = x[i];
    }
    return true;
}

// Body-fixed X-Y-Z angles q[0..2]: cos, sin and 1/cos(q1) into the cache
// (performQPrecalculations, RigidBodyNodeSpec_Gimbal.h) and R_FM
// (Rotation::setRotationToBodyFixedXYZ(c, s), Rotation.h:342-349).
template <class R> inline void bodyFixedXYZ(BodyCache<R>& c, const R* q) {
    const R cy = cos(q[1]);
    c.ca[0] = cos(q[0]); c.ca[1] = cy; c.ca[2] = cos(q[2]);
    c.sa[0] = sin(q[0]); c.sa[1] = sin(q[1]); c.sa[2] = sin(q[2]);
    c.ooc1 = R(1) / cy;
    const R* cc = c.ca;
    const R* ss = c.sa;
    const R s0s1 = ss[0] * ss[1], s2c0 = ss[2] * cc[0], c0c2 = cc[0] * cc[2], nc1 = -cc[1];
    c.R_FM(0, 0) = cc[1] * cc[2];           c.R_FM(0, 1) = ss[2] * nc1;           c.R_FM(0, 2) = ss[1];
    c.R_FM(1, 0) = s2c0 + s0s1 * cc[2];     c.R_FM(1, 1) = c0c2 - s0s1 * ss[2];   c.R_FM(1, 2) = ss[0] * nc1;
    c.R_FM(2, 0) = ss[0] * ss[2] - ss[1] * c0c2; c.R_FM(2, 1) = ss[0] * cc[2] + ss[1] * s2c0; c.R_FM(2, 2) = cc[0] * cc[1];
}

// Rotation::multiplyByBodyXYZ_N_P (Rotation.h:395-406): qdot of body-fixed
// X-Y-Z angles from the angular velocity w in the parent frame.
template <class R> inline void bodyXYZ_N_P(const R* cc, const R* ss, R ooc1, const R* w, R* qd) {
    const R s0 = ss[0], c0 = cc[0], s1 = ss[1];
    const R t = (s0 * w[1] - c0 * w[2]) * ooc1;
    qd[0] = w[0] + t * s1;
    qd[1] = c0 * w[1] + s0 * w[2];
    qd[2] = -t;
}

// ------------------------------------------------------- position stage
// RigidBodyNodeSpec::realizePosition (RigidBodyNodeSpec.h:229-288) driven
// base-to-tip by realizePositionKinematics (SimbodyMatterSubsystemRep.cpp:1112-1144).
template <class R> void realizePosition(const Topology& t, const R* q, Work<R>& w) {
    BodyCache<R>& g = w.c[0];
    g.R_GB = ident33<R>(); g.p_GB = zero3<R>();
    g.Vw = zero3<R>(); g.Vv = zero3<R>();
    g.Aw = zero3<R>(); g.Av = zero3<R>();
    int quat = 0;
    for (const auto& lev : t.levels)
        for (int bi : lev) {
            const Body& b = t.b[bi];
            BodyCache<R>& c = w.c[bi];
            const BodyCache<R>& pc = w.c[b.parent];
            const R* qb = q + b.qoff;
            // performQPrecalculations + calcX_FM (mobilizer specific)
            for (int j = 0; j < 6; ++j) { c.HFw[j] = zero3<R>(); c.HFv[j] = zero3<R>(); }
            c.p_FM = zero3<R>();
            switch (b.type) {
            case SBG_WELD:  // RigidBodyNode_Weld.cpp:389-396: X_FM = identity, no q
                c.R_FM = ident33<R>();
                break;
            case SBG_SCREW: {  // RigidBodyNodeSpec_Screw.h:121-140: about Fz, p_FM = (0, 0, q pitch)
                const R cq = cos(qb[0]), sq = sin(qb[0]);
                c.R_FM = ident33<R>();
                c.R_FM(0, 0) = cq; c.R_FM(1, 1) = cq; c.R_FM(1, 0) = sq; c.R_FM(0, 1) = -sq;
                c.p_FM = v3<R>(R(0), R(0), qb[0] * R(b.pitch));
                c.HFw[0] = v3<R>(R(0), R(0), R(1));
                c.HFv[0] = v3<R>(R(0), R(0), R(b.pitch));
                break;
            }
            case SBG_PIN: {  // RigidBodyNodeSpec_Pin.h:103-131; Rotation.h:210-213
                const R cq = cos(qb[0]), sq = sin(qb[0]);
                c.R_FM = ident33<R>();
                c.R_FM(0, 0) = cq; c.R_FM(1, 1) = cq; c.R_FM(1, 0) = sq; c.R_FM(0, 1) = -sq;
                c.HFw[0] = v3<R>(R(0), R(0), R(1));
                break;
            }
            case SBG_SLIDER:  // RigidBodyNodeSpec_Slider.h:100-128
                c.R_FM = ident33<R>();
                c.p_FM = v3<R>(qb[0], R(0), R(0));
                c.HFv[0] = v3<R>(R(1), R(0), R(0));
                break;
            case SBG_UNIVERSAL: {  // RigidBodyNodeSpec_Universal.h:124-166; Rotation.cpp:241-264
                const R c1 = cos(qb[0]), s1 = sin(qb[0]), c2 = cos(qb[1]), s2 = sin(qb[1]);
                c.R_FM(0, 0) = c2;       c.R_FM(0, 1) = R(0); c.R_FM(0, 2) = s2;
                c.R_FM(1, 0) = s2 * s1;  c.R_FM(1, 1) = c1;   c.R_FM(1, 2) = -s1 * c2;
                c.R_FM(2, 0) = -s2 * c1; c.R_FM(2, 1) = s1;   c.R_FM(2, 2) = c1 * c2;
                c.HFw[0] = v3<R>(R(1), R(0), R(0));
                c.HFw[1] = col(c.R_FM, 1);
                break;
            }
            case SBG_BALL:
            case SBG_FREE:
                if (b.euler) {  // RigidBodyNodeSpec_Ball.h:118-127, _Free.h Euler branch
                    bodyFixedXYZ(c, qb);
                    for (int j = 0; j < 3; ++j) { V3<R> e = zero3<R>(); e[j] = R(1); c.HFw[j] = e; }
                    if (b.type == SBG_FREE) {
                        c.p_FM = v3<R>(qb[3], qb[4], qb[5]);
                        for (int j = 0; j < 3; ++j) { V3<R> e = zero3<R>(); e[j] = R(1); c.HFv[3 + j] = e; }
                    }
                    break;
                }
                {  // RigidBodyNodeSpec_Ball.h:134-180, _Free.h:142-188
                const R len = sqrt(qb[0] * qb[0] + qb[1] * qb[1] + qb[2] * qb[2] + qb[3] * qb[3]);
                w.qerr[quat++] = len - R(1);
                c.ooNorm = R(1) / len;
                const R e0 = qb[0] * c.ooNorm, e1 = qb[1] * c.ooNorm, e2 = qb[2] * c.ooNorm, e3 = qb[3] * c.ooNorm;
                // Rotation::setRotationFromQuaternion (Rotation.cpp:600-610)
                const R q00 = e0 * e0, q11 = e1 * e1, q22 = e2 * e2, q33 = e3 * e3;
                const R q01 = e0 * e1, q02 = e0 * e2, q03 = e0 * e3, q12 = e1 * e2, q13 = e1 * e3, q23 = e2 * e3;
                const R q00mq11 = q00 - q11, q22mq33 = q22 - q33;
                c.R_FM(0, 0) = q00 + q11 - q22 - q33; c.R_FM(0, 1) = R(2) * (q12 - q03); c.R_FM(0, 2) = R(2) * (q13 + q02);
                c.R_FM(1, 0) = R(2) * (q12 + q03); c.R_FM(1, 1) = q00mq11 + q22mq33; c.R_FM(1, 2) = R(2) * (q23 - q01);
                c.R_FM(2, 0) = R(2) * (q13 - q02); c.R_FM(2, 1) = R(2) * (q23 + q01); c.R_FM(2, 2) = q00mq11 - q22mq33;
                for (int j = 0; j < 3; ++j) { V3<R> e = zero3<R>(); e[j] = R(1); c.HFw[j] = e; }
                if (b.type == SBG_FREE) {
                    c.p_FM = v3<R>(qb[4], qb[5], qb[6]);
                    for (int j = 0; j < 3; ++j) { V3<R> e = zero3<R>(); e[j] = R(1); c.HFv[3 + j] = e; }
                }
                break;
                }
            case SBG_GIMBAL:
            case SBG_BUSHING:  // RigidBodyNodeSpec_Gimbal.h, _Bushing.h: calcX_FM, H_FM columns
                bodyFixedXYZ(c, qb);
                c.HFw[0] = v3<R>(R(1), R(0), R(0));
                c.HFw[1] = v3<R>(R(0), c.ca[0], c.sa[0]);
                c.HFw[2] = v3<R>(c.sa[1], -c.sa[0] * c.ca[1], c.ca[0] * c.ca[1]);
                if (b.type == SBG_BUSHING) {
                    c.p_FM = v3<R>(qb[3], qb[4], qb[5]);
                    for (int j = 0; j < 3; ++j) { V3<R> e = zero3<R>(); e[j] = R(1); c.HFv[3 + j] = e; }
                }
                break;
            case SBG_TRANSLATION:  // RigidBodyNodeSpec_Translation.h
                c.R_FM = ident33<R>();
                c.p_FM = v3<R>(qb[0], qb[1], qb[2]);
                for (int j = 0; j < 3; ++j) { V3<R> e = zero3<R>(); e[j] = R(1); c.HFv[j] = e; }
                break;
            case SBG_CYLINDER:  // RigidBodyNodeSpec_Cylinder.h
            case SBG_PLANAR: {  // RigidBodyNodeSpec_Planar.h
                const R cq = cos(qb[0]), sq = sin(qb[0]);
                c.R_FM = ident33<R>();
                c.R_FM(0, 0) = cq; c.R_FM(1, 1) = cq; c.R_FM(1, 0) = sq; c.R_FM(0, 1) = -sq;
                c.HFw[0] = v3<R>(R(0), R(0), R(1));
                if (b.type == SBG_CYLINDER) {
                    c.p_FM = v3<R>(R(0), R(0), qb[1]);
                    c.HFv[1] = v3<R>(R(0), R(0), R(1));
                } else {
                    c.p_FM = v3<R>(qb[1], qb[2], R(0));
                    c.HFv[1] = v3<R>(R(1), R(0), R(0));
                    c.HFv[2] = v3<R>(R(0), R(1), R(0));
                }
                break;
            }
            }
            // calcBodyTransforms (RigidBodyNodeSpec.h:554-569)
            const M33<R> RMB = loadR<R>(b.RMB), RPF = loadR<R>(b.RPF);
            const V3<R> pMB = loadV<R>(b.pMB), pPF = loadV<R>(b.pPF);
            const M33<R> R_FB = c.R_FM * RMB;
            const V3<R> p_FB = c.R_FM * pMB + c.p_FM;
            const M33<R> R_PB = RPF * R_FB;
            c.p_PB = RPF * p_FB + pPF;
            c.R_GB = pc.R_GB * R_PB;
            c.p_GB = pc.R_GB * c.p_PB + pc.p_GB;
            // calcParentToChildVelocityJacobianInGround (RigidBodyNodeSpec.cpp:44-74)
            const M33<R> R_GF = pc.R_GB * RPF;
            const V3<R> r_MB_F = c.R_FM * pMB;
            for (int j = 0; j < b.nu; ++j) {
                c.Hw[j] = R_GF * c.HFw[j];
                c.Hv[j] = R_GF * (c.HFv[j] - cross(r_MB_F, c.HFw[j]));
            }
            // calcJointIndependentKinematicsPos (RigidBodyNode.cpp:54-84)
            c.l = pc.R_GB * c.p_PB;
            c.m = R(b.mass);
            c.Gi = reexpress(c.R_GB, s33<R>(R(b.G[0]), R(b.G[3]), R(b.G[1]), R(b.G[4]), R(b.G[5]), R(b.G[2])));
            c.pc = c.R_GB * loadV<R>(b.com);
        }
}

// ------------------------------------------------------- velocity stage
// RigidBodyNodeSpec::realizeVelocity (RigidBodyNodeSpec.h:305-333) and
// calcJointIndependentKinematicsVel (RigidBodyNode.cpp:98-174), base to tip.
// qdot=N(q)u (RigidBodyNodeSpec_Ball.h:187-214, Rotation.h:712-719, 990-992).
template <class R> void realizeVelocity(const Topology& t, const R* q, const R* u, Work<R>& w, R* qdot) {
    for (const auto& lev : t.levels)
        for (int bi : lev) {
            const Body& b = t.b[bi];
            BodyCache<R>& c = w.c[bi];
            const BodyCache<R>& pc = w.c[b.parent];
            const R* qb = q + b.qoff;
            const R* ub = u + b.uoff;
            if (qdot) {
                R* qd = qdot + b.qoff;
                if (b.euler) {  // RigidBodyNodeSpec_Ball.h:198-209: convertAngVelInParentToBodyXYZDot
                    bodyXYZ_N_P(c.ca, c.sa, c.ooc1, ub, qd);
                    if (b.type == SBG_FREE) { qd[3] = ub[3]; qd[4] = ub[4]; qd[5] = ub[5]; qd[6] = R(0); }
                    else qd[3] = R(0);  // the unused slot
                } else if (b.quat) {
                    // calcUnnormalizedNForQuaternion: e = q/2 (Rotation.h:712-719)
                    const R e0 = qb[0] / R(2), e1 = qb[1] / R(2), e2 = qb[2] / R(2), e3 = qb[3] / R(2);
                    const R ne1 = -e1, ne2 = -e2, ne3 = -e3;
                    qd[0] = ne1 * ub[0] + ne2 * ub[1] + ne3 * ub[2];
                    qd[1] = e0 * ub[0] + e3 * ub[1] + ne2 * ub[2];
                    qd[2] = ne3 * ub[0] + e0 * ub[1] + e1 * ub[2];
                    qd[3] = e2 * ub[0] + ne1 * ub[1] + e0 * ub[2];
                    if (b.type == SBG_FREE) { qd[4] = ub[3]; qd[5] = ub[4]; qd[6] = ub[5]; }
                } else {
                    for (int j = 0; j < b.nu; ++j) qd[j] = ub[j];
                }
            }
            // V_FM = H_FM*u, V_PB_G = H*u
            V3<R> VPw = zero3<R>(), VPv = zero3<R>();
            c.VFw = zero3<R>(); c.VFv = zero3<R>();
            for (int j = 0; j < b.nu; ++j) {
                c.VFw = c.VFw + ub[j] * c.HFw[j]; c.VFv = c.VFv + ub[j] * c.HFv[j];
                VPw = VPw + ub[j] * c.Hw[j];     VPv = VPv + ub[j] * c.Hv[j];
            }
            // HDot_FM: zero except Universal (RigidBodyNodeSpec_Universal.h:174-188)
            V3<R> HDFw[6], HDFv[6];
            for (int j = 0; j < 6; ++j) { HDFw[j] = zero3<R>(); HDFv[j] = zero3<R>(); }
            if (b.type == SBG_UNIVERSAL) HDFw[1] = cross(c.VFw, col(c.R_FM, 1));
            if (b.type == SBG_GIMBAL || b.type == SBG_BUSHING) {  // RigidBodyNodeSpec_Gimbal.h HDot_FM, qdot = u
                const R c0 = c.ca[0], c1 = c.ca[1], s0 = c.sa[0], s1 = c.sa[1];
                const R qd0 = ub[0], qd1 = ub[1];
                const R dc0 = -s0 * qd0, dc1 = -s1 * qd1;
                const R ds0 = c0 * qd0, ds1 = c1 * qd1;
                HDFw[1] = v3<R>(R(0), dc0, ds0);
                HDFw[2] = v3<R>(ds1, -ds0 * c1 - s0 * dc1, dc0 * c1 + c0 * dc1);
            }
            // calcParentToChildVelocityJacobianInGroundDot (RigidBodyNodeSpec.cpp:82-129)
            const M33<R> RPF = loadR<R>(b.RPF);
            const M33<R> R_GF = pc.R_GB * RPF;
            const V3<R> w_GF = pc.Vw;
            const V3<R> r_MB_F = c.R_FM * loadV<R>(b.pMB);
            const V3<R> wxr = cross(c.VFw, r_MB_F);
            V3<R> VDw = zero3<R>(), VDv = zero3<R>();
            for (int j = 0; j < b.nu; ++j) {
                const V3<R> hv = HDFv[j] - cross(r_MB_F, HDFw[j]) - cross(wxr, c.HFw[j]);
                c.HDw[j] = R_GF * HDFw[j] + cross(w_GF, c.Hw[j]);
                c.HDv[j] = R_GF * hv + cross(w_GF, c.Hv[j]);
                VDw = VDw + ub[j] * c.HDw[j]; VDv = VDv + ub[j] * c.HDv[j];
            }
            // V_GB = ~Phi*V_GP + V_PB_G (PhiMatrixTranspose*SpatialVec, SpatialAlgebra.h:757-763)
            c.Vw = pc.Vw + VPw;
            c.Vv = (pc.Vv + cross(pc.Vw, c.l)) + VPv;
            // gyroscopic force b
            const V3<R> wB = c.Vw;
            c.bw = c.m * cross(wB, c.Gi * wB);
            c.bv = c.m * cross(wB, cross(wB, c.pc));
            // mobilizer coriolis acceleration A
            c.aw = VDw;
            c.av = VDv + cross(pc.Vw, c.Vv - pc.Vv);
        }
}

// ------------------------------------------------------------ forces
// SmoothSphereHalfSpaceForceImpl::calcForce (SmoothSphereHalfSpaceForce.cpp:
// 252-336) with the half-space on Ground: the (moment, force) at the body
// origin of -force applied at the contact point, which is midway through the
// indentation. Needs the body's position and velocity.
template <class R> void contactBodyForce(const sbg_contact_desc& k, const BodyCache<R>& c, V3<R>& Mw, V3<R>& Fv) {
    using std::pow; using std::tanh; using std::min;
    const V3<R> nrm = v3<R>(R(k.halfspace[0]), R(k.halfspace[3]), R(k.halfspace[6]));  // frame x axis in Ground
    const V3<R> pH = v3<R>(R(k.halfspace[9]), R(k.halfspace[10]), R(k.halfspace[11]));
    const R radius = R(k.radius);
    const V3<R> centre = c.R_GB * loadV<R>(k.station) + c.p_GB;
    const V3<R> d = centre - pH;
    const R indentation = -(dot(d, -nrm) - radius);
    const V3<R> pc = centre + radius * nrm;
    const V3<R> pa = pc - (R(1) / R(2)) * indentation * nrm;
    const V3<R> station1 = mulT(c.R_GB, pa - c.p_GB);
    const V3<R> rG = c.R_GB * station1;
    const V3<R> v = c.Vv + cross(c.Vw, rG);  // findStationVelocityInGround; Ground's is zero
    const R vnormal = dot(v, nrm);
    const V3<R> vtangent = v - vnormal * nrm;
    const R kk = (R(1) / R(2)) * pow(R(k.stiffness), R(2) / R(3));
    const R fh_pos = (R(4) / R(3)) * kk * sqrt(radius * kk) * pow(sqrt(indentation * indentation + R(k.cf)), R(3) / R(2));
    const R fh_smooth = fh_pos * (R(1) / R(2) + (R(1) / R(2)) * tanh(R(k.bd) * indentation));
    const R cdis = R(k.dissipation);
    const R fhc_pos = fh_smooth * (R(1) + (R(3) / R(2)) * cdis * vnormal);
    const R fhc_smooth = fhc_pos * (R(1) / R(2) + (R(1) / R(2)) * tanh(R(k.bv) * (vnormal + (R(2) / (R(3) * cdis)))));
    V3<R> force = fhc_smooth * nrm;
    const R aux = dot(vtangent, vtangent) + R(k.cf);
    const R vslip = pow(aux, R(1) / R(2));
    const R vrel = vslip / R(k.transition_velocity);
    const R us = R(k.static_friction), ud = R(k.dynamic_friction), uv = R(k.viscous_friction);
    const R ff = fhc_smooth * (min(vrel, R(1)) * (ud + R(2) * (us - ud) / (R(1) + vrel * vrel)) + uv * vslip);
    force = force + (ff / vslip) * vtangent;
    // applyForceToBodyPoint(station1, -force)
    Mw = Mw + cross(rG, -force);
    Fv = Fv - force;
}

// Force::Gravity (Force_Gravity.cpp:531-556), the mobility forces
// (Force.cpp:339-351, 434-443) and the contact spheres, accumulated in
// element order.
template <class R> void calcForces(const Topology& t, const R* q, const R* u, Work<R>& w) {
    const V3<R> g = loadV<R>(t.gravity);
    for (int bi = 1; bi <= t.nb; ++bi) {
        BodyCache<R>& c = w.c[bi];
        const V3<R> F = c.m * g;
        c.Fw = cross(c.pc, F);
        c.Fv = F;
    }
    for (const auto& k : t.contacts) contactBodyForce(k, w.c[k.body], w.c[k.body].Fw, w.c[k.body].Fv);
    for (int i = 0; i < t.nu; ++i) w.f[i] = R(0);
    for (const auto& fe : t.forces) {
        const Body& b = t.b[fe.body];
        if (fe.kind == 0) {
            const R frc = -R(fe.coef) * (q[b.qoff + fe.which] - R(fe.q0));
            w.f[b.uoff + fe.which] = w.f[b.uoff + fe.which] + frc;
        } else {
            const R frc = -R(fe.coef) * u[b.uoff + fe.which];
            w.f[b.uoff + fe.which] = w.f[b.uoff + fe.which] + frc;
        }
    }
}

// ---------------------------------------------- articulated body inertias
// realizeArticulatedBodyInertiasInward (RigidBodyNodeSpec.cpp:249-325),
// tip to base (SimbodyMatterSubsystemRep.cpp:1217-1246). Returns false on a
// singular D.
template <class R> bool realizeABI(const Topology& t, Work<R>& w) {
    bool ok = true;
    for (int li = (int)t.levels.size() - 1; li >= 0; --li)
        for (int bi : t.levels[li]) {
            const Body& b = t.b[bi];
            BodyCache<R>& c = w.c[bi];
            ABI<R>& P = c.P;
            // ArticulatedInertia(Mk): M = m, J = m*G, F = crossMat(m*p) (MassProperties.h:1255-1256)
            P.M = s33<R>(c.m, R(0), c.m, R(0), R(0), c.m);
            P.J = c.m * c.Gi;
            const V3<R> mp = c.m * c.pc;
            P.F = zero33<R>();
            P.F(0, 1) = -mp[2]; P.F(0, 2) = mp[1]; P.F(1, 0) = mp[2]; P.F(1, 2) = -mp[0]; P.F(2, 0) = -mp[1]; P.F(2, 1) = mp[0];
            for (int ch : b.children) abiAdd(P, abiShift(w.c[ch].PP, w.c[ch].l));
            const int n = b.nu;
            V3<R> PHw[6], PHv[6];
            for (int j = 0; j < n; ++j) abiMul(P, c.Hw[j], c.Hv[j], PHw[j], PHv[j]);
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) c.D[i * n + j] = dot(c.Hw[i], PHw[j]) + dot(c.Hv[i], PHv[j]);
            if (!invertD(n, c.D, c.DI)) ok = false;
            for (int j = 0; j < n; ++j) {
                c.Gw[j] = zero3<R>(); c.Gv[j] = zero3<R>();
                for (int k = 0; k < n; ++k) {
                    c.Gw[j] = c.Gw[j] + c.DI[k * n + j] * PHw[k];
                    c.Gv[j] = c.Gv[j] + c.DI[k * n + j] * PHv[k];
                }
            }
            M33<R> mm = zero33<R>(), ms = zero33<R>(), in = zero33<R>();
            for (int r = 0; r < 3; ++r)
                for (int s = 0; s < 3; ++s)
                    for (int j = 0; j < n; ++j) {
                        mm(r, s) = mm(r, s) + c.Gw[j][r] * PHv[j][s];
                        ms(r, s) = ms(r, s) + c.Gv[j][r] * PHv[j][s];
                        in(r, s) = in(r, s) + c.Gw[j][r] * PHw[j][s];
                    }
            const S33<R> symMass = s33<R>(ms(0, 0), (ms(1, 0) + ms(0, 1)) / R(2), ms(1, 1),
                                          (ms(2, 0) + ms(0, 2)) / R(2), (ms(2, 1) + ms(1, 2)) / R(2), ms(2, 2));
            const S33<R> symIn = s33<R>(in(0, 0), (in(1, 0) + in(0, 1)) / R(2), in(1, 1),
                                        (in(2, 0) + in(0, 2)) / R(2), (in(2, 1) + in(1, 2)) / R(2), in(2, 2));
            c.PP.M = P.M - symMass;
            c.PP.J = P.J - symIn;
            c.PP.F = P.F - mm;
        }
    return ok;
}

// realizeArticulatedBodyVelocityCache (RigidBodyNode.cpp:201-213): P*a + b.
template <class R> void realizeABVelocity(const Topology& t, Work<R>& w) {
    for (int bi = 1; bi <= t.nb; ++bi) {
        BodyCache<R>& c = w.c[bi];
        V3<R> pw, pv;
        abiMul(c.P, c.aw, c.av, pw, pv);
        c.cw = pw + c.bw;
        c.cv = pv + c.bv;
    }
}

// calcTreeAccelerations (SimbodyMatterSubsystemRep.cpp:5258-5343):
// calcUDotPass1Inward (RigidBodyNodeSpec.cpp:355-400), calcUDotPass2Outward
// (:408-446). f = mobility forces; body forces from w (gravity).
template <class R> void calcTreeUDot(const Topology& t, Work<R>& w, const R* f, R* udot) {
    for (int li = (int)t.levels.size() - 1; li >= 0; --li)
        for (int bi : t.levels[li]) {
            const Body& b = t.b[bi];
            BodyCache<R>& c = w.c[bi];
            c.zw = c.cw - c.Fw;
            c.zv = c.cv - c.Fv;
            for (int ch : b.children) {  // Phi*v = (v0 + l % v1, v1)
                const BodyCache<R>& cc = w.c[ch];
                c.zw = c.zw + (cc.zpw + cross(cc.l, cc.zpv));
                c.zv = c.zv + cc.zpv;
            }
            const int n = b.nu;
            for (int j = 0; j < n; ++j) c.eps[j] = f[b.uoff + j] - (dot(c.Hw[j], c.zw) + dot(c.Hv[j], c.zv));
            c.zpw = c.zw; c.zpv = c.zv;
            V3<R> gw = zero3<R>(), gv = zero3<R>();
            for (int j = 0; j < n; ++j) { gw = gw + c.eps[j] * c.Gw[j]; gv = gv + c.eps[j] * c.Gv[j]; }
            c.zpw = c.zpw + gw; c.zpv = c.zpv + gv;
        }
    for (const auto& lev : t.levels)
        for (int bi : lev) {
            const Body& b = t.b[bi];
            BodyCache<R>& c = w.c[bi];
            const BodyCache<R>& pc = w.c[b.parent];
            // APlus = ~Phi*A_GP (SpatialAlgebra.h:757-763)
            const V3<R> Apw = pc.Aw;
            const V3<R> Apv = pc.Av + cross(pc.Aw, c.l);
            const int n = b.nu;
            R* ud = udot + b.uoff;
            for (int i = 0; i < n; ++i) {
                R s = R(0);
                for (int k = 0; k < n; ++k) s = s + c.DI[i * n + k] * c.eps[k];
                ud[i] = s - (dot(c.Gw[i], Apw) + dot(c.Gv[i], Apv));
            }
            V3<R> hw = zero3<R>(), hv = zero3<R>();
            for (int j = 0; j < n; ++j) { hw = hw + ud[j] * c.Hw[j]; hv = hv + ud[j] * c.Hv[j]; }
            c.Aw = (Apw + hw) + c.aw;
            c.Av = (Apv + hv) + c.av;
        }
}

// multiplyByMInv (SimbodyMatterSubsystemRep.cpp:5357-5400; RigidBodyNodeSpec.cpp:483-552).
// Needs realizePosition and realizeABI on the same q.
template <class R> void multiplyByMInv(const Topology& t, Work<R>& w, const R* f, R* out) {
    for (int li = (int)t.levels.size() - 1; li >= 0; --li)
        for (int bi : t.levels[li]) {
            const Body& b = t.b[bi];
            BodyCache<R>& c = w.c[bi];
            c.zw = zero3<R>(); c.zv = zero3<R>();
            for (int ch : b.children) {
                const BodyCache<R>& cc = w.c[ch];
                c.zw = c.zw + (cc.zpw + cross(cc.l, cc.zpv));
                c.zv = c.zv + cc.zpv;
            }
            const int n = b.nu;
            for (int j = 0; j < n; ++j) c.eps[j] = f[b.uoff + j] - (dot(c.Hw[j], c.zw) + dot(c.Hv[j], c.zv));
            c.zpw = c.zw; c.zpv = c.zv;
            V3<R> gw = zero3<R>(), gv = zero3<R>();
            for (int j = 0; j < n; ++j) { gw = gw + c.eps[j] * c.Gw[j]; gv = gv + c.eps[j] * c.Gv[j]; }
            c.zpw = c.zpw + gw; c.zpv = c.zpv + gv;
        }
    for (const auto& lev : t.levels)
        for (int bi : lev) {
            const Body& b = t.b[bi];
            BodyCache<R>& c = w.c[bi];
            const BodyCache<R>& pc = w.c[b.parent];
            const V3<R> Apw = pc.Aw;
            const V3<R> Apv = pc.Av + cross(pc.Aw, c.l);
            const int n = b.nu;
            R* ud = out + b.uoff;
            for (int i = 0; i < n; ++i) {
                R s = R(0);
                for (int k = 0; k < n; ++k) s = s + c.DI[i * n + k] * c.eps[k];
                ud[i] = s - (dot(c.Gw[i], Apw) + dot(c.Gv[i], Apv));
            }
            V3<R> hw = zero3<R>(), hv = zero3<R>();
            for (int j = 0; j < n; ++j) { hw = hw + ud[j] * c.Hw[j]; hv = hv + ud[j] * c.Hv[j]; }
            c.Aw = Apw + hw;
            c.Av = Apv + hv;
        }
}

// ------------------------------------------------------- tree operators
// Body accelerations from a u-like vector x, base to tip:
//   calcBodyAccelerationsFromUdotOutward (RigidBodyNodeSpec.cpp:566-582):
//     A = ~Phi A_parent + H x + a (coriolis = true, Stage::Velocity);
//   multiplyByMPass1Outward (:658-669), multiplyBySystemJacobian (:762-775):
//     A = ~Phi A_parent + H x (coriolis = false, Stage::Position).
template <class R> void accelerationsOutward(const Topology& t, Work<R>& w, const R* x, bool coriolis) {
    w.c[0].Aw = zero3<R>(); w.c[0].Av = zero3<R>();
    for (const auto& lev : t.levels)
        for (int bi : lev) {
            const Body& b = t.b[bi];
            BodyCache<R>& c = w.c[bi];
            const BodyCache<R>& pc = w.c[b.parent];
            const V3<R> Apw = pc.Aw;
            const V3<R> Apv = pc.Av + cross(pc.Aw, c.l);
            V3<R> hw = zero3<R>(), hv = zero3<R>();
            for (int j = 0; j < b.nu; ++j) { hw = hw + x[b.uoff + j] * c.Hw[j]; hv = hv + x[b.uoff + j] * c.Hv[j]; }
            c.Aw = Apw + hw;
            c.Av = Apv + hv;
            if (coriolis) { c.Aw = c.Aw + c.aw; c.Av = c.Av + c.av; }
        }
}

// Tip-to-base force sweep F = own + sum over children of Phi_c F_c, then
// tau = ~H F - f (f may be null). The body's own term is
//   kind 0  Mk A + b - F_applied   calcInverseDynamicsPass2Inward (RigidBodyNodeSpec.cpp:611-642)
//   kind 1  Mk A                   multiplyByMPass2Inward (:675-697)
//   kind 2  F_applied              multiplyBySystemJacobianTranspose (:795-818)
// with Mk A = m (G A_w + p x A_v, A_v - p x A_w) (MassProperties.h:1071-1072).
// F_applied holds 6 values (moment, force) per mobilized body in body order
// (may be null: zero).
template <class R> void forcesInward(const Topology& t, Work<R>& w, int kind, const R* F_applied, const R* f, R* tau) {
    for (int li = (int)t.levels.size() - 1; li >= 0; --li)
        for (int bi : t.levels[li]) {
            const Body& b = t.b[bi];
            BodyCache<R>& c = w.c[bi];
            V3<R> Fw = zero3<R>(), Fv = zero3<R>();
            if (kind != 2) {
                Fw = c.m * (c.Gi * c.Aw + cross(c.pc, c.Av));
                Fv = c.m * (c.Av - cross(c.pc, c.Aw));
                if (kind == 0) { Fw = Fw + c.bw; Fv = Fv + c.bv; }
            }
            if (F_applied) {
                const R* Fb = F_applied + 6 * (bi - 1);
                const V3<R> aw = v3<R>(Fb[0], Fb[1], Fb[2]), av = v3<R>(Fb[3], Fb[4], Fb[5]);
                if (kind == 2) { Fw = Fw + aw; Fv = Fv + av; }
                else { Fw = Fw - aw; Fv = Fv - av; }
            }
            for (int ch : b.children) {  // Phi*F = (F_w + l % F_v, F_v)
                const BodyCache<R>& cc = w.c[ch];
                Fw = Fw + (cc.zw + cross(cc.l, cc.zv));
                Fv = Fv + cc.zv;
            }
            c.zw = Fw; c.zv = Fv;
            for (int j = 0; j < b.nu; ++j) {
                R s = dot(c.Hw[j], Fw) + dot(c.Hv[j], Fv);
                if (f) s = s - f[b.uoff + j];
                tau[b.uoff + j] = s;
            }
        }
}

// Unit inertia of a unit point mass at p (UnitInertia::pointMassAt,
// MassProperties.h:866-867, element order of Inertia::pointMassAt :458-466).
template <class R> inline S33<R> pointMassUnit(const V3<R>& p) {
    const R xx = p[0] * p[0], yy = p[1] * p[1], zz = p[2] * p[2];
    return s33<R>(yy + zz, -p[0] * p[1], xx + zz, -p[0] * p[2], -p[1] * p[2], xx + yy);
}
// Spatial inertia (m, p = mass center from the origin, G = unit inertia about
// the origin), all in Ground.
template <class R> struct SpatialInertia {
    R m;
    V3<R> p;
    S33<R> G;
};
// SpatialInertia::shiftInPlace (MassProperties.h:1110-1116): origin OF -> OF + S.
template <class R> inline SpatialInertia<R> siShift(SpatialInertia<R> s, const V3<R>& S) {
    s.G = s.G - pointMassUnit(s.p);
    const V3<R> pNew = s.p - S;
    s.G = s.G + pointMassUnit(pNew);
    s.p = pNew;
    return s;
}
// SpatialInertia::operator+= (MassProperties.h:1037-1044).
template <class R> inline void siAdd(SpatialInertia<R>& a, const SpatialInertia<R>& b) {
    const R mtot = a.m + b.m, oom = R(1) / mtot;
    a.p = oom * (a.m * a.p + b.m * b.p);
    a.G = oom * (a.m * a.G + b.m * b.G);
    a.m = mtot;
}
// calcCompositeBodyInertias (SimbodyMatterSubsystemRep.cpp:5196-5205),
// RigidBodyNode::calcCompositeBodyInertiasInward (RigidBodyNode.cpp:232-243):
// R = Mk_G + sum over children of R_c.shift(-l_c). out: 10 values per body
// (m, p[3], G xx yy zz xy xz yz), body order.
template <class R> void compositeInertias(const Topology& t, const Work<R>& w, R* out) {
    std::vector<SpatialInertia<R>> Rb(t.nb + 1);
    for (int li = (int)t.levels.size() - 1; li >= 0; --li)
        for (int bi : t.levels[li]) {
            const BodyCache<R>& c = w.c[bi];
            SpatialInertia<R> r{c.m, c.pc, c.Gi};
            for (int ch : t.b[bi].children) siAdd(r, siShift(Rb[ch], -w.c[ch].l));
            Rb[bi] = r;
            R* o = out + 10 * (bi - 1);
            o[0] = r.m; o[1] = r.p[0]; o[2] = r.p[1]; o[3] = r.p[2];
            o[4] = r.G.xx; o[5] = r.G.yy; o[6] = r.G.zz; o[7] = r.G.yx; o[8] = r.G.zx; o[9] = r.G.zy;
        }
}

// Full realize(Stage::Acceleration) of one unconstrained instance:
// ydot = [qdot, udot]. Returns false on a singular D.
template <class R> bool realizeAcceleration(const Topology& t, const R* y, Work<R>& w, R* ydot) {
    const R* q = y;
    const R* u = y + t.nq;
    realizePosition(t, q, w);
    realizeVelocity(t, q, u, w, ydot);
    calcForces(t, q, u, w);
    const bool ok = realizeABI(t, w);
    realizeABVelocity(t, w);
    calcTreeUDot(t, w, w.f.data(), ydot + t.nq);
    return ok;
}

// qdotdot = N(q) udot + NDot(q, qdot) u per mobilizer, the quantity
// State::getQDotDot() returns at Stage::Acceleration
// (SimbodyMatterSubsystemRep.cpp calcQDotDot over the nodes):
//   Pin, Slider, Universal  q = angles/displacement with qdot = u, so
//                           qdotdot = udot (RigidBodyNodeSpec.h calcQDotDot)
//   Ball (quaternion)       convertAngVelDotToQuaternionDotDot(q, w_FM, b_FM)
//                           = N(q) b + (-1/4 |w|^2) q with the unnormalized q
//                           (RigidBodyNodeSpec_Ball.h:355-390,
//                           Rotation.h:1006-1013)
//   Free                    the quaternion part as Ball, then the translational
//                           udot (RigidBodyNodeSpec_Free.h:418-455)
template <class R> void calcQDotDot(const Topology& t, const R* y, const R* udot, R* qdotdot) {
    const R* q = y;
    const R* u = y + t.nq;
    for (int bi = 1; bi <= t.nb; ++bi) {
        const Body& b = t.b[bi];
        const R* qq = q + b.qoff;
        const R* ub = u + b.uoff;
        const R* bd = udot + b.uoff;
        R* o = qdotdot + b.qoff;
        if (b.euler) {
            // Rotation::convertAngAccInParentToBodyXYZDotDot (Rotation.h:1041-1060)
            // with qdot = N_P(q) w (RigidBodyNodeSpec_Ball.h:355-390 Euler branch)
            const R cy = cos(qq[1]);
            const R cc[2] = {cos(qq[0]), cy}, ss[2] = {sin(qq[0]), sin(qq[1])};
            const R ooc1 = R(1) / cy;
            R qd[3], Nb[3];
            bodyXYZ_N_P(cc, ss, ooc1, ub, qd);
            bodyXYZ_N_P(cc, ss, ooc1, bd, Nb);
            const R q1oc1 = qd[1] * ooc1;
            o[0] = Nb[0] + (qd[0] * ss[1] - qd[2]) * q1oc1;
            o[1] = Nb[1] + qd[0] * qd[2] * cc[1];
            o[2] = Nb[2] + (qd[2] * ss[1] - qd[0]) * q1oc1;
            if (b.type == SBG_FREE) {
                for (int k = 0; k < 3; ++k) o[3 + k] = bd[3 + k];
                o[6] = R(0);
            } else {
                o[3] = R(0);  // the unused slot
            }
            continue;
        }
        if (!b.quat) {  // u = qdot
            for (int k = 0; k < b.nu; ++k) o[k] = bd[k];
            continue;
        }
        // Rotation.h: calcUnnormalizedNForQuaternion is 0.5 * the rows below;
        // N b is a row-by-row product (Mat43 * Vec3)
        const R e0 = R(0.5) * qq[0], e1 = R(0.5) * qq[1], e2 = R(0.5) * qq[2], e3 = R(0.5) * qq[3];
        const R Nb0 = -e1 * bd[0] + -e2 * bd[1] + -e3 * bd[2];
        const R Nb1 = e0 * bd[0] + e3 * bd[1] + -e2 * bd[2];
        const R Nb2 = -e3 * bd[0] + e0 * bd[1] + e1 * bd[2];
        const R Nb3 = e2 * bd[0] + -e1 * bd[1] + e0 * bd[2];
        const R s = R(-0.25) * (ub[0] * ub[0] + ub[1] * ub[1] + ub[2] * ub[2]);
        o[0] = Nb0 + s * qq[0];
        o[1] = Nb1 + s * qq[1];
        o[2] = Nb2 + s * qq[2];
        o[3] = Nb3 + s * qq[3];
        if (b.type == SBG_FREE)
            for (int k = 0; k < 3; ++k) o[4 + k] = bd[3 + k];
    }
}

}  // namespace sbgo
