// sbg_oracle.hpp -- CPU restatement of Simbody's articulated-body forward
// dynamics and fixed-step Runge-Kutta-Merson integration.
//
// TEST INFRASTRUCTURE ONLY. This is the checker the CUDA path is compared
// against; it is never linked into or called by the product library. Only
// tests/, the smoke check and bench.py's CPU-baseline / reference legs use it.
//
// Parity status: pinned against the reference's own known-answer tests
// (TestMassMatrix.cpp M*M^-1 = I and udot = M^-1 f at u = 0, TestForces.cpp
// spring/damper closed forms and RK-Merson energy conservation,
// TestConstraints.cpp Ball errors) restated in tests/, against golden vectors
// recorded from a build of the reference (tests/golden/reference_vectors.npz:
// realize, M^-1 f and RK-Merson states of the seeded workloads) and against a
// trajectory value recorded from the reference itself (double pendulum,
// instance 0 of the 1024-instance workload, y(1 s)). The tree operators
// (inverse dynamics, M x, J x, ~J F, composite inertias) are pinned through
// the identities the reference's TestMassMatrix.cpp checks, on the golden
// states and the golden M^-1 f and udot. The error-controlled RK-Merson is
// pinned through its fixed-limit case, which reproduces the golden
// fixed-step states.
//
// Every routine follows the reference formulas and evaluation order closely
// and cites the reference file:line (paths relative to the Simbody source
// tree). The scalar type is a template parameter so that a counting scalar can
// produce exact per-body flop counts for the roofline.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

#include "../include/simbody_gb300.h"

namespace sbgo {

using std::abs;
using std::cos;
using std::sin;
using std::sqrt;

// ------------------------------------------------------------------ algebra
template <class R> struct V3 {
    R x[3];
    R& operator[](int i) { return x[i]; }
    const R& operator[](int i) const { return x[i]; }
};
template <class R> inline V3<R> v3(R a, R b, R c) { V3<R> r; r[0] = a; r[1] = b; r[2] = c; return r; }
template <class R> inline V3<R> zero3() { return v3<R>(R(0), R(0), R(0)); }
template <class R> inline V3<R> operator+(const V3<R>& a, const V3<R>& b) { return v3<R>(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
template <class R> inline V3<R> operator-(const V3<R>& a, const V3<R>& b) { return v3<R>(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
template <class R> inline V3<R> operator-(const V3<R>& a) { return v3<R>(-a[0], -a[1], -a[2]); }
template <class R> inline V3<R> operator*(R s, const V3<R>& a) { return v3<R>(s * a[0], s * a[1], s * a[2]); }
template <class R> inline R dot(const V3<R>& a, const V3<R>& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
// SmallMatrixMixed.h:404-410
template <class R> inline V3<R> cross(const V3<R>& a, const V3<R>& b) {
    return v3<R>(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}

// Full 3x3, row-major.
template <class R> struct M33 {
    R m[3][3];
    R& operator()(int i, int j) { return m[i][j]; }
    const R& operator()(int i, int j) const { return m[i][j]; }
};
template <class R> inline M33<R> ident33() {
    M33<R> r;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r(i, j) = R(i == j ? 1 : 0);
    return r;
}
template <class R> inline M33<R> zero33() {
    M33<R> r;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r(i, j) = R(0);
    return r;
}
template <class R> inline V3<R> operator*(const M33<R>& A, const V3<R>& v) {
    return v3<R>(A(0, 0) * v[0] + A(0, 1) * v[1] + A(0, 2) * v[2],
                 A(1, 0) * v[0] + A(1, 1) * v[1] + A(1, 2) * v[2],
                 A(2, 0) * v[0] + A(2, 1) * v[1] + A(2, 2) * v[2]);
}
template <class R> inline M33<R> operator*(const M33<R>& A, const M33<R>& B) {
    M33<R> C;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C(i, j) = A(i, 0) * B(0, j) + A(i, 1) * B(1, j) + A(i, 2) * B(2, j);
    return C;
}
template <class R> inline M33<R> transpose(const M33<R>& A) {
    M33<R> T;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) T(i, j) = A(j, i);
    return T;
}
template <class R> inline V3<R> mulT(const M33<R>& A, const V3<R>& v) {  // ~A * v
    return v3<R>(A(0, 0) * v[0] + A(1, 0) * v[1] + A(2, 0) * v[2],
                 A(0, 1) * v[0] + A(1, 1) * v[1] + A(2, 1) * v[2],
                 A(0, 2) * v[0] + A(1, 2) * v[1] + A(2, 2) * v[2]);
}
template <class R> inline M33<R> operator+(const M33<R>& A, const M33<R>& B) {
    M33<R> C; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) C(i, j) = A(i, j) + B(i, j); return C;
}
template <class R> inline M33<R> operator-(const M33<R>& A, const M33<R>& B) {
    M33<R> C; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) C(i, j) = A(i, j) - B(i, j); return C;
}
template <class R> inline V3<R> col(const M33<R>& A, int j) { return v3<R>(A(0, j), A(1, j), A(2, j)); }

// Symmetric 3x3 stored as its lower triangle (SimTK SymMat<3>).
template <class R> struct S33 {
    R xx, yx, yy, zx, zy, zz;
    R at(int i, int j) const {
        if (i < j) std::swap(i, j);
        if (i == 0) return xx;
        if (i == 1) return j == 0 ? yx : yy;
        return j == 0 ? zx : (j == 1 ? zy : zz);
    }
};
template <class R> inline S33<R> s33(R xx, R yx, R yy, R zx, R zy, R zz) { S33<R> s; s.xx = xx; s.yx = yx; s.yy = yy; s.zx = zx; s.zy = zy; s.zz = zz; return s; }
template <class R> inline V3<R> operator*(const S33<R>& S, const V3<R>& v) {
    return v3<R>(S.xx * v[0] + S.yx * v[1] + S.zx * v[2],
                 S.yx * v[0] + S.yy * v[1] + S.zy * v[2],
                 S.zx * v[0] + S.zy * v[1] + S.zz * v[2]);
}
template <class R> inline S33<R> operator+(const S33<R>& a, const S33<R>& b) { return s33<R>(a.xx + b.xx, a.yx + b.yx, a.yy + b.yy, a.zx + b.zx, a.zy + b.zy, a.zz + b.zz); }
template <class R> inline S33<R> operator-(const S33<R>& a, const S33<R>& b) { return s33<R>(a.xx - b.xx, a.yx - b.yx, a.yy - b.yy, a.zx - b.zx, a.zy - b.zy, a.zz - b.zz); }
template <class R> inline S33<R> operator*(R s, const S33<R>& a) { return s33<R>(s * a.xx, s * a.yx, s * a.yy, s * a.zx, s * a.zy, s * a.zz); }

// R*S*~R, the re-expression of a symmetric tensor (Rotation.cpp:780-804 does
// the same product with a flop-saving factorization).
template <class R> inline S33<R> reexpress(const M33<R>& Rm, const S33<R>& S) {
    M33<R> RS;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) RS(i, j) = Rm(i, 0) * S.at(0, j) + Rm(i, 1) * S.at(1, j) + Rm(i, 2) * S.at(2, j);
    R o[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j <= i; ++j) o[i][j] = RS(i, 0) * Rm(j, 0) + RS(i, 1) * Rm(j, 1) + RS(i, 2) * Rm(j, 2);
    return s33<R>(o[0][0], o[1][0], o[1][1], o[2][0], o[2][1], o[2][2]);
}

// crossMat(v)*S for symmetric S (SmallMatrixMixed.h:512-524, "v % s").
template <class R> inline M33<R> crossSym(const V3<R>& v, const S33<R>& s) {
    const R x = v[0], y = v[1], z = v[2];
    const R a = s.xx, b = s.yx, d = s.yy, c = s.zx, e = s.zy, f = s.zz;
    const R xe = x * e, yc = y * c, zb = z * b;
    M33<R> r;
    r(0, 0) = yc - zb;      r(0, 1) = y * e - z * d; r(0, 2) = y * f - z * e;
    r(1, 0) = z * a - x * c; r(1, 1) = zb - xe;       r(1, 2) = z * c - x * f;
    r(2, 0) = x * b - y * a; r(2, 1) = x * d - y * b; r(2, 2) = xe - yc;
    return r;
}

// Lower half of v_x*F - G*v_x (MassProperties.cpp:100-113, halfCrossDiff).
template <class R> inline S33<R> halfCrossDiff(const V3<R>& v, const M33<R>& F, const M33<R>& G) {
    return s33<R>(v[1] * (F(2, 0) + G(0, 2)) - v[2] * (F(1, 0) + G(0, 1)),
                  v[2] * (F(0, 0) - G(1, 1)) - v[0] * F(2, 0) + v[1] * G(1, 2),
                  v[2] * (F(0, 1) + G(1, 0)) - v[0] * (F(2, 1) + G(1, 2)),
                  v[0] * F(1, 0) - v[2] * G(2, 1) - v[1] * (F(0, 0) - G(2, 2)),
                  v[0] * (F(1, 1) - G(2, 2)) - v[1] * F(0, 1) + v[2] * G(2, 0),
                  v[0] * (F(1, 2) + G(2, 1)) - v[1] * (F(0, 2) + G(2, 0)));
}

// Articulated body inertia {M sym, J sym, F full}: P = [J F; ~F M]
// (MassProperties.h:1235-1330).
template <class R> struct ABI {
    S33<R> M, J;
    M33<R> F;
};
template <class R> inline void abiMul(const ABI<R>& P, const V3<R>& w, const V3<R>& v, V3<R>& ow, V3<R>& ov) {
    // MassProperties.h:1285-1287: (J*w + F*v, ~F*w + M*v)
    ow = P.J * w + P.F * v;
    ov = mulT(P.F, w) + P.M * v;
}
// ArticulatedInertia::shift(s) (MassProperties.cpp:123-127): shift by -s.
template <class R> inline ABI<R> abiShift(const ABI<R>& P, const V3<R>& s) {
    ABI<R> out;
    out.M = P.M;
    out.F = P.F + crossSym(s, P.M);
    out.J = P.J + halfCrossDiff(s, transpose(P.F), out.F);
    return out;
}
template <class R> inline void abiAdd(ABI<R>& a, const ABI<R>& b) { a.M = a.M + b.M; a.J = a.J + b.J; a.F = a.F + b.F; }

// ---------------------------------------------------------------- topology
struct Body {
    int parent = 0, type = 0, nq = 0, nu = 0, qoff = 0, uoff = 0, level = 0;
    bool quat = false;   // Ball/Free with quaternion coordinates
    bool euler = false;  // Ball/Free with body-fixed X-Y-Z angles (SimbodyMatterSubsystem::setUseEulerAngles)
    std::vector<int> children;
    double mass = 0, com[3] = {0, 0, 0}, G[6] = {0, 0, 0, 0, 0, 0};  // unit inertia xx yy zz xy xz yz
    double RPF[9], pPF[3], RMB[9], pMB[3];                               // X_PF and X_MB = ~X_BM
    double pitch = 0;                                                    // Screw
};

struct Topology {
    int nb = 0;  // mobilized bodies (Ground excluded)
    int nq = 0, nu = 0, nquat = 0;
    std::vector<Body> b;                 // index 0 = Ground
    std::vector<std::vector<int>> levels;  // rbNodeLevels without Ground
    double gravity[3] = {0, 0, 0};
    std::vector<sbg_mobility_force_desc> forces;
    std::vector<sbg_ball_constraint_desc> constraints;
    std::vector<sbg_contact_desc> contacts;  // parameters defaulted as the reference's
};

// q and u counts per mobilizer (quaternion mode for Ball and Free)
inline int mobNQ(int t) { static const int n[12] = {1, 1, 2, 4, 7, 3, 3, 2, 3, 6, 0, 1}; return n[t]; }
inline int mobNU(int t) { static const int n[12] = {1, 1, 2, 3, 6, 3, 3, 2, 3, 6, 0, 1}; return n[t]; }

// Node creation and slot assignment (SimbodyMatterSubsystemRep.cpp:256-330,
// RigidBodyNodeSpec.h:76-86): q/u slots consecutive in body order.
bool buildTopology(const sbg_system_desc& d, Topology& t, const char** err);

// --------------------------------------------------------------- caches
template <class R> struct BodyCache {
    // position
    M33<R> R_FM, R_GB;
    V3<R> p_FM, p_GB, p_PB;
    V3<R> HFw[6], HFv[6];  // H_FM
    V3<R> Hw[6], Hv[6];    // H_PB_G
    V3<R> l;               // Phi
    R m;
    V3<R> pc;              // Mk mass center offset p_BBc_G
    S33<R> Gi;             // unit inertia about Bo, in G
    R ooNorm;
    R ca[3], sa[3], ooc1;  // body-fixed X-Y-Z angles: cos, sin, 1/cos(q1)
    // velocity
    V3<R> Vw, Vv, VFw, VFv;
    V3<R> HDw[6], HDv[6];
    V3<R> bw, bv, aw, av;  // gyroscopic force b, mobilizer coriolis acceleration
    // dynamics
    V3<R> Fw, Fv;          // gravity body force
    ABI<R> P, PP;          // P and P+
    R D[36], DI[36];
    V3<R> Gw[6], Gv[6];
    V3<R> cw, cv;          // P*a + b
    // acceleration
    V3<R> zw, zv, zpw, zpv, Aw, Av;
    R eps[6];
};

template <class R> struct Work {
    std::vector<BodyCache<R>> c;
    std::vector<R> qerr;  // per quaternion |q|-1
    std::vector<R> f;     // mobility forces (nu)
    void resize(const Topology& t) { c.resize(t.nb + 1); qerr.resize(t.nquat); f.resize(t.nu); }
};

}  // namespace sbgo
