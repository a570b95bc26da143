// sbg_oracle.cpp -- CPU oracle: topology, RK-Merson driver, loop closures and
// a C API for the tests and the CPU-baseline legs of bench.py.
// TEST INFRASTRUCTURE ONLY (see sbg_oracle.hpp).
#include "sbg_oracle_impl.hpp"
#include "sbg_oracle_api.h"
#include "flopcount.hpp"

#include <atomic>
#include <chrono>
#include <limits>
#include <string>
#include <thread>

namespace sbgo {

bool buildTopology(const sbg_system_desc& d, Topology& t, const char** err) {
    static thread_local std::string msg;
    auto fail = [&](const std::string& m) { msg = m; if (err) *err = msg.c_str(); return false; };
    if (d.nbodies < 1 || !d.bodies) return fail("system has no bodies");
    t = Topology();
    t.nb = d.nbodies;
    t.b.resize(t.nb + 1);
    for (int k = 0; k < 3; ++k) t.gravity[k] = d.gravity[k];
    int qn = 0, un = 0;
    for (int i = 1; i <= t.nb; ++i) {
        const sbg_body_desc& bd = d.bodies[i - 1];
        Body& b = t.b[i];
        if (bd.parent < 0 || bd.parent >= i) return fail("body parent must precede the body");
        if (bd.mobilizer < 0 || bd.mobilizer >= SBG_NUM_MOBILIZERS) return fail("unknown mobilizer");
        b.parent = bd.parent;
        b.type = bd.mobilizer;
        const bool ballOrFree = b.type == SBG_BALL || b.type == SBG_FREE;
        b.euler = ballOrFree && (d.flags & SBG_SYSTEM_EULER_ANGLES);
        b.quat = ballOrFree && !b.euler;
        // Euler-angle mode keeps Simbody's q slots (4 and 7) and leaves the
        // last one unused (RigidBodyNodeSpec_Ball.h:393-395, _Free.h getMaxNQ)
        b.nq = mobNQ(b.type);
        b.nu = mobNU(b.type);
        b.qoff = qn; b.uoff = un;
        qn += b.nq; un += b.nu;
        if (b.quat) t.nquat++;
        b.level = t.b[b.parent].level + 1;
        t.b[b.parent].children.push_back(i);
        b.mass = bd.mass;
        b.pitch = bd.pitch;
        for (int k = 0; k < 3; ++k) b.com[k] = bd.com[k];
        for (int k = 0; k < 6; ++k) b.G[k] = bd.unit_inertia[k];
        for (int k = 0; k < 9; ++k) b.RPF[k] = bd.X_PF[k];
        for (int k = 0; k < 3; ++k) b.pPF[k] = bd.X_PF[9 + k];
        // X_MB = ~X_BM: R_MB = ~R_BM, p_MB = -(~R_BM p_BM)
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) b.RMB[3 * r + c] = bd.X_BM[3 * c + r];
        for (int r = 0; r < 3; ++r)
            b.pMB[r] = -(b.RMB[3 * r + 0] * bd.X_BM[9] + b.RMB[3 * r + 1] * bd.X_BM[10] + b.RMB[3 * r + 2] * bd.X_BM[11]);
    }
    t.nq = qn; t.nu = un;
    if (d.ncontacts < 0 || (d.ncontacts > 0 && !d.contacts)) return fail("bad contact list");
    for (int i = 0; i < d.ncontacts; ++i) {
        sbg_contact_desc c = d.contacts[i];
        if (c.body < 1 || c.body > t.nb) return fail("contact sphere on a bad body");
        if (!(c.radius > 0)) return fail("contact sphere radius must be positive");
        const double* par = &c.stiffness;
        bool zero = true;
        for (int k = 0; k < 9; ++k) zero &= par[k] == 0;
        if (zero) {  // SmoothSphereHalfSpaceForceImpl::Parameters() defaults
            c.stiffness = 1; c.dissipation = 0; c.static_friction = 0; c.dynamic_friction = 0;
            c.viscous_friction = 0; c.transition_velocity = 0.01; c.cf = 1e-5; c.bd = 300; c.bv = 50;
        }
        t.contacts.push_back(c);
    }
    int maxLevel = 0;
    for (int i = 1; i <= t.nb; ++i) maxLevel = std::max(maxLevel, t.b[i].level);
    t.levels.assign(maxLevel, {});
    for (int i = 1; i <= t.nb; ++i) t.levels[t.b[i].level - 1].push_back(i);
    for (int i = 0; i < d.nforces; ++i) {
        const sbg_mobility_force_desc& f = d.forces[i];
        if (f.body < 1 || f.body > t.nb) return fail("force on a bad body");
        if (f.kind != 0 && f.kind != 1) return fail("unknown mobility force kind");
        if (f.which < 0 || f.which >= t.b[f.body].nu) return fail("mobility index out of range");
        t.forces.push_back(f);
    }
    for (int i = 0; i < d.nconstraints; ++i) {
        const sbg_ball_constraint_desc& c = d.constraints[i];
        if (c.body1 < 0 || c.body1 > t.nb || c.body2 < 0 || c.body2 > t.nb || c.body1 == c.body2)
            return fail("Ball constraint on bad bodies");
        t.constraints.push_back(c);
    }
    return true;
}

// ======================================================== loop closures
// Constraint::Ball (ConstraintImpl.h:1835-1993). Station S1 on body1 and S2
// on body2 must coincide: perr = p_G(S2) - p_G(S1) (3 equations each).
// The loop forward dynamics (SimbodyMatterSubsystemRep.cpp:5076-5152) solves
// (G M^-1 G^T) lambda = aerr(udot_tree) by the rank-revealing QTZ at
// conditioning tolerance m Eps^(3/4) (:5116-5135), restated in qtzSolve
// below, so redundant closures (G rank-deficient) solve as well.
template <class R> struct LoopWork {
    std::vector<R> G;  // m x nu constraint Jacobian (rows)
};

// Station location and its velocity / acceleration (all in G).
template <class R> static void stationKin(const Work<R>& w, int body, const double* st, V3<R>& p, V3<R>& v,
                                          V3<R>* a, const V3<R>* Aw, const V3<R>* Av) {
    const BodyCache<R>& c = w.c[body];
    const V3<R> s_G = c.R_GB * loadV<R>(st);
    p = c.p_GB + s_G;
    v = c.Vv + cross(c.Vw, s_G);
    if (a) *a = Av[body] + cross(Aw[body], s_G) + cross(c.Vw, cross(c.Vw, s_G));
}

// Kinematics of the material point of `body` now at Ground location pG.
template <class R> static void pointKin(const Work<R>& w, int body, const V3<R>& pG, V3<R>& v, V3<R>* a,
                                        const V3<R>* Aw, const V3<R>* Av) {
    const BodyCache<R>& c = w.c[body];
    const V3<R> r = pG - c.p_GB;
    v = c.Vv + cross(c.Vw, r);
    if (a) *a = Av[body] + cross(Aw[body], r) + cross(c.Vw, cross(c.Vw, r));
}

// Jacobian row block d(v)/du of the material point of `body` at Ground
// location pS, added with `sign`: each mobility j of an ancestor a
// contributes Hv + Hw x (pS - p_a) (the transpose of applying a station
// force, SimbodyMatterSubsystemRep.cpp:2227).
template <class R> static void pointJacobian(const Topology& t, const Work<R>& w, int body, const V3<R>& pS, R sign,
                                             R* Grow /* 3 x nu */) {
    for (int a = body; a != 0; a = t.b[a].parent) {
        const Body& ab = t.b[a];
        const BodyCache<R>& ac = w.c[a];
        const V3<R> r = pS - ac.p_GB;
        for (int j = 0; j < ab.nu; ++j) {
            const V3<R> col = ac.Hv[j] + cross(ac.Hw[j], r);
            for (int k = 0; k < 3; ++k) Grow[k * t.nu + ab.uoff + j] = Grow[k * t.nu + ab.uoff + j] + sign * col[k];
        }
    }
}

// Ground location of station S (station2 on body2).
template <class R> static V3<R> pointS(const Work<R>& w, const sbg_ball_constraint_desc& c) {
    return w.c[c.body2].p_GB + w.c[c.body2].R_GB * loadV<R>(c.station2);
}

// The Ball constraint (ConstraintImpl.h:1835-1993) keeps station P
// (station1 on body1) and S (station2 on body2) together. perr = p_S - p_P;
// the velocity and acceleration errors and the constraint forces use the
// material point C of body1 coincident with S, not P (:1915-1991):
// verr = v_S - v_C, aerr = a_S - a_C, +lambda at S on body2, -lambda at C.
template <class R> static void constraintJacobian(const Topology& t, const Work<R>& w, std::vector<R>& G) {
    const int m = 3 * (int)t.constraints.size();
    G.assign((size_t)m * t.nu, R(0));
    for (size_t ci = 0; ci < t.constraints.size(); ++ci) {
        const auto& c = t.constraints[ci];
        R* rows = G.data() + 3 * ci * t.nu;
        const V3<R> pS = pointS(w, c);
        pointJacobian(t, w, c.body2, pS, R(1), rows);
        pointJacobian(t, w, c.body1, pS, R(-1), rows);
    }
}

template <class R> static void perrAll(const Topology& t, const Work<R>& w, R* perr) {
    for (size_t ci = 0; ci < t.constraints.size(); ++ci) {
        const auto& c = t.constraints[ci];
        V3<R> p1, v1, p2, v2;
        stationKin(w, c.body1, c.station1, p1, v1, (V3<R>*)nullptr, (const V3<R>*)nullptr, (const V3<R>*)nullptr);
        stationKin(w, c.body2, c.station2, p2, v2, (V3<R>*)nullptr, (const V3<R>*)nullptr, (const V3<R>*)nullptr);
        for (int k = 0; k < 3; ++k) perr[3 * ci + k] = p2[k] - p1[k];
    }
}

// ------------------------------------------------- rank-revealing solve
// The minimum-norm least-squares solution x of A x = b (A nr x nc, row-major)
// through a complete orthogonal factorization, as FactorQTZ does
// (SimTKmath/LinearAlgebra/src/FactorQTZ.cpp:355-430 factor, :225-290 solve;
// it calls LAPACK's dgeqp3, dlaic1, dtzrzf, dormqr and dormrz the way dgelsy
// does, LAPACK 3.x, not part of the reference's sources):
//  1. A P = Q R by Householder QR with column pivoting, the remaining column
//     of largest norm first;
//  2. the rank r: 0 if R00 = 0, else the leading blocks R[0:k,0:k] are taken
//     in turn while smin/smax > rcond, stopping at the first that fails;
//  3. x = P [R11 R12]^+ (Q^T b)[0:r], the minimum-norm solution of the kept
//     rows (R22 is dropped).
// LAPACK estimates smin and smax incrementally; this restatement takes them
// exactly (one-sided Jacobi on the leading block), so the two can decide
// differently only for a block whose condition lies within the estimate's
// error of 1/rcond. LAPACK reduces [R11 R12] to [T 0] Z by right-side
// reflections; here [R11 R12]^+ c comes from a QR of its transpose, which is
// the same minimum-norm solution. Returns r.

// Householder reflector of (alpha, x[0..n)) in the convention of dlarfg:
// H = I - tau v v^T with v = (1, x'), H (alpha, x) = (beta, 0).
static void householder(double& alpha, double* x, int n, int stride, double& tau) {
    double xn = 0;
    for (int i = 0; i < n; ++i) xn += x[i * stride] * x[i * stride];
    xn = std::sqrt(xn);
    if (xn == 0) { tau = 0; return; }
    const double beta = -std::copysign(std::hypot(alpha, xn), alpha);
    tau = (beta - alpha) / beta;
    const double sc = 1.0 / (alpha - beta);
    for (int i = 0; i < n; ++i) x[i * stride] *= sc;
    alpha = beta;
}

// Extreme singular values of the leading k x k block of an upper-triangular
// matrix (row stride ld), by one-sided Jacobi rotations (Hestenes).
static void extremeSingularValues(const std::vector<double>& R, int ld, int k, double& smin, double& smax) {
    std::vector<double> B((size_t)k * k);
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) B[(size_t)j * k + i] = j >= i ? R[(size_t)i * ld + j] : 0.0;  // column j
    const double eps = std::numeric_limits<double>::epsilon();
    for (int sweep = 0; sweep < 60; ++sweep) {
        bool rotated = false;
        for (int i = 0; i < k - 1; ++i)
            for (int j = i + 1; j < k; ++j) {
                double a = 0, b = 0, g = 0;
                double* ci = &B[(size_t)i * k];
                double* cj = &B[(size_t)j * k];
                for (int r = 0; r < k; ++r) { a += ci[r] * ci[r]; b += cj[r] * cj[r]; g += ci[r] * cj[r]; }
                if (!(std::abs(g) > eps * std::sqrt(a * b))) continue;
                rotated = true;
                const double zeta = (b - a) / (2 * g);
                const double t = std::copysign(1.0, zeta) / (std::abs(zeta) + std::sqrt(1 + zeta * zeta));
                const double c = 1 / std::sqrt(1 + t * t), sn = c * t;
                for (int r = 0; r < k; ++r) {
                    const double u = ci[r], v = cj[r];
                    ci[r] = c * u - sn * v;
                    cj[r] = sn * u + c * v;
                }
            }
        if (!rotated) break;
    }
    smin = std::numeric_limits<double>::infinity();
    smax = 0;
    for (int j = 0; j < k; ++j) {
        double n = 0;
        for (int r = 0; r < k; ++r) n += B[(size_t)j * k + r] * B[(size_t)j * k + r];
        n = std::sqrt(n);
        smin = std::min(smin, n);
        smax = std::max(smax, n);
    }
}

static int qtzSolve(int nr, int nc, std::vector<double> A, double rcond, const double* b, double* x) {
    const int mn = std::min(nr, nc);
    std::vector<int> piv(nc);
    for (int j = 0; j < nc; ++j) piv[j] = j;
    std::vector<double> tau(mn, 0.0);
    for (int k = 0; k < mn; ++k) {
        int jmax = k;
        double best = -1;
        for (int j = k; j < nc; ++j) {
            double n = 0;
            for (int i = k; i < nr; ++i) n += A[(size_t)i * nc + j] * A[(size_t)i * nc + j];
            if (n > best) { best = n; jmax = j; }
        }
        if (jmax != k) {
            for (int i = 0; i < nr; ++i) std::swap(A[(size_t)i * nc + k], A[(size_t)i * nc + jmax]);
            std::swap(piv[k], piv[jmax]);
        }
        householder(A[(size_t)k * nc + k], &A[(size_t)(k + 1) * nc + k], nr - k - 1, nc, tau[k]);
        if (tau[k] == 0) continue;
        for (int j = k + 1; j < nc; ++j) {
            double w = A[(size_t)k * nc + j];
            for (int i = k + 1; i < nr; ++i) w += A[(size_t)i * nc + k] * A[(size_t)i * nc + j];
            w *= tau[k];
            A[(size_t)k * nc + j] -= w;
            for (int i = k + 1; i < nr; ++i) A[(size_t)i * nc + j] -= w * A[(size_t)i * nc + k];
        }
    }
    int r = 0;
    if (mn > 0 && A[0] != 0) {
        r = 1;
        while (r < mn) {
            double smin, smax;
            extremeSingularValues(A, nc, r + 1, smin, smax);
            if (!(smax * rcond < smin)) break;
            ++r;
        }
    }
    // c = Q^T b
    std::vector<double> c(b, b + nr);
    for (int k = 0; k < mn; ++k) {
        if (tau[k] == 0) continue;
        double w = c[k];
        for (int i = k + 1; i < nr; ++i) w += A[(size_t)i * nc + k] * c[i];
        w *= tau[k];
        c[k] -= w;
        for (int i = k + 1; i < nr; ++i) c[i] -= w * A[(size_t)i * nc + k];
    }
    std::vector<double> z(nc, 0.0);
    if (r == nc) {
        for (int i = r - 1; i >= 0; --i) {
            double v = c[i];
            for (int j = i + 1; j < r; ++j) v -= A[(size_t)i * nc + j] * z[j];
            z[i] = v / A[(size_t)i * nc + i];
        }
    } else if (r > 0) {
        // T^T = [R11 R12]^T (nc x r) = Q2 R2; z = Q2 [R2^-T c; 0].
        std::vector<double> Tt((size_t)nc * r);
        for (int i = 0; i < r; ++i)
            for (int j = 0; j < nc; ++j) Tt[(size_t)j * r + i] = j >= i ? A[(size_t)i * nc + j] : 0.0;
        std::vector<double> tau2(r, 0.0);
        for (int k = 0; k < r; ++k) {
            householder(Tt[(size_t)k * r + k], &Tt[(size_t)(k + 1) * r + k], nc - k - 1, r, tau2[k]);
            if (tau2[k] == 0) continue;
            for (int j = k + 1; j < r; ++j) {
                double w = Tt[(size_t)k * r + j];
                for (int i = k + 1; i < nc; ++i) w += Tt[(size_t)i * r + k] * Tt[(size_t)i * r + j];
                w *= tau2[k];
                Tt[(size_t)k * r + j] -= w;
                for (int i = k + 1; i < nc; ++i) Tt[(size_t)i * r + j] -= w * Tt[(size_t)i * r + k];
            }
        }
        for (int i = 0; i < r; ++i) {  // R2^T w = c, R2 upper
            double v = c[i];
            for (int j = 0; j < i; ++j) v -= Tt[(size_t)j * r + i] * z[j];
            z[i] = v / Tt[(size_t)i * r + i];
        }
        for (int k = r - 1; k >= 0; --k) {  // z = Q2 z
            if (tau2[k] == 0) continue;
            double w = z[k];
            for (int i = k + 1; i < nc; ++i) w += Tt[(size_t)i * r + k] * z[i];
            w *= tau2[k];
            z[k] -= w;
            for (int i = k + 1; i < nc; ++i) z[i] -= w * Tt[(size_t)i * r + k];
        }
    }
    for (int j = 0; j < nc; ++j) x[piv[j]] = z[j];
    return r;
}

// realize(Acceleration) with Ball loop closures (double only). Returns
// SBG_INST_* bits.
static int realizeAccelerationLoops(const Topology& t, const double* y, Work<double>& w, double* ydot) {
    int st = 0;
    if (!realizeAcceleration(t, y, w, ydot)) st |= SBG_INST_SINGULAR_D;
    const int m = 3 * (int)t.constraints.size();
    if (m == 0) return st;
    const int nu = t.nu;
    double* udot = ydot + t.nq;
    // Acceleration errors of the tree solution: aerr = a_S2 - a_S1.
    std::vector<V3<double>> Aw(t.nb + 1), Av(t.nb + 1);
    for (int b = 0; b <= t.nb; ++b) { Aw[b] = w.c[b].Aw; Av[b] = w.c[b].Av; }
    std::vector<double> aerr(m);
    for (size_t ci = 0; ci < t.constraints.size(); ++ci) {
        const auto& c = t.constraints[ci];
        const V3<double> pS = pointS(w, c);
        V3<double> v1, a1, v2, a2;
        pointKin(w, c.body1, pS, v1, &a1, Aw.data(), Av.data());
        pointKin(w, c.body2, pS, v2, &a2, Aw.data(), Av.data());
        for (int k = 0; k < 3; ++k) aerr[3 * ci + k] = a2[k] - a1[k];
    }
    std::vector<double> G;
    constraintJacobian(t, w, G);
    // G M^-1 G^T column by column: m multiplyByMInv calls (:3512-3558).
    std::vector<double> A((size_t)m * m), x(nu);
    for (int j = 0; j < m; ++j) {
        multiplyByMInv(t, w, &G[(size_t)j * nu], x.data());
        for (int i = 0; i < m; ++i) {
            double s = 0;
            for (int k = 0; k < nu; ++k) s += G[(size_t)i * nu + k] * x[k];
            A[(size_t)i * m + j] = s;
        }
    }
    // FactorQTZ(GMInvGt, m Eps^(3/4)) and solve (:5116-5135).
    for (double v : A)
        if (!std::isfinite(v)) return st | SBG_INST_CHOLESKY_FAIL;
    std::vector<double> lam(m);
    const double eps = std::numeric_limits<double>::epsilon();
    qtzSolve(m, m, A, m * std::sqrt(eps) * std::sqrt(std::sqrt(eps)), aerr.data(), lam.data());
    // udot -= M^-1 G^T lambda
    std::vector<double> gtl(nu, 0.0);
    for (int i = 0; i < m; ++i)
        for (int k = 0; k < nu; ++k) gtl[k] += G[(size_t)i * nu + k] * lam[i];
    multiplyByMInv(t, w, gtl.data(), x.data());
    for (int k = 0; k < nu; ++k) udot[k] -= x[k];
    return st;
}

// ================================================================ RK Merson
struct IntegOpts {
    double accuracy = 1e-3, consTol = 1e-4;
    bool projectEveryStep = false;
};

static double normRMS(const double* v, int n) {
    if (n == 0) return 0;
    double s = 0;
    for (int i = 0; i < n; ++i) s += v[i] * v[i];
    return std::sqrt(s / n);
}

// calcErrorNorm (IntegratorRep.h:454-488) with unit u weights
// (SimbodyMatterSubsystemRep.cpp:1625-1634); the q part is N*Wu*NInv*dq
// (IntegratorRep.h:500-523, Rotation.h:742-748).
static double errorNorm(const Topology& t, const double* y1, const double* yerr, const double* uScale) {
    std::vector<double> dqw(t.nq);
    for (int bi = 1; bi <= t.nb; ++bi) {
        const Body& b = t.b[bi];
        const double* q = y1 + b.qoff;
        const double* dq = yerr + b.qoff;
        double* o = dqw.data() + b.qoff;
        if (b.quat) {
            const double e0 = 2 * q[0], e1 = 2 * q[1], e2 = 2 * q[2], e3 = 2 * q[3];
            const double ne1 = -e1, ne2 = -e2, ne3 = -e3;
            const double du0 = ne1 * dq[0] + e0 * dq[1] + ne3 * dq[2] + e2 * dq[3];
            const double du1 = ne2 * dq[0] + e3 * dq[1] + e0 * dq[2] + ne1 * dq[3];
            const double du2 = ne3 * dq[0] + ne2 * dq[1] + e1 * dq[2] + e0 * dq[3];
            const double h0 = q[0] / 2, h1 = q[1] / 2, h2 = q[2] / 2, h3 = q[3] / 2;
            o[0] = -h1 * du0 + -h2 * du1 + -h3 * du2;
            o[1] = h0 * du0 + h3 * du1 + -h2 * du2;
            o[2] = -h3 * du0 + h0 * du1 + h1 * du2;
            o[3] = h2 * du0 + -h1 * du1 + h0 * du2;
            if (b.type == SBG_FREE) { o[4] = dq[4]; o[5] = dq[5]; o[6] = dq[6]; }
        } else {
            for (int j = 0; j < b.nq; ++j) o[j] = dq[j];
        }
    }
    const double qn = normRMS(dqw.data(), t.nq);
    std::vector<double> us(t.nu);
    for (int i = 0; i < t.nu; ++i) us[i] = uScale[i] * yerr[t.nq + i];
    const double un = normRMS(us.data(), t.nu);
    return qn >= un ? qn : un;
}

// normalizeQuaternions (SimbodyMatterSubsystemRep.cpp:4448-4475,
// RigidBodyNodeSpec_Ball.h:417-434): q /= |q|.
static void normalizeQuaternions(const Topology& t, double* q) {
    for (int bi = 1; bi <= t.nb; ++bi) {
        const Body& b = t.b[bi];
        if (!b.quat) continue;
        double* qq = q + b.qoff;
        const double n = std::sqrt(qq[0] * qq[0] + qq[1] * qq[1] + qq[2] * qq[2] + qq[3] * qq[3]);
        for (int k = 0; k < 4; ++k) qq[k] = qq[k] / n;
    }
}

// ---------------------------------------------------------- projection
// Both projections take the minimum-norm solution of a scaled constraint
// Jacobian through FactorQTZ (qtzSolve above), as the reference does.
//
// Position (projectQ, SimbodyMatterSubsystemRep.cpp:4096-4442): the reference
// solves (P NInv) x = perr for the minimum-norm x, at conditioning tolerance
// m Eps^(1/2) (:4256-4281), and steps q -= N NInv x (Wu = 1, Tp = 1;
// :4282-4300). Here the same solution is taken in u space: with S
// any square factor of NInv NInv^T (S S^T = NInv NInv^T), the minimum-norm x'
// of (G S) x' = perr gives du = S x' = NInv x, and G S has the singular values
// of P NInv. S is 2|q| I on the rotational mobilities of a quaternion joint
// (NInv NInv^T = 4|q|^2 I for the unnormalized NInv, Rotation.h:742-748), the
// 3x3 NInv itself on those of a joint in body-fixed X-Y-Z angles (NInv =
// [x, Rx y, Rx Ry z], RigidBodyNodeSpec_Ball.h:266-300) and 1 elsewhere. Full
// Newton until RMS(perr) <= 0.1 tol, at most 20 iterations; with localOnly
// the iteration stops when the norm grows (:4310-4321); the entry q is
// restored if the result is worse than on entry (:4336-4341); then
// quaternions are normalized (:4411-4413).
//
// Velocity (projectU, :4664-4943): E = diag(uRelScale), uRelScale_i =
// max(|u_i|, 1) taken at entry (:4778-4784); the minimum-norm x of (G E) x =
// verr at tolerance m Eps^(1/2) (:4793-4812), du = E x, the factorization
// made once; at most 7 iterations.

static double normRMSv(const std::vector<double>& v) { return normRMS(v.data(), (int)v.size()); }

// Block-diagonal nu x nu scale: diag, overridden by 3x3 blocks (row-major)
// at the u offsets in uoff.
struct ScaleFactor {
    std::vector<double> diag;
    std::vector<int> uoff;
    std::vector<double> B;  // 9 per block
};

// S with S S^T = NInv NInv^T for the current (unnormalized) q.
static void projectionFactorQ(const Topology& t, const double* q, ScaleFactor& S) {
    S.diag.assign(t.nu, 1.0);
    S.uoff.clear();
    S.B.clear();
    for (int bi = 1; bi <= t.nb; ++bi) {
        const Body& b = t.b[bi];
        const double* qq = q + b.qoff;
        if (b.euler) {
            const double c0 = std::cos(qq[0]), s0 = std::sin(qq[0]), c1 = std::cos(qq[1]), s1 = std::sin(qq[1]);
            // NInv columns: (1,0,0), (0,c0,s0), (s1,-s0 c1,c0 c1)
            const double N[9] = {1, 0, s1, 0, c0, -s0 * c1, 0, s0, c0 * c1};
            S.uoff.push_back(b.uoff);
            S.B.insert(S.B.end(), N, N + 9);
            continue;
        }
        if (!b.quat) continue;
        const double n = std::sqrt(qq[0] * qq[0] + qq[1] * qq[1] + qq[2] * qq[2] + qq[3] * qq[3]);
        for (int k = 0; k < 3; ++k) S.diag[b.uoff + k] = 2 * n;
    }
}

// A = G S (m x nu).
static void scaledJacobian(int m, int nu, const std::vector<double>& G, const ScaleFactor& S, std::vector<double>& A) {
    A.assign((size_t)m * nu, 0.0);
    for (int i = 0; i < m; ++i)
        for (int k = 0; k < nu; ++k) A[(size_t)i * nu + k] = G[(size_t)i * nu + k] * S.diag[k];
    for (size_t bk = 0; bk < S.uoff.size(); ++bk) {
        const int u = S.uoff[bk];
        const double* B = &S.B[9 * bk];
        for (int i = 0; i < m; ++i) {
            const double* g = &G[(size_t)i * nu + u];
            for (int c = 0; c < 3; ++c) A[(size_t)i * nu + u + c] = g[0] * B[c] + g[1] * B[3 + c] + g[2] * B[6 + c];
        }
    }
}

// du = S x.
static void applyScale(int nu, const ScaleFactor& S, const std::vector<double>& x, std::vector<double>& du) {
    du.assign(nu, 0.0);
    for (int k = 0; k < nu; ++k) du[k] = S.diag[k] * x[k];
    for (size_t bk = 0; bk < S.uoff.size(); ++bk) {
        const int u = S.uoff[bk];
        const double* B = &S.B[9 * bk];
        for (int a = 0; a < 3; ++a) du[u + a] = B[3 * a] * x[u] + B[3 * a + 1] * x[u + 1] + B[3 * a + 2] * x[u + 2];
    }
}

// qtzSolve of a finite system; false (the projection fails) otherwise.
static bool qtzSolveFinite(int m, int nu, const std::vector<double>& A, double rcond, const double* b,
                           std::vector<double>& x) {
    for (double v : A)
        if (!std::isfinite(v)) return false;
    for (int i = 0; i < m; ++i)
        if (!std::isfinite(b[i])) return false;
    x.assign(nu, 0.0);
    qtzSolve(m, nu, A, rcond, b, x.data());
    return true;
}

// dq = N(q) du with the unnormalized N of Rotation.h:712-719.
static void multiplyByN(const Topology& t, const double* q, const double* du, double* dq) {
    for (int bi = 1; bi <= t.nb; ++bi) {
        const Body& b = t.b[bi];
        const double* qb = q + b.qoff;
        const double* ub = du + b.uoff;
        double* d = dq + b.qoff;
        if (b.quat) {
            const double e0 = qb[0] / 2, e1 = qb[1] / 2, e2 = qb[2] / 2, e3 = qb[3] / 2;
            d[0] = -e1 * ub[0] - e2 * ub[1] - e3 * ub[2];
            d[1] = e0 * ub[0] + e3 * ub[1] - e2 * ub[2];
            d[2] = -e3 * ub[0] + e0 * ub[1] + e1 * ub[2];
            d[3] = e2 * ub[0] - e1 * ub[1] + e0 * ub[2];
            if (b.type == SBG_FREE) { d[4] = ub[3]; d[5] = ub[4]; d[6] = ub[5]; }
        } else if (b.euler) {  // N_P of body-fixed X-Y-Z angles; the last q slot is unused
            const double cc[2] = {std::cos(qb[0]), std::cos(qb[1])}, ss[2] = {std::sin(qb[0]), std::sin(qb[1])};
            bodyXYZ_N_P(cc, ss, 1.0 / cc[1], ub, d);
            if (b.type == SBG_FREE) { d[3] = ub[3]; d[4] = ub[4]; d[5] = ub[5]; d[6] = 0; }
            else d[3] = 0;
        } else {
            for (int j = 0; j < b.nq; ++j) d[j] = ub[j];
        }
    }
}

static void perrAt(const Topology& t, const double* q, Work<double>& w, std::vector<double>& perr) {
    realizePosition(t, q, w);
    perr.resize(3 * t.constraints.size());
    perrAll(t, w, perr.data());
}

// Velocity errors v_G(S2) - v_G(S1) at (q, u); realizePosition must be current.
static void verrAt(const Topology& t, const double* q, const double* u, Work<double>& w, std::vector<double>& verr) {
    std::vector<double> qdot(t.nq);
    realizeVelocity(t, q, u, w, qdot.data());
    verr.resize(3 * t.constraints.size());
    for (size_t ci = 0; ci < t.constraints.size(); ++ci) {
        const auto& c = t.constraints[ci];
        const V3<double> pS = pointS(w, c);
        V3<double> v1, v2;
        pointKin(w, c.body1, pS, v1, (V3<double>*)nullptr, (const V3<double>*)nullptr, (const V3<double>*)nullptr);
        pointKin(w, c.body2, pS, v2, (V3<double>*)nullptr, (const V3<double>*)nullptr, (const V3<double>*)nullptr);
        for (int k = 0; k < 3; ++k) verr[3 * ci + k] = v2[k] - v1[k];
    }
}

// Newton iteration of projectQ (loops present, perr not yet acceptable).
static bool projectQNewton(const Topology& t, double* q, Work<double>& w, double tol, bool localOnly) {
    const int m = 3 * (int)t.constraints.size();
    std::vector<double> perr, G, A, x(t.nu), du, dq(t.nq);
    ScaleFactor S;
    perrAt(t, q, w, perr);
    const double normOnEntry = normRMSv(perr);
    const std::vector<double> saveQ(q, q + t.nq);
    const double tryFor = std::max(0.1 * tol, std::pow(std::numeric_limits<double>::epsilon(), 0.875));
    double achieved = normOnEntry, prev = normOnEntry;
    int its = 0;
    const double condTol = m * std::sqrt(std::numeric_limits<double>::epsilon());
    do {
        constraintJacobian(t, w, G);
        projectionFactorQ(t, q, S);
        scaledJacobian(m, t.nu, G, S, A);
        if (!qtzSolveFinite(m, t.nu, A, condTol, perr.data(), x)) return false;
        applyScale(t.nu, S, x, du);
        multiplyByN(t, q, du.data(), dq.data());
        for (int k = 0; k < t.nq; ++k) q[k] -= dq[k];
        perrAt(t, q, w, perr);
        achieved = normRMSv(perr);
        ++its;
        if (localOnly && its >= 2 && achieved > prev) {
            for (int k = 0; k < t.nq; ++k) q[k] += dq[k];
            perrAt(t, q, w, perr);
            achieved = normRMSv(perr);
            break;
        }
        prev = achieved;
    } while (achieved > tryFor && its < 20);
    if (achieved > tol) {
        if (achieved >= normOnEntry) std::copy(saveQ.begin(), saveQ.end(), q);
        return false;
    }
    normalizeQuaternions(t, q);
    return true;
}

// projectU with loops present; force = ProjectOptions::ForceProjection.
static bool projectULoops(const Topology& t, const double* q, double* u, Work<double>& w, double tol, bool force,
                          double limit, bool localOnly) {
    const int m = 3 * (int)t.constraints.size();
    std::vector<double> verr, G, E2(t.nu), A, du;
    realizePosition(t, q, w);
    verrAt(t, q, u, w, verr);
    const double normOnEntry = normRMSv(verr);
    if (normOnEntry > limit) return false;
    if (normOnEntry == 0 || (normOnEntry <= tol && !force)) return true;
    for (int k = 0; k < t.nu; ++k) {
        const double e = std::abs(u[k]) > 1 ? std::abs(u[k]) : 1.0;
        E2[k] = e * e;
    }
    constraintJacobian(t, w, G);
    ScaleFactor E;
    E.diag = E2;
    for (double& e : E.diag) e = std::sqrt(e);
    scaledJacobian(m, t.nu, G, E, A);
    const double condTol = m * std::sqrt(std::numeric_limits<double>::epsilon());
    std::vector<double> x(t.nu);
    const std::vector<double> saveU(u, u + t.nu);
    const double tryFor = std::max(0.1 * tol, std::pow(std::numeric_limits<double>::epsilon(), 0.875));
    double achieved = normOnEntry, prev = normOnEntry;
    int its = 0;
    do {
        if (!qtzSolveFinite(m, t.nu, A, condTol, verr.data(), x)) return false;
        applyScale(t.nu, E, x, du);
        for (int k = 0; k < t.nu; ++k) u[k] -= du[k];
        verrAt(t, q, u, w, verr);
        achieved = normRMSv(verr);
        ++its;
        if (localOnly && its >= 2 && achieved > prev) {
            for (int k = 0; k < t.nu; ++k) u[k] += du[k];
            verrAt(t, q, u, w, verr);
            achieved = normRMSv(verr);
            break;
        }
        prev = achieved;
    } while (achieved > tryFor && its < 7);
    if (achieved > tol) {
        if (achieved >= normOnEntry) std::copy(saveU.begin(), saveU.end(), u);
        return false;
    }
    return true;
}

int rkMersonRun(const Topology& t, double* y, double* time, double h, int nsteps, double tReport, bool initialize,
                const IntegOpts& o, Work<double>& w, int64_t* nProjections);

// One instance: Integrator::initialize (Integrator.cpp:333-377, which forces a
// projection: quaternions are normalized) then nsteps fixed RK-Merson steps
// (RungeKuttaMersonIntegrator.cpp:86-140, AbstractIntegratorRep.cpp:137-207,
// 341-577). Step k runs from t to t1 = t + h (FP64 sum, tMax = infinity as
// with interpolation allowed) with stage step hs = t1 - t.
int rkMerson(const Topology& t, double* y, double* time, double h, int nsteps, const IntegOpts& o, Work<double>& w,
             int64_t* nProjections) {
    return rkMersonRun(t, y, time, h, nsteps, 0.0, true, o, w, nProjections);
}

// One call of the fixed-step integrator. initialize: Integrator::initialize
// first (as above); otherwise the integration continues from y and *time as
// the previous call left them -- a second Integrator::stepTo() on the same
// integrator: the first stage derivative is recomputed from y, which is what
// the reference's realizeStateDerivatives at the top of the main loop does
// (AbstractIntegratorRep.cpp:395-404), and nothing is normalized or projected
// at entry. nsteps >= 0: exactly nsteps steps of h (tMax = infinity).
// nsteps < 0: stepTo(tReport) with setAllowInterpolation(false), i.e. tMax =
// tReport (AbstractIntegratorRep.cpp:229-240): each step's t1 follows
// takeOneStep (:536-544) -- tReport when it lies within 0.95 h of t0, t0 + h
// when it lies beyond 1.001 h, else tReport -- until t reaches tReport; with
// a fixed step size adjustStepSize keeps h for the next step (min = max = h).
int rkMersonRun(const Topology& t, double* y, double* time, double h, int nsteps, double tReport, bool initialize,
                const IntegOpts& o, Work<double>& w, int64_t* nProjections) {
    const int ny = t.nq + t.nu;
    const bool loops = !t.constraints.empty();
    int status = 0;
    std::vector<double> y0(ny), f0(ny), fa(ny), fb(ny), ysave(ny), ytmp(ny), yerr(ny), uScale(t.nu);
    auto rhs = [&](const double* yy, double* f) {
        int st = loops ? realizeAccelerationLoops(t, yy, w, f) : (realizeAcceleration(t, yy, w, f) ? 0 : SBG_INST_SINGULAR_D);
        status |= st;
    };
    if (initialize) {
        // initialize: ForceProjection, not LocalOnly, no projection limit
        // (IntegratorRep.h:856-895): with loops at least one Newton iteration
        // runs unless perr is exactly 0.
        std::vector<double> perr0;
        if (loops) perrAt(t, y, w, perr0);
        if (!loops || normRMSv(perr0) == 0) normalizeQuaternions(t, y);
        else if (!projectQNewton(t, y, w, o.consTol, false)) status |= SBG_INST_PROJECTION_FAILED;
        if (loops) {
            if (!projectULoops(t, y, y + t.nq, w, o.consTol, true, HUGE_VAL, false))
                status |= SBG_INST_PROJECTION_FAILED;
        }
    }
    double tc = *time;
    for (int step = 0;; ++step) {
        const double t0 = tc;
        double t1;
        if (nsteps >= 0) {
            if (step >= nsteps) break;
            t1 = t0 + h;
        } else {
            if (!(t0 < tReport)) break;
            if (tReport < t0 + 0.95 * h) t1 = tReport;
            else if (tReport > t0 + 1.001 * h) t1 = t0 + h;
            else t1 = tReport;
            if (!(t1 > t0)) { status |= SBG_INST_TIMEOUT; break; }
        }
        for (int i = 0; i < ny; ++i) y0[i] = y[i];
        for (int i = 0; i < t.nu; ++i) {  // calcRelativeScaling (IntegratorRep.h:644-655), w = 1
            const double vi = std::abs(y0[t.nq + i]);
            uScale[i] = vi > 1 ? 1 / vi : 1.0;
        }
        rhs(y0.data(), f0.data());
        const double hs = t1 - t0;
        const double h3 = hs / 3, h6 = hs / 6, h8 = hs / 8, h2 = hs / 2;
        for (int i = 0; i < ny; ++i) ytmp[i] = y0[i] + h3 * f0[i];
        rhs(ytmp.data(), fa.data());  // f1
        for (int i = 0; i < ny; ++i) ytmp[i] = y0[i] + h6 * (f0[i] + fa[i]);
        rhs(ytmp.data(), fa.data());  // f2
        for (int i = 0; i < ny; ++i) ytmp[i] = y0[i] + h8 * (f0[i] + 3 * fa[i]);
        rhs(ytmp.data(), fb.data());  // f3
        for (int i = 0; i < ny; ++i) ysave[i] = y0[i] + h2 * ((f0[i] - 3 * fa[i]) + 4 * fb[i]);
        rhs(ysave.data(), fa.data());  // f4
        for (int i = 0; i < ny; ++i) y[i] = y0[i] + h6 * ((f0[i] + 4 * fb[i]) + fa[i]);
        for (int i = 0; i < ny; ++i) yerr[i] = 0.2 * std::abs(y[i] - ysave[i]);
        for (int i = 0; i < ny; ++i)
            if (!std::isfinite(y[i])) status |= SBG_INST_NONFINITE;
        // attemptDAEStep gate (AbstractIntegratorRep.cpp:158-166)
        const double errNorm = errorNorm(t, y, yerr.data(), uScale.data());
        if (errNorm <= 16 * o.accuracy) {
            const double projLimit = std::max(2 * o.consTol, std::sqrt(o.consTol));
            // quaternion errors of y1 (realizePosition qErr)
            double s = 0;
            int nqt = 0;
            for (int bi = 1; bi <= t.nb; ++bi) {
                const Body& b = t.b[bi];
                if (!b.quat) continue;
                const double* qq = y + b.qoff;
                const double e = std::sqrt(qq[0] * qq[0] + qq[1] * qq[1] + qq[2] * qq[2] + qq[3] * qq[3]) - 1;
                s += e * e;
                ++nqt;
            }
            const double quatNorm = nqt ? std::sqrt(s / nqt) : 0.0;
            double perrNorm = 0;
            std::vector<double> perr;
            if (loops) {
                realizePosition(t, y, w);
                perr.resize(3 * t.constraints.size());
                perrAll(t, w, perr.data());
                perrNorm = normRMS(perr.data(), (int)perr.size());
            }
            const double normOnEntry = std::max(perrNorm, quatNorm);
            // A failed projection fails attemptDAEStep (:185-187, :197-199);
            // a fixed step cannot shrink, so the step stands and the status
            // records the failure.
            bool qok = true;
            if (normOnEntry > projLimit) {
                qok = false;
            } else if (perrNorm == 0 || (perrNorm <= o.consTol && !o.projectEveryStep)) {
                if (quatNorm > o.consTol || o.projectEveryStep) {
                    normalizeQuaternions(t, y);
                    if (nProjections) ++*nProjections;
                }
            } else {
                qok = projectQNewton(t, y, w, o.consTol, true);
                if (nProjections) ++*nProjections;
            }
            if (qok && loops) qok = projectULoops(t, y, y + t.nq, w, o.consTol, o.projectEveryStep, projLimit, true);
            if (!qok) status |= SBG_INST_PROJECTION_FAILED;
        }
        tc = t1;
    }
    *time = tc;
    return status;
}

// ======================================================= variable step
// AbstractIntegratorRep::adjustStepSize (AbstractIntegratorRep.cpp:448-502):
// the next step size from the error norm of the step just attempted (order
// errOrder). Returns whether the step succeeded: the new size is not smaller.
// hMin / hMax <= 0: no user limit (the reference's -1).
bool adjustStepSize(double err, int errOrder, bool hWasArtificiallyLimited, double accuracy, double hMin,
                    double hMax, double& h) {
    const double Safety = 0.9, MinShrink = 0.1, MaxGrow = 5, HysteresisLow = 0.9, HysteresisHigh = 1.2;
    double hNew;
    if (!std::isfinite(err)) hNew = MinShrink * h;
    else if (err == 0) hNew = MaxGrow * h;
    else hNew = Safety * h * std::pow(accuracy / err, 1 / double(errOrder));
    if (hNew > h && (hWasArtificiallyLimited || hNew < HysteresisHigh * h)) hNew = h;
    if (hNew < h) {
        if (err <= accuracy) hNew = h;
        else hNew = std::min(hNew, HysteresisLow * h);
    }
    hNew = std::min(hNew, MaxGrow * h);
    hNew = std::max(hNew, MinShrink * h);
    if (hMin > 0) hNew = std::max(hNew, hMin);
    if (hMax > 0) hNew = std::min(hNew, hMax);
    const bool success = hNew >= h;
    h = hNew;
    return success;
}

// Error-controlled RK-Merson for an instance without constraints:
// Integrator::setFinalTime(tFinal), initialize(state) (quaternions
// normalized), then stepTo(tFinal) until reached. The first step size is the
// system timescale / 10 = 0.01 (AbstractIntegratorRep.cpp:41-49,
// SystemGutsRep.h:50) unless hInit > 0. Each internal step
// (AbstractIntegratorRep.cpp:513-577) picks t1 against tMax = tFinal,
// attempts the RK-Merson step (the stages and yErr as in rkMerson), projects
// when errNorm <= 2^4 accuracy: quaternions are normalized when their RMS error
// exceeds consTol (or projectEveryStep), removing the radial component of
// their error estimate (RigidBodyNodeSpec_Ball.h:417-434); an RMS error above
// max(2 consTol, sqrt(consTol)) fails the attempt (errNorm = infinity). The
// error norm after projection decides through adjustStepSize; a failed
// attempt restores y and retries with the smaller step. Returns SBG_INST_*
// bits; SBG_INST_TIMEOUT when maxSteps accepted steps did not reach tFinal or
// the step size no longer advances time.
int rkMersonAdaptive(const Topology& t, double* y, double* time, double tFinal, double hInit, double hMin,
                     double hMax, const IntegOpts& o, Work<double>& w, int maxSteps, int64_t* accepted,
                     int64_t* rejected) {
    const int ny = t.nq + t.nu;
    int status = 0;
    std::vector<double> y0(ny), f0(ny), fa(ny), fb(ny), ysave(ny), ytmp(ny), yerr(ny), uScale(t.nu);
    auto rhs = [&](const double* yy, double* f) {
        if (!realizeAcceleration(t, yy, w, f)) status |= SBG_INST_SINGULAR_D;
    };
    normalizeQuaternions(t, y);
    double h = hInit > 0 ? hInit : 0.1 / 10;
    if (hMin > 0) h = std::max(h, hMin);
    if (hMax > 0) h = std::min(h, hMax);
    const double projLimit = std::max(2 * o.consTol, std::sqrt(o.consTol));
    double tc = *time;
    int64_t nAcc = 0, nRej = 0;
    while (tc < tFinal) {
        if (nAcc >= maxSteps) { status |= SBG_INST_TIMEOUT; break; }
        const double t0 = tc;
        for (int i = 0; i < ny; ++i) y0[i] = y[i];
        for (int i = 0; i < t.nu; ++i) {  // calcRelativeScaling (IntegratorRep.h:644-655), w = 1
            const double vi = std::abs(y0[t.nq + i]);
            uScale[i] = vi > 1 ? 1 / vi : 1.0;
        }
        rhs(y0.data(), f0.data());
        double t1 = t0;
        for (;;) {
            bool limited = false;
            if (tFinal < t0 + 0.95 * h) { limited = true; t1 = tFinal; }
            else if (tFinal > t0 + 1.001 * h) t1 = t0 + h;
            else t1 = tFinal;
            if (!(t1 > t0)) { status |= SBG_INST_TIMEOUT; break; }
            const double hs = t1 - t0;
            const double h3 = hs / 3, h6 = hs / 6, h8 = hs / 8, h2 = hs / 2;
            for (int i = 0; i < ny; ++i) ytmp[i] = y0[i] + h3 * f0[i];
            rhs(ytmp.data(), fa.data());  // f1
            for (int i = 0; i < ny; ++i) ytmp[i] = y0[i] + h6 * (f0[i] + fa[i]);
            rhs(ytmp.data(), fa.data());  // f2
            for (int i = 0; i < ny; ++i) ytmp[i] = y0[i] + h8 * (f0[i] + 3 * fa[i]);
            rhs(ytmp.data(), fb.data());  // f3
            for (int i = 0; i < ny; ++i) ysave[i] = y0[i] + h2 * ((f0[i] - 3 * fa[i]) + 4 * fb[i]);
            rhs(ysave.data(), fa.data());  // f4
            for (int i = 0; i < ny; ++i) y[i] = y0[i] + h6 * ((f0[i] + 4 * fb[i]) + fa[i]);
            for (int i = 0; i < ny; ++i) yerr[i] = 0.2 * std::abs(y[i] - ysave[i]);
            double errNorm = errorNorm(t, y, yerr.data(), uScale.data());
            if (errNorm <= 16 * o.accuracy) {  // attemptDAEStep (AbstractIntegratorRep.cpp:158-199)
                double sq = 0;
                int nqt = 0;
                for (int bi = 1; bi <= t.nb; ++bi) {
                    const Body& b = t.b[bi];
                    if (!b.quat) continue;
                    const double* qq = y + b.qoff;
                    const double e = std::sqrt(qq[0] * qq[0] + qq[1] * qq[1] + qq[2] * qq[2] + qq[3] * qq[3]) - 1;
                    sq += e * e;
                    ++nqt;
                }
                const double quatNorm = nqt ? std::sqrt(sq / nqt) : 0.0;
                if (quatNorm > projLimit) {
                    errNorm = HUGE_VAL;  // the step did not converge
                } else if (quatNorm > o.consTol || o.projectEveryStep) {
                    for (int bi = 1; bi <= t.nb; ++bi) {
                        const Body& b = t.b[bi];
                        if (!b.quat) continue;
                        double* qq = y + b.qoff;
                        double* qe = yerr.data() + b.qoff;
                        const double n = std::sqrt(qq[0] * qq[0] + qq[1] * qq[1] + qq[2] * qq[2] + qq[3] * qq[3]);
                        for (int k = 0; k < 4; ++k) qq[k] = qq[k] / n;
                        const double d = qe[0] * qq[0] + qe[1] * qq[1] + qe[2] * qq[2] + qe[3] * qq[3];
                        for (int k = 0; k < 4; ++k) qe[k] = qe[k] - d * qq[k];
                    }
                    errNorm = errorNorm(t, y, yerr.data(), uScale.data());
                }
            }
            if (adjustStepSize(errNorm, 4, limited, o.accuracy, hMin, hMax, h)) break;
            ++nRej;
            for (int i = 0; i < ny; ++i) y[i] = y0[i];
            if (nRej > 64 * (int64_t)maxSteps) { status |= SBG_INST_TIMEOUT; break; }
        }
        if (status & SBG_INST_TIMEOUT) break;
        for (int i = 0; i < ny; ++i)
            if (!std::isfinite(y[i])) status |= SBG_INST_NONFINITE;
        tc = t1;
        ++nAcc;
    }
    *time = tc;
    if (accepted) *accepted = nAcc;
    if (rejected) *rejected = nRej;
    return status;
}

}  // namespace sbgo

// ===================================================================== C API
using namespace sbgo;

namespace {
thread_local std::string g_err;
int setErr(const char* m) { g_err = m ? m : "error"; return SBG_ERR_INVALID; }

struct Inst {
    Topology topo;
};

// Parallel for over instances with nthreads workers (0 = hardware).
template <class F> void parallelFor(int n, int nthreads, F&& fn) {
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    nthreads = std::min(nthreads, std::max(1, n));
    if (nthreads == 1) { for (int i = 0; i < n; ++i) fn(i, 0); return; }
    std::atomic<int> next(0);
    std::vector<std::thread> th;
    for (int w = 0; w < nthreads; ++w)
        th.emplace_back([&, w] {
            for (;;) {
                const int i = next.fetch_add(1);
                if (i >= n) break;
                fn(i, w);
            }
        });
    for (auto& x : th) x.join();
}
}  // namespace

extern "C" {

const char* oracle_last_error(void) { return g_err.c_str(); }

int oracle_system_sizes(const sbg_system_desc* d, int32_t* nq, int32_t* nu, int32_t* nquat) {
    Topology t;
    const char* e = nullptr;
    if (!buildTopology(*d, t, &e)) return setErr(e);
    if (nq) *nq = t.nq;
    if (nu) *nu = t.nu;
    if (nquat) *nquat = t.nquat;
    return 0;
}

// Batch realize(Acceleration): systems[sys_of[i]] for instance i; y and ydot
// packed [q,u] per instance at y_off[i]. status may be NULL.
int oracle_realize_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                         const int64_t* y_off, const double* y, double* ydot, int32_t* status, int32_t nthreads) {
    std::vector<Topology> topo(nsys);
    for (int s = 0; s < nsys; ++s) {
        const char* e = nullptr;
        if (!buildTopology(systems[s], topo[s], &e)) return setErr(e);
    }
    parallelFor(ninst, nthreads, [&](int i, int) {
        const Topology& t = topo[sys_of[i]];
        Work<double> w;
        w.resize(t);
        int st = t.constraints.empty()
                     ? (realizeAcceleration(t, y + y_off[i], w, ydot + y_off[i]) ? 0 : SBG_INST_SINGULAR_D)
                     : realizeAccelerationLoops(t, y + y_off[i], w, ydot + y_off[i]);
        for (int k = 0; k < t.nq + t.nu; ++k)
            if (!std::isfinite(ydot[y_off[i] + k])) st |= SBG_INST_NONFINITE;
        if (status) status[i] = st;
    });
    return 0;
}

// multiplyByMInv for a batch: f/out packed per instance (nu values) at u_off[i].
int oracle_minv_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                      const int64_t* y_off, const double* y, const int64_t* u_off, const double* f, double* out,
                      int32_t nthreads) {
    std::vector<Topology> topo(nsys);
    for (int s = 0; s < nsys; ++s) {
        const char* e = nullptr;
        if (!buildTopology(systems[s], topo[s], &e)) return setErr(e);
    }
    parallelFor(ninst, nthreads, [&](int i, int) {
        const Topology& t = topo[sys_of[i]];
        Work<double> w;
        w.resize(t);
        realizePosition(t, y + y_off[i], w);
        realizeABI(t, w);
        multiplyByMInv(t, w, f + u_off[i], out + u_off[i]);
    });
    return 0;
}

int oracle_rk_merson_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                           const int64_t* y_off, double* y, double* t, double h, int32_t nsteps, double accuracy,
                           double consTol, int32_t projectEveryStep, int32_t* status, int64_t* nproj,
                           int32_t nthreads) {
    std::vector<Topology> topo(nsys);
    for (int s = 0; s < nsys; ++s) {
        const char* e = nullptr;
        if (!buildTopology(systems[s], topo[s], &e)) return setErr(e);
    }
    IntegOpts o;
    if (accuracy > 0) o.accuracy = accuracy;
    o.consTol = consTol > 0 ? consTol : o.accuracy / 10;
    o.projectEveryStep = projectEveryStep != 0;
    std::atomic<int64_t> np(0);
    parallelFor(ninst, nthreads, [&](int i, int) {
        const Topology& tp = topo[sys_of[i]];
        Work<double> w;
        w.resize(tp);
        double tt = t ? t[i] : 0.0;
        int64_t p = 0;
        const int st = rkMerson(tp, y + y_off[i], &tt, h, nsteps, o, w, &p);
        if (t) t[i] = tt;
        if (status) status[i] = st;
        np += p;
    });
    if (nproj) *nproj = np.load();
    return 0;
}

// One integration call per instance (rkMersonRun): nsteps >= 0 steps of h, or
// nsteps < 0 stepTo(t_report) with interpolation off; initialize = 0
// continues the integration y and t describe.
int oracle_rk_merson_run_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                               const int64_t* y_off, double* y, double* t, double h, int32_t nsteps, double t_report,
                               int32_t initialize, double accuracy, double consTol, int32_t projectEveryStep,
                               int32_t* status, int32_t nthreads) {
    std::vector<Topology> topo(nsys);
    for (int s = 0; s < nsys; ++s) {
        const char* e = nullptr;
        if (!buildTopology(systems[s], topo[s], &e)) return setErr(e);
    }
    IntegOpts o;
    if (accuracy > 0) o.accuracy = accuracy;
    o.consTol = consTol > 0 ? consTol : o.accuracy / 10;
    o.projectEveryStep = projectEveryStep != 0;
    parallelFor(ninst, nthreads, [&](int i, int) {
        const Topology& tp = topo[sys_of[i]];
        Work<double> w;
        w.resize(tp);
        double tt = t ? t[i] : 0.0;
        const int st = rkMersonRun(tp, y + y_off[i], &tt, h, nsteps, t_report, initialize != 0, o, w, nullptr);
        if (t) t[i] = tt;
        if (status) status[i] = st;
    });
    return 0;
}

// State::getQDotDot() after realize(Acceleration) for a batch: y and ydot in
// the [q,u] packing at y_off[i], qdotdot nq values per instance at q_off[i].
int oracle_qdotdot_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                         const int64_t* y_off, const double* y, const double* ydot, const int64_t* q_off,
                         double* qdotdot) {
    std::vector<Topology> topo(nsys);
    for (int s = 0; s < nsys; ++s) {
        const char* e = nullptr;
        if (!buildTopology(systems[s], topo[s], &e)) return setErr(e);
    }
    for (int i = 0; i < ninst; ++i) {
        const Topology& tp = topo[sys_of[i]];
        calcQDotDot(tp, y + y_off[i], ydot + y_off[i] + tp.nq, qdotdot + q_off[i]);
    }
    return 0;
}

// Tree operators for a batch (body arrays: b_off[i] = bodies before instance
// i; SpatialVecs take 6 values per body, spatial inertias 10):
//   op 0  calcResidualForceIgnoringConstraints: out(u) = M x + C(q,u) - fmob - ~J Fbody
//   op 1  multiplyByM: out(u) = M x
//   op 2  multiplyBySystemJacobian: out(6 per body) = J x
//   op 3  multiplyBySystemJacobianTranspose: out(u) = ~J Fbody
//   op 4  calcCompositeBodyInertias: out(10 per body)
// fmob and Fbody may be NULL (zero); x may be NULL for ops 0 and 1 (zero).
int oracle_tree_op_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                         const int64_t* y_off, const double* y, const int64_t* u_off, const int64_t* b_off,
                         int32_t op, const double* x, const double* fmob, const double* Fbody, double* out,
                         int32_t nthreads) {
    if (op < 0 || op > 4) return setErr("unknown tree operator");
    std::vector<Topology> topo(nsys);
    for (int s = 0; s < nsys; ++s) {
        const char* e = nullptr;
        if (!buildTopology(systems[s], topo[s], &e)) return setErr(e);
    }
    parallelFor(ninst, nthreads, [&](int i, int) {
        const Topology& t = topo[sys_of[i]];
        Work<double> w;
        w.resize(t);
        const double* q = y + y_off[i];
        realizePosition(t, q, w);
        std::vector<double> zero(t.nu, 0.0);
        const double* xi = x ? x + u_off[i] : zero.data();
        const double* Fi = Fbody ? Fbody + 6 * b_off[i] : nullptr;
        const double* fi = fmob ? fmob + u_off[i] : nullptr;
        switch (op) {
        case 0:
            realizeVelocity(t, q, q + t.nq, w, (double*)nullptr);
            accelerationsOutward(t, w, xi, true);
            forcesInward(t, w, 0, Fi, fi, out + u_off[i]);
            break;
        case 1:
            accelerationsOutward(t, w, xi, false);
            forcesInward(t, w, 1, (const double*)nullptr, (const double*)nullptr, out + u_off[i]);
            break;
        case 2: {
            accelerationsOutward(t, w, xi, false);
            double* o = out + 6 * b_off[i];
            for (int bi = 1; bi <= t.nb; ++bi)
                for (int k = 0; k < 3; ++k) { o[6 * (bi - 1) + k] = w.c[bi].Aw[k]; o[6 * (bi - 1) + 3 + k] = w.c[bi].Av[k]; }
            break;
        }
        case 3:
            forcesInward(t, w, 2, Fi, (const double*)nullptr, out + u_off[i]);
            break;
        default:
            compositeInertias(t, w, out + 10 * b_off[i]);
            break;
        }
    });
    return 0;
}

// The forces of each system's own force elements at its state: Force::Gravity
// body forces (6 per body, moment and force in Ground) and the mobility
// springs and dampers (nu per instance), as realize(Dynamics) accumulates them.
int oracle_system_forces_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                               const int64_t* y_off, const double* y, const int64_t* u_off, const int64_t* b_off,
                               double* fmob, double* Fbody, int32_t nthreads) {
    std::vector<Topology> topo(nsys);
    for (int s = 0; s < nsys; ++s) {
        const char* e = nullptr;
        if (!buildTopology(systems[s], topo[s], &e)) return setErr(e);
    }
    parallelFor(ninst, nthreads, [&](int i, int) {
        const Topology& t = topo[sys_of[i]];
        Work<double> w;
        w.resize(t);
        const double* q = y + y_off[i];
        realizePosition(t, q, w);
        realizeVelocity(t, q, q + t.nq, w, (double*)nullptr);  // contact forces depend on velocities
        calcForces(t, q, q + t.nq, w);
        for (int k = 0; k < t.nu; ++k) fmob[u_off[i] + k] = w.f[k];
        for (int bi = 1; bi <= t.nb; ++bi)
            for (int k = 0; k < 3; ++k) {
                Fbody[6 * (b_off[i] + bi - 1) + k] = w.c[bi].Fw[k];
                Fbody[6 * (b_off[i] + bi - 1) + 3 + k] = w.c[bi].Fv[k];
            }
    });
    return 0;
}

// Error-controlled RK-Merson to tFinal for every instance (no constraints;
// rkMersonAdaptive). hInit / hMin / hMax <= 0: the reference's defaults.
// stats (may be NULL): accepted and rejected steps, 2 per instance.
int oracle_rk_merson_adaptive_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of,
                                    int32_t ninst, const int64_t* y_off, double* y, double* t, double tFinal,
                                    double hInit, double hMin, double hMax, double accuracy, double consTol,
                                    int32_t projectEveryStep, int32_t maxSteps, int32_t* status, int64_t* stats,
                                    int32_t nthreads) {
    std::vector<Topology> topo(nsys);
    for (int s = 0; s < nsys; ++s) {
        const char* e = nullptr;
        if (!buildTopology(systems[s], topo[s], &e)) return setErr(e);
    }
    for (int i = 0; i < ninst; ++i)
        if (!topo[sys_of[i]].constraints.empty())
            return setErr("variable-step integration of loop closures is not restated");
    IntegOpts o;
    if (accuracy > 0) o.accuracy = accuracy;
    o.consTol = consTol > 0 ? consTol : o.accuracy / 10;
    o.projectEveryStep = projectEveryStep != 0;
    parallelFor(ninst, nthreads, [&](int i, int) {
        const Topology& tp = topo[sys_of[i]];
        Work<double> w;
        w.resize(tp);
        double tt = t ? t[i] : 0.0;
        int64_t acc = 0, rej = 0;
        const int st = rkMersonAdaptive(tp, y + y_off[i], &tt, tFinal, hInit, hMin, hMax, o, w, maxSteps, &acc, &rej);
        if (t) t[i] = tt;
        if (status) status[i] = st;
        if (stats) { stats[2 * i] = acc; stats[2 * i + 1] = rej; }
    });
    return 0;
}

// Step-size controller alone (adjustStepSize), for its unit tests.
int oracle_adjust_step_size(double err, int32_t errOrder, int32_t limited, double accuracy, double hMin, double hMax,
                            double* h) {
    return adjustStepSize(err, errOrder, limited != 0, accuracy, hMin, hMax, *h) ? 1 : 0;
}

// Invariants of one instance at y, for the restated known-answer tests:
// energy[0] kinetic energy u.M u / 2 (multiplyByM, as above); energy[1]
// gravity's potential energy -sum m g.p_C (Force_Gravity.cpp:531-556, zero
// height 0); energy[2] the mobility springs' sum k (q[which] - q0)^2 / 2
// (Force.cpp:353-360). perr, verr, aerr (3 per Ball closure; may be null when
// there are none): the closure errors of ConstraintImpl.h:1896-1960 at y, the
// accelerations those of the constrained realize(Acceleration). Returns the
// realize's SBG_INST_* bits.
int oracle_instance_invariants(const sbg_system_desc* d, const double* y, double* energy, double* perr, double* verr,
                               double* aerr) {
    Topology t;
    const char* e = nullptr;
    if (!buildTopology(*d, t, &e)) return -setErr(e);
    Work<double> w;
    w.resize(t);
    const double* q = y;
    const double* u = y + t.nq;
    std::vector<double> ydot(t.nq + t.nu), Mu(t.nu);
    const int st = t.constraints.empty() ? (realizeAcceleration(t, y, w, ydot.data()) ? 0 : SBG_INST_SINGULAR_D)
                                         : realizeAccelerationLoops(t, y, w, ydot.data());
    realizePosition(t, q, w);
    realizeVelocity(t, q, u, w, (double*)nullptr);
    accelerationsOutward(t, w, u, false);
    forcesInward(t, w, 1, (const double*)nullptr, (const double*)nullptr, Mu.data());
    double ke = 0;
    for (int k = 0; k < t.nu; ++k) ke += u[k] * Mu[k];
    energy[0] = ke / 2;
    // accelerationsOutward overwrote the body accelerations; positions and
    // velocities are unchanged.
    double pe = 0;
    const V3<double> g = loadV<double>(d->gravity);
    for (int bi = 1; bi <= t.nb; ++bi) {
        const BodyCache<double>& c = w.c[bi];
        const V3<double> pC = c.p_GB + c.R_GB * loadV<double>(d->bodies[bi - 1].com);
        pe -= d->bodies[bi - 1].mass * dot(g, pC);
    }
    energy[1] = pe;
    double ps = 0;
    for (int i = 0; i < d->nforces; ++i) {
        const sbg_mobility_force_desc& f = d->forces[i];
        if (f.kind != 0) continue;
        const double dq = q[t.b[f.body].qoff + f.which] - f.q0;
        ps += f.coef * dq * dq / 2;
    }
    energy[2] = ps;
    if (!t.constraints.empty()) {
        accelerationsOutward(t, w, ydot.data() + t.nq, true);
        std::vector<V3<double>> Aw(t.nb + 1), Av(t.nb + 1);
        for (int b = 0; b <= t.nb; ++b) { Aw[b] = w.c[b].Aw; Av[b] = w.c[b].Av; }
        perrAll(t, w, perr);
        for (size_t ci = 0; ci < t.constraints.size(); ++ci) {
            const auto& c = t.constraints[ci];
            const V3<double> pS = pointS(w, c);
            V3<double> v1, a1, v2, a2;
            pointKin(w, c.body1, pS, v1, &a1, Aw.data(), Av.data());
            pointKin(w, c.body2, pS, v2, &a2, Aw.data(), Av.data());
            for (int k = 0; k < 3; ++k) {
                verr[3 * ci + k] = v2[k] - v1[k];
                aerr[3 * ci + k] = a2[k] - a1[k];
            }
        }
    }
    return st;
}

// The rank-revealing minimum-norm solve alone (qtzSolve), for its unit tests:
// A nr x nc row-major, x gets nc values; returns the rank.
int oracle_qtz_solve(int32_t nr, int32_t nc, const double* A, double rcond, const double* b, double* x) {
    if (nr < 0 || nc < 0) return setErr("negative size");
    return qtzSolve(nr, nc, std::vector<double>(A, A + (size_t)nr * nc), rcond, b, x);
}

// Exact operation counts of one realize(Acceleration) of one instance with
// the counting scalar: counts[0]=add/sub, [1]=mul, [2]=div, [3]=sqrt,
// [4]=sin/cos, [5]=abs/compare.
int oracle_count_realize(const sbg_system_desc* d, const double* y, int64_t* counts) {
    Topology t;
    const char* e = nullptr;
    if (!buildTopology(*d, t, &e)) return setErr(e);
    const int ny = t.nq + t.nu;
    std::vector<CReal> yy(ny), yd(ny);
    for (int i = 0; i < ny; ++i) yy[i] = CReal(y[i]);
    Work<CReal> w;
    w.resize(t);
    CReal::reset();
    realizeAcceleration(t, yy.data(), w, yd.data());
    CReal::get(counts);
    return 0;
}

// Wall-clock seconds of nreps realize(Acceleration) passes over all instances
// with nthreads workers (the reference's CPU path restated; used as the CPU
// baseline when the reference itself cannot be built).
double oracle_time_realize(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                           const int64_t* y_off, const double* y, double* ydot, int32_t nreps, int32_t nthreads) {
    std::vector<Topology> topo(nsys);
    for (int s = 0; s < nsys; ++s) {
        const char* e = nullptr;
        if (!buildTopology(systems[s], topo[s], &e)) { setErr(e); return -1; }
    }
    const auto t0 = std::chrono::steady_clock::now();
    parallelFor(ninst, nthreads, [&](int i, int) {
        const Topology& t = topo[sys_of[i]];
        Work<double> w;
        w.resize(t);
        for (int r = 0; r < nreps; ++r) realizeAcceleration(t, y + y_off[i], w, ydot + y_off[i]);
    });
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

int oracle_hardware_threads(void) { return (int)std::thread::hardware_concurrency(); }

}  // extern "C"
