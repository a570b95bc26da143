// workloads.cpp -- seeded synthetic workloads with the shapes, sizes and value
// distributions of the benchmark configurations of the batched
// forward-dynamics path. Host-only C++ (std::mt19937_64 and the libstdc++
// distributions, so the streams are identical on every gcc host).
//
// Seeds: system parameters and states of instance i of workload c come from
// std::mt19937_64(c << 32 | i); the shared 32-Ball chain draws its body
// parameters from std::mt19937_64(2).
//
//  1  double pendulum: 2 Pin links, mass 1, UnitInertia(1), X_BM = (I,(0,1,0)),
//     gravity 9.8 along -Y; q ~ U[-pi,pi], u ~ N(0,1); h = 1e-3, 1000 steps.
//  2  unbranched chain of 32 Ball bodies, mass lognormal(0,0.5), brick inertia
//     with sides U[0.05,0.3], X_BM = (I,(0,0.1,0)); random unit quaternions,
//     u ~ N(0,0.5); realize(Acceleration) only.
//  3  random trees of 20..40 bodies: Free root, children uniform over
//     Pin/Slider/Universal/Ball, parent uniform over earlier bodies; gravity,
//     one MobilityLinearSpring (k ~ U[10,100], q0 = 0) and one
//     MobilityLinearDamper (c ~ U[0.1,1]) per mobility; h = 5e-4, 2000 steps.
//  4  uneven batch: as 3 with body count log-uniform in [4,256]; 1000 steps.
//  5  serving requests: trees as 4, horizon log-uniform in [100,10000] steps,
//     20% with 1..4 Constraint::Ball closures to Ground, assembled at t = 0.
// Test workloads of the wider mobilizer set (no benchmark counterpart):
//  6  random trees as 3 whose children are uniform over Pin, Slider,
//     Universal, Ball, Gimbal, Translation, Cylinder, Planar, Bushing, Weld and
//     Screw (pitch U[-0.05,0.05]), the
//     root a Free body (even instances) or a Bushing (odd ones); angles
//     U[-0.5,0.5], displacements U[-0.05,0.05].
//  7  random trees as 3 in Euler-angle mode (SBG_SYSTEM_EULER_ANGLES): Ball
//     and Free bodies with body-fixed X-Y-Z angles U[-0.5,0.5].
//  9  random trees as 7 (Euler-angle mode) where 20% get 1..4 Ball loop
//     closures to Ground as in 5, assembled at t = 0.
//  8  random trees as 3 on a ground half-space: a SmoothSphereHalfSpaceForce
//     sphere on every body (station U[-0.05,0.05]^3, radius U[0.02,0.06]), the
//     half-space normal tilted U[-0.2,0.2] rad from -Y, the lowest sphere
//     indented 3 mm at t = 0; 2000 steps of 5e-4.
// 10  random trees as 3, each closed by 1..2 Ball closures to Ground and made
//     redundant: a repeated closure, a second pinned point of the same body,
//     or both (instance % 3), so G M^-1 G^T is rank-deficient.
#include "../../include/simbody_gb300.h"
#include "sbg_workloads.h"

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace {

const double kPi = 3.14159265358979323846;

struct Sys {
    bool euler = false;  // Ball and Free bodies in body-fixed X-Y-Z angles
    std::vector<sbg_body_desc> bodies;
    std::vector<sbg_mobility_force_desc> forces;
    std::vector<sbg_ball_constraint_desc> cons;
    std::vector<sbg_contact_desc> contacts;
    double gravity[3] = {0, -9.8, 0};
    int32_t flags = 0;
};

}  // namespace

struct sbg_workload_s {
    int config = 0;
    std::vector<Sys> sys;
    std::vector<sbg_system_desc> desc;
    std::vector<int32_t> inst_sys;
    std::vector<int64_t> y_off;
    std::vector<double> y0;
    std::vector<int32_t> horizon;     // serving: steps per request
    std::vector<double> arrival;      // serving: arrival time (s)
    double h = 0;
    int32_t nsteps = 0;
};

namespace {

thread_local std::string g_wl_err;

void setIdentity(double* X) {
    std::memset(X, 0, 12 * sizeof(double));
    X[0] = X[4] = X[8] = 1;
}

int nq_of(int t) { static const int n[12] = {1, 1, 2, 4, 7, 3, 3, 2, 3, 6, 0, 1}; return n[t]; }
int nu_of(int t) { static const int n[12] = {1, 1, 2, 3, 6, 3, 3, 2, 3, 6, 0, 1}; return n[t]; }

sbg_body_desc makeBody(int parent, int mob, double m, const double G[6], const double pPF[3], const double pBM[3]) {
    sbg_body_desc b;
    std::memset(&b, 0, sizeof b);
    b.parent = parent;
    b.mobilizer = mob;
    b.mass = m;
    for (int k = 0; k < 6; ++k) b.unit_inertia[k] = G[k];
    setIdentity(b.X_PF);
    setIdentity(b.X_BM);
    for (int k = 0; k < 3; ++k) { b.X_PF[9 + k] = pPF[k]; b.X_BM[9 + k] = pBM[k]; }
    return b;
}

// UnitInertia::brick(hx,hy,hz) with half lengths (MassProperties.h:897-901).
void brick(double a, double b, double c, double* G) {
    const double hx = a / 2, hy = b / 2, hz = c / 2;
    const double oo3 = 1.0 / 3.0;
    G[0] = oo3 * (hy * hy + hz * hz);
    G[1] = oo3 * (hx * hx + hz * hz);
    G[2] = oo3 * (hx * hx + hy * hy);
    G[3] = G[4] = G[5] = 0;
}

void randomUnitQuat(std::mt19937_64& r, double* q) {
    std::normal_distribution<double> N(0, 1);
    double n2 = 0;
    for (int k = 0; k < 4; ++k) { q[k] = N(r); n2 += q[k] * q[k]; }
    const double n = std::sqrt(n2);
    for (int k = 0; k < 4; ++k) q[k] /= n;
}

// Random tree (workloads 3-8) and its initial state. wide: children over
// all eleven non-Free mobilizers and rootType for the root (workload 6);
// euler: Ball and Free bodies with body-fixed X-Y-Z angles (workload 7).
// Workloads 3-5 (wide = euler = false) draw exactly the stream they always did.
void randomTree(std::mt19937_64& r, int nb, Sys& s, std::vector<double>& y, bool wide = false,
                int rootType = SBG_FREE, bool euler = false) {
    static const int kWide[11] = {SBG_PIN, SBG_SLIDER, SBG_UNIVERSAL, SBG_BALL, SBG_GIMBAL, SBG_TRANSLATION,
                                  SBG_CYLINDER, SBG_PLANAR, SBG_BUSHING, SBG_WELD, SBG_SCREW};
    std::uniform_int_distribution<int> typeD(0, wide ? 10 : 3);
    std::lognormal_distribution<double> LN(0, 0.5);
    std::uniform_real_distribution<double> US(0.05, 0.3), UK(10, 100), UC(0.1, 1), UP(-0.1, 0.1);
    std::uniform_real_distribution<double> UA(-0.5, 0.5), UL(-0.05, 0.05);
    std::normal_distribution<double> NU(0, 0.5);
    const double pBM[3] = {0, 0.1, 0};
    for (int i = 1; i <= nb; ++i) {
        int parent = 0, mob = rootType;
        if (i > 1) {
            std::uniform_int_distribution<int> parD(1, i - 1);
            parent = parD(r);
            const int t = typeD(r);
            mob = wide ? kWide[t] : t == 0 ? SBG_PIN : t == 1 ? SBG_SLIDER : t == 2 ? SBG_UNIVERSAL : SBG_BALL;
        }
        const double m = LN(r);
        const double a = US(r), b = US(r), c = US(r);
        double G[6];
        brick(a, b, c, G);
        double pPF[3] = {0, 0, 0};
        if (i > 1) { pPF[0] = UP(r); pPF[1] = UP(r); pPF[2] = UP(r); }
        s.bodies.push_back(makeBody(parent, mob, m, G, pPF, pBM));
        if (mob == SBG_SCREW) s.bodies.back().pitch = UL(r);  // U[-0.05, 0.05] per radian
        for (int j = 0; j < nu_of(mob); ++j) {
            sbg_mobility_force_desc sp{0, i, j, 0, UK(r), 0.0};
            sbg_mobility_force_desc dp{1, i, j, 0, UC(r), 0.0};
            s.forces.push_back(sp);
            s.forces.push_back(dp);
        }
    }
    // state
    std::vector<double> q, u;
    for (int i = 1; i <= nb; ++i) {
        const int mob = s.bodies[i - 1].mobilizer;
        if (mob == SBG_PIN || mob == SBG_SCREW) q.push_back(UA(r));
        else if (mob == SBG_SLIDER) q.push_back(UL(r));
        else if (mob == SBG_UNIVERSAL) { q.push_back(UA(r)); q.push_back(UA(r)); }
        else if (mob == SBG_GIMBAL || mob == SBG_BUSHING || (euler && (mob == SBG_BALL || mob == SBG_FREE))) {
            for (int k = 0; k < 3; ++k) q.push_back(UA(r));
            if (mob == SBG_BUSHING || mob == SBG_FREE)
                for (int k = 0; k < 3; ++k) q.push_back(i == 1 ? 0.0 : UL(r));
            // Euler-angle Ball and Free keep the quaternion's slot count; the last is unused
            if (mob == SBG_BALL || mob == SBG_FREE) q.push_back(0.0);
        } else if (mob == SBG_TRANSLATION) {
            for (int k = 0; k < 3; ++k) q.push_back(UL(r));
        } else if (mob == SBG_CYLINDER) {
            q.push_back(UA(r)); q.push_back(UL(r));
        } else if (mob == SBG_PLANAR) {
            q.push_back(UA(r)); q.push_back(UL(r)); q.push_back(UL(r));
        } else if (mob == SBG_WELD) {
            // no coordinates
        } else {
            double qq[4];
            randomUnitQuat(r, qq);
            for (double v : qq) q.push_back(v);
            if (mob == SBG_FREE) { q.push_back(0); q.push_back(0); q.push_back(0); }
        }
        for (int j = 0; j < nu_of(mob); ++j) u.push_back(NU(r));
    }
    y.insert(y.end(), q.begin(), q.end());
    y.insert(y.end(), u.begin(), u.end());
}

// -------- host forward kinematics (for assembling loop closures at t = 0)
struct Xf { double R[9], p[3]; };
Xf compose(const Xf& A, const Xf& B) {
    Xf C;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            C.R[3 * i + j] = A.R[3 * i] * B.R[j] + A.R[3 * i + 1] * B.R[3 + j] + A.R[3 * i + 2] * B.R[6 + j];
    for (int i = 0; i < 3; ++i)
        C.p[i] = A.R[3 * i] * B.p[0] + A.R[3 * i + 1] * B.p[1] + A.R[3 * i + 2] * B.p[2] + A.p[i];
    return C;
}
Xf fromArr(const double* X) { Xf x; std::memcpy(x.R, X, 9 * sizeof(double)); std::memcpy(x.p, X + 9, 3 * sizeof(double)); return x; }
Xf inverse(const Xf& A) {
    Xf B;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) B.R[3 * i + j] = A.R[3 * j + i];
    for (int i = 0; i < 3; ++i) B.p[i] = -(B.R[3 * i] * A.p[0] + B.R[3 * i + 1] * A.p[1] + B.R[3 * i + 2] * A.p[2]);
    return B;
}
Xf jointX(int mob, const double* q, bool euler) {
    Xf X;
    std::memset(&X, 0, sizeof X);
    X.R[0] = X.R[4] = X.R[8] = 1;
    if (euler && (mob == SBG_BALL || mob == SBG_FREE)) {
        // body-fixed X-Y-Z angles: R = Rx(q0) Ry(q1) Rz(q2)
        const double c0 = std::cos(q[0]), s0 = std::sin(q[0]), c1 = std::cos(q[1]), s1 = std::sin(q[1]),
                     c2 = std::cos(q[2]), s2 = std::sin(q[2]);
        const double R[9] = {c1 * c2, -c1 * s2, s1,
                             c0 * s2 + s0 * s1 * c2, c0 * c2 - s0 * s1 * s2, -s0 * c1,
                             s0 * s2 - c0 * s1 * c2, s0 * c2 + c0 * s1 * s2, c0 * c1};
        std::memcpy(X.R, R, sizeof R);
        if (mob == SBG_FREE) { X.p[0] = q[3]; X.p[1] = q[4]; X.p[2] = q[5]; }
    } else if (mob == SBG_PIN) {
        const double c = std::cos(q[0]), s = std::sin(q[0]);
        X.R[0] = c; X.R[1] = -s; X.R[3] = s; X.R[4] = c;
    } else if (mob == SBG_SLIDER) {
        X.p[0] = q[0];
    } else if (mob == SBG_UNIVERSAL) {
        const double c1 = std::cos(q[0]), s1 = std::sin(q[0]), c2 = std::cos(q[1]), s2 = std::sin(q[1]);
        const double R[9] = {c2, 0, s2, s2 * s1, c1, -s1 * c2, -s2 * c1, s1, c1 * c2};
        std::memcpy(X.R, R, sizeof R);
    } else {
        const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
        const double w = q[0] / n, x = q[1] / n, y = q[2] / n, z = q[3] / n;
        const double R[9] = {w * w + x * x - y * y - z * z, 2 * (x * y - w * z), 2 * (x * z + w * y),
                             2 * (x * y + w * z), w * w - x * x + y * y - z * z, 2 * (y * z - w * x),
                             2 * (x * z - w * y), 2 * (y * z + w * x), w * w - x * x - y * y + z * z};
        std::memcpy(X.R, R, sizeof R);
        if (mob == SBG_FREE) { X.p[0] = q[4]; X.p[1] = q[5]; X.p[2] = q[6]; }
    }
    return X;
}
std::vector<Xf> bodyTransforms(const Sys& s, const double* q) {
    const int nb = (int)s.bodies.size();
    std::vector<Xf> X(nb + 1);
    X[0] = fromArr(std::vector<double>{1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0}.data());
    int qo = 0;
    for (int i = 1; i <= nb; ++i) {
        const sbg_body_desc& b = s.bodies[i - 1];
        const Xf X_PB = compose(compose(fromArr(b.X_PF), jointX(b.mobilizer, q + qo, s.euler)), inverse(fromArr(b.X_BM)));
        X[i] = compose(X[b.parent], X_PB);
        qo += nq_of(b.mobilizer);
    }
    return X;
}

// 20% of serving requests get 1..4 Ball closures from a deep body to Ground,
// with the Ground station at the body station's t = 0 location.
void addLoops(std::mt19937_64& r, Sys& s, const double* q, bool always = false, int maxLoops = 4) {
    std::uniform_real_distribution<double> U01(0, 1), UP(-0.05, 0.05);
    if (!always && U01(r) >= 0.2) return;
    std::uniform_int_distribution<int> nl(1, maxLoops);
    int want = nl(r);
    const int nb = (int)s.bodies.size();
    // depth and dofs along the path from Ground
    std::vector<int> pathDof(nb + 1, 0);
    for (int i = 1; i <= nb; ++i) pathDof[i] = pathDof[s.bodies[i - 1].parent] + nu_of(s.bodies[i - 1].mobilizer);
    // Each closure removes 3 dofs; keep at least 3 free dofs per closure and
    // never close two loops through the same body.
    int totalDof = 0;
    for (int i = 1; i <= nb; ++i) totalDof += nu_of(s.bodies[i - 1].mobilizer);
    want = std::min(want, std::max(0, (totalDof - 6) / 6));
    if (want == 0) return;
    std::vector<int> cand;
    for (int i = 2; i <= nb; ++i)
        if (pathDof[i] >= 9) cand.push_back(i);
    const std::vector<Xf> X = bodyTransforms(s, q);
    for (int l = 0; l < want && !cand.empty(); ++l) {
        std::uniform_int_distribution<int> pick(0, (int)cand.size() - 1);
        const int k = pick(r);
        const int b = cand[k];
        cand.erase(cand.begin() + k);
        sbg_ball_constraint_desc c;
        std::memset(&c, 0, sizeof c);
        c.body1 = b;
        c.body2 = 0;
        for (int j = 0; j < 3; ++j) c.station1[j] = UP(r);
        const Xf& Xb = X[b];
        for (int j = 0; j < 3; ++j)
            c.station2[j] = Xb.R[3 * j] * c.station1[0] + Xb.R[3 * j + 1] * c.station1[1] + Xb.R[3 * j + 2] * c.station1[2] + Xb.p[j];
        s.cons.push_back(c);
    }
}

// Workload 10: every tree closed by one or two Ball closures to Ground, then
// made redundant (kind = instance % 3): 0 repeats the first closure exactly
// (G M^-1 G^T loses rank 3), 1 pins a second point of the first closure's body
// (two points fix all but the rotation about the line through them: 6
// equations of rank 5), 2 does both. The added closures hold at t = 0.
void addRedundantLoops(std::mt19937_64& r, Sys& s, const double* q, int kind) {
    addLoops(r, s, q, true, 2);
    if (s.cons.empty()) return;
    const sbg_ball_constraint_desc c0 = s.cons[0];
    if (kind != 1) s.cons.push_back(c0);
    if (kind != 0) {
        std::uniform_real_distribution<double> UA(0.1, 0.2), US(-1, 1);
        sbg_ball_constraint_desc c = c0;
        double dir[3], n = 0;
        for (int j = 0; j < 3; ++j) { dir[j] = US(r); n += dir[j] * dir[j]; }
        n = std::sqrt(n);
        const double len = UA(r);
        for (int j = 0; j < 3; ++j) c.station1[j] = c0.station1[j] + len * dir[j] / n;
        const Xf& Xb = bodyTransforms(s, q)[c0.body1];
        for (int j = 0; j < 3; ++j)
            c.station2[j] = Xb.R[3 * j] * c.station1[0] + Xb.R[3 * j + 1] * c.station1[1] + Xb.R[3 * j + 2] * c.station1[2] + Xb.p[j];
        s.cons.push_back(c);
    }
}

// Workload 8: a contact sphere on every body and a ground half-space,
// slightly tilted, whose contact normal (the half-space frame's x axis)
// points down into it and whose surface lies so that the lowest sphere is
// indented by 3 mm at t = 0. Parameters in the range of gait models (Hertz
// stiffness 1e6, Hunt-Crossley dissipation 2, static / dynamic / viscous
// friction 0.8 / 0.5 / 0.1, transition velocity 0.2: with viscous friction
// 0.5 a few light bodies' friction is too stiff for the fixed step of 5e-4 s);
// every eighth instance leaves the parameter block zero, which stands for the
// reference's defaults.
void addContacts(std::mt19937_64& r, Sys& s, const double* q, bool defaults) {
    std::uniform_real_distribution<double> UP(-0.05, 0.05), UR(0.02, 0.06), UT(-0.2, 0.2);
    const int nb = (int)s.bodies.size();
    const std::vector<Xf> X = bodyTransforms(s, q);
    const double th = -kPi / 2 + UT(r);
    const double c = std::cos(th), sn = std::sin(th);
    const double nrm[3] = {c, sn, 0};
    double lowest = 1e300;
    for (int b = 1; b <= nb; ++b) {
        sbg_contact_desc k;
        std::memset(&k, 0, sizeof k);
        k.body = b;
        for (int j = 0; j < 3; ++j) k.station[j] = UP(r);
        k.radius = UR(r);
        const Xf& Xb = X[b];
        double ctr[3];
        for (int j = 0; j < 3; ++j)
            ctr[j] = Xb.R[3 * j] * k.station[0] + Xb.R[3 * j + 1] * k.station[1] + Xb.R[3 * j + 2] * k.station[2] + Xb.p[j];
        lowest = std::min(lowest, -(ctr[0] * nrm[0] + ctr[1] * nrm[1] + ctr[2] * nrm[2]) - k.radius);
        if (!defaults) {
            k.stiffness = 1e6; k.dissipation = 2; k.static_friction = 0.8; k.dynamic_friction = 0.5;
            k.viscous_friction = 0.1; k.transition_velocity = 0.2; k.cf = 1e-5; k.bd = 300; k.bv = 50;
        }
        s.contacts.push_back(k);
    }
    // rotation about z by th (row-major), origin at depth d along the normal
    const double d = -0.003 - lowest;
    for (auto& k : s.contacts) {
        const double R[9] = {c, -sn, 0, sn, c, 0, 0, 0, 1};
        for (int j = 0; j < 9; ++j) k.halfspace[j] = R[j];
        for (int j = 0; j < 3; ++j) k.halfspace[9 + j] = d * nrm[j];
    }
}

}  // namespace

extern "C" {

const char* sbg_workload_last_error(void) { return g_wl_err.c_str(); }

int sbg_workload_create(int32_t config, int32_t ninstances, sbg_workload* out) {
    if (!out || ninstances < 0 || config < 1 || config > 10) { g_wl_err = "bad workload arguments"; return SBG_ERR_INVALID; }
    auto* w = new sbg_workload_s();
    w->config = config;
    w->y_off.push_back(0);
    if (config == 1) {
        Sys s;
        const double G[6] = {1, 1, 1, 0, 0, 0};
        const double z[3] = {0, 0, 0}, pBM[3] = {0, 1, 0};
        s.bodies.push_back(makeBody(0, SBG_PIN, 1.0, G, z, pBM));
        s.bodies.push_back(makeBody(1, SBG_PIN, 1.0, G, z, pBM));
        w->sys.push_back(s);
        w->h = 1e-3;
        w->nsteps = 1000;
        for (int32_t i = 0; i < ninstances; ++i) {
            std::mt19937_64 r((1ull << 32) | (uint64_t)i);
            std::uniform_real_distribution<double> U(-kPi, kPi);
            std::normal_distribution<double> N(0, 1);
            double q[2], u[2];
            for (int k = 0; k < 2; ++k) { q[k] = U(r); u[k] = N(r); }
            w->y0.insert(w->y0.end(), {q[0], q[1], u[0], u[1]});
            w->inst_sys.push_back(0);
            w->y_off.push_back((int64_t)w->y0.size());
        }
    } else if (config == 2) {
        Sys s;
        std::mt19937_64 r(2);
        std::lognormal_distribution<double> LN(0, 0.5);
        std::uniform_real_distribution<double> US(0.05, 0.3);
        const double z[3] = {0, 0, 0}, pBM[3] = {0, 0.1, 0};
        for (int i = 1; i <= 32; ++i) {
            const double m = LN(r);
            const double a = US(r), b = US(r), c = US(r);
            double G[6];
            brick(a, b, c, G);
            s.bodies.push_back(makeBody(i - 1, SBG_BALL, m, G, z, pBM));
        }
        w->sys.push_back(s);
        for (int32_t i = 0; i < ninstances; ++i) {
            std::mt19937_64 rr((2ull << 32) | (uint64_t)i);
            std::normal_distribution<double> Nu(0, 0.5);
            for (int b = 0; b < 32; ++b) {
                double qq[4];
                randomUnitQuat(rr, qq);
                w->y0.insert(w->y0.end(), qq, qq + 4);
            }
            for (int k = 0; k < 96; ++k) w->y0.push_back(Nu(rr));
            w->inst_sys.push_back(0);
            w->y_off.push_back((int64_t)w->y0.size());
        }
    } else {
        w->h = 5e-4;
        w->nsteps = config == 4 || config == 5 ? 1000 : 2000;
        std::uniform_int_distribution<int> n34(20, 40);
        std::uniform_real_distribution<double> ULogN(std::log(4.0), std::log(256.0));
        std::uniform_real_distribution<double> ULogH(std::log(100.0), std::log(10000.0));
        std::exponential_distribution<double> inter(2000.0);
        double tArr = 0;
        for (int32_t i = 0; i < ninstances; ++i) {
            std::mt19937_64 r(((uint64_t)config << 32) | (uint64_t)i);
            int nb = 0;
            if (config == 3 || config >= 6) nb = n34(r);
            else nb = (int)std::lround(std::exp(ULogN(r)));
            nb = std::max(4, std::min(256, nb));
            Sys s;
            std::vector<double> y;
            if (config == 6) randomTree(r, nb, s, y, true, (i & 1) ? SBG_BUSHING : SBG_FREE);
            else if (config == 7 || config == 9) randomTree(r, nb, s, y, false, SBG_FREE, true);
            else randomTree(r, nb, s, y);
            if (config == 7 || config == 9) {
                s.flags = SBG_SYSTEM_EULER_ANGLES;
                s.euler = true;
            }
            if (config == 9) addLoops(r, s, y.data());
            if (config == 10) addRedundantLoops(r, s, y.data(), (int)(i % 3));
            if (config == 8) addContacts(r, s, y.data(), (i & 7) == 7);
            if (config == 5) {
                addLoops(r, s, y.data());
                w->horizon.push_back((int32_t)std::lround(std::exp(ULogH(r))));
                tArr += inter(r);
                w->arrival.push_back(tArr);
            }
            w->sys.push_back(s);
            w->inst_sys.push_back(i);
            w->y0.insert(w->y0.end(), y.begin(), y.end());
            w->y_off.push_back((int64_t)w->y0.size());
        }
    }
    for (auto& s : w->sys) {
        sbg_system_desc d;
        std::memset(&d, 0, sizeof d);
        d.nbodies = (int32_t)s.bodies.size();
        d.nforces = (int32_t)s.forces.size();
        d.nconstraints = (int32_t)s.cons.size();
        d.flags = s.flags;
        for (int k = 0; k < 3; ++k) d.gravity[k] = s.gravity[k];
        d.bodies = s.bodies.data();
        d.forces = s.forces.empty() ? nullptr : s.forces.data();
        d.constraints = s.cons.empty() ? nullptr : s.cons.data();
        d.ncontacts = (int32_t)s.contacts.size();
        d.contacts = s.contacts.empty() ? nullptr : s.contacts.data();
        w->desc.push_back(d);
    }
    *out = w;
    return SBG_OK;
}

int sbg_workload_destroy(sbg_workload w) { delete w; return SBG_OK; }
int32_t sbg_workload_num_systems(sbg_workload w) { return (int32_t)w->desc.size(); }
int32_t sbg_workload_num_instances(sbg_workload w) { return (int32_t)w->inst_sys.size(); }
const sbg_system_desc* sbg_workload_systems(sbg_workload w) { return w->desc.data(); }
const int32_t* sbg_workload_instance_system(sbg_workload w) { return w->inst_sys.data(); }
const int64_t* sbg_workload_y_offsets(sbg_workload w) { return w->y_off.data(); }
const double* sbg_workload_y0(sbg_workload w) { return w->y0.data(); }
double sbg_workload_h(sbg_workload w) { return w->h; }
int32_t sbg_workload_nsteps(sbg_workload w) { return w->nsteps; }
const int32_t* sbg_workload_horizons(sbg_workload w) { return w->horizon.empty() ? nullptr : w->horizon.data(); }
const double* sbg_workload_arrivals(sbg_workload w) { return w->arrival.empty() ? nullptr : w->arrival.data(); }

}  // extern "C"
