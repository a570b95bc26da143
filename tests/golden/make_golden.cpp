// make_golden.cpp -- writes golden input/output vectors for the hot path by
// running a built Simbody (the reference) on the seeded synthetic workloads.
//
// Built and run by make_golden.py next to this file; it is not part of the
// library and nothing at test time compiles or runs it. For each selected
// instance of the workload configs it records:
//   y0                      the seeded state (from libsbg_workloads)
//   ydot                    System::realize(s, Stage::Acceleration); s.getYDot()
//   f, minv_f               SimbodyMatterSubsystem::multiplyByMInv(s, f, out)
//   y_rk, t_rk              RungeKuttaMersonIntegrator with setFixedStepSize(h),
//                           default accuracy, the default constraint tolerance
//                           or cons_tol when it is nonzero (tight tolerances
//                           make the in-step projections run), stepped for
//                           exactly nsteps steps
//   qdd                     s.getQDotDot() after the realize above
//   adapter_gdev            the Simbody-side adapter (simbody_gb300_simtk.hpp)
//                           reads the built system back into descriptors: all
//                           fields equal the workload's bit for bit (else the
//                           run stops), gravity to this relative deviation
// and, into a second file, integrator continuation records: with
// setFixedStepSize(h) and setAllowInterpolation(false), after initialize(s)
//   mode 0  stepTo(t_mid); stepTo(t_end)     (a second call continues)
//   mode 1  stepTo(t_end)
//   mode 2  stepTo(t_end + 0.3 h)            (a shortened last step)
// and, into a third file, error-controlled records: a RungeKuttaMersonIntegrator
// with the given accuracy, setFinalTime(t_final), initialize(s) and stepTo
// looped until t_final, with the numbers of steps taken and attempted;
// and, into a fourth, the number of systems outside the GPU path (one
// unsupported element each) that the Simbody-side adapter refused.
// Reference calls used (paths relative to the Simbody source tree):
//   MobilizedBody::{Pin,Slider,Universal,Ball,Free} (Simbody/include/simbody/internal/MobilizedBody_*.h)
//   Force::Gravity, Force::MobilityLinearSpring/Damper (Simbody/include/simbody/internal/Force*.h)
//   Constraint::Ball (Simbody/include/simbody/internal/Constraint_Ball.h)
//   SmoothSphereHalfSpaceForce (Simbody/include/simbody/internal/SmoothSphereHalfSpaceForce.h)
//   RungeKuttaMersonIntegrator (SimTKmath/Integrators/include/simmath/RungeKuttaMersonIntegrator.h)
//
// Output: one binary file of records
//   int64 cfg, inst, ny, nu, nsteps, status   double h, t_rk, cons_tol, adapter_gdev
//   double y0[ny], ydot[ny], f[nu], minv_f[nu], y_rk[ny], qdd[ny - nu]
// and a second of continuation records
//   int64 cfg, inst, ny, mode, status, nsteps_taken   double h, t_mid, t_end, t_out
//   double y0[ny], y_out[ny]
// and a third of error-controlled records
//   int64 cfg, inst, ny, status, steps_taken, steps_attempted   double accuracy, t_final, t_out
//   double y0[ny], y_out[ny]
#include "Simbody.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "sbg_workloads.h"
#include "simbody_gb300_simtk.hpp"

using namespace SimTK;

namespace {

Transform toTransform(const double* x) { return sbg::simtk::unpackTransform(x); }

// One MultibodySystem per described system; body index 0 is Ground and body
// k >= 1 is desc.bodies[k-1].
struct Model {
    MultibodySystem sys;
    SimbodyMatterSubsystem matter;
    GeneralForceSubsystem forces;
    std::vector<MobilizedBody> mobods;
    sbg::simtk::ForceLog log;  // the elements whose parameters Simbody does not expose

    explicit Model(const sbg_system_desc& d) : matter(sys), forces(sys) {
        const Vec3 g(d.gravity[0], d.gravity[1], d.gravity[2]);
        Force::Gravity(forces, matter, UnitVec3(g), g.norm());
        mobods.push_back(matter.Ground());
        for (int i = 0; i < d.nbodies; ++i) {
            const sbg_body_desc& b = d.bodies[i];
            const UnitInertia G(b.unit_inertia[0], b.unit_inertia[1], b.unit_inertia[2], b.unit_inertia[3],
                                b.unit_inertia[4], b.unit_inertia[5]);
            Body::Rigid body(MassProperties(b.mass, Vec3(b.com[0], b.com[1], b.com[2]), G));
            MobilizedBody& P = mobods[b.parent];
            const Transform X_PF = toTransform(b.X_PF), X_BM = toTransform(b.X_BM);
            switch (b.mobilizer) {
            case SBG_PIN: mobods.push_back(MobilizedBody::Pin(P, X_PF, body, X_BM)); break;
            case SBG_SLIDER: mobods.push_back(MobilizedBody::Slider(P, X_PF, body, X_BM)); break;
            case SBG_UNIVERSAL: mobods.push_back(MobilizedBody::Universal(P, X_PF, body, X_BM)); break;
            case SBG_BALL: mobods.push_back(MobilizedBody::Ball(P, X_PF, body, X_BM)); break;
            case SBG_GIMBAL: mobods.push_back(MobilizedBody::Gimbal(P, X_PF, body, X_BM)); break;
            case SBG_TRANSLATION: mobods.push_back(MobilizedBody::Translation(P, X_PF, body, X_BM)); break;
            case SBG_CYLINDER: mobods.push_back(MobilizedBody::Cylinder(P, X_PF, body, X_BM)); break;
            case SBG_PLANAR: mobods.push_back(MobilizedBody::Planar(P, X_PF, body, X_BM)); break;
            case SBG_BUSHING: mobods.push_back(MobilizedBody::Bushing(P, X_PF, body, X_BM)); break;
            case SBG_WELD: mobods.push_back(MobilizedBody::Weld(P, X_PF, body, X_BM)); break;
            case SBG_SCREW: mobods.push_back(MobilizedBody::Screw(P, X_PF, body, X_BM, b.pitch)); break;
            default: mobods.push_back(MobilizedBody::Free(P, X_PF, body, X_BM)); break;
            }
        }
        for (int i = 0; i < d.nforces; ++i) {
            const sbg_mobility_force_desc& f = d.forces[i];
            if (f.kind == 0)
                log.addMobilityLinearSpring(forces, mobods[f.body], MobilizerQIndex(f.which), f.coef, f.q0);
            else
                log.addMobilityLinearDamper(forces, mobods[f.body], MobilizerUIndex(f.which), f.coef);
        }
        for (int i = 0; i < d.ncontacts; ++i) {
            const sbg_contact_desc& k = d.contacts[i];
            const double* par = &k.stiffness;
            sbg::simtk::ContactParameters p;
            bool zero = true;
            for (int j = 0; j < 9; ++j) {
                p[j] = par[j];
                zero = zero && par[j] == 0;
            }
            // a zero block keeps the force's own defaults
            log.addSmoothSphereHalfSpaceForce(forces, mobods[k.body], Vec3(k.station[0], k.station[1], k.station[2]),
                                              k.radius, matter.Ground(), toTransform(k.halfspace), zero ? nullptr : &p);
        }
        for (int i = 0; i < d.nconstraints; ++i) {
            const sbg_ball_constraint_desc& c = d.constraints[i];
            Constraint::Ball(mobods[c.body1], Vec3(c.station1[0], c.station1[1], c.station1[2]), mobods[c.body2],
                             Vec3(c.station2[0], c.station2[1], c.station2[2]));
        }
        sys.realizeTopology();
        euler = (d.flags & SBG_SYSTEM_EULER_ANGLES) != 0;
    }
    bool euler = false;
    // The default state with the system's model-stage choices applied
    // (SimbodyMatterSubsystem::setUseEulerAngles).
    State defaultState() {
        State st = sys.getDefaultState();
        if (euler) {
            matter.setUseEulerAngles(st, true);
            sys.realizeModel(st);
        }
        return st;
    }
};

// The Simbody-side adapter (include/simbody_gb300_simtk.hpp) reads the
// built system back into descriptors; they must equal the ones it was built
// from, every field bit for bit except gravity, which Force::Gravity keeps as
// a unit direction and a magnitude. Returns gravity's relative deviation;
// exits on any other difference.
double adapterRoundTrip(const sbg_system_desc& d, Model& m, int cfg, int inst) {
    const State st = m.defaultState();
    const sbg::simtk::SystemDescription a = sbg::simtk::describe(m.matter, m.forces, m.log, st);
    const sbg_system_desc& e = a.desc;
    int bad = 0;
    auto same = [&](const double* x, const double* y, int n) {
        for (int k = 0; k < n; ++k) bad += x[k] != y[k];
    };
    bad += e.nbodies != d.nbodies || e.nforces != d.nforces || e.nconstraints != d.nconstraints ||
           e.ncontacts != d.ncontacts || e.flags != d.flags;
    if (!bad) {
        for (int i = 0; i < d.nbodies; ++i) {
            const sbg_body_desc &x = e.bodies[i], &y = d.bodies[i];
            bad += x.parent != y.parent || x.mobilizer != y.mobilizer || x.mass != y.mass;
            same(x.com, y.com, 3);
            same(x.unit_inertia, y.unit_inertia, 6);
            same(x.X_PF, y.X_PF, 12);
            same(x.X_BM, y.X_BM, 12);
            if (y.mobilizer == SBG_SCREW) bad += x.pitch != y.pitch;
        }
        for (int i = 0; i < d.nforces; ++i) {
            const sbg_mobility_force_desc &x = e.forces[i], &y = d.forces[i];
            bad += x.kind != y.kind || x.body != y.body || x.which != y.which || x.coef != y.coef;
            if (y.kind == 0) bad += x.q0 != y.q0;
        }
        for (int i = 0; i < d.nconstraints; ++i) {
            const sbg_ball_constraint_desc &x = e.constraints[i], &y = d.constraints[i];
            bad += x.body1 != y.body1 || x.body2 != y.body2;
            same(x.station1, y.station1, 3);
            same(x.station2, y.station2, 3);
        }
        for (int i = 0; i < d.ncontacts; ++i) {
            const sbg_contact_desc &x = e.contacts[i], &y = d.contacts[i];
            bad += x.body != y.body || x.radius != y.radius;
            same(x.station, y.station, 3);
            same(x.halfspace, y.halfspace, 12);
            same(&x.stiffness, &y.stiffness, 9);
        }
    }
    if (bad) {
        fprintf(stderr, "cfg %d inst %d: the adapter's descriptors differ in %d fields\n", cfg, inst, bad);
        std::exit(1);
    }
    double gn = 0, dn = 0;
    for (int k = 0; k < 3; ++k) {
        gn += d.gravity[k] * d.gravity[k];
        dn += (e.gravity[k] - d.gravity[k]) * (e.gravity[k] - d.gravity[k]);
    }
    return gn > 0 ? std::sqrt(dn / gn) : std::sqrt(dn);
}

// describe() must refuse what the GPU path does not cover. Each case is a
// two-Pin pendulum plus one such element; returns how many were refused
// (exits if one is not).
int adapterRefusals() {
    int refused = 0;
    for (int c = 0; c < 6; ++c) {
        MultibodySystem sys;
        SimbodyMatterSubsystem matter(sys);
        GeneralForceSubsystem forces(sys);
        sbg::simtk::ForceLog log;
        Force::Gravity gravity(forces, matter, -YAxis, 9.8);
        Body::Rigid body(MassProperties(1.0, Vec3(0), UnitInertia(1)));
        MobilizedBody::Pin b1(matter.Ground(), Transform(), body, Transform(Vec3(0, 1, 0)));
        MobilizedBody::Pin b2(b1, Transform(), body, Transform(Vec3(0, 1, 0)));
        const char* what = "";
        switch (c) {
        case 0: Force::TwoPointLinearSpring(forces, b1, Vec3(0), b2, Vec3(0), 1.0, 0.5); what = "a two-point spring"; break;
        case 1: Force::MobilityLinearSpring(forces, b1, MobilizerQIndex(0), 1.0, 0.0); what = "a spring outside the log"; break;
        case 2: gravity.setDefaultBodyIsExcluded(b2, true); what = "gravity excluding a body"; break;
        case 3: log.addSmoothSphereHalfSpaceForce(forces, b2, Vec3(0), 0.1, b1, Transform()); what = "a moving half-space"; break;
        case 4: Constraint::Rod(b1, Vec3(0), b2, Vec3(0.1, 0, 0), 1.0); what = "a Rod constraint"; break;
        default: MobilizedBody::Ellipsoid(b2, Transform(), body, Transform()); what = "an Ellipsoid mobilizer"; break;
        }
        sys.realizeTopology();
        const State st = sys.getDefaultState();
        try {
            sbg::simtk::describe(matter, forces, log, st);
        } catch (const std::runtime_error&) {
            ++refused;
            continue;
        }
        fprintf(stderr, "the adapter took %s\n", what);
        std::exit(1);
    }
    return refused;
}

void put(FILE* fp, const void* p, size_t bytes) {
    if (fwrite(p, 1, bytes, fp) != bytes) {
        fprintf(stderr, "write failed\n");
        std::exit(1);
    }
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: make_golden OUT.bin CONT.bin ADAPT.bin REFUSALS.txt\n");
        return 2;
    }
    FILE* fp = fopen(argv[1], "wb");
    if (!fp) return 1;
    FILE* fc = fopen(argv[2], "wb");
    if (!fc) return 1;
    struct Sel { int cfg, ninst, nsteps; double h; std::vector<int> pick; double consTol; };
    // cfgs 5 and 9 draw 1-4 Ball loops for about one tree in five; for an
    // empty list, four instances that carry loops and two that do not.
    const Sel sels[] = {
        {1, 8, 1000, 1e-3, {0, 1, 2, 3}, 0},
        {1, 8, 20, 1e-3, {4, 5, 6, 7}, 0},
        {2, 4, 20, 5e-4, {0, 1, 2, 3}, 0},
        {3, 6, 20, 5e-4, {0, 1, 2, 3, 4, 5}, 0},
        {4, 8, 20, 5e-4, {0, 1, 2, 3, 4, 5, 6, 7}, 0},
        {5, 64, 20, 5e-4, {}, 0},
        {5, 64, 200, 5e-4, {}, 1e-9},
        {6, 8, 20, 5e-4, {0, 1, 2, 3, 4, 5, 6, 7}, 0},
        {7, 6, 20, 5e-4, {0, 1, 2, 3, 4, 5}, 0},
        {8, 8, 20, 5e-4, {0, 1, 2, 3, 4, 5, 6, 7}, 0},
        {8, 8, 400, 5e-4, {0, 1}, 0},
        {9, 64, 20, 5e-4, {}, 0},
        {9, 64, 100, 2e-3, {}, 1e-9},
        {10, 6, 20, 5e-4, {0, 1, 2, 3, 4, 5}, 0},
        {10, 6, 100, 2e-3, {0, 1, 2, 3, 4, 5}, 1e-9},
    };
    int written = 0;
    for (const Sel& s : sels) {
        sbg_workload w;
        if (sbg_workload_create(s.cfg, s.ninst, &w)) {
            fprintf(stderr, "workload %d: %s\n", s.cfg, sbg_workload_last_error());
            return 1;
        }
        const sbg_system_desc* systems = sbg_workload_systems(w);
        const int32_t* isys = sbg_workload_instance_system(w);
        const int64_t* yo = sbg_workload_y_offsets(w);
        const double* y0 = sbg_workload_y0(w);
        std::vector<int> pick = s.pick;
        if (pick.empty()) {  // configs 5 and 9: four instances with loops and two without
            int withLoops = 0, without = 0;
            for (int i = 0; i < s.ninst; ++i) {
                const bool loops = systems[isys[i]].nconstraints > 0;
                if (loops && withLoops < 4) { pick.push_back(i); ++withLoops; }
                if (!loops && without < 2) { pick.push_back(i); ++without; }
            }
        }
        for (int i : pick) {
            const sbg_system_desc& d = systems[isys[i]];
            Model m(d);
            const double gdev = adapterRoundTrip(d, m, s.cfg, i);
            const int64_t ny = yo[i + 1] - yo[i];
            int64_t status = 0;
            State st = m.defaultState();
            if (st.getNY() != ny) {
                fprintf(stderr, "cfg %d inst %d: ny %d != %lld\n", s.cfg, i, st.getNY(), (long long)ny);
                return 1;
            }
            const int64_t nu = st.getNU();
            sbg::simtk::setY(&y0[yo[i]], st);
            std::vector<double> ydot(ny), f(nu), minv(nu), yrk(ny);
            m.sys.realize(st, Stage::Acceleration);
            for (int k = 0; k < ny; ++k) ydot[k] = st.getYDot()[k];
            std::vector<double> qdd(ny - nu);
            for (int k = 0; k < ny - nu; ++k) qdd[k] = st.getQDotDot()[k];
            Vector fv((int)nu), out;
            for (int k = 0; k < nu; ++k) fv[k] = f[k] = std::cos(0.7 * k + 0.3 * i + s.cfg);
            m.matter.multiplyByMInv(st, fv, out);
            for (int k = 0; k < nu; ++k) minv[k] = out[k];
            double trk = 0;
            try {
                State s2 = m.defaultState();
                sbg::simtk::setY(&y0[yo[i]], s2);
                RungeKuttaMersonIntegrator integ(m.sys);
                integ.setFixedStepSize(s.h);
                integ.setReturnEveryInternalStep(true);
                if (s.consTol > 0) integ.setConstraintTolerance(s.consTol);
                integ.initialize(s2);
                while (integ.getNumStepsTaken() < s.nsteps) integ.stepTo(1e9);
                sbg::simtk::getY(integ.getState(), yrk.data());
                trk = integ.getTime();
            } catch (const std::exception& e) {
                fprintf(stderr, "cfg %d inst %d: integrator failed: %s\n", s.cfg, i, e.what());
                status = 1;
            }
            const int64_t hdr[6] = {s.cfg, i, ny, nu, s.nsteps, status};
            const double hd[4] = {s.h, trk, s.consTol, gdev};
            put(fp, hdr, sizeof hdr);
            put(fp, hd, sizeof hd);
            put(fp, &y0[yo[i]], ny * 8);
            put(fp, ydot.data(), ny * 8);
            put(fp, f.data(), nu * 8);
            put(fp, minv.data(), nu * 8);
            put(fp, yrk.data(), ny * 8);
            put(fp, qdd.data(), (ny - nu) * 8);
            ++written;
        }
        sbg_workload_destroy(w);
    }
    fclose(fp);

    // integrator continuation: one or two stepTo calls, interpolation off
    struct ContSel { int cfg, ninst; double h, tMid, tEnd; std::vector<int> pick; };
    const ContSel cont[] = {
        {1, 8, 1e-3, 0.5, 1.0, {0, 1}},
        {2, 4, 5e-4, 0.005, 0.01, {0, 1}},
        {3, 6, 5e-4, 0.005, 0.01, {0, 1}},
        {4, 8, 5e-4, 0.005, 0.01, {2, 3}},
        {5, 64, 5e-4, 0.005, 0.01, {}},
        {8, 8, 5e-4, 0.005, 0.01, {0, 7}},
    };
    int contWritten = 0;
    for (const ContSel& c : cont) {
        sbg_workload w;
        if (sbg_workload_create(c.cfg, c.ninst, &w)) {
            fprintf(stderr, "workload %d: %s\n", c.cfg, sbg_workload_last_error());
            return 1;
        }
        const sbg_system_desc* systems = sbg_workload_systems(w);
        const int32_t* isys = sbg_workload_instance_system(w);
        const int64_t* yo = sbg_workload_y_offsets(w);
        const double* y0 = sbg_workload_y0(w);
        std::vector<int> pick = c.pick;
        if (pick.empty()) {  // config 5: two requests with loop closures, one without
            int withLoops = 0, without = 0;
            for (int i = 0; i < c.ninst; ++i) {
                const bool loops = systems[isys[i]].nconstraints > 0;
                if (loops && withLoops < 2) { pick.push_back(i); ++withLoops; }
                if (!loops && without < 1) { pick.push_back(i); ++without; }
            }
        }
        for (int i : pick) {
            const sbg_system_desc& d = systems[isys[i]];
            Model m(d);
            const int64_t ny = yo[i + 1] - yo[i];
            for (int mode = 0; mode < 3; ++mode) {
                int64_t status = 0, taken = 0;
                std::vector<double> yout(ny, 0.0);
                double tout = 0;
                try {
                    State s2 = m.defaultState();
                    sbg::simtk::setY(&y0[yo[i]], s2);
                    RungeKuttaMersonIntegrator integ(m.sys);
                    integ.setFixedStepSize(c.h);
                    integ.setAllowInterpolation(false);
                    integ.initialize(s2);
                    auto to = [&](double t) { while (integ.getTime() < t) integ.stepTo(t); };
                    if (mode == 0) { to(c.tMid); to(c.tEnd); }
                    else if (mode == 1) to(c.tEnd);
                    else to(c.tEnd + 0.3 * c.h);
                    sbg::simtk::getY(integ.getState(), yout.data());
                    tout = integ.getTime();
                    taken = integ.getNumStepsTaken();
                } catch (const std::exception& e) {
                    fprintf(stderr, "cfg %d inst %d mode %d: integrator failed: %s\n", c.cfg, i, mode, e.what());
                    status = 1;
                }
                const int64_t hdr[6] = {c.cfg, i, ny, mode, status, taken};
                const double hd[4] = {c.h, c.tMid, c.tEnd, tout};
                put(fc, hdr, sizeof hdr);
                put(fc, hd, sizeof hd);
                put(fc, &y0[yo[i]], ny * 8);
                put(fc, yout.data(), ny * 8);
                ++contWritten;
            }
        }
        sbg_workload_destroy(w);
    }
    fclose(fc);

    // error-controlled integration
    FILE* fa = fopen(argv[3], "wb");
    if (!fa) return 1;
    struct AdaptSel { int cfg, ninst; double acc, tFinal; std::vector<int> pick; };
    const AdaptSel adapt[] = {
        {1, 8, 1e-3, 1.0, {0, 1}},
        {1, 8, 1e-6, 0.5, {2}},
        {2, 4, 1e-3, 0.05, {0, 1}},
        {3, 6, 1e-3, 0.05, {0, 1, 2}},
        {3, 6, 1e-5, 0.02, {3}},
        {4, 8, 1e-3, 0.03, {2, 3}},
        {6, 8, 1e-3, 0.03, {0, 1}},
        {7, 6, 1e-3, 0.03, {0, 1}},
        {8, 8, 1e-3, 0.03, {0, 1}},
    };
    int adaptWritten = 0;
    for (const AdaptSel& c : adapt) {
        sbg_workload w;
        if (sbg_workload_create(c.cfg, c.ninst, &w)) {
            fprintf(stderr, "workload %d: %s\n", c.cfg, sbg_workload_last_error());
            return 1;
        }
        const sbg_system_desc* systems = sbg_workload_systems(w);
        const int32_t* isys = sbg_workload_instance_system(w);
        const int64_t* yo = sbg_workload_y_offsets(w);
        const double* y0 = sbg_workload_y0(w);
        for (int i : c.pick) {
            Model m(systems[isys[i]]);
            const int64_t ny = yo[i + 1] - yo[i];
            int64_t status = 0, taken = 0, attempted = 0;
            std::vector<double> yout(ny, 0.0);
            double tout = 0;
            try {
                State s2 = m.defaultState();
                sbg::simtk::setY(&y0[yo[i]], s2);
                RungeKuttaMersonIntegrator integ(m.sys);
                integ.setAccuracy(c.acc);
                integ.setFinalTime(c.tFinal);
                integ.initialize(s2);
                while (integ.getTime() < c.tFinal) integ.stepTo(c.tFinal);
                sbg::simtk::getY(integ.getState(), yout.data());
                tout = integ.getTime();
                taken = integ.getNumStepsTaken();
                attempted = integ.getNumStepsAttempted();
            } catch (const std::exception& e) {
                fprintf(stderr, "cfg %d inst %d: error-controlled integrator failed: %s\n", c.cfg, i, e.what());
                status = 1;
            }
            const int64_t hdr[6] = {c.cfg, i, ny, status, taken, attempted};
            const double hd[3] = {c.acc, c.tFinal, tout};
            put(fa, hdr, sizeof hdr);
            put(fa, hd, sizeof hd);
            put(fa, &y0[yo[i]], ny * 8);
            put(fa, yout.data(), ny * 8);
            ++adaptWritten;
        }
        sbg_workload_destroy(w);
    }
    fclose(fa);
    const int refusals = adapterRefusals();
    FILE* fr = fopen(argv[4], "w");
    if (!fr) return 1;
    fprintf(fr, "%d\n", refusals);
    fclose(fr);
    printf("%d records, %d continuation records, %d error-controlled records, %d adapter refusals\n", written,
           contWritten, adaptWritten, refusals);
    return 0;
}
