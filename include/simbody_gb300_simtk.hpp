// simbody_gb300_simtk.hpp -- Simbody (SimTK) side of the drop-in: reads a
// MultibodySystem into the C ABI's descriptors and moves State y vectors to
// and from the ABI's packing. Header-only C++17; include after "Simbody.h"
// and link Simbody as usual. The batch calls go through simbody_gb300.hpp
// (sbg::Topology, sbg::StateBatch, ...), which this header includes; the
// helpers at the end move batches of States through them.
//
//   sbg::simtk::ForceLog log;                          // next to the GeneralForceSubsystem
//   log.addMobilityLinearSpring(forces, mobod, MobilizerQIndex(0), k, q0);
//   ...
//   system.realizeTopology();
//   State s = system.getDefaultState();
//   sbg::simtk::SystemDescription d = sbg::simtk::describe(matter, forces, log, s);
//   sbg::Topology topo(d.desc);
//   sbg::simtk::getY(s, y.data() + offset);            // one instance of the batch
//
// What Simbody exposes through public getters is read from the system: every
// mobilized body (parent, mobilizer type, Screw pitch, default mass
// properties, X_PF, X_BM), Force::Gravity, each Constraint::Ball, and the
// bodies, station, radius and half-space frame of a SmoothSphereHalfSpaceForce.
// What it does not expose is recorded by ForceLog when the model builder
// creates the element through it: the mobilized body and coordinate of a
// Force::MobilityLinearSpring / MobilityLinearDamper and the parameters of a
// SmoothSphereHalfSpaceForce (MobilityLinearSpring.h, MobilityLinearDamper.h
// and SmoothSphereHalfSpaceForce.h have setters but no getters for those).
//
// describe() throws std::runtime_error for anything outside the GPU path: a
// mobilizer, force or constraint type it does not cover, a Gravity that
// excludes bodies, a spring, damper or contact force created without the log,
// a half-space not fixed in Ground, or a system with auxiliary (z) states.
#ifndef SIMBODY_GB300_SIMTK_HPP
#define SIMBODY_GB300_SIMTK_HPP

#include <array>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "simbody_gb300.hpp"

namespace sbg {
namespace simtk {

// Row-major 3x3 rotation followed by the translation, the ABI's transform.
inline void packTransform(const SimTK::Transform& X, double out[12]) {
    const SimTK::Mat33& R = X.R().asMat33();
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out[3 * i + j] = R(i, j);
    for (int k = 0; k < 3; ++k) out[9 + k] = X.p()[k];
}

// The inverse of packTransform; the rotation is taken as given (it must be
// orthonormal), as Rotation(Mat33, true) does.
inline SimTK::Transform unpackTransform(const double x[12]) {
    const SimTK::Mat33 R(x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7], x[8]);
    return SimTK::Transform(SimTK::Rotation(R, true), SimTK::Vec3(x[9], x[10], x[11]));
}

// The nine parameters of SmoothSphereHalfSpaceForce::setParameters in its
// order: stiffness, dissipation, static / dynamic / viscous friction,
// transition velocity, cf, bd, bv.
using ContactParameters = std::array<double, 9>;

// Creates the force elements whose descriptors Simbody does not expose, and
// records them by ForceIndex.
class ForceLog {
public:
    SimTK::Force::MobilityLinearSpring addMobilityLinearSpring(SimTK::GeneralForceSubsystem& forces,
                                                               const SimTK::MobilizedBody& mobod,
                                                               SimTK::MobilizerQIndex which, SimTK::Real stiffness,
                                                               SimTK::Real qZero) {
        SimTK::Force::MobilityLinearSpring f(forces, mobod, which, stiffness, qZero);
        sbg_mobility_force_desc d{};
        d.kind = 0;
        d.body = (int32_t)mobod.getMobilizedBodyIndex();
        d.which = (int32_t)which;
        d.coef = stiffness;
        d.q0 = qZero;
        mobility_[(int)f.getForceIndex()] = d;
        return f;
    }

    SimTK::Force::MobilityLinearDamper addMobilityLinearDamper(SimTK::GeneralForceSubsystem& forces,
                                                               const SimTK::MobilizedBody& mobod,
                                                               SimTK::MobilizerUIndex which, SimTK::Real damping) {
        SimTK::Force::MobilityLinearDamper f(forces, mobod, which, damping);
        sbg_mobility_force_desc d{};
        d.kind = 1;
        d.body = (int32_t)mobod.getMobilizedBodyIndex();
        d.which = (int32_t)which;
        d.coef = damping;
        mobility_[(int)f.getForceIndex()] = d;
        return f;
    }

    // A sphere on sphereBody against a half-space fixed in Ground (its frame's
    // x axis is the contact normal). params == nullptr keeps the force's own
    // defaults, which the ABI writes as an all-zero block.
    SimTK::SmoothSphereHalfSpaceForce addSmoothSphereHalfSpaceForce(SimTK::GeneralForceSubsystem& forces,
                                                                    const SimTK::MobilizedBody& sphereBody,
                                                                    const SimTK::Vec3& station, SimTK::Real radius,
                                                                    const SimTK::MobilizedBody& ground,
                                                                    const SimTK::Transform& halfSpaceFrame,
                                                                    const ContactParameters* params = nullptr) {
        SimTK::SmoothSphereHalfSpaceForce f(forces);
        f.setContactSphereBody(sphereBody);
        f.setContactSphereLocationInBody(station);
        f.setContactSphereRadius(radius);
        f.setContactHalfSpaceBody(ground);
        f.setContactHalfSpaceFrame(halfSpaceFrame);
        ContactParameters p{};
        if (params) {
            p = *params;
            f.setParameters(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8]);
        }
        contact_[(int)f.getForceIndex()] = p;
        return f;
    }

    const sbg_mobility_force_desc* mobility(SimTK::ForceIndex i) const {
        auto it = mobility_.find((int)i);
        return it == mobility_.end() ? nullptr : &it->second;
    }
    const ContactParameters* contact(SimTK::ForceIndex i) const {
        auto it = contact_.find((int)i);
        return it == contact_.end() ? nullptr : &it->second;
    }

private:
    std::map<int, sbg_mobility_force_desc> mobility_;
    std::map<int, ContactParameters> contact_;
};

// Owns the arrays desc points into; movable, not copyable (desc holds
// pointers into the vectors).
struct SystemDescription {
    std::vector<sbg_body_desc> bodies;
    std::vector<sbg_mobility_force_desc> forces;
    std::vector<sbg_ball_constraint_desc> constraints;
    std::vector<sbg_contact_desc> contacts;
    sbg_system_desc desc{};

    SystemDescription() = default;
    SystemDescription(const SystemDescription&) = delete;
    SystemDescription& operator=(const SystemDescription&) = delete;
    SystemDescription(SystemDescription&& o) noexcept { *this = std::move(o); }
    SystemDescription& operator=(SystemDescription&& o) noexcept {
        bodies = std::move(o.bodies);
        forces = std::move(o.forces);
        constraints = std::move(o.constraints);
        contacts = std::move(o.contacts);
        desc = o.desc;
        link();
        return *this;
    }
    void link() {
        desc.nbodies = (int32_t)bodies.size();
        desc.bodies = bodies.empty() ? nullptr : bodies.data();
        desc.nforces = (int32_t)forces.size();
        desc.forces = forces.empty() ? nullptr : forces.data();
        desc.nconstraints = (int32_t)constraints.size();
        desc.constraints = constraints.empty() ? nullptr : constraints.data();
        desc.ncontacts = (int32_t)contacts.size();
        desc.contacts = contacts.empty() ? nullptr : contacts.data();
    }
};

namespace detail {
inline int32_t mobilizerOf(const SimTK::MobilizedBody& mb) {
    using MB = SimTK::MobilizedBody;
    if (MB::Pin::isInstanceOf(mb)) return SBG_PIN;
    if (MB::Slider::isInstanceOf(mb)) return SBG_SLIDER;
    if (MB::Universal::isInstanceOf(mb)) return SBG_UNIVERSAL;
    if (MB::Ball::isInstanceOf(mb)) return SBG_BALL;
    if (MB::Free::isInstanceOf(mb)) return SBG_FREE;
    if (MB::Gimbal::isInstanceOf(mb)) return SBG_GIMBAL;
    if (MB::Translation::isInstanceOf(mb)) return SBG_TRANSLATION;
    if (MB::Cylinder::isInstanceOf(mb)) return SBG_CYLINDER;
    if (MB::Planar::isInstanceOf(mb)) return SBG_PLANAR;
    if (MB::Bushing::isInstanceOf(mb)) return SBG_BUSHING;
    if (MB::Weld::isInstanceOf(mb)) return SBG_WELD;
    if (MB::Screw::isInstanceOf(mb)) return SBG_SCREW;
    return -1;
}
[[noreturn]] inline void unsupported(const std::string& what) {
    throw std::runtime_error("simbody_gb300: " + what + " is outside the GPU path");
}
}  // namespace detail

// Reads the system behind matter and forces (realizeTopology done) into ABI
// descriptors. modelState supplies the model-stage choice of Euler angles
// (SimbodyMatterSubsystem::setUseEulerAngles) and must be realized to Model.
inline SystemDescription describe(const SimTK::SimbodyMatterSubsystem& matter,
                                  const SimTK::GeneralForceSubsystem& forces, const ForceLog& log,
                                  const SimTK::State& modelState) {
    SystemDescription out;
    if (modelState.getNZ() != 0) detail::unsupported("a system with auxiliary (z) states");
    for (SimTK::MobilizedBodyIndex i(1); i < matter.getNumBodies(); ++i) {
        const SimTK::MobilizedBody& mb = matter.getMobilizedBody(i);
        sbg_body_desc b{};
        b.parent = (int32_t)mb.getParentMobilizedBody().getMobilizedBodyIndex();
        b.mobilizer = detail::mobilizerOf(mb);
        if (b.mobilizer < 0) detail::unsupported("the mobilizer of body " + std::to_string((int)i));
        if (b.mobilizer == SBG_SCREW) b.pitch = SimTK::MobilizedBody::Screw::downcast(mb).getDefaultPitch();
        const SimTK::MassProperties& mp = mb.getDefaultMassProperties();
        b.mass = mp.getMass();
        for (int k = 0; k < 3; ++k) b.com[k] = mp.getMassCenter()[k];
        const SimTK::UnitInertia& G = mp.getUnitInertia();
        const SimTK::Vec3 mom = G.getMoments(), prod = G.getProducts();
        for (int k = 0; k < 3; ++k) {
            b.unit_inertia[k] = mom[k];
            b.unit_inertia[3 + k] = prod[k];
        }
        packTransform(mb.getDefaultInboardFrame(), b.X_PF);
        packTransform(mb.getDefaultOutboardFrame(), b.X_BM);
        out.bodies.push_back(b);
    }
    bool gravitySeen = false;
    for (SimTK::ForceIndex fi(0); fi < forces.getNumForces(); ++fi) {
        const SimTK::Force& f = forces.getForce(fi);
        if (f.isDisabledByDefault()) continue;
        if (SimTK::Force::Gravity::isInstanceOf(f)) {
            const SimTK::Force::Gravity& g = SimTK::Force::Gravity::downcast(f);
            if (gravitySeen) detail::unsupported("a second Force::Gravity");
            for (SimTK::MobilizedBodyIndex i(1); i < matter.getNumBodies(); ++i)
                if (g.getDefaultBodyIsExcluded(i)) detail::unsupported("a Gravity that excludes bodies");
            const SimTK::Vec3 gv = g.getDefaultGravityVector();
            for (int k = 0; k < 3; ++k) out.desc.gravity[k] = gv[k];
            gravitySeen = true;
        } else if (SimTK::Force::MobilityLinearSpring::isInstanceOf(f) ||
                   SimTK::Force::MobilityLinearDamper::isInstanceOf(f)) {
            const sbg_mobility_force_desc* d = log.mobility(fi);
            if (!d) detail::unsupported("a mobility spring or damper created without ForceLog");
            out.forces.push_back(*d);
        } else if (SimTK::SmoothSphereHalfSpaceForce::isInstanceOf(f)) {
            const ContactParameters* p = log.contact(fi);
            if (!p) detail::unsupported("a SmoothSphereHalfSpaceForce created without ForceLog");
            SimTK::SmoothSphereHalfSpaceForce h = SimTK::SmoothSphereHalfSpaceForce::downcast(f);
            if (h.getBodyHalfSpace().getMobilizedBodyIndex() != 0) detail::unsupported("a half-space on a moving body");
            sbg_contact_desc c{};
            c.body = (int32_t)h.getBodySphere().getMobilizedBodyIndex();
            const SimTK::Vec3 st = h.getContactSphereLocationInBody();
            for (int k = 0; k < 3; ++k) c.station[k] = st[k];
            c.radius = h.getContactSphereRadius();
            packTransform(h.getContactHalfSpaceTransform(), c.halfspace);
            double* par = &c.stiffness;
            for (int k = 0; k < 9; ++k) par[k] = (*p)[k];
            out.contacts.push_back(c);
        } else {
            detail::unsupported("force element " + std::to_string((int)fi));
        }
    }
    for (SimTK::ConstraintIndex ci(0); ci < matter.getNumConstraints(); ++ci) {
        const SimTK::Constraint& c = matter.getConstraint(ci);
        if (c.isDisabledByDefault()) continue;
        if (!SimTK::Constraint::Ball::isInstanceOf(c)) detail::unsupported("constraint " + std::to_string((int)ci));
        const SimTK::Constraint::Ball& b = SimTK::Constraint::Ball::downcast(c);
        sbg_ball_constraint_desc d{};
        d.body1 = (int32_t)b.getBody1MobilizedBodyIndex();
        d.body2 = (int32_t)b.getBody2MobilizedBodyIndex();
        const SimTK::Vec3 &s1 = b.getDefaultPointOnBody1(), &s2 = b.getDefaultPointOnBody2();
        for (int k = 0; k < 3; ++k) {
            d.station1[k] = s1[k];
            d.station2[k] = s2[k];
        }
        out.constraints.push_back(d);
    }
    out.desc.flags = matter.getUseEulerAngles(modelState) ? SBG_SYSTEM_EULER_ANGLES : 0;
    out.link();
    return out;
}

// One instance's y in the ABI packing: q (nq slots, Simbody's own slot
// counts) then u (nu), which is Simbody's y = [q u] for a system without z.
inline int ny(const SimTK::State& s) { return s.getNQ() + s.getNU(); }
inline void getY(const SimTK::State& s, double* y) {
    const SimTK::Vector& Y = s.getY();
    const int n = ny(s);
    for (int k = 0; k < n; ++k) y[k] = Y[k];
}
inline void setY(const double* y, SimTK::State& s) {
    SimTK::Vector& Y = s.updY();
    const int n = ny(s);
    for (int k = 0; k < n; ++k) Y[k] = y[k];
}

// ------------------------------------------------- batches of States
// Instance i of the batch is states[i]; each State's system must be the
// instance's topology (the batch's instanceTopology).

// State::getY and getTime of every State into the batch.
inline void loadStates(StateBatch& batch, const std::vector<const SimTK::State*>& states) {
    const std::vector<int64_t>& off = batch.getYOffsets();
    if ((int)states.size() != batch.getNumInstances()) throw Error(SBG_ERR_INVALID, "one State per instance");
    std::vector<double> y((size_t)off.back()), t(states.size());
    for (size_t i = 0; i < states.size(); ++i) {
        if (ny(*states[i]) != off[i + 1] - off[i]) throw Error(SBG_ERR_INVALID, "State size differs from its topology");
        getY(*states[i], y.data() + off[i]);
        t[i] = states[i]->getTime();
    }
    batch.setY(y, t);
}

// The batch's y and times back into the States (after an integration).
inline void storeStates(const StateBatch& batch, const std::vector<SimTK::State*>& states) {
    const std::vector<int64_t>& off = batch.getYOffsets();
    if ((int)states.size() != batch.getNumInstances()) throw Error(SBG_ERR_INVALID, "one State per instance");
    const std::vector<double> y = batch.getY(), t = batch.getTime();
    for (size_t i = 0; i < states.size(); ++i) {
        if (ny(*states[i]) != off[i + 1] - off[i]) throw Error(SBG_ERR_INVALID, "State size differs from its topology");
        setY(y.data() + off[i], *states[i]);
        states[i]->setTime(t[i]);
    }
}

// System::realize(s, Stage::Acceleration) and s.getYDot() for every State:
// ydot[i] of states[i]; status (may be null) gets the SBG_INST_* words.
inline std::vector<SimTK::Vector> realizeAcceleration(StateBatch& batch, const std::vector<const SimTK::State*>& states,
                                                      std::vector<int32_t>* status = nullptr) {
    loadStates(batch, states);
    const std::vector<double> yd = batch.realizeAcceleration(status);
    const std::vector<int64_t>& off = batch.getYOffsets();
    std::vector<SimTK::Vector> out(states.size());
    for (size_t i = 0; i < states.size(); ++i) {
        const int n = (int)(off[i + 1] - off[i]);
        out[i].resize(n);
        for (int k = 0; k < n; ++k) out[i][k] = yd[off[i] + k];
    }
    return out;
}

// RungeKuttaMersonIntegrator::initialize(s) and stepTo(tReport) for every
// State, the results written back into the States. Configure integ
// (setFixedStepSize, setAccuracy, ...) before; the States' common time is the
// start. Returns the SBG_INST_* word of each (Integrator::StepFailed analogue).
inline std::vector<int32_t> integrateTo(RungeKuttaMersonBatchIntegrator& integ, StateBatch& batch,
                                        const std::vector<SimTK::State*>& states, double tReport) {
    const std::vector<const SimTK::State*> in(states.begin(), states.end());
    loadStates(batch, in);
    integ.initialize(states.empty() ? 0.0 : states[0]->getTime());
    std::vector<int32_t> st = integ.stepTo(tReport);
    storeStates(batch, states);
    return st;
}

}  // namespace simtk
}  // namespace sbg

#endif  // SIMBODY_GB300_SIMTK_HPP
