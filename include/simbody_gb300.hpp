// simbody_gb300.hpp -- header-only C++17 surface over the C ABI
// (simbody_gb300.h), named after the Simbody calls it stands in for, so that a
// Simbody-based program can hand a batch of States to the GPU with the
// vocabulary it already uses. Errors are thrown as sbg::Error, as SimTK throws
// (the integrator's failure per instance is a status word instead, like
// Integrator::StepFailed without the exception: AbstractIntegratorRep.cpp:426-431).
//
//   Topology                      System::realizeTopology of one system
//   StateBatch                    a device-resident batch of States
//     setY / getY / setTime       State::updY / getY / setTime (State.h:962-1034)
//     realizeAcceleration         System::realize(s, Stage::Acceleration) + getYDot
//     getQDotDot                  State::getQDotDot after that realize
//     multiplyByMInv / multiplyByM / calcResidualForceIgnoringConstraints /
//     multiplyBySystemJacobian(Transpose) / calcCompositeBodyInertias
//                                 SimbodyMatterSubsystem operators (.h:1262-2323)
//   RungeKuttaMersonBatchIntegrator
//                                 RungeKuttaMersonIntegrator with setFixedStepSize,
//                                 setAccuracy, setConstraintTolerance,
//                                 setProjectEveryStep, initialize, stepTo, stepBy;
//                                 without a fixed step size, error-controlled
//                                 (setInitial/Minimum/MaximumStepSize,
//                                 getNumStepsTaken/Attempted per instance)
#ifndef SIMBODY_GB300_HPP_
#define SIMBODY_GB300_HPP_

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "simbody_gb300.h"

namespace sbg {

// A failing C-ABI call: its sbg_status code and message.
class Error : public std::runtime_error {
public:
    Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

inline void check(int rc) {
    if (rc != SBG_OK) {
        const char* m = sbg_last_error();
        throw Error(rc, m && *m ? m : "simbody_gb300 call failed");
    }
}

enum class Precision { FP64 = SBG_PRECISION_FP64, Mixed = SBG_PRECISION_MIXED, MixedFast = SBG_PRECISION_MIXED_FAST };

// System::realizeTopology of one system: validated and flattened. Host only.
class Topology {
public:
    explicit Topology(const sbg_system_desc& system) {
        check(sbg_topology_create(&system, &h_));
        check(sbg_topology_info(h_, &nq_, &nu_, &nb_, &nlev_, &nquat_, &ncons_));
    }
    ~Topology() {
        if (h_) sbg_topology_destroy(h_);
    }
    Topology(const Topology&) = delete;
    Topology& operator=(const Topology&) = delete;
    Topology(Topology&& o) noexcept { *this = std::move(o); }
    Topology& operator=(Topology&& o) noexcept {
        std::swap(h_, o.h_);
        nq_ = o.nq_; nu_ = o.nu_; nb_ = o.nb_; nlev_ = o.nlev_; nquat_ = o.nquat_; ncons_ = o.ncons_;
        return *this;
    }
    int getNQ() const { return nq_; }
    int getNU() const { return nu_; }
    int getNY() const { return nq_ + nu_; }
    int getNumBodies() const { return nb_; }
    int getNumLevels() const { return nlev_; }
    int getNumQuaternions() const { return nquat_; }
    int getNumConstraintEquations() const { return ncons_; }
    // Simbody's default state: quaternions identity, everything else zero.
    std::vector<double> getDefaultY() const {
        std::vector<double> y(getNY());
        check(sbg_topology_default_state(h_, y.data()));
        return y;
    }
    sbg_topology handle() const { return h_; }

private:
    sbg_topology h_ = nullptr;
    int32_t nq_ = 0, nu_ = 0, nb_ = 0, nlev_ = 0, nquat_ = 0, ncons_ = 0;
};

// A batch of States on one GPU: instance i is a state of
// *topologies[instanceTopology[i]]. Host vectors use the packing of
// State::getY per instance, instances back to back (getYOffsets).
class StateBatch {
public:
    StateBatch(const std::vector<const Topology*>& topologies, const std::vector<int32_t>& instanceTopology,
               Precision precision = Precision::FP64, int device = 0, int64_t deviceBudgetBytes = 0) {
        std::vector<sbg_topology> hs;
        for (const Topology* t : topologies) hs.push_back(t->handle());
        const sbg_batch_config cfg{static_cast<int32_t>(precision), device, deviceBudgetBytes};
        check(sbg_batch_create(hs.data(), (int32_t)hs.size(), instanceTopology.data(),
                               (int32_t)instanceTopology.size(), &cfg, &h_));
        n_ = (int)instanceTopology.size();
        yOff_.resize(n_ + 1);
        int64_t ny = 0;
        check(sbg_batch_layout(h_, yOff_.data(), &ny));
        uOff_.assign(n_ + 1, 0);
        bOff_.assign(n_ + 1, 0);
        qOff_.assign(n_ + 1, 0);
        for (int i = 0; i < n_; ++i) {
            const Topology* t = topologies[instanceTopology[i]];
            uOff_[i + 1] = uOff_[i] + t->getNU();
            bOff_[i + 1] = bOff_[i] + t->getNumBodies();
            qOff_[i + 1] = qOff_[i] + t->getNQ();
        }
    }
    ~StateBatch() {
        if (h_) sbg_batch_destroy(h_);
    }
    StateBatch(const StateBatch&) = delete;
    StateBatch& operator=(const StateBatch&) = delete;

    int getNumInstances() const { return n_; }
    const std::vector<int64_t>& getYOffsets() const { return yOff_; }
    const std::vector<int64_t>& getUOffsets() const { return uOff_; }
    const std::vector<int64_t>& getBodyOffsets() const { return bOff_; }

    // State::updY (and setTime: t may be empty = all zero) for every instance.
    void setY(const std::vector<double>& y, const std::vector<double>& t = {}) {
        need(y.size() == (size_t)yOff_[n_], "y");
        need(t.empty() || t.size() == (size_t)n_, "t");
        check(sbg_batch_set_state(h_, t.empty() ? nullptr : t.data(), y.data()));
    }
    std::vector<double> getY() const {
        std::vector<double> y(yOff_[n_]), t(n_);
        check(sbg_batch_get_state(h_, t.data(), y.data()));
        return y;
    }
    std::vector<double> getTime() const {
        std::vector<double> y(yOff_[n_]), t(n_);
        check(sbg_batch_get_state(h_, t.data(), y.data()));
        return t;
    }

    // System::realize(s, Stage::Acceleration) then State::getYDot.
    std::vector<double> realizeAcceleration(std::vector<int32_t>* status = nullptr) {
        std::vector<double> ydot(yOff_[n_]);
        std::vector<int32_t> st(n_);
        check(sbg_realize_acceleration(h_, ydot.data(), st.data()));
        if (status) *status = std::move(st);
        return ydot;
    }

    // State::getQDotDot() of every instance after realizeAcceleration() of
    // the current state (nq values per instance, back to back: getQOffsets).
    std::vector<double> getQDotDot() const {
        std::vector<double> qdd(qOff_[n_]);
        check(sbg_batch_get_qdotdot(h_, qdd.data()));
        return qdd;
    }
    const std::vector<int64_t>& getQOffsets() const { return qOff_; }

    // SimbodyMatterSubsystem operators (u-like vectors packed like the u
    // parts of y; body vectors 6 values per body, inertias 10).
    std::vector<double> multiplyByMInv(const std::vector<double>& f) {
        need(f.size() == (size_t)uOff_[n_], "f");
        std::vector<double> out(f.size());
        check(sbg_multiply_by_minv(h_, f.data(), out.data()));
        return out;
    }
    std::vector<double> multiplyByM(const std::vector<double>& a) {
        need(a.size() == (size_t)uOff_[n_], "a");
        std::vector<double> out(a.size());
        check(sbg_multiply_by_m(h_, a.data(), out.data(), nullptr));
        return out;
    }
    // Empty inputs act as all zero, as zero-length Vectors do for the reference.
    std::vector<double> calcResidualForceIgnoringConstraints(const std::vector<double>& appliedMobilityForces,
                                                             const std::vector<double>& appliedBodyForces,
                                                             const std::vector<double>& knownUdot) {
        need(appliedMobilityForces.empty() || appliedMobilityForces.size() == (size_t)uOff_[n_], "mobility forces");
        need(appliedBodyForces.empty() || appliedBodyForces.size() == (size_t)(6 * bOff_[n_]), "body forces");
        need(knownUdot.empty() || knownUdot.size() == (size_t)uOff_[n_], "udot");
        std::vector<double> out(uOff_[n_]);
        check(sbg_calc_residual_force(h_, opt(appliedMobilityForces), opt(appliedBodyForces), opt(knownUdot),
                                      out.data(), nullptr));
        return out;
    }
    std::vector<double> multiplyBySystemJacobian(const std::vector<double>& u) {
        need(u.size() == (size_t)uOff_[n_], "u");
        std::vector<double> out(6 * bOff_[n_]);
        check(sbg_multiply_by_system_jacobian(h_, u.data(), out.data(), nullptr));
        return out;
    }
    std::vector<double> multiplyBySystemJacobianTranspose(const std::vector<double>& F_G) {
        need(F_G.size() == (size_t)(6 * bOff_[n_]), "F_G");
        std::vector<double> out(uOff_[n_]);
        check(sbg_multiply_by_system_jacobian_transpose(h_, F_G.data(), out.data(), nullptr));
        return out;
    }
    std::vector<double> calcCompositeBodyInertias() {
        std::vector<double> out(10 * bOff_[n_]);
        check(sbg_calc_composite_body_inertias(h_, out.data(), nullptr));
        return out;
    }

    sbg_batch handle() const { return h_; }

private:
    static void need(bool ok, const char* what) {
        if (!ok) throw Error(SBG_ERR_INVALID, std::string("wrong length: ") + what);
    }
    static const double* opt(const std::vector<double>& v) { return v.empty() ? nullptr : v.data(); }

    sbg_batch h_ = nullptr;
    int n_ = 0;
    std::vector<int64_t> yOff_, uOff_, bOff_, qOff_;
};

// RungeKuttaMersonIntegrator over every state of a batch, with a fixed step
// size (Integrator::setFixedStepSize) and interpolation off
// (Integrator::setAllowInterpolation(false)): stepTo(t) lands every instance
// exactly on t, its last step shortened when t is not a whole number of steps
// away (AbstractIntegratorRep.cpp:536-544). initialize() starts a new
// integration of the batch's current state: the first stepTo after it does
// Integrator::initialize's projection (quaternions normalized, loop closures
// projected); later calls continue the integration, as repeated stepTo calls
// on one Simbody integrator do. stepTo returns one SBG_INST_* word per
// instance.
//
// Without setFixedStepSize the integrator is error-controlled, as Simbody's
// is by default: each instance takes its own steps (accuracy, initial,
// minimum and maximum step size as set), and stepTo(t) brings every instance
// to exactly t (Integrator::setFinalTime(t) + stepTo(t); FP64 batches
// without loop closures). Each such stepTo starts the step-size control anew
// from the initial step size.
class RungeKuttaMersonBatchIntegrator {
public:
    explicit RungeKuttaMersonBatchIntegrator(StateBatch& batch) : b_(batch) {}
    void setFixedStepSize(double h) {
        if (!(h > 0) || !std::isfinite(h)) throw Error(SBG_ERR_INVALID, "step size must be positive");
        h_ = h;
    }
    void setAccuracy(double a) { opts_.accuracy = a; aopts_.accuracy = a; }
    void setConstraintTolerance(double c) { opts_.constraint_tolerance = c; aopts_.constraint_tolerance = c; }
    void setProjectEveryStep(bool p) { opts_.project_every_step = p ? 1 : 0; aopts_.project_every_step = p ? 1 : 0; }
    void setInitialStepSize(double h) { aopts_.initial_step = h; }
    void setMinimumStepSize(double h) { aopts_.min_step = h; }
    void setMaximumStepSize(double h) { aopts_.max_step = h; }
    // Accepted and attempted steps of each instance in the last
    // error-controlled stepTo (Integrator::getNumStepsTaken / Attempted).
    const std::vector<int64_t>& getNumStepsTaken() const { return taken_; }
    const std::vector<int64_t>& getNumStepsAttempted() const { return attempted_; }
    // Integrator::initialize: the next stepTo starts the integration from
    // the batch's current state, whose time is t0 (StateBatch::setY).
    void initialize(double t0 = 0.0) {
        t_ = t0;
        started_ = false;
    }
    double getTime() const { return t_; }
    std::vector<int32_t> stepTo(double tReport) {
        if (!std::isfinite(tReport)) throw Error(SBG_ERR_INVALID, "stepTo: the report time must be finite");
        std::vector<int32_t> st(b_.getNumInstances());
        if (h_ <= 0) {  // error-controlled
            std::vector<int64_t> stats(2 * st.size());
            check(sbg_rk_merson_adaptive(b_.handle(), tReport, &aopts_, st.data(), stats.data()));
            taken_.resize(st.size());
            attempted_.resize(st.size());
            for (size_t i = 0; i < st.size(); ++i) {
                taken_[i] = stats[2 * i];
                attempted_[i] = stats[2 * i] + stats[2 * i + 1];
            }
            t_ = std::max(t_, tReport);
            return st;
        }
        opts_.continue_integration = started_ ? 1 : 0;
        check(sbg_rk_merson_step_to(b_.handle(), h_, tReport, &opts_, st.data()));
        started_ = true;
        t_ = std::max(t_, tReport);
        return st;
    }
    std::vector<int32_t> stepBy(double dt) { return stepTo(t_ + dt); }

private:
    StateBatch& b_;
    double h_ = 0, t_ = 0;
    bool started_ = false;
    sbg_integ_opts opts_{0, 0, 0, 0};
    sbg_adaptive_opts aopts_{0, 0, 0, 0, 0, 0, 0};
    std::vector<int64_t> taken_, attempted_;
};

}  // namespace sbg

#endif  // SIMBODY_GB300_HPP_
