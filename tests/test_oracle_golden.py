"""The CPU oracle against golden vectors recorded from the reference.

tests/golden/reference_vectors.npz holds, for seeded instances of workload
configs 1-5, the outputs of a built Simbody (make_golden.py / .cpp beside it):
realize(Stage::Acceleration) y-derivatives, multiplyByMInv(f), and the state
after a fixed number of RungeKuttaMersonIntegrator steps (fixed step size,
default accuracy; some config-5 records with loop closures use a 1e-9
constraint tolerance so that the in-step position and velocity projections
run). These pin the oracle, which in turn is the reference the CUDA engine
is checked against.

Tolerances (relative 2-norm per record): 1e-12 for realize and M^-1 f;
1e-11 for trajectories (20-1000 steps; roundoff grows along a trajectory).
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from simbody_gb300 import Workload
from simbody_gb300 import _native as N

GOLD = Path(__file__).resolve().parent / "golden" / "reference_vectors.npz"
WORKLOAD_SIZES = {1: 8, 2: 4, 3: 6, 4: 8, 5: 64, 6: 8, 7: 6, 8: 8, 9: 64, 10: 6}


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


@pytest.fixture(scope="module")
def workloads():
    return {c: Workload(c, n) for c, n in WORKLOAD_SIZES.items()}


def _records(g):
    for r in range(len(g["cfg"])):
        ys = slice(int(g["y_off"][r]), int(g["y_off"][r + 1]))
        us = slice(int(g["u_off"][r]), int(g["u_off"][r + 1]))
        yield r, int(g["cfg"][r]), int(g["inst"][r]), ys, us


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_fixture_inputs_match_generator(gold, workloads):
    """The seeded generator still produces the recorded inputs bit for bit."""
    for r, cfg, inst, ys, _ in _records(gold):
        w = workloads[cfg]
        assert np.array_equal(w.y0[w.instance_slice(inst)], gold["y0"][ys]), (cfg, inst)


def test_fixture_covers_every_mobilizer_and_loops(gold, workloads):
    kinds, loops = set(), 0
    for r, cfg, inst, ys, _ in _records(gold):
        d = workloads[cfg].systems[int(workloads[cfg].instance_system[inst])]
        kinds |= {d.bodies[k].mobilizer for k in range(d.nbodies)}
        loops += d.nconstraints > 0
    assert kinds == set(range(12)) and loops >= 4
    # and the Euler-angle mode of Ball and Free
    assert any(workloads[cfg].systems[int(workloads[cfg].instance_system[inst])].flags & 1
               for r, cfg, inst, ys, _ in _records(gold))


def test_realize_matches_reference(gold, workloads):
    for r, cfg, inst, ys, _ in _records(gold):
        ydot, st = O.realize_workload(workloads[cfg], [inst])
        assert st[0] == 0
        assert _rel(ydot, gold["ydot"][ys]) <= 1e-12, (cfg, inst)


def test_multiply_by_minv_matches_reference(gold, workloads):
    for r, cfg, inst, ys, us in _records(gold):
        w = workloads[cfg]
        y0 = gold["y0"][ys]
        out = O.multiply_by_minv(w.systems, w.nsys, w.instance_system[[inst]], np.array([0, len(y0)]), y0,
                                 np.array([0, us.stop - us.start]), gold["f"][us])
        assert _rel(out, gold["minv_f"][us]) <= 1e-12, (cfg, inst)


def test_rk_merson_matches_reference(gold, workloads):
    for r, cfg, inst, ys, _ in _records(gold):
        ctol = float(gold["cons_tol"][r])
        kw = {"cons_tol": ctol} if ctol > 0 else {}
        y, t, st, _ = O.rk_workload(workloads[cfg], float(gold["h"][r]), int(gold["nsteps"][r]), [inst], **kw)
        assert st[0] == 0
        assert t[0] == gold["t_rk"][r]
        assert _rel(y, gold["y_rk"][ys]) <= 1e-11, (cfg, inst, _rel(y, gold["y_rk"][ys]))


def test_double_pendulum_one_second_recorded_value(gold):
    """Config 1, instance 0, 1000 steps of h = 1e-3: the reference gives
    q0(1 s) = 0.47628747478039263 and u0(1 s) = 4.3677176498038577."""
    w = Workload(1, 1)
    y, t, st, _ = O.rk_workload(w, 1e-3, 1000)
    assert abs(y[0] - 0.47628747478039263) <= 1e-13
    assert abs(y[2] - 4.3677176498038577) <= 1e-12


def test_tight_tolerance_records_project_in_steps(gold, workloads):
    """With a 1e-9 constraint tolerance the oracle projects during the steps
    (the reference does too), so the fixture exercises projectQ/projectU."""
    done = 0
    for r, cfg, inst, ys, _ in _records(gold):
        if gold["cons_tol"][r] == 0:
            continue
        w = workloads[cfg]
        if w.systems[int(w.instance_system[inst])].nconstraints == 0:
            continue
        _, _, _, nproj = O.rk_workload(w, float(gold["h"][r]), int(gold["nsteps"][r]), [inst],
                                       cons_tol=float(gold["cons_tol"][r]))
        done += nproj > 0
    assert done >= 3


def test_redundant_closures_solve_like_reference(gold, workloads):
    """Workload 10 repeats a closure or pins a second point of a closed body,
    so G M^-1 G^T is rank-deficient. The oracle's QTZ minimum-norm solve (the reference's FactorQTZ) matches the
    reference's records, the tight-tolerance ones with projections in every
    few steps."""
    w = workloads[10]
    kinds = set()
    projected = 0
    for r, cfg, inst, ys, _ in _records(gold):
        if cfg != 10:
            continue
        s = w.systems[int(w.instance_system[inst])]
        cons = [(s.constraints[k].body1, tuple(s.constraints[k].station1)) for k in range(s.nconstraints)]
        repeated = len(set(cons)) < len(cons)
        two_points = len({b for b, _ in cons}) < len(set(cons))
        kinds.add((repeated, two_points))
        ydot, st = O.realize_workload(w, [inst])
        assert st[0] == 0 and gold["status"][r] == 0
        ref = gold["ydot"][ys]
        assert np.linalg.norm(ydot - ref) / np.linalg.norm(ref) <= 1e-12
        y, _, st, nproj = O.rk_workload(w, float(gold["h"][r]), int(gold["nsteps"][r]), [inst],
                                        cons_tol=float(gold["cons_tol"][r]))
        ref = gold["y_rk"][ys]
        assert st[0] == 0 and np.linalg.norm(y - ref) / np.linalg.norm(ref) <= 1e-11
        projected += nproj > 0
    assert kinds == {(True, False), (False, True), (True, True)}
    assert projected >= 6


def test_qdotdot_matches_reference(gold, workloads):
    """State::getQDotDot() recorded after realize(Acceleration): the oracle's
    calcQDotDot from the recorded ydot, every mobilizer type (quaternion
    second derivatives of Ball and Free bodies included)."""
    for r, cfg, inst, ys, _ in _records(gold):
        w = workloads[cfg]
        qs = slice(int(gold["q_off"][r]), int(gold["q_off"][r + 1]))
        y0, yd = gold["y0"][ys], gold["ydot"][ys]
        qdd = O.qdotdot(w.systems, w.nsys, w.instance_system[[inst]], np.array([0, len(y0)]), y0, yd,
                        np.array([0, qs.stop - qs.start]))
        assert _rel(qdd, gold["qdd"][qs]) <= 1e-13, (cfg, inst, _rel(qdd, gold["qdd"][qs]))


def _cont_records(g):
    for r in range(len(g["c_cfg"])):
        ys = slice(int(g["c_y_off"][r]), int(g["c_y_off"][r + 1]))
        yield r, int(g["c_cfg"][r]), int(g["c_inst"][r]), int(g["c_mode"][r]), ys


def oracle_continuation(w, inst, mode, h, t_mid, t_end, y0):
    """The oracle driven as the continuation records were: initialize, then
    stepTo(t_mid); stepTo(t_end) (mode 0), stepTo(t_end) (1) or
    stepTo(t_end + 0.3 h) (2), interpolation off."""
    off = np.array([0, len(y0)])
    so = w.instance_system[[inst]]
    if mode == 0:
        y, t, st = O.rk_merson_run(w.systems, w.nsys, so, off, y0, h, t_report=t_mid)
        y, t, st2 = O.rk_merson_run(w.systems, w.nsys, so, off, y, h, t_report=t_end, t=t, initialize=False)
        return y, t, st | st2
    target = t_end if mode == 1 else t_end + 0.3 * h
    return O.rk_merson_run(w.systems, w.nsys, so, off, y0, h, t_report=target)


def test_integrator_continuation_matches_reference(gold, workloads):
    """Integrator::stepTo twice on one integrator, once, and to a time that
    is not a whole number of steps (setAllowInterpolation(false): the last
    step is shortened): the oracle's continuation against the reference's
    records, final time exactly and state to 1e-11."""
    for r, cfg, inst, mode, ys in _cont_records(gold):
        assert gold["c_status"][r] == 0
        w = workloads[cfg]
        assert np.array_equal(w.y0[w.instance_slice(inst)], gold["c_y0"][ys])
        y, t, st = oracle_continuation(w, inst, mode, float(gold["c_h"][r]), float(gold["c_t_mid"][r]),
                                       float(gold["c_t_end"][r]), gold["c_y0"][ys])
        assert st[0] == 0
        assert t[0] == gold["c_t_out"][r], (cfg, inst, mode, t[0], gold["c_t_out"][r])
        assert _rel(y, gold["c_y_out"][ys]) <= 1e-11, (cfg, inst, mode, _rel(y, gold["c_y_out"][ys]))


def test_continuation_records_cover_loops_and_quaternions(gold, workloads):
    """The continuation records include quaternion bodies (a re-initialize
    would renormalize them) and loop closures (it would re-project)."""
    quats = loops = 0
    for r, cfg, inst, mode, ys in _cont_records(gold):
        d = workloads[cfg].systems[int(workloads[cfg].instance_system[inst])]
        quats += any(d.bodies[k].mobilizer in (3, 4) for k in range(d.nbodies))
        loops += d.nconstraints > 0
    assert quats >= 6 and loops >= 2


def test_contact_records_engage_the_contact_force(gold, workloads):
    """The records of the ground-contact trees (SmoothSphereHalfSpaceForce)
    realize with the spheres pressing on the half-space: dropping the contact
    elements changes the recorded accelerations well beyond the tolerance,
    and one record uses the force's default parameters (a zero block)."""
    w = workloads[8]
    seen_defaults = checked = 0
    for r, cfg, inst, ys, _ in _records(gold):
        if cfg != 8:
            continue
        d = w.systems[int(w.instance_system[inst])]
        assert d.ncontacts == d.nbodies
        seen_defaults += d.contacts[0].stiffness == 0
        bare = N.SystemDesc.from_buffer_copy(d)
        bare.ncontacts = 0
        off = np.array([0, ys.stop - ys.start])
        ydot, st = O.realize((N.SystemDesc * 1)(bare), 1, np.zeros(1, np.int32), off, gold["y0"][ys])
        assert st[0] == 0
        # one indented sphere among 20-40 bodies (the default stiffness, 1,
        # gives about 1e-4 N): small against the whole ydot, but a hundred
        # times the agreement of the realize records
        assert _rel(ydot, gold["ydot"][ys]) > 1e-10, (inst, _rel(ydot, gold["ydot"][ys]))
        checked += 1
    assert checked >= 8 and seen_defaults >= 1
