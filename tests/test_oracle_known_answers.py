"""Known-answer checks of the CPU oracle, after the reference's own tests:

  TestForces.cpp:177-191     MobilityLinearSpring / MobilityLinearDamper
                             closed forms (to 1e-10)
  TestMassMatrix.cpp:658-800 M^-1 consistent with M: symmetric, and
                             M^-1 f reproduced by the forward dynamics
  Force.cpp:339-351          the spring reads q[which] and writes u[which],
                             also for quaternion joints
  TestForces.cpp:244-290     energy conservation under RK Merson (Gimbal
                             chain, mobility spring, gravity)
  TestConstraints.cpp:49-127 Ball closure errors after projection: position
                             and velocity within the tolerance, acceleration
                             to machine precision
"""
import ctypes as C

import numpy as np

from oracle import oracle as O
from simbody_gb300 import Workload
from simbody_gb300 import _native as N

IDENT = [1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0]


def one_body_system(mobilizer, mass=2.0, forces=(), gravity=(0.0, 0.0, 0.0)):
    bodies = (N.BodyDesc * 1)()
    b = bodies[0]
    b.parent, b.mobilizer, b.mass = 0, mobilizer, mass
    b.com[:] = [0.0, 0.0, 0.0]
    b.unit_inertia[:] = [1.0, 1.0, 1.0, 0.0, 0.0, 0.0]
    b.X_PF[:] = IDENT
    b.X_BM[:] = IDENT
    fs = (N.MobilityForceDesc * max(1, len(forces)))()
    for i, (kind, which, coef, q0) in enumerate(forces):
        fs[i].kind, fs[i].body, fs[i].which, fs[i].coef, fs[i].q0 = kind, 1, which, coef, q0
    d = N.SystemDesc()
    d.nbodies, d.nforces, d.nconstraints = 1, len(forces), 0
    d.gravity[:] = list(gravity)
    d.bodies = C.cast(bodies, C.POINTER(N.BodyDesc))
    d.forces = C.cast(fs, C.POINTER(N.MobilityForceDesc))
    d.constraints = None
    arr = (N.SystemDesc * 1)(d)
    return arr, (bodies, fs)


def realize_one(arr, y):
    y = np.asarray(y, dtype=np.float64)
    ydot, st = O.realize(arr, 1, np.zeros(1, np.int32), np.array([0, len(y)], np.int64), y)
    assert st[0] == 0
    return ydot


def test_slider_spring_and_damper_closed_form():
    k, q0, c, m = 37.0, 0.25, 0.6, 2.0
    arr, keep = one_body_system(N.SBG_SLIDER, m, [(0, 0, k, q0), (1, 0, c, 0.0)])
    for q, u in [(0.0, 0.0), (1.3, -0.7), (-2.0, 4.0)]:
        ydot = realize_one(arr, [q, u])
        assert abs(ydot[0] - u) <= 1e-15
        assert abs(ydot[1] - (-k * (q - q0) - c * u) / m) <= 1e-10 * max(1.0, abs(ydot[1]))


def test_pin_spring_about_z_axis():
    k, m = 12.0, 3.0  # unit inertia 1 about z, so I_zz = m
    arr, keep = one_body_system(N.SBG_PIN, m, [(0, 0, k, 0.0)])
    ydot = realize_one(arr, [0.4, 0.0])
    assert abs(ydot[1] - (-k * 0.4 / m)) <= 1e-12


def test_ball_spring_reads_quaternion_component():
    """MobilityLinearSpring on a Ball with which = 0 uses q[0], the scalar
    part of the quaternion, and pushes u[0] (the reference's behaviour)."""
    k, m = 5.0, 1.0
    arr, keep = one_body_system(N.SBG_BALL, m, [(0, 0, k, 0.0)])
    ydot = realize_one(arr, [1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0])
    assert abs(ydot[4] - (-k * 1.0 / m)) <= 1e-12   # udot[0] = -k q[0] / I
    assert abs(ydot[5]) <= 1e-15 and abs(ydot[6]) <= 1e-15


def test_minv_is_symmetric_positive_definite():
    w = Workload(3, 2)
    i = 1
    y0 = w.y0[w.instance_slice(i)]
    d = w.systems[int(w.instance_system[i])]
    nq = sum(N.NQ[d.bodies[b].mobilizer] for b in range(d.nbodies))
    nu = len(y0) - nq
    cols = []
    for j in range(nu):
        e = np.zeros(nu)
        e[j] = 1.0
        cols.append(O.multiply_by_minv(w.systems, w.nsys, w.instance_system[[i]], np.array([0, len(y0)]), y0,
                                       np.array([0, nu]), e))
    Minv = np.array(cols).T
    assert np.abs(Minv - Minv.T).max() <= 1e-12 * np.abs(Minv).max()
    assert np.linalg.eigvalsh(0.5 * (Minv + Minv.T)).min() > 0


def test_forward_dynamics_is_minv_of_applied_forces():
    """With u = 0 the velocity terms vanish, so udot = M^-1 f for the
    spring force f = -k (q - q0) of a one-body Slider."""
    k, q0, m = 8.0, -0.5, 1.5
    arr, keep = one_body_system(N.SBG_SLIDER, m, [(0, 0, k, q0)])
    ydot = realize_one(arr, [0.75, 0.0])
    f = np.array([-k * (0.75 - q0)])
    minv = O.multiply_by_minv(arr, 1, np.zeros(1, np.int32), np.array([0, 2]), np.array([0.75, 0.0]),
                              np.array([0, 1]), f)
    assert abs(ydot[1] - minv[0]) <= 1e-14


def rotation(angle, axis):
    """Rotation(angle, UnitVec3(axis)): right-handed about the unit axis,
    row-major."""
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) * np.cos(angle) + (1 - np.cos(angle)) * np.outer(a, a) + np.sin(angle) * K


def chain_system(mobilizers, mass, com, unit_inertia, X_PF, X_BM, gravity=(0.0, 0.0, 0.0), forces=(), balls=()):
    """A chain, body k+1 on body k, every body alike; X_* = (R 3x3, p)."""
    n = len(mobilizers)
    bodies = (N.BodyDesc * n)()
    for k, mob in enumerate(mobilizers):
        b = bodies[k]
        b.parent, b.mobilizer, b.mass = k, mob, mass
        b.com[:] = list(com)
        b.unit_inertia[:] = list(unit_inertia)
        b.X_PF[:] = list(np.ravel(X_PF[0])) + list(X_PF[1])
        b.X_BM[:] = list(np.ravel(X_BM[0])) + list(X_BM[1])
    fs = (N.MobilityForceDesc * max(1, len(forces)))()
    for i, (kind, body, which, coef, q0) in enumerate(forces):
        fs[i].kind, fs[i].body, fs[i].which, fs[i].coef, fs[i].q0 = kind, body, which, coef, q0
    cs = (N.BallConstraintDesc * max(1, len(balls)))()
    for i, (b1, s1, b2, s2) in enumerate(balls):
        cs[i].body1, cs[i].body2 = b1, b2
        cs[i].station1[:] = list(s1)
        cs[i].station2[:] = list(s2)
    d = N.SystemDesc()
    d.nbodies, d.nforces, d.nconstraints = n, len(forces), len(balls)
    d.gravity[:] = list(gravity)
    d.bodies = C.cast(bodies, C.POINTER(N.BodyDesc))
    d.forces = C.cast(fs, C.POINTER(N.MobilityForceDesc)) if forces else None
    d.constraints = C.cast(cs, C.POINTER(N.BallConstraintDesc)) if balls else None
    return (N.SystemDesc * 1)(d), (bodies, fs, cs)


def test_conservative_forces_conserve_energy_under_rk_merson():
    """TestForces.cpp:244-290: a chain of ten unit Gimbal bodies (bond 0.5)
    with a MobilityLinearSpring (body 1, q 1, k 0.1, q0 1) and gravity
    (0, -1, 0), from a random state, keeps its energy within 0.5 % over
    10 s of RK Merson at accuracy 1e-4. (The reference adds a
    TwoPointLinearSpring, which is not on this path.)"""
    I3 = np.eye(3)
    arr, keep = chain_system([N.SBG_GIMBAL] * 10, 1.0, (0, 0, 0), (1, 1, 1, 0, 0, 0), (I3, (0, 0, 0)),
                             (I3, (0.5, 0, 0)), gravity=(0, -1.0, 0), forces=[(0, 1, 1, 0.1, 1.0)])
    ny = 60
    y0 = np.random.default_rng(244).uniform(0, 1, ny)

    def energy(y):
        e = O.invariants(arr[0], y)
        assert e["status"] == 0
        return e["ke"] + e["pe_gravity"] + e["pe_springs"]

    y, t, st, stats = O.rk_merson_adaptive(arr, 1, np.zeros(1, np.int32), np.array([0, ny], np.int64), y0, 10.0,
                                           accuracy=1e-4)
    assert st[0] == 0 and t[0] == 10.0 and stats[0, 0] > 100
    e0, e1 = energy(y0), energy(y)
    assert abs(e0 / e1 - 1) < 0.005, (e0, e1)


def test_ball_constraint_errors_after_projection():
    """TestConstraints.cpp:49-127: a chain of ten bodies (Gimbal, with a
    Universal at 5 and a Ball at 7; mass 1.23, COM (.1,.2,-.03), rotated
    inboard and outboard frames) closed by a Ball between the origins of
    bodies 1 and 10. From a random state, projection to 1e-10 leaves
    position and velocity errors within 1e-10, and the accelerations of
    the constrained realize meet the closure to machine precision times
    the problem size (10 nu SignificantReal)."""
    mobs = [N.SBG_GIMBAL] * 10
    mobs[5], mobs[7] = N.SBG_UNIVERSAL, N.SBG_BALL
    X_PF = (rotation(np.pi / 20, (1, 2, 3)), (-0.1, 0.3, 0.2))
    X_BM = (rotation(-np.pi / 17, (2, 0.2, 3)), (0.5, 0, 0))
    arr, keep = chain_system(mobs, 1.23, (0.1, 0.2, -0.03), (1.1, 1.2, 1.3, 0.01, -0.02, 0.07), X_PF, X_BM,
                             balls=[(1, (0, 0, 0), 10, (0, 0, 0))])
    nq, nu = 8 * 3 + 2 + 4, 8 * 3 + 2 + 3
    y0 = np.random.default_rng(100).uniform(0, 1, nq + nu)
    before = O.invariants(arr[0], y0)
    assert np.abs(before["perr"]).max() > 0.1  # the random state violates the closure
    y, _, st = O.rk_merson_run(arr, 1, np.zeros(1, np.int32), np.array([0, nq + nu], np.int64), y0, 1e-3,
                               nsteps=0, initialize=True, cons_tol=1e-10)
    assert st[0] == 0
    inv = O.invariants(arr[0], y)
    assert inv["status"] == 0
    assert np.linalg.norm(inv["perr"]) <= 1e-10
    assert np.linalg.norm(inv["verr"]) <= 1e-10
    ydot = realize_one(arr, y)
    scale = max(1.0, np.abs(ydot[nq:]).max())
    assert np.linalg.norm(inv["aerr"]) <= 10 * nu * np.finfo(float).eps ** 0.875 * scale, inv["aerr"]
