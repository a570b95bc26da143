"""Known-answer checks of the CPU oracle, after the reference's own tests:

  TestForces.cpp:177-191     MobilityLinearSpring / MobilityLinearDamper
                             closed forms (to 1e-10)
  TestMassMatrix.cpp:658-800 M^-1 consistent with M: symmetric, and
                             M^-1 f reproduced by the forward dynamics
  Force.cpp:339-351          the spring reads q[which] and writes u[which],
                             also for quaternion joints
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
