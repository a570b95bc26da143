"""Host-side topology flattening (sbg_topology_create): the validation the
reference performs when a System is built (SimbodyMatterSubsystemRep.cpp:
256-330, MobilizedBody/Force/Constraint constructors), the state sizes and
the default state. No GPU is needed for any of it."""
import ctypes as C

import numpy as np
import pytest

from simbody_gb300 import _native as N
from simbody_gb300.engine import Topology


def chain(n, mob=N.SBG_PIN):
    bodies = (N.BodyDesc * n)()
    for k in range(n):
        b = bodies[k]
        b.parent, b.mobilizer, b.mass = k, mob, 1.0
        b.unit_inertia[0] = b.unit_inertia[1] = b.unit_inertia[2] = 1.0
        for j in (0, 4, 8):
            b.X_PF[j] = b.X_BM[j] = 1.0
        b.X_BM[10] = 0.5
    return bodies


def make(bodies, n, forces=None, nf=0, cons=None, nc=0):
    return N.SystemDesc(n, nf, nc, 0, (C.c_double * 3)(0, -9.8, 0), bodies, forces, cons)


def create(desc):
    h = C.c_void_p()
    rc = N.engine_lib().sbg_topology_create(C.byref(desc), C.byref(h))
    if rc == 0:
        N.engine_lib().sbg_topology_destroy(h)
    return rc, (N.engine_lib().sbg_last_error() or b"").decode()


@pytest.mark.parametrize("mob,nq,nu,nquat", [(N.SBG_PIN, 1, 1, 0), (N.SBG_SLIDER, 1, 1, 0),
                                              (N.SBG_UNIVERSAL, 2, 2, 0), (N.SBG_BALL, 4, 3, 1),
                                              (N.SBG_FREE, 7, 6, 1), (N.SBG_WELD, 0, 0, 0),
                                              (N.SBG_SCREW, 1, 1, 0)])
def test_sizes_and_default_state(mob, nq, nu, nquat):
    b = chain(3, mob)
    t = Topology(make(b, 3), keepalive=b)
    assert (t.nq, t.nu, t.nbodies, t.nlevels, t.nquaternions) == (3 * nq, 3 * nu, 3, 3, 3 * nquat)
    y = t.default_state()
    # quaternions start at the identity (RigidBodyNodeSpec_Ball.h:405-415), all else zero
    expect = np.zeros(3 * (nq + nu))
    if nquat:
        expect[[k * nq for k in range(3)]] = 1.0
    assert np.array_equal(y, expect)


def test_levels_of_a_branched_tree():
    b = chain(5)
    b[1].parent = 1
    b[2].parent = 1  # bodies 2 and 3 hang off body 1
    b[3].parent = 3
    b[4].parent = 0  # a second root
    t = Topology(make(b, 5), keepalive=b)
    assert t.nlevels == 3


@pytest.mark.parametrize("field,value,msg", [("parent", 2, "parent must precede"), ("parent", -1, "parent must precede"),
                                             ("mobilizer", 12, "unknown mobilizer"), ("mass", 0.0, "mass must be positive"),
                                             ("mass", float("nan"), "mass must be positive")])
def test_invalid_bodies_are_rejected(field, value, msg):
    b = chain(3)
    setattr(b[1], field, value)
    rc, err = create(make(b, 3))
    assert rc == 1 and msg in err  # SBG_ERR_INVALID


def test_invalid_forces_and_constraints_are_rejected():
    b = chain(3)
    f = (N.MobilityForceDesc * 1)()
    f[0].kind, f[0].body, f[0].which, f[0].coef = 0, 2, 1, 10.0  # a Pin has one mobility: which = 1 is out of range
    assert create(make(b, 3, f, 1))[0] == 1
    f[0].which, f[0].body = 0, 4  # no body 4
    assert create(make(b, 3, f, 1))[0] == 1
    f[0].body, f[0].kind = 2, 5  # unknown kind
    assert create(make(b, 3, f, 1))[0] == 1
    c = (N.BallConstraintDesc * 1)()
    c[0].body1, c[0].body2 = 2, 2  # a body constrained to itself
    assert create(make(b, 3, None, 0, c, 1))[0] == 1
    assert create(N.SystemDesc(0, 0, 0, 0, (C.c_double * 3)(0, 0, 0), None, None, None))[0] == 1


def test_largest_serving_tree_flattens():
    b = chain(256, N.SBG_BALL)
    for k in range(2, 256):
        b[k].parent = (k * 7919 + 3) % (k + 1)  # any earlier body: a random-looking tree
    t = Topology(make(b, 256), keepalive=b)
    assert t.nbodies == 256 and t.nq == 1024 and t.nu == 768


def test_euler_angle_flag_sizes_and_default_state():
    """SBG_SYSTEM_EULER_ANGLES keeps Ball/Free q slot counts (the last slot
    unused, as Simbody's State does), drops their quaternions, and takes
    loop closures; unknown flags are refused."""
    import ctypes as C

    from simbody_gb300 import _native as N
    from simbody_gb300.build import build_engine

    build_engine()
    lib = N.engine_lib()
    bodies = (N.BodyDesc * 2)()
    for k, mob in enumerate((N.SBG_FREE, N.SBG_BALL)):
        b = bodies[k]
        b.parent, b.mobilizer, b.mass = k, mob, 1.0
        b.unit_inertia[0] = b.unit_inertia[1] = b.unit_inertia[2] = 1.0
        for i in (0, 4, 8):
            b.X_PF[i] = b.X_BM[i] = 1.0
    for flags, nquat in ((0, 2), (N.SYSTEM_EULER_ANGLES, 0)):
        d = N.SystemDesc(2, 0, 0, flags, (C.c_double * 3)(0, -9.8, 0), bodies, None, None)
        h = C.c_void_p()
        assert lib.sbg_topology_create(C.byref(d), C.byref(h)) == 0
        nq, nu, nb, nl, nqt, nc = (C.c_int32() for _ in range(6))
        lib.sbg_topology_info(h, *(C.byref(v) for v in (nq, nu, nb, nl, nqt, nc)))
        assert (nq.value, nu.value, nqt.value) == (11, 9, nquat)
        y = (C.c_double * 20)()
        lib.sbg_topology_default_state(h, y)
        assert list(y[:11]) == ([1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0] if nquat else [0] * 11)
        lib.sbg_topology_destroy(h)
    d = N.SystemDesc(2, 0, 0, 4, (C.c_double * 3)(0, -9.8, 0), bodies, None, None)
    h = C.c_void_p()
    assert lib.sbg_topology_create(C.byref(d), C.byref(h)) == 1  # unknown flag
    cons = (N.BallConstraintDesc * 1)()
    cons[0].body1, cons[0].body2 = 2, 0
    d = N.SystemDesc(2, 0, 1, N.SYSTEM_EULER_ANGLES, (C.c_double * 3)(0, -9.8, 0), bodies, None, cons)
    assert lib.sbg_topology_create(C.byref(d), C.byref(h)) == 0  # loop closures in Euler-angle mode
    lib.sbg_topology_destroy(h)


def test_contact_spheres_are_validated_and_refused_where_unsupported():
    """SmoothSphereHalfSpaceForce spheres: a bad body or a non-positive
    radius is SBG_ERR_INVALID; a valid list flattens; the allocation-free
    realize refuses a topology with spheres (SBG_ERR_UNSUPPORTED) before it
    touches the device."""
    b = chain(3)
    k = (N.ContactDesc * 2)()
    for j in range(2):
        k[j].body, k[j].radius = j + 1, 0.05
        k[j].halfspace[1], k[j].halfspace[3], k[j].halfspace[8] = 1.0, -1.0, 1.0  # normal -Y
    d = make(b, 3)
    d.ncontacts, d.contacts = 2, k
    assert create(d)[0] == 0
    k[1].body = 4
    rc, err = create(d)
    assert rc == 1 and "contact" in err
    k[1].body, k[1].radius = 2, 0.0
    rc, err = create(d)
    assert rc == 1 and "radius" in err
    d.contacts = None
    assert create(d)[0] == 1
    k[1].radius = 0.05
    d.contacts = k
    lib = N.engine_lib()
    h = C.c_void_p()
    assert lib.sbg_topology_create(C.byref(d), C.byref(h)) == 0
    try:
        y = (C.c_double * 6)()
        st = (C.c_int32 * 1)()
        assert lib.sbg_realize_acceleration_noalloc(h, 1, y, y, st, None) == 6
        assert b"contact" in lib.sbg_noalloc_last_error()
    finally:
        lib.sbg_topology_destroy(h)


def test_closure_counts_and_redundant_closures():
    """Redundant closures are taken as Simbody builds them: a repeated
    closure and a second pinned point of the same body. Batches hold up to
    four closures per system (12 equations, the multiplier solve's fixed
    size); a batch of a system with five is refused SBG_ERR_UNSUPPORTED
    before any device is touched (the server refuses it at submit)."""
    lib = N.engine_lib()
    b = chain(8, N.SBG_BALL)
    c = (N.BallConstraintDesc * 5)()
    for k, (body, s) in enumerate([(8, 0.0), (8, 0.0), (8, 0.1), (6, 0.0), (4, 0.0)]):
        c[k].body1, c[k].body2 = body, 0
        c[k].station1[0] = s
    t4 = Topology(make(b, 8, None, 0, c, 4), keepalive=(b, c))
    assert t4.nbodies == 8
    t5 = Topology(make(b, 8, None, 0, c, 5), keepalive=(b, c))
    which = (C.c_int32 * 1)(0)
    cfg = N.BatchConfig(N.PRECISION_FP64, 0, 0)
    h = C.c_void_p()
    topos = (C.c_void_p * 1)(t5.handle)
    assert lib.sbg_batch_create(topos, 1, which, 1, C.byref(cfg), C.byref(h)) == 6  # SBG_ERR_UNSUPPORTED
    assert b"at most 4" in lib.sbg_last_error()
