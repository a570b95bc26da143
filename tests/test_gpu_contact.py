"""SmoothSphereHalfSpaceForce on the GPU (workload 8: trees of 20-40 bodies,
a contact sphere on every body, a tilted ground half-space, the lowest
sphere indented at t = 0), through the C ABI.

  - FP64 integration against the oracle, whose contact force is pinned to
    the reference's records (test_oracle_golden.py), over 400 steps of
    5e-4 s, during which the trees land and slide: <= 1e-9 relative, or, for
    an instance whose landing amplifies rounding (a body that bounces or
    starts to slip near a smoothing threshold amplifies 1e-15 into 1e-4),
    within 100 times the oracle's own response to a 1e-14 relative
    perturbation of the initial state.
  - The mixed form against FP64 over the same horizon, by the same rule with
    1e-5. The indentation is a small difference of body positions that FP32
    kinematics resolve only to about 1e-5 of it, so the mixed form takes
    instances with contact spheres through its FP64 path.
  - A zero parameter block stands for the reference's defaults: the engine
    gives the same accelerations as with the defaults written out.
  - The server integrates contact requests like the batch path, the same
    alone and in a mix; the allocation-free realize refuses them
    (test_topology_host.py).
"""
import numpy as np
import pytest

from oracle import oracle as O
from simbody_gb300 import Server, Workload, engine_batch
from simbody_gb300 import _native as N
from simbody_gb300.engine import Topology

pytestmark = pytest.mark.gpu


def _rel(a, b, off):
    return np.array([np.linalg.norm(a[off[i]:off[i + 1]] - b[off[i]:off[i + 1]]) /
                     max(np.linalg.norm(b[off[i]:off[i + 1]]), 1e-300) for i in range(len(off) - 1)])


@pytest.fixture(scope="module")
def w8():
    return Workload(8, 96)


STEPS = 400


@pytest.fixture(scope="module")
def oracle_runs(w8):
    """The oracle's trajectory and its response to a 1e-14 relative
    perturbation of y0 (per instance, relative): how much the instance
    amplifies rounding over the horizon."""
    ref, rt, rst, _ = O.rk_workload(w8, w8.h, STEPS)
    rng = np.random.default_rng(8)
    yp = w8.y0 * (1 + 1e-14 * rng.choice([-1.0, 1.0], size=w8.y0.size))
    pert, _, _, _ = O.rk_merson(w8.systems, w8.nsys, w8.instance_system, w8.y_offsets, yp, w8.h, STEPS)
    return ref, rt, rst, _rel(pert, ref, w8.y_offsets)


def test_contact_trajectory_fp64_matches_oracle(engine, w8, oracle_runs):
    ref, rt, rst, sens = oracle_runs
    b, y0 = engine_batch(w8, "fp64")
    b.set_state(y0)
    st = b.rk_merson_fixed(w8.h, STEPS)
    y, t = b.get_state()
    np.testing.assert_array_equal(st, rst)
    assert (st == 0).all()
    np.testing.assert_array_equal(t, rt)
    err = _rel(y, ref, b.y_offsets)
    bound = np.maximum(1e-9, 100 * sens)
    assert (err <= bound).all(), (err / bound).max()
    assert (err <= 1e-9).mean() >= 0.9, np.sort(err)[-10:]
    # the trees moved by more than the tolerance: contact and gravity acted
    assert _rel(y, y0, b.y_offsets).min() > 1e-3


def test_contact_trajectory_mixed_close_to_fp64(engine, w8, oracle_runs):
    sens = oracle_runs[3]
    b64, y0 = engine_batch(w8, "fp64")
    bm, _ = engine_batch(w8, "mixed")
    b64.set_state(y0)
    bm.set_state(y0)
    st64 = b64.rk_merson_fixed(w8.h, STEPS)
    st = bm.rk_merson_fixed(w8.h, STEPS)
    np.testing.assert_array_equal(st, st64)
    assert (st == 0).all()
    y64, _ = b64.get_state()
    ym, _ = bm.get_state()
    err = _rel(ym, y64, b64.y_offsets)
    bound = np.maximum(1e-5, 100 * sens)
    assert (err <= bound).all(), (err / bound).max()
    assert (err <= 1e-5).mean() >= 0.9, np.sort(err)[-10:]


def test_zero_parameter_block_is_the_reference_defaults(engine, w8):
    i = 7  # every eighth instance of workload 8 leaves the block zero
    d = w8.systems[int(w8.instance_system[i])]
    assert d.contacts[0].stiffness == 0
    spelled = (N.ContactDesc * d.ncontacts)()
    for k in range(d.ncontacts):
        spelled[k] = N.ContactDesc.from_buffer_copy(d.contacts[k])
        c = spelled[k]
        c.stiffness, c.dissipation, c.static_friction, c.dynamic_friction = 1.0, 0.0, 0.0, 0.0
        c.viscous_friction, c.transition_velocity, c.cf, c.bd, c.bv = 0.0, 0.01, 1e-5, 300.0, 50.0
    d2 = N.SystemDesc.from_buffer_copy(d)
    d2.contacts = spelled
    y0 = w8.y0[w8.instance_slice(i)]
    out = []
    for desc in (d, d2):
        from simbody_gb300.engine import Batch
        b = Batch([Topology(desc, keepalive=(w8, spelled))], np.zeros(1, np.int32), precision="fp64")
        b.set_state(y0)
        ydot, st = b.realize_acceleration()
        assert st[0] == 0
        out.append(ydot.copy())
    np.testing.assert_array_equal(out[0], out[1])


def test_server_integrates_contact_spheres(engine, w8):
    """Contact requests in the server: FP64 results match the batch path
    (1e-9: the server's level-parallel driver sums children in another
    order over 40 steps of landing trees); in a mixed server they switch to
    FP64 within their first step (the indentation is beyond FP32) and match
    to 1e-8; and a
    request's result is the same alone and among tree requests without
    spheres (bit for bit)."""
    idx = list(range(8))
    topos = {i: Topology(w8.systems[int(w8.instance_system[i])], keepalive=w8) for i in idx}
    steps = 40
    ref = {}
    for i in idx:
        b, y0 = engine_batch(w8, "fp64", instances=[i])
        b.set_state(y0)
        st = b.rk_merson_fixed(w8.h, steps)
        assert st[0] == 0
        ref[i] = b.get_state()[0]
    w5 = Workload(5, 24)
    t5 = [Topology(w5.systems[int(w5.instance_system[i])], keepalive=w5) for i in range(24)]
    for precision in ("fp64", "mixed"):
        srv = Server(precision, device_budget_bytes=1 << 30, chunk_steps=16)
        ids = {i: srv.submit(topos[i], w8.y0[w8.instance_slice(i)], w8.h, steps) for i in idx}
        srv.drain()
        alone = {}
        for i in idx:
            y, inf = srv.result(ids[i])
            assert inf["status"] == 0, (precision, i, inf["status"])
            if precision == "mixed":
                assert inf["fp64_steps"] == 1
            err = np.linalg.norm(y - ref[i]) / np.linalg.norm(ref[i])
            # mixed: the switch to FP64 comes within the request's first step
            assert err <= (1e-9 if precision == "fp64" else 1e-8), (precision, i, err)
            alone[i] = y
        srv.close()
        srv = Server(precision, device_budget_bytes=1 << 30, chunk_steps=16)
        mix = {}
        for k, i in enumerate(idx):
            mix[i] = srv.submit(topos[i], w8.y0[w8.instance_slice(i)], w8.h, steps)
            for j in range(3 * k, 3 * k + 3):
                srv.submit(t5[j], w5.y0[w5.instance_slice(j)], w5.h, 30)
            srv.tick()
        srv.drain()
        for i in idx:
            y, _ = srv.result(mix[i])
            assert np.array_equal(y, alone[i]), (precision, i)
        srv.close()


def _with_spheres(w, every=2, seed=3):
    """Put a contact sphere on each body of every `every`-th system of
    workload w (in place), over a ground half-space whose surface lies at
    y = -0.1, so that the lower bodies of about half of those trees press
    into it; returns the arrays to keep alive."""
    rng = np.random.default_rng(seed)
    keep = []
    for k in range(0, w.nsys, every):
        d = w.systems[k]
        arr = (N.ContactDesc * d.nbodies)()
        for j in range(d.nbodies):
            c = arr[j]
            c.body, c.radius = j + 1, 0.05
            c.station[0], c.station[1], c.station[2] = rng.uniform(-0.05, 0.05, 3)
            c.halfspace[1], c.halfspace[3], c.halfspace[8] = 1.0, -1.0, 1.0  # x axis (the normal) = -Y
            c.halfspace[10] = -0.1  # surface at y = -0.1: the lower bodies start below it
            c.stiffness, c.dissipation, c.static_friction, c.dynamic_friction = 1e5, 1.0, 0.6, 0.4
            c.viscous_friction, c.transition_velocity, c.cf, c.bd, c.bv = 0.1, 0.2, 1e-5, 300.0, 50.0
        d.ncontacts, d.contacts = d.nbodies, arr
        keep.append(arr)
    return keep


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_contacts_with_loop_closures_and_mixed_batches(engine, precision):
    """Contact spheres on every other system of the serving mix (trees with
    and without Ball loop closures) in one batch: realize against the
    oracle (FP64 1e-12; mixed 1e-5), and a short integration (1e-9)."""
    w = Workload(5, 48)
    keep = _with_spheres(w)
    assert any(w.systems[k].nconstraints > 0 and w.systems[k].ncontacts > 0 for k in range(w.nsys))
    b, y0 = engine_batch(w, precision)
    b.set_state(y0)
    ydot, st = b.realize_acceleration()
    ref, rst = O.realize_workload(w)
    assert (st == 0).all() and (rst == 0).all()
    err = _rel(ydot, ref, b.y_offsets)
    assert err.max() <= (1e-12 if precision == "fp64" else 1e-5), err.max()
    if precision == "fp64":
        b.set_state(y0)
        st = b.rk_merson_fixed(w.h, 20)
        y, _ = b.get_state()
        ry, _, rst, _ = O.rk_workload(w, w.h, 20)
        assert (st == 0).all() and (rst == 0).all()
        assert _rel(y, ry, b.y_offsets).max() <= 1e-9
    del keep
