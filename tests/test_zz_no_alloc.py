"""The allocation-free realize entry point (sbg_realize_acceleration_noalloc).

Callers that may not allocate device memory (a control loop that allocates only
at start-up, a framework that hands out device buffers from its own pool) get
a realize(Stage::Acceleration) whose scratch lives in a fixed file-scope device
array. This test drives it through the C ABI with device buffers it owns and
checks two calls in a row against the regular entry point
(sbg_realize_acceleration), to the FP64 parity tolerance 1e-12. The file is
named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from simbody_gb300 import Workload, engine_batch
from simbody_gb300 import _native as N
from simbody_gb300.engine import Topology

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _noalloc(topo, n, y_host):
    import torch

    lib = N.engine_lib()
    ny = y_host.size // n
    y = torch.from_numpy(y_host).cuda()
    ydot = torch.full((n * ny,), float("nan"), dtype=torch.float64, device="cuda")
    st = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.sbg_realize_acceleration_noalloc(topo.handle, n, C.c_void_p(y.data_ptr()), C.c_void_p(ydot.data_ptr()),
                                              C.c_void_p(st.data_ptr()), None)
    assert rc == 0, lib.sbg_noalloc_last_error().decode()
    torch.cuda.synchronize()
    return ydot.cpu().numpy(), st.cpu().numpy()


def _regular(w, y0):
    b, _ = engine_batch(w, "fp64")
    b.set_state(y0)
    return b.realize_acceleration()


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_noalloc_matches_regular_entry_point_twice(engine):
    pytest.importorskip("torch")
    w = Workload(2, 2048)  # more instances than the 16 MiB scratch holds at once
    topo = Topology(w.systems[0], keepalive=w)
    y0 = w.y0.copy()
    ref1, rst1 = _regular(w, y0)
    got1, st1 = _noalloc(topo, w.ninst, y0)
    assert (st1 == 0).all() and (rst1 == 0).all()
    assert _rel(got1, ref1) <= TOL

    # second call in a row, different states: nothing left over from the first
    rng = np.random.default_rng(11)
    y1 = y0.copy()
    nq = 128
    for i in range(w.ninst):
        s = slice(int(w.y_offsets[i]) + nq, int(w.y_offsets[i + 1]))
        y1[s] += rng.normal(scale=0.3, size=s.stop - s.start)
    w.y0[:] = y1
    ref2, _ = _regular(w, y1)
    got2, st2 = _noalloc(topo, w.ninst, y1)
    assert (st2 == 0).all()
    assert _rel(got2, ref2) <= TOL
    assert _rel(got2, got1) > 1e-6  # the inputs really differed


def _one_topology_batch(w, inst, n, seed):
    """n states of instance inst's topology: its seeded state plus noise."""
    from simbody_gb300.engine import Batch

    k = int(w.instance_system[inst])
    topo = Topology(w.systems[k], keepalive=w)
    y0 = w.y0[w.instance_slice(inst)]
    rng = np.random.default_rng(seed)
    y = np.tile(y0, n) + rng.normal(scale=0.05, size=n * y0.size)
    b = Batch([topo], np.zeros(n, dtype=np.int32), precision="fp64")
    return topo, b, y


@pytest.mark.parametrize("config,inst,n", [
    (3, 0, 1500),    # branched tree, Free base: 6-wide Free records, children pushed into a parent's record
    (3, 5, 1500),    # another random tree
    (1, 0, 20000),   # two-Pin chain: one-mobility records; more instances than the scratch holds at once
])
def test_noalloc_matches_regular_on_trees_and_pin_chains(engine, config, inst, n):
    """Two calls in a row on one topology of a workload, against the regular
    entry point. The instance counts exceed what the 16 MiB scratch holds at
    once, so the kernel's threads loop over several instances each."""
    pytest.importorskip("torch")
    w = Workload(config, max(inst + 1, 8))
    topo, b, y = _one_topology_batch(w, inst, n, seed=config * 100 + inst)
    assert topo.nbodies > 1
    for call in range(2):
        yy = y if call == 0 else y + 0.01 * np.sin(np.arange(y.size))
        b.set_state(yy)
        ref, rst = b.realize_acceleration()
        got, st = _noalloc(topo, n, yy)
        assert (st == rst).all()
        assert (st == 0).mean() > 0.99
        ok = st == 0
        ny = y.size // n
        e = np.abs(got - ref).reshape(n, ny)[ok].max() / np.abs(ref.reshape(n, ny)[ok]).max()
        assert e <= TOL, (call, e)


def test_noalloc_rejects_oversized_topology(engine):
    bodies = (N.BodyDesc * 300)()
    for i in range(300):
        b = bodies[i]
        b.parent, b.mobilizer, b.mass = i, N.SBG_PIN, 1.0
        b.unit_inertia[0] = b.unit_inertia[1] = b.unit_inertia[2] = 1.0
        for k in (0, 4, 8):
            b.X_PF[k] = b.X_BM[k] = 1.0
        b.X_BM[10] = 0.1
    d = N.SystemDesc(300, 0, 0, 0, (C.c_double * 3)(0, -9.8, 0), bodies, None, None)
    topo = Topology(d, keepalive=bodies)
    import torch

    y = torch.zeros(topo.nq + topo.nu, dtype=torch.float64, device="cuda")
    ydot = torch.zeros_like(y)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib = N.engine_lib()
    rc = lib.sbg_realize_acceleration_noalloc(topo.handle, 1, C.c_void_p(y.data_ptr()), C.c_void_p(ydot.data_ptr()),
                                              C.c_void_p(st.data_ptr()), None)
    assert rc == 1
    assert b"at most 256" in lib.sbg_noalloc_last_error()


def test_noalloc_refuses_a_capturing_stream(engine):
    """Its table uploads read host memory that ends with the call, so on a
    stream that is being captured it returns SBG_ERR_UNSUPPORTED before it
    enqueues anything, and the capture stays valid."""
    torch = pytest.importorskip("torch")
    w = Workload(2, 64)
    topo = Topology(w.systems[0], keepalive=w)
    ny = w.y0.size // w.ninst
    y = torch.from_numpy(w.y0.copy()).cuda()
    ydot = torch.zeros(w.ninst * ny, dtype=torch.float64, device="cuda")
    st = torch.zeros(w.ninst, dtype=torch.int32, device="cuda")
    _noalloc(topo, w.ninst, w.y0.copy())  # the first call's set-up, outside any capture
    lib = N.engine_lib()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    x = torch.zeros(4, device="cuda")
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        rc = lib.sbg_realize_acceleration_noalloc(topo.handle, w.ninst, C.c_void_p(y.data_ptr()),
                                                  C.c_void_p(ydot.data_ptr()), C.c_void_p(st.data_ptr()),
                                                  C.c_void_p(s.cuda_stream))
        x += 1
    assert rc == 6, rc  # SBG_ERR_UNSUPPORTED
    assert b"capturing" in lib.sbg_noalloc_last_error()
    g.replay()
    torch.cuda.synchronize()
    assert float(x[0]) == 1.0  # the capture held the other work (recorded, run once by the replay)
