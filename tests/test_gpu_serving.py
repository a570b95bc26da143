"""The serving loop on the GPU (sbg_server_* through the C ABI): requests of
different topologies and horizons, 20% with Ball loop closures, admitted
while others run.

  - A request's result is the same alone and in the mix: bit for bit, since
    its arithmetic depends only on its own tables and state (tolerance 0).
  - It matches the batch path (sbg_rk_merson_fixed of the same instance):
    FP64 requests to 1e-10 relative (the server runs every tree on the
    level-parallel driver, the batch may pick the one-thread driver, whose
    sums over children run in another order), mixed ones to 1e-5 against
    the FP64 batch over these short horizons.
  - A small device budget bounds how many requests are resident, and the
    results do not change.
"""
import ctypes as C

import numpy as np
import pytest

from simbody_gb300 import Server, Workload, engine_batch
from simbody_gb300 import _native as N
from simbody_gb300.engine import Topology

pytestmark = pytest.mark.gpu

NREQ = 40


@pytest.fixture(scope="module")
def w5():
    return Workload(5, NREQ)


@pytest.fixture(scope="module")
def topos(w5):
    return [Topology(w5.systems[int(w5.instance_system[i])], keepalive=w5) for i in range(NREQ)]


def horizons(w5):
    # the stream's log-uniform horizons, scaled down to keep the test short
    return np.maximum(1, (w5.horizons // 40)).astype(int)


def run(server, w5, topos, idx, stagger=0):
    """Submit requests idx (optionally a few per tick) and drain."""
    hz = horizons(w5)
    ids = {}
    for k, i in enumerate(idx):
        ids[i] = server.submit(topos[i], w5.y0[w5.instance_slice(i)], w5.h, int(hz[i]))
        if stagger and k % stagger == stagger - 1:
            server.tick()
    server.drain()
    out = {}
    for i, rid in ids.items():
        res = server.result(rid)
        assert res is not None
        out[i] = res
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_result_alone_equals_result_in_the_mix(engine, w5, topos, precision):
    assert sum(w5.systems[int(w5.instance_system[i])].nconstraints > 0 for i in range(NREQ)) >= 4
    mix = run(Server(precision, device_budget_bytes=1 << 30, chunk_steps=16), w5, topos, range(NREQ), stagger=3)
    picks = [i for i in range(NREQ) if w5.systems[int(w5.instance_system[i])].nconstraints > 0][:3] + [0, 1, 7]
    for i in picks:
        alone = run(Server(precision, device_budget_bytes=1 << 30, chunk_steps=16), w5, topos, [i])[i]
        y_mix, inf_mix = mix[i]
        y_alone, inf_alone = alone
        assert inf_mix["status"] == 0 and inf_alone["status"] == 0
        assert np.array_equal(y_mix, y_alone), (i, np.abs(y_mix - y_alone).max())
        assert inf_mix["t"] == inf_alone["t"]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
def test_server_matches_batch_integration(engine, w5, topos, precision, tol):
    hz = horizons(w5)
    res = run(Server(precision, device_budget_bytes=1 << 30, chunk_steps=16), w5, topos, range(NREQ), stagger=5)
    for i in range(0, NREQ, 3):
        b, y0 = engine_batch(w5, "fp64", instances=[i])
        b.set_state(y0)
        st = b.rk_merson_fixed(w5.h, int(hz[i]))
        yb, tb = b.get_state()
        y, inf = res[i]
        assert st[0] == 0 and inf["status"] == 0
        err = np.linalg.norm(y - yb) / np.linalg.norm(yb)
        assert err <= tol, (i, err)
        assert abs(inf["t"] - tb[0]) <= 1e-12


def test_small_budget_limits_residency_not_results(engine, w5, topos):
    big = run(Server("mixed", device_budget_bytes=1 << 30, chunk_steps=16), w5, topos, range(NREQ))
    small = Server("mixed", device_budget_bytes=48 << 20, max_slots=6, chunk_steps=16)
    res = run(small, w5, topos, range(NREQ))
    st = small.stats()
    assert st["peak_resident"] <= 6 and st["completed"] == NREQ
    for i in range(NREQ):
        assert np.array_equal(res[i][0], big[i][0])
        assert res[i][1]["admit_s"] >= res[i][1]["submit_s"]
        assert res[i][1]["done_s"] >= res[i][1]["admit_s"]


def test_request_larger_than_the_budget_is_rejected(engine, w5, topos):
    srv = Server("mixed", device_budget_bytes=48 << 20, max_slots=4)
    big = max(range(NREQ), key=lambda i: topos[i].nbodies)
    # a small budget still has room for the largest tree of the stream...
    srv.submit(topos[big], w5.y0[w5.instance_slice(big)], w5.h, 3)
    srv.drain()
    assert srv.result(1) is not None
    # ...but a 20,000-body chain does not fit it
    n = 20000
    bodies = (N.BodyDesc * n)()
    for k in range(n):
        b = bodies[k]
        b.parent, b.mobilizer, b.mass = k, N.SBG_PIN, 1.0
        b.unit_inertia[0] = b.unit_inertia[1] = b.unit_inertia[2] = 1.0
        for j in (0, 4, 8):
            b.X_PF[j] = b.X_BM[j] = 1.0
        b.X_BM[10] = 0.1
    d = N.SystemDesc(n, 0, 0, 0, (C.c_double * 3)(0, -9.8, 0), bodies, None, None)
    chain = Topology(d, keepalive=bodies)
    with pytest.raises(N.EngineError) as e:
        srv.submit(chain, chain.default_state(), 1e-3, 10)
    assert e.value.code == 4  # SBG_ERR_BUDGET


def test_failed_mixed_request_is_rerun_in_fp64(engine, w5, topos):
    """A mixed-precision request that ends non-finite is rerun from its
    initial state in the FP64 lane (attempts == 2): here the state itself
    holds a NaN, so the rerun fails too and reports it; its neighbours are
    unaffected and keep attempts == 1."""
    srv = Server("mixed", device_budget_bytes=1 << 30, chunk_steps=16)
    i_bad, i_ok = 0, 1
    assert w5.systems[int(w5.instance_system[i_bad])].nconstraints == 0
    y_bad = w5.y0[w5.instance_slice(i_bad)].copy()
    y_bad[2] = np.nan
    rb = srv.submit(topos[i_bad], y_bad, w5.h, 20)
    ro = srv.submit(topos[i_ok], w5.y0[w5.instance_slice(i_ok)], w5.h, 20)
    srv.drain()
    yb, ib = srv.result(rb)
    yo, io = srv.result(ro)
    assert ib["attempts"] == 2 and ib["status"] & N.INST_NONFINITE
    assert io["attempts"] == 1 and io["status"] == 0 and np.isfinite(yo).all()
    assert srv.stats()["submitted"] == 2


def test_loop_requests_with_tight_tolerance_match_batch_integration(engine, w5, topos):
    """A constraint tolerance of 1e-9 makes the position and velocity
    projections run at every step. In the server they spread the Gram over
    the request's first three lanes; the batch path runs them on one thread.
    Both integrate to the same states (1e-10)."""
    loops = [i for i in range(NREQ) if w5.systems[int(w5.instance_system[i])].nconstraints > 0][:4]
    assert loops
    srv = Server("fp64", device_budget_bytes=1 << 30, chunk_steps=16)
    ids = {i: srv.submit(topos[i], w5.y0[w5.instance_slice(i)], w5.h, 60, constraint_tolerance=1e-9) for i in loops}
    srv.drain()
    for i in loops:
        y, inf = srv.result(ids[i])
        b, y0 = engine_batch(w5, "fp64", instances=[i])
        b.set_state(y0)
        st = b.rk_merson_fixed(w5.h, 60, constraint_tolerance=1e-9)
        yb, _ = b.get_state()
        assert st[0] == 0 and inf["status"] == 0
        err = np.linalg.norm(y - yb) / np.linalg.norm(yb)
        assert err <= 1e-10, (i, err)
    srv.close()
