"""The mixed form on ill-conditioned states: detection and FP64 fallback.

FP32 recursions plus one double-float refinement step reach the 1e-5 udot bar
only while the FP32 factorisation of M is good enough. Along random-tree
trajectories M becomes ill-conditioned often enough that the refinement
correction grows to the size of udot itself. The kernels detect this from the
size of the correction. Then:
  * a mixed realize recomputes those instances in FP64 (status 0, counted by
    sbg_batch_fallback_count); threshold 1e-4 of udot;
  * a mixed batch integration takes the step in FP64, and the next 15 of that
    instance; threshold 1e-5;
  * the server's mixed lane continues such a request in FP64
    (info fp64_steps = 1, status 0); threshold 1e-5.

Along FP64 trajectories of the random-tree and uneven workloads (108,000
states sampled on a GB300) a 1e-5 threshold flagged 14-17 % of the states and
left none above 1e-5; 1e-4 flagged 3-4 % and let three states per workload
through, up to 3.5e-5 (their error comes from the FP32 position kinematics,
which the correction does not see).

The states here come from FP64 integrations of the serving stream's trees
(2,000 steps), where such states are common. The bar is the mixed form's:
every instance within 1e-5.
"""
import numpy as np
import pytest

from simbody_gb300 import Server, Workload, engine_batch
from simbody_gb300.engine import Topology

pytestmark = pytest.mark.gpu



def _udot(d, b):
    return [d[b.y_offsets[i] + b.nq[i]:b.y_offsets[i + 1]] for i in range(b.ninst)]


@pytest.fixture(scope="module")
def trees():
    w = Workload(5, 320)
    idx = [i for i in range(w.ninst) if w.systems[int(w.instance_system[i])].nconstraints == 0][:192]
    b64, y0 = engine_batch(w, "fp64", instances=idx)
    b64.set_state(y0)
    st = b64.rk_merson_fixed(w.h, 2000)
    assert (st == 0).all()
    y, _ = b64.get_state()
    return w, idx, y


def test_mixed_realize_falls_back_to_fp64_on_ill_conditioned_states(engine, trees):
    w, idx, y = trees
    b64, _ = engine_batch(w, "fp64", instances=idx)
    bmx, _ = engine_batch(w, "mixed", instances=idx)
    b64.set_state(y)
    bmx.set_state(y)
    d64, s64 = b64.realize_acceleration()
    dmx, smx = bmx.realize_acceleration()
    assert (s64 == 0).all() and (smx == 0).all()
    assert bmx.fallback_count() > 0
    err = np.array([np.linalg.norm(a - r) / np.linalg.norm(r) for a, r in zip(_udot(dmx, bmx), _udot(d64, b64))])
    assert err.max() <= 1e-5, np.sort(err)[-5:]


def test_mixed_batch_integration_takes_ill_conditioned_steps_in_fp64(engine, trees):
    """From ill-conditioned states a mixed batch integration takes the
    affected steps in FP64: no instance reports the bit, every instance ends
    at the same time as the FP64 integration, within the mixed bar of it, and
    two calls of 15 steps give the bits of one call of 30."""
    w, idx, y = trees
    bmx, _ = engine_batch(w, "mixed", instances=idx)
    b64, _ = engine_batch(w, "fp64", instances=idx)
    bmx.set_state(y)
    b64.set_state(y)
    st = bmx.rk_merson_fixed(w.h, 30)
    s64 = b64.rk_merson_fixed(w.h, 30)
    assert (st & ~4 == 0).all() and (s64 & ~4 == 0).all()
    ym, tm = bmx.get_state()
    y64, t64 = b64.get_state()
    np.testing.assert_array_equal(tm, t64)
    err = np.array([np.linalg.norm(ym[a:e] - y64[a:e]) / np.linalg.norm(y64[a:e])
                    for a, e in zip(bmx.y_offsets[:-1], bmx.y_offsets[1:])])
    assert err.max() <= 1e-6, np.sort(err)[-5:]
    b2, _ = engine_batch(w, "mixed", instances=idx)
    b2.set_state(y)
    b2.rk_merson_fixed(w.h, 15)
    b2.rk_merson_fixed(w.h, 15, continue_integration=True)
    yb, tb = b2.get_state()
    np.testing.assert_array_equal(yb, ym)
    np.testing.assert_array_equal(tb, tm)
    # the states were ill-conditioned: the unrefined FP32 form is far off on some
    probe, _ = engine_batch(w, "mixed_fast", instances=idx)
    probe.set_state(y)
    dfa, _ = probe.realize_acceleration()
    b64.set_state(y)
    d64, _ = b64.realize_acceleration()
    efa = [np.linalg.norm(a - r) / np.linalg.norm(r) for a, r in zip(_udot(dfa, probe), _udot(d64, b64))]
    assert max(efa) > 1e-4


def test_server_continues_ill_conditioned_requests_in_fp64(engine, trees):
    """Requests that start in an ill-conditioned state: the mixed lane runs
    them in FP64 and they match the FP64 batch integration to the mixed
    bar; each is the same alone and in the mix."""
    w, idx, y = trees
    bfa, _ = engine_batch(w, "mixed_fast", instances=idx)
    b64, _ = engine_batch(w, "fp64", instances=idx)
    bfa.set_state(y)
    b64.set_state(y)
    dfa, _ = bfa.realize_acceleration()
    d64, _ = b64.realize_acceleration()
    efa = np.array([np.linalg.norm(a - r) / np.linalg.norm(r) for a, r in zip(_udot(dfa, bfa), _udot(d64, b64))])
    flagged = np.argsort(-efa)[:8]  # the worst-conditioned states (unrefined FP32 error)
    assert efa[flagged[1]] > 1e-4
    bmx = bfa
    steps = 20
    srv = Server("mixed", device_budget_bytes=1 << 30, chunk_steps=8)
    topos, ids = {}, {}
    for k in flagged:
        i = idx[k]
        topos[k] = Topology(w.systems[int(w.instance_system[i])], keepalive=w)
        ids[k] = srv.submit(topos[k], y[bmx.y_offsets[k]:bmx.y_offsets[k + 1]], w.h, steps)
    srv.drain()
    switched = 0
    for k in flagged:
        ys, inf = srv.result(ids[k])
        assert inf["status"] == 0
        switched += inf["fp64_steps"]
        b64, _ = engine_batch(w, "fp64", instances=[idx[k]])
        b64.set_state(y[bmx.y_offsets[k]:bmx.y_offsets[k + 1]])
        assert b64.rk_merson_fixed(w.h, steps)[0] == 0
        yb, _ = b64.get_state()
        assert np.linalg.norm(ys - yb) / np.linalg.norm(yb) <= 1e-5, k
    assert switched >= len(flagged) // 2
    k = flagged[0]
    alone = Server("mixed", device_budget_bytes=1 << 30, chunk_steps=8)
    rid = alone.submit(topos[k], y[bmx.y_offsets[k]:bmx.y_offsets[k + 1]], w.h, steps)
    alone.drain()
    assert np.array_equal(alone.result(rid)[0], srv.result(ids[k])[0])


def test_mixed_integration_switches_to_fp64_when_most_steps_need_it(engine, trees):
    """From the ill-conditioned states a quarter or more of the instance steps
    need FP64: after its first 64-launch window the integration continues on
    the FP64 kernels (a few launches instead of two per step), and it stays
    within the mixed bar of the FP64 integration."""
    w, idx, y = trees
    bmx, _ = engine_batch(w, "mixed", instances=idx)
    b64, _ = engine_batch(w, "fp64", instances=idx)
    bmx.set_state(y)
    b64.set_state(y)
    bmx.realize_acceleration()  # tunes the batch (its timing launches are counted too)
    steps = 256
    l0, f0 = bmx.launch_count, bmx.fp64_steps()
    st = bmx.rk_merson_fixed(w.h, steps)
    launches, fp64 = bmx.launch_count - l0, bmx.fp64_steps() - f0
    assert (st & ~4 == 0).all()
    assert fp64 > len(idx) * 64 // 4, fp64  # the first window's share was above a quarter
    # ... so the rest ran on the FP64 kernels: a few launches, not two or more per step
    assert launches < 1.5 * steps, launches
    b64.rk_merson_fixed(w.h, steps)
    ym, tm = bmx.get_state()
    y64, t64 = b64.get_state()
    np.testing.assert_array_equal(tm, t64)
    err = np.array([np.linalg.norm(ym[a:e] - y64[a:e]) / np.linalg.norm(y64[a:e])
                    for a, e in zip(bmx.y_offsets[:-1], bmx.y_offsets[1:])])
    assert np.median(err) <= 1e-6, np.median(err)
