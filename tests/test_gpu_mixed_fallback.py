"""The mixed form on ill-conditioned states: detection and FP64 fallback.

FP32 recursions plus one double-float refinement step reach the 1e-5 udot bar
only while the FP32 factorisation of M is good enough. Along random-tree
trajectories M becomes ill-conditioned often enough that the refinement
correction grows to the size of udot itself. The kernels detect this: a
correction above 1e-4 of udot sets SBG_INST_ILL_CONDITIONED. Then:
  * a mixed realize recomputes those instances in FP64 (status 0, counted by
    sbg_batch_fallback_count);
  * the server's mixed lane continues such a request in FP64
    (info fp64_steps = 1, status 0);
  * a mixed batch integration reports the bit.

The states come from FP64 integrations of the serving stream's trees (2,000
steps), where such states are common. A CPU emulation of the mixed RHS along
those trajectories flagged 18 % of the states; the unflagged ones stayed
within 2.2e-5 (a floor set by the FP32 kinematics, which the correction does
not see). So the bar here is: every instance within 3e-5, and 99 % within
1e-5.
"""
import numpy as np
import pytest

from simbody_gb300 import Server, Workload, engine_batch
from simbody_gb300.engine import Topology

pytestmark = pytest.mark.gpu

ILL = 32


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
    assert err.max() <= 3e-5, err.max()
    assert np.mean(err <= 1e-5) >= 0.99, np.sort(err)[-5:]


def test_mixed_batch_integration_reports_ill_conditioning(engine, trees):
    w, idx, y = trees
    bmx, _ = engine_batch(w, "mixed", instances=idx)
    bmx.set_state(y)
    st = bmx.rk_merson_fixed(w.h, 1)
    assert (st & ~(ILL | 4) == 0).all()
    assert (st & ILL).any()


def test_server_continues_ill_conditioned_requests_in_fp64(engine, trees):
    """Requests that start in an ill-conditioned state: the mixed lane runs
    them in FP64 and they match the FP64 batch integration to the mixed
    bar; each is the same alone and in the mix."""
    w, idx, y = trees
    bmx, _ = engine_batch(w, "mixed", instances=idx)
    bmx.set_state(y)
    flagged = np.nonzero(bmx.rk_merson_fixed(w.h, 1) & ILL)[0][:8]
    assert len(flagged) >= 2
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
