"""Integrator continuation, stepTo with a shortened last step, and qdotdot on
the CUDA engine, through the C ABI.

* sbg_rk_merson_step_to with interpolation off (tMax = the report time): the
  reference's stepTo(t_mid); stepTo(t_end), stepTo(t_end) and
  stepTo(t_end + 0.3 h) records (tests/golden/reference_vectors.npz, made by a
  build of the reference) and the oracle's continuation, final time exactly
  and state to 1e-10 (FP64 trajectories).
* continue_integration on sbg_rk_merson_fixed: two calls of n steps equal one
  call of 2n steps bit for bit, and a call that re-initializes does not.
* sbg_batch_get_qdotdot: the reference's getQDotDot() records and the oracle
  to 1e-12.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from simbody_gb300 import Workload, engine_batch

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "reference_vectors.npz"
WORKLOAD_SIZES = {1: 8, 2: 4, 3: 6, 4: 8, 5: 64, 6: 8, 7: 6, 8: 8, 9: 64, 10: 6}


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _engine_continuation(w, mode, h, t_mid, t_end, precision="fp64"):
    b, y0 = engine_batch(w, precision)
    b.set_state(y0)
    if mode == 0:
        st = b.rk_merson_step_to(h, t_mid)
        st |= b.rk_merson_step_to(h, t_end, continue_integration=True)
    else:
        st = b.rk_merson_step_to(h, t_end if mode == 1 else t_end + 0.3 * h)
    y, t = b.get_state()
    return b, y, t, st


def test_step_to_matches_reference_records(engine, gold):
    workloads = {c: Workload(c, n) for c, n in WORKLOAD_SIZES.items()}
    done = set()
    for r in range(len(gold["c_cfg"])):
        cfg, inst, mode = int(gold["c_cfg"][r]), int(gold["c_inst"][r]), int(gold["c_mode"][r])
        if (cfg, mode) in done:
            continue
        done.add((cfg, mode))
        w = workloads[cfg]
        h, t_mid, t_end = float(gold["c_h"][r]), float(gold["c_t_mid"][r]), float(gold["c_t_end"][r])
        b, y, t, st = _engine_continuation(w, mode, h, t_mid, t_end)
        # every recorded instance of this config and mode
        for rr in range(len(gold["c_cfg"])):
            if int(gold["c_cfg"][rr]) != cfg or int(gold["c_mode"][rr]) != mode:
                continue
            i = int(gold["c_inst"][rr])
            ys = slice(int(gold["c_y_off"][rr]), int(gold["c_y_off"][rr + 1]))
            got = y[b.y_offsets[i]:b.y_offsets[i + 1]]
            assert st[i] == 0, (cfg, i, mode, st[i])
            assert t[i] == gold["c_t_out"][rr], (cfg, i, mode, t[i], gold["c_t_out"][rr])
            assert _rel(got, gold["c_y_out"][ys]) <= 1e-10, (cfg, i, mode, _rel(got, gold["c_y_out"][ys]))


@pytest.mark.parametrize("config,n", [(2, 64), (3, 64), (4, 32), (5, 64)])
def test_step_to_matches_oracle(engine, config, n):
    w = Workload(config, n)
    h = w.h if w.h > 0 else 5e-4  # the Ball-chain workload is realize-only
    t_mid, t_end = 7 * h, 15.5 * h
    for mode in (0, 2):
        b, y, t, st = _engine_continuation(w, mode, h, t_mid, t_end)
        off = b.y_offsets
        so = w.instance_system[:n]
        y0 = w.y0[: int(off[-1])]
        if mode == 0:
            ry, rt, rs = O.rk_merson_run(w.systems, w.nsys, so, off, y0, h, t_report=t_mid)
            ry, rt, rs2 = O.rk_merson_run(w.systems, w.nsys, so, off, ry, h, t_report=t_end, t=rt, initialize=False)
        else:
            ry, rt, rs = O.rk_merson_run(w.systems, w.nsys, so, off, y0, h, t_report=t_end + 0.3 * h)
        np.testing.assert_array_equal(t, rt)
        errs = [_rel(y[off[i]:off[i + 1]], ry[off[i]:off[i + 1]]) for i in range(n)]
        assert max(errs) <= 1e-10, (mode, max(errs))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_continue_fixed_equals_one_call(engine, precision):
    """n steps then n more with continue_integration = 2n steps in one call,
    bit for bit; re-initializing in between (quaternions renormalised) is a
    different trajectory."""
    w = Workload(3, 128)
    b1, y0 = engine_batch(w, precision)
    b1.set_state(y0)
    b1.rk_merson_fixed(w.h, 40)
    ya, ta = b1.get_state()
    b2, _ = engine_batch(w, precision)
    b2.set_state(y0)
    b2.rk_merson_fixed(w.h, 20)
    b2.rk_merson_fixed(w.h, 20, continue_integration=True)
    yb, tb = b2.get_state()
    np.testing.assert_array_equal(ya, yb)
    np.testing.assert_array_equal(ta, tb)
    b3, _ = engine_batch(w, precision)
    b3.set_state(y0)
    b3.rk_merson_fixed(w.h, 20)
    b3.rk_merson_fixed(w.h, 20)
    yc, _ = b3.get_state()
    assert not np.array_equal(ya, yc)


def test_continue_needs_a_started_integration(engine):
    import simbody_gb300._native as N

    w = Workload(1, 32)
    b, y0 = engine_batch(w, "fp64")
    b.set_state(y0)
    with pytest.raises(N.EngineError) as e:
        b.rk_merson_fixed(w.h, 5, continue_integration=True)
    assert e.value.code == 5  # SBG_ERR_STATE
    b.rk_merson_fixed(w.h, 5)
    b.set_state(y0)  # a new state ends the integration
    with pytest.raises(N.EngineError):
        b.rk_merson_step_to(w.h, 0.5, continue_integration=True)


def test_qdotdot_matches_reference_records(engine, gold):
    workloads = {c: Workload(c, n) for c, n in {**WORKLOAD_SIZES, 6: 8, 7: 6}.items()}
    for c, w in workloads.items():
        b, y0 = engine_batch(w, "fp64")
        b.set_state(y0)
        b.realize_acceleration()
        qdd = b.get_qdotdot()
        qoff = b.y_offsets - b.u_offsets
        for r in range(len(gold["cfg"])):
            if int(gold["cfg"][r]) != c:
                continue
            i = int(gold["inst"][r])
            qs = slice(int(gold["q_off"][r]), int(gold["q_off"][r + 1]))
            got = qdd[qoff[i]:qoff[i + 1]]
            assert _rel(got, gold["qdd"][qs]) <= 1e-12, (c, i, _rel(got, gold["qdd"][qs]))


@pytest.mark.parametrize("config,n", [(2, 256), (3, 256), (4, 64), (8, 64)])
def test_qdotdot_matches_oracle(engine, config, n):
    import simbody_gb300._native as N

    w = Workload(config, n)
    b, y0 = engine_batch(w, "fp64")
    b.set_state(y0)
    with pytest.raises(N.EngineError):
        b.get_qdotdot()  # nothing realized yet
    ydot, st = b.realize_acceleration()
    qdd = b.get_qdotdot()
    qoff = b.y_offsets - b.u_offsets
    ref = O.qdotdot(w.systems, w.nsys, w.instance_system[:n], b.y_offsets, y0, ydot, qoff)
    errs = [_rel(qdd[qoff[i]:qoff[i + 1]], ref[qoff[i]:qoff[i + 1]]) for i in range(n)]
    assert max(errs) <= 1e-12, max(errs)
