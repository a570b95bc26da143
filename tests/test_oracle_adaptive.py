"""The oracle's error-controlled RK-Merson (the next row after the fixed-step
path): the step-size controller and the accept/reject loop of the reference's
AbstractIntegratorRep, restated for instances without constraints.

Pinned two ways:
  * With hMin = hMax = hInit = h (what Integrator::setFixedStepSize does,
    Integrator.cpp:263-267) the loop must take the fixed-step path: every
    attempt is accepted and the last step lands on the final time. It then
    reproduces the reference's recorded RK-Merson states
    (tests/golden/reference_vectors.npz), and the fixed-step oracle bit for
    bit.
  * The controller adjustStepSize (AbstractIntegratorRep.cpp:448-502) is a
    pure function; its cases are checked against the reference formula
    evaluated by hand: safety 0.9, shrink at least to 0.9 h and at most to
    0.1 h, grow at most 5 h and only beyond 1.2 h, keep h after an accepted
    error, and clamp to the user's limits.
Error control itself is checked on the double pendulum: the global error
falls with the requested accuracy, and so does the step size.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from simbody_gb300 import Workload

GOLD = Path(__file__).resolve().parent / "golden" / "reference_vectors.npz"
ACC = 1e-3


@pytest.mark.parametrize("err,limited,h_min,h_max,ok,factor", [
    (0.0, False, 0, 0, True, 5.0),                                    # perfect step: grow 5x
    (0.0, True, 0, 0, True, 1.0),                                     # ... unless h was limited
    (ACC, False, 0, 0, True, 1.0),                                    # accepted error: keep h
    (2 * ACC, False, 0, 0, False, 0.9 * 0.5 ** 0.25),                 # 0.9 (acc/err)^(1/4)
    (1.01 * ACC, False, 0, 0, False, 0.9 * (1 / 1.01) ** 0.25),       # shrink at least to 0.9 h
    (1e-3 * ACC, False, 0, 0, True, 5.0),                             # growth capped at 5x
    (ACC * (0.9 / 1.1) ** 4, False, 0, 0, True, 1.0),                 # growth below 1.2x: keep
    (ACC * (0.9 / 1.3) ** 4, False, 0, 0, True, 1.3),                 # growth above 1.2x: take it
    (1e6 * ACC, False, 0, 0, False, 0.1),                             # shrink at most to 0.1 h
    (float("nan"), False, 0, 0, False, 0.1),                          # non-finite error
    (float("inf"), False, 0, 0, False, 0.1),
    (1e6 * ACC, False, 0.5, 0, False, 0.5),                           # user minimum
    (0.0, False, 0, 2.0, True, 2.0),                                  # user maximum
])
def test_step_size_controller(err, limited, h_min, h_max, ok, factor):
    h = 0.01
    got_ok, h_new = O.adjust_step_size(err, h, accuracy=ACC, limited=limited, h_min=h_min * h, h_max=h_max * h)
    assert got_ok == ok
    assert h_new == pytest.approx(factor * h, rel=1e-14)


def test_fixed_limits_reproduce_the_reference_fixed_step_states():
    g = dict(np.load(GOLD))
    w_all = {c: Workload(c, n) for c, n in {1: 8, 2: 4, 3: 6, 4: 8, 5: 64, 6: 8, 7: 6, 8: 8, 9: 64, 10: 6}.items()}
    checked = 0
    for r in range(len(g["cfg"])):
        cfg, inst = int(g["cfg"][r]), int(g["inst"][r])
        w = w_all[cfg]
        if w.systems[int(w.instance_system[inst])].nconstraints or g["nsteps"][r] == 0:
            continue
        ys = slice(int(g["y_off"][r]), int(g["y_off"][r + 1]))
        h, t_final, ctol = float(g["h"][r]), float(g["t_rk"][r]), float(g["cons_tol"][r])
        off = np.array([0, ys.stop - ys.start])
        ya, ta, sa, stats = O.rk_merson_adaptive(w.systems, w.nsys, w.instance_system[[inst]], off, g["y0"][ys],
                                                 t_final, h_init=h, h_min=h, h_max=h, cons_tol=ctol)
        yf, _, _, _ = O.rk_merson(w.systems, w.nsys, w.instance_system[[inst]], off, g["y0"][ys], h,
                                  int(g["nsteps"][r]), cons_tol=ctol)
        assert sa[0] == 0 and ta[0] == t_final
        assert tuple(stats[0]) == (int(g["nsteps"][r]), 0)
        assert np.array_equal(ya, yf)
        assert np.linalg.norm(ya - g["y_rk"][ys]) <= 1e-11 * np.linalg.norm(g["y_rk"][ys]), (cfg, inst)
        checked += 1
    assert checked >= 20


def test_error_control_on_the_double_pendulum():
    w = Workload(1, 16)
    off = w.y_offsets[:17]
    y0 = w.y0[: int(off[-1])]
    yref, tref, st, _ = O.rk_merson(w.systems, w.nsys, w.instance_system, off, y0, 1e-4, 10000)
    assert (st == 0).all() and np.allclose(tref, 1.0)

    def run(acc):
        y, t, s, stats = O.rk_merson_adaptive(w.systems, w.nsys, w.instance_system, off, y0, 1.0, accuracy=acc)
        assert (s == 0).all() and (t == 1.0).all()
        err = max(np.linalg.norm(y[off[i]:off[i + 1]] - yref[off[i]:off[i + 1]]) /
                  np.linalg.norm(yref[off[i]:off[i + 1]]) for i in range(16))
        return err, stats[:, 0].mean()

    e3, n3 = run(1e-3)
    e6, n6 = run(1e-6)
    e8, n8 = run(1e-8)
    assert e8 < e6 < e3 and n3 < n6 < n8
    assert e6 <= 1e-4 and e8 <= 1e-6
    # far fewer steps than the fixed 1,000 of the benchmark configuration
    assert n3 < 50


def test_loop_closures_are_refused():
    w = Workload(5, 64)
    i = next(k for k in range(w.ninst) if w.systems[int(w.instance_system[k])].nconstraints)
    sl = w.instance_slice(i)
    with pytest.raises(RuntimeError, match="loop closures"):
        O.rk_merson_adaptive(w.systems, w.nsys, w.instance_system[[i]], np.array([0, sl.stop - sl.start]),
                             w.y0[sl], 0.1)


def _adaptive_records(g):
    for r in range(len(g["a_cfg"])):
        ys = slice(int(g["a_y_off"][r]), int(g["a_y_off"][r + 1]))
        yield r, int(g["a_cfg"][r]), int(g["a_inst"][r]), ys


def test_error_controlled_matches_reference_records():
    """The reference's error-controlled RungeKuttaMersonIntegrator
    (setAccuracy, setFinalTime, stepTo; default initial step, no step limits)
    recorded on the seeded workloads, double pendulum to the trees: the oracle
    takes the same numbers of accepted and rejected steps, ends on the final
    time and reproduces the final state to 1e-11."""
    g = dict(np.load(GOLD))
    sizes = {1: 8, 2: 4, 3: 6, 4: 8, 6: 8, 7: 6, 8: 8, 9: 64, 10: 6}
    ws = {c: Workload(c, n) for c, n in sizes.items()}
    for r, cfg, inst, ys in _adaptive_records(g):
        assert g["a_status"][r] == 0
        w = ws[cfg]
        y0 = g["a_y0"][ys]
        assert np.array_equal(w.y0[w.instance_slice(inst)], y0)
        y, t, st, stats = O.rk_merson_adaptive(w.systems, w.nsys, w.instance_system[[inst]], np.array([0, len(y0)]),
                                               y0, float(g["a_t_final"][r]), accuracy=float(g["a_accuracy"][r]))
        assert st[0] == 0
        assert t[0] == g["a_t_out"][r]
        assert stats[0, 0] == g["a_taken"][r], (cfg, inst, stats[0], g["a_taken"][r], g["a_attempted"][r])
        assert stats[0, 0] + stats[0, 1] == g["a_attempted"][r], (cfg, inst, stats[0], g["a_attempted"][r])
        rel = np.linalg.norm(y - g["a_y_out"][ys]) / np.linalg.norm(g["a_y_out"][ys])
        assert rel <= 1e-11, (cfg, inst, rel)
