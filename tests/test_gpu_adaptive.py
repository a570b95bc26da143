"""The error-controlled RK-Merson kernel (sbg_rk_merson_adaptive) against the
reference's recorded error-controlled runs and the oracle.

Every instance keeps its own step size, accept/reject decisions and time in
one persistent kernel. Against the reference's records
(tests/golden/reference_vectors.npz: setAccuracy, setFinalTime, stepTo) and
against the oracle on whole batches (configs 1-4, several accuracies, step
limits, project-every-step), the kernel must take the same numbers of accepted
and rejected steps, end on the final time, and reach the same state to 1e-10
(FP64).
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from simbody_gb300 import Workload, engine_batch

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "reference_vectors.npz"


def _worst(a, b, off):
    return max(np.linalg.norm(a[off[i]:off[i + 1]] - b[off[i]:off[i + 1]]) / np.linalg.norm(b[off[i]:off[i + 1]])
               for i in range(len(off) - 1))


def test_adaptive_matches_reference_records(engine):
    g = dict(np.load(GOLD))
    sizes = {1: 8, 2: 4, 3: 6, 4: 8, 6: 8, 7: 6, 8: 8, 9: 64, 10: 6}
    for r in range(len(g["a_cfg"])):
        cfg, inst = int(g["a_cfg"][r]), int(g["a_inst"][r])
        w = Workload(cfg, sizes[cfg])
        b, y0 = engine_batch(w, "fp64", instances=[inst])
        b.set_state(y0)
        st, stats = b.rk_merson_adaptive(float(g["a_t_final"][r]), accuracy=float(g["a_accuracy"][r]))
        y, t = b.get_state()
        ys = slice(int(g["a_y_off"][r]), int(g["a_y_off"][r + 1]))
        assert st[0] == 0
        assert t[0] == g["a_t_out"][r]
        assert stats[0, 0] == g["a_taken"][r] and stats[0].sum() == g["a_attempted"][r], (cfg, inst, stats[0])
        rel = np.linalg.norm(y - g["a_y_out"][ys]) / np.linalg.norm(g["a_y_out"][ys])
        assert rel <= 1e-10, (cfg, inst, rel)


@pytest.mark.parametrize("config,n,t_final,kw", [
    (1, 512, 1.0, dict(accuracy=1e-4)),
    (2, 128, 0.05, dict()),
    (3, 256, 0.05, dict(accuracy=1e-4)),
    (3, 128, 0.03, dict(initial_step=1e-3, max_step=4e-3, project_every_step=True)),
    (4, 64, 0.02, dict(min_step=1e-4)),
    (8, 64, 0.03, dict()),
])
def test_adaptive_matches_oracle(engine, config, n, t_final, kw):
    w = Workload(config, n)
    b, y0 = engine_batch(w, "fp64")
    b.set_state(y0)
    st, stats = b.rk_merson_adaptive(t_final, **kw)
    y, t = b.get_state()
    okw = {k: v for k, v in kw.items() if k != "initial_step"}
    if "initial_step" in kw:
        okw["h_init"] = kw["initial_step"]
    if "min_step" in okw:
        okw["h_min"] = okw.pop("min_step")
    if "max_step" in okw:
        okw["h_max"] = okw.pop("max_step")
    ry, rt, rst, rstats = O.rk_merson_adaptive(w.systems, w.nsys, w.instance_system[:n], b.y_offsets, y0, t_final,
                                               **okw)
    np.testing.assert_array_equal(st, rst)
    ok = st == 0
    assert ok.mean() > 0.95
    np.testing.assert_array_equal(stats[ok], rstats[ok])
    np.testing.assert_array_equal(t[ok], rt[ok])
    off = b.y_offsets
    errs = [np.linalg.norm(y[off[i]:off[i + 1]] - ry[off[i]:off[i + 1]]) / np.linalg.norm(ry[off[i]:off[i + 1]])
            for i in np.nonzero(ok)[0]]
    assert max(errs) <= 1e-10, max(errs)
    assert stats[ok, 1].sum() > 0 or config == 2  # the controller rejected some attempts


def test_adaptive_refuses_mixed_batches(engine):
    import simbody_gb300._native as N

    w = Workload(3, 32)
    b, y0 = engine_batch(w, "mixed")
    b.set_state(y0)
    with pytest.raises(N.EngineError) as e:
        b.rk_merson_adaptive(0.01)
    assert e.value.code == 6  # SBG_ERR_UNSUPPORTED
