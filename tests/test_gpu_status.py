"""Failure reporting on the GPU, injected through the inputs (no fault is
provoked on the device): the kernels set per-instance SBG_INST_* status bits
where Simbody would throw, and the host returns ABI error codes.

  - a NaN in one instance's state flags that instance NONFINITE and leaves
    its neighbours' results intact (the reference's integrator would restore
    y and throw Integrator::StepFailed, AbstractIntegratorRep.cpp:426-431);
  - a Ball body with no rotational inertia about its joint makes D = H^T P H
    singular: SINGULAR_D (the reference's Mat::invert throws,
    SmallMatrixMixed.h:878-892);
  - a batch larger than its device budget is refused with SBG_ERR_BUDGET.
"""
import ctypes as C

import numpy as np
import pytest

from simbody_gb300 import Batch, Workload, engine_batch
from simbody_gb300 import _native as N
from simbody_gb300.engine import Topology

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_state_flags_only_that_instance(engine, precision):
    w = Workload(3, 96)
    b, y0 = engine_batch(w, precision)
    b.set_state(y0)
    ref, st0 = b.realize_acceleration()
    assert (st0 == 0).all()
    bad = 17
    y1 = y0.copy()
    y1[b.y_offsets[bad] + 2] = np.nan
    b.set_state(y1)
    yd, st = b.realize_acceleration()
    assert st[bad] & N.INST_NONFINITE
    ok = np.arange(b.ninst) != bad
    assert (st[ok] == 0).all()
    for i in np.nonzero(ok)[0]:
        s = slice(b.y_offsets[i], b.y_offsets[i + 1])
        assert np.array_equal(yd[s], ref[s])


def point_mass_on_ball():
    bodies = (N.BodyDesc * 2)()
    for k in range(2):
        b = bodies[k]
        b.parent, b.mass = k, 1.0
        for j in (0, 4, 8):
            b.X_PF[j] = b.X_BM[j] = 1.0
    bodies[0].mobilizer = N.SBG_PIN
    bodies[0].unit_inertia[0] = bodies[0].unit_inertia[1] = bodies[0].unit_inertia[2] = 1.0
    bodies[0].X_BM[10] = 0.5
    bodies[1].mobilizer = N.SBG_BALL  # point mass at the joint centre: no inertia about the joint
    d = N.SystemDesc(2, 0, 0, 0, (C.c_double * 3)(0, -9.8, 0), bodies, None, None)
    return Topology(d, keepalive=bodies)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_singular_articulated_inertia_is_reported(engine, precision):
    t = point_mass_on_ball()
    b = Batch([t], np.zeros(4, dtype=np.int32), precision=precision)
    y = np.tile(t.default_state(), 4)
    b.set_state(y)
    _, st = b.realize_acceleration()
    assert (st & N.INST_SINGULAR_D).all()


def test_batch_over_budget_is_refused(engine):
    w = Workload(2, 4096)
    with pytest.raises(N.EngineError) as e:
        engine_batch(w, "fp64", device_budget_bytes=1 << 20)
    assert e.value.code == 4  # SBG_ERR_BUDGET
