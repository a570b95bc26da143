"""The staged chain driver (kernel variant 8: record fields of the next body
copied to shared memory while the warp computes the current one) against the
plain chain driver (variant 7) on the batches it applies to: one shared
chain topology without Free bodies (the 32-Ball chain, the double pendulum).
Same arithmetic, so the same results bit for bit (tolerance 0), for full and
partial warp tiles, in both FP32 forms, and through the pipelined host call.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from simbody_gb300 import Workload, engine_batch

pytestmark = pytest.mark.gpu


def _batch(w, precision, variant):
    old = os.environ.get("SBG_VARIANT")
    os.environ["SBG_VARIANT"] = str(variant)
    try:
        return engine_batch(w, precision)
    finally:
        if old is None:
            del os.environ["SBG_VARIANT"]
        else:
            os.environ["SBG_VARIANT"] = old


@pytest.mark.parametrize("precision", ["mixed", "mixed_fast"])
@pytest.mark.parametrize("config,n", [(2, 4096), (2, 1000), (2, 5), (1, 777)])
def test_staged_equals_plain_chain_driver(engine, config, n, precision):
    w = Workload(config, n)
    out = {}
    for v in (7, 8):
        b, y0 = _batch(w, precision, v)
        b.set_state(y0)
        ydot, st = b.realize_acceleration()
        assert b.kernel_variant == v
        out[v] = (ydot.copy(), st.copy())
    np.testing.assert_array_equal(out[8][1], out[7][1])
    np.testing.assert_array_equal(out[8][0], out[7][0])


def test_staged_mixed_matches_oracle_and_host_pipeline(engine):
    w = Workload(2, 2048)
    b, y0 = _batch(w, "mixed", 8)
    b.set_state(y0)
    ydot, st = b.realize_acceleration()
    assert b.kernel_variant == 8 and (st == 0).all()
    ref, _ = O.realize_workload(w)
    off = b.y_offsets
    err = max(np.linalg.norm(ydot[off[i]:off[i + 1]] - ref[off[i]:off[i + 1]]) / np.linalg.norm(ref[off[i]:off[i + 1]])
              for i in range(w.ninst))
    assert err <= 1e-5, err
    # the pipelined host call (tile-aligned chunks) gives the same numbers
    ydot2, st2 = b.realize_acceleration_from(y0)
    np.testing.assert_array_equal(ydot2, ydot)
    np.testing.assert_array_equal(st2, st)


def test_staged_variant_only_where_it_applies(engine):
    """Trees (not chains) and FP64 batches keep their own drivers."""
    w = Workload(3, 64)
    b, y0 = _batch(w, "mixed", 8)
    b.set_state(y0)
    b.realize_acceleration()
    assert b.kernel_variant == 7
