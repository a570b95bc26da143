"""Parity of the CUDA engine (through the C ABI) with the CPU oracle.

Workloads 6 (trees over all nine non-Free mobilizers: Gimbal, Translation,
Cylinder, Planar and Bushing beside the benchmark's four, Free or Bushing
roots) and 7 (trees in Euler-angle mode) cover the wider mobilizer set, and 8
(trees with a SmoothSphereHalfSpaceForce sphere on every body, pressing on a
ground half-space) the contact force.

Tolerances: the plain FP64 form must reproduce realize(Acceleration) to
<= 1e-12 relative (norm-wise per instance) and short trajectories to <= 1e-12;
the mixed form must keep the relative udot error <= 1e-5 against FP64.
"""
import numpy as np
import pytest

from oracle import oracle as O
from simbody_gb300 import Workload, engine_batch

pytestmark = pytest.mark.gpu


def rel_err_per_instance(a, b, offsets, part=None):
    errs = []
    for i in range(len(offsets) - 1):
        s = slice(offsets[i], offsets[i + 1])
        x, y = a[s], b[s]
        errs.append(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))
    return np.array(errs)


@pytest.mark.parametrize("config,n", [(1, 256), (2, 512), (3, 128), (4, 64), (6, 128), (7, 128), (8, 128)])
def test_realize_fp64_matches_oracle(engine, config, n):
    w = Workload(config, n)
    b, y0 = engine_batch(w, "fp64")
    b.set_state(y0)
    ydot, st = b.realize_acceleration()
    ref, rst = O.realize_workload(w)
    assert (st == 0).all() and (rst == 0).all()
    err = rel_err_per_instance(ydot, ref, b.y_offsets)
    assert err.max() <= 1e-12, err.max()


def _udot(d, b):
    return np.concatenate([d[b.y_offsets[i] + b.nq[i]:b.y_offsets[i + 1]] for i in range(b.ninst)])


@pytest.mark.parametrize("config,n", [(1, 512), (2, 2048), (3, 512), (4, 256), (6, 256), (7, 256), (8, 256)])
def test_realize_mixed_udot_error(engine, config, n):
    """Mixed form (FP32 recursions + double-float residual refinement):
    relative udot error per instance <= 1e-5 against FP64."""
    w = Workload(config, n)
    b64, y0 = engine_batch(w, "fp64")
    b32, _ = engine_batch(w, "mixed")
    b64.set_state(y0)
    b32.set_state(y0)
    d64, _ = b64.realize_acceleration()
    d32, st = b32.realize_acceleration()
    assert (st == 0).all()
    err = rel_err_per_instance(_udot(d32, b32), _udot(d64, b64), b64.u_offsets)
    assert err.max() <= 1e-5, err.max()
    # qdot = N(q) u is part of the same RHS
    assert rel_err_per_instance(d32, d64, b64.y_offsets).max() <= 1e-5


@pytest.mark.parametrize("config,n", [(2, 512), (3, 256)])
def test_realize_mixed_fast_is_plain_fp32(engine, config, n):
    """Without refinement the FP32 recursion alone is within FP32 reach."""
    w = Workload(config, n)
    b64, y0 = engine_batch(w, "fp64")
    bf, _ = engine_batch(w, "mixed_fast")
    b64.set_state(y0)
    bf.set_state(y0)
    d64, _ = b64.realize_acceleration()
    df, st = bf.realize_acceleration()
    assert (st == 0).all()
    err = rel_err_per_instance(_udot(df, bf), _udot(d64, b64), b64.u_offsets)
    assert err.max() <= 1e-3, err.max()


@pytest.mark.parametrize("config,n,steps,tol", [(1, 256, 50, 1e-6), (3, 64, 20, 1e-6), (4, 32, 20, 1e-6),
                                                  (6, 64, 20, 1e-6), (7, 64, 20, 1e-6), (8, 64, 20, 1e-6)])
def test_rk_merson_mixed_short_horizon(engine, config, n, steps, tol):
    """FP32 recursions with FP64 state accumulation stay close to the FP64
    trajectory over a short horizon."""
    w = Workload(config, n)
    b64, y0 = engine_batch(w, "fp64")
    bm, _ = engine_batch(w, "mixed")
    b64.set_state(y0)
    bm.set_state(y0)
    b64.rk_merson_fixed(w.h, steps)
    st = bm.rk_merson_fixed(w.h, steps)
    assert (st & ~4 == 0).all()  # steps that met an ill-conditioned M were taken in FP64
    y64, t64 = b64.get_state()
    ym, tm = bm.get_state()
    np.testing.assert_array_equal(tm, t64)
    err = rel_err_per_instance(ym, y64, b64.y_offsets)
    assert err.max() <= tol, err.max()


@pytest.mark.parametrize("config,n,steps", [(1, 256, 50), (3, 64, 20), (4, 32, 20), (6, 64, 20), (7, 64, 20),
                                             (8, 64, 20)])
def test_rk_merson_fp64_short_horizon(engine, config, n, steps):
    w = Workload(config, n)
    b, y0 = engine_batch(w, "fp64")
    b.set_state(y0)
    st = b.rk_merson_fixed(w.h, steps)
    y, t = b.get_state()
    ref, rt, rst, _ = O.rk_workload(w, w.h, steps)
    assert (st & ~4 == 0).all()
    err = rel_err_per_instance(y, ref, b.y_offsets)
    assert err.max() <= 1e-12, err.max()
    np.testing.assert_array_equal(t, rt)


def test_multiply_by_minv_fp64(engine):
    w = Workload(3, 64)
    b, y0 = engine_batch(w, "fp64")
    b.set_state(y0)
    rng = np.random.default_rng(7)
    f = rng.normal(size=int(b.u_offsets[-1]))
    out = b.multiply_by_minv(f)
    ref = O.multiply_by_minv(w.systems, w.nsys, w.instance_system[:64], b.y_offsets, y0, b.u_offsets, f)
    err = rel_err_per_instance(out, ref, b.u_offsets)
    assert err.max() <= 1e-12, err.max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pipelined_host_realize_equals_separate_calls(engine, precision):
    """sbg_realize_acceleration_host (chunked upload / realize / download on
    several streams) gives the bits of set_state + realize_acceleration, with
    pageable and with page-locked host buffers."""
    import torch

    w = Workload(2, 4096)
    b, y0 = engine_batch(w, precision)
    b.set_state(y0)
    ref, st0 = b.realize_acceleration()  # also tunes the batch
    y1 = y0 * (1 + 1e-3 * np.random.default_rng(5).standard_normal(y0.size))
    b.set_state(y1)
    ref1, _ = b.realize_acceleration()
    got, st = b.realize_acceleration_from(y0)
    assert (st == 0).all() and np.array_equal(got, ref)
    yp = torch.from_numpy(y1).pin_memory().numpy()
    dp = torch.empty(b.ny_total, dtype=torch.float64).pin_memory().numpy()
    sp = torch.empty(b.ninst, dtype=torch.int32).pin_memory().numpy()
    got1, st1 = b.realize_acceleration_from(yp, dp, sp)
    assert (st1 == 0).all() and np.array_equal(got1, ref1)
    # the same buffers again: from the second such call on, the call replays
    # a captured graph, which must read the buffers' new contents each time
    for k, (yin, want) in enumerate([(y0, ref), (y1, ref1), (y0, ref)]):
        yp[:] = yin
        got2, st2 = b.realize_acceleration_from(yp, dp, sp)
        assert (st2 == 0).all() and np.array_equal(got2, want), k
    # pageable buffers go through the batch's own staging: the same holds
    for yin, want in [(y1, ref1), (y0, ref), (y1, ref1)]:
        got3, _ = b.realize_acceleration_from(yin.copy())
        assert np.array_equal(got3, want)


def test_full_size_ball_chain_fp64_matches_oracle(engine):
    """The headline workload at its full size (65,536 32-Ball chains): every
    instance's FP64 udot against the oracle, and the mixed form within 1e-5."""
    w = Workload(2, 65536)
    b, y0 = engine_batch(w, "fp64")
    b.set_state(y0)
    ydot, st = b.realize_acceleration()
    ref, rst = O.realize_workload(w, nthreads=O.hardware_threads())
    assert (st == 0).all() and (rst == 0).all()
    err = rel_err_per_instance(ydot, ref, b.y_offsets)
    assert err.max() <= 1e-12, err.max()
    bm, _ = engine_batch(w, "mixed")
    bm.set_state(y0)
    dm, _ = bm.realize_acceleration()
    nq = 128
    errs = [np.linalg.norm(dm[o + nq:e] - ydot[o + nq:e]) / np.linalg.norm(ydot[o + nq:e])
            for o, e in zip(b.y_offsets[:-1:97], b.y_offsets[1::97])]
    assert max(errs) <= 1e-5, max(errs)


def test_largest_tree_single_instance_matches_oracle(engine):
    """One instance of the largest tree of the uneven distribution (the
    level-parallel driver alone on the GPU)."""
    w = Workload(4, 400)
    i = int(np.argmax(w.nbodies()))
    assert w.nbodies()[i] >= 200
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-5)):
        b, y0 = engine_batch(w, prec, instances=[i])
        b.set_state(y0)
        ydot, st = b.realize_acceleration()
        ref, _ = O.realize_workload(w, [i])
        assert st[0] == 0
        err = np.linalg.norm(ydot - ref) / np.linalg.norm(ref)
        assert err <= tol, (prec, err)


def test_empty_batch(engine):
    """A batch of no instances: every operation is a no-op."""
    from simbody_gb300 import Batch
    from simbody_gb300.engine import Topology

    w = Workload(1, 1)
    t = Topology(w.systems[0], keepalive=w)
    b = Batch([t], np.zeros(0, dtype=np.int32), precision="mixed")
    assert b.ninst == 0 and b.ny_total == 0
    b.set_state(np.zeros(0))
    ydot, st = b.realize_acceleration()
    assert ydot.size == 0 and st.size == 0
    b.rk_merson_fixed(1e-3, 3)
