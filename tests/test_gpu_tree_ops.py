"""The CUDA tree operators against the oracle's, through the C ABI.

The operators are inverse dynamics (calcResidualForceIgnoringConstraints),
M x, J x, ~J F and the composite body inertias. They run in FP64 in every
batch precision, so both an FP64 and a mixed batch must match the oracle to
<= 1e-12 relative, per instance and norm-wise. The oracle's operators are
pinned to the reference's golden vectors in test_oracle_tree_ops.py.

The workloads cover every segment of a batch:
  * Pin chains (one-thread driver, width 1);
  * Ball chains (width 3);
  * random and uneven trees (one-thread and level-parallel drivers);
  * the serving mix with Ball loop closures (the FP64 loop-closure segment,
    whose constraints the operators ignore).
"""
import numpy as np
import pytest

from oracle import oracle as O
from simbody_gb300 import Workload, engine_batch

pytestmark = pytest.mark.gpu

CASES = [(1, 64), (2, 96), (3, 64), (4, 48), (5, 64), (6, 64), (7, 64), (8, 64)]


def _per_instance_rel(a, b, off):
    errs = []
    for i in range(len(off) - 1):
        s = slice(int(off[i]), int(off[i + 1]))
        errs.append(np.linalg.norm(a[s] - b[s]) / max(np.linalg.norm(b[s]), 1e-300))
    return np.array(errs)


def _setup(config, n, precision):
    w = Workload(config, n)
    b, y0 = engine_batch(w, precision)
    b.set_state(y0)
    ref = lambda op, **kw: O.tree_op(w.systems, w.nsys, w.instance_system, b.y_offsets, y0, b.u_offsets,
                                     b.body_offsets, op, **kw)
    return w, b, y0, ref


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("config,n", CASES)
def test_tree_operators_match_oracle(engine, config, n, precision):
    w, b, y0, ref = _setup(config, n, precision)
    rng = np.random.default_rng(config)
    nu, nb = int(b.u_offsets[-1]), int(b.body_offsets[-1])
    x, f, F = rng.standard_normal(nu), rng.standard_normal(nu), rng.standard_normal(6 * nb)
    uo, bo6, bo10 = b.u_offsets, 6 * b.body_offsets, 10 * b.body_offsets

    r, st = b.calc_residual_force(f, F, x)
    assert (st == 0).all()
    assert _per_instance_rel(r, ref("residual", x=x, fmob=f, fbody=F), uo).max() <= 1e-12

    r0, st = b.calc_residual_force()   # all inputs absent: the velocity-dependent forces alone
    assert (st == 0).all()
    assert _per_instance_rel(r0, ref("residual"), uo).max() <= 1e-12

    mv, st = b.multiply_by_m(x)
    assert (st == 0).all()
    assert _per_instance_rel(mv, ref("mv", x=x), uo).max() <= 1e-12

    jv, st = b.multiply_by_system_jacobian(x)
    assert (st == 0).all()
    assert _per_instance_rel(jv, ref("jv", x=x), bo6).max() <= 1e-12

    jtf, st = b.multiply_by_system_jacobian_transpose(F)
    assert (st == 0).all()
    assert _per_instance_rel(jtf, ref("jtf", fbody=F), uo).max() <= 1e-12

    R, st = b.calc_composite_body_inertias()
    assert (st == 0).all()
    assert _per_instance_rel(R, ref("composite"), bo10).max() <= 1e-12
    assert b.last_operator_ms() > 0.0


def test_tree_operators_leave_the_state_and_realize_untouched(engine):
    """The operators share the batch's scratch but not its state: a realize
    after them gives the same derivatives as before."""
    w, b, y0, ref = _setup(4, 48, "mixed")
    d0, _ = b.realize_acceleration()
    b.calc_residual_force(known_udot=np.ones(int(b.u_offsets[-1])))
    b.calc_composite_body_inertias()
    d1, _ = b.realize_acceleration()
    assert np.array_equal(d0, d1)
    y, _ = b.get_state()
    assert np.array_equal(y, y0)


def test_inverse_dynamics_inverts_the_engines_forward_dynamics(engine):
    """residual(udot from realize, the systems' own forces) = 0: the GPU's
    forward and inverse dynamics agree with each other (FP64 batch)."""
    w, b, y0, ref = _setup(3, 128, "fp64")
    ydot, st = b.realize_acceleration()
    assert (st == 0).all()
    udot = np.concatenate([ydot[b.y_offsets[i] + b.nq[i]:b.y_offsets[i + 1]] for i in range(b.ninst)])
    fm, fb = O.system_forces(w.systems, w.nsys, w.instance_system, b.y_offsets, y0, b.u_offsets, b.body_offsets)
    r, st = b.calc_residual_force(fm, fb, udot)
    mv, _ = b.multiply_by_m(udot)
    scale = np.linalg.norm(mv) + np.linalg.norm(fm)
    assert np.linalg.norm(r) / scale <= 1e-12


def test_nonfinite_state_is_flagged_per_instance(engine):
    w, b, y0, ref = _setup(3, 32, "fp64")
    y = y0.copy()
    y[b.y_offsets[5]] = np.nan
    b.set_state(y)
    _, st = b.multiply_by_m(np.ones(int(b.u_offsets[-1])))
    assert st[5] != 0 and (np.delete(st, 5) == 0).all()
