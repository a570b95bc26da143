"""The oracle's O(n) tree operators, pinned through the reference's golden vectors.

The operators (the reference's inverse dynamics, M x, J x, ~J F and composite
body inertias) have no recorded outputs of their own. They are pinned by the
identities the reference's own tests check (TestMassMatrix.cpp:682-870), built
on quantities the golden vectors do pin:
  * M (M^-1 f) = f, with M^-1 f recorded from the reference;
  * the residual force of the recorded udot, with the systems' own forces
    applied, is zero (forward and inverse dynamics agree);
  * inverse dynamics is M x plus a part independent of x, and re-applying the
    residual leaves nothing (TestMassMatrix.cpp:772-778);
  * <J v, F> = <v, ~J F>, and at u = 0 the residual of zero udot is -~J F;
  * M_jj = V^T R V, with R the composite body inertia of the body that owns
    mobility j and V = J e_j at that body (the kinetic energy of the rigid
    body made by locking every joint outboard of it).
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from simbody_gb300 import Workload
from simbody_gb300 import _native as N

GOLD = Path(__file__).resolve().parent / "golden" / "reference_vectors.npz"
WORKLOAD_SIZES = {1: 8, 2: 4, 3: 6, 4: 8, 5: 64, 6: 8, 7: 6, 8: 8, 9: 64, 10: 6}


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


@pytest.fixture(scope="module")
def workloads():
    return {c: Workload(c, n) for c, n in WORKLOAD_SIZES.items()}


def _records(g, workloads, loops=True):
    for r in range(len(g["cfg"])):
        cfg, inst = int(g["cfg"][r]), int(g["inst"][r])
        w = workloads[cfg]
        d = w.systems[int(w.instance_system[inst])]
        if not loops and d.nconstraints > 0:
            continue
        ys = slice(int(g["y_off"][r]), int(g["y_off"][r + 1]))
        us = slice(int(g["u_off"][r]), int(g["u_off"][r + 1]))
        yield cfg, inst, w, d, ys, us


class One:
    """Operator calls on one instance."""

    def __init__(self, w, inst, y):
        self.w, self.inst, self.y = w, inst, np.ascontiguousarray(y, dtype=np.float64)
        d = w.systems[int(w.instance_system[inst])]
        self.nb = d.nbodies
        self.nu = None
        self.sys_of = w.instance_system[[inst]]
        self.y_off = np.array([0, len(y)], dtype=np.int64)
        self.b_off = np.array([0, self.nb], dtype=np.int64)

    def with_nu(self, nu):
        self.nu = nu
        self.u_off = np.array([0, nu], dtype=np.int64)
        return self

    def op(self, name, x=None, fmob=None, fbody=None, y=None):
        return O.tree_op(self.w.systems, self.w.nsys, self.sys_of, self.y_off, self.y if y is None else y,
                         self.u_off, self.b_off, name, x=x, fmob=fmob, fbody=fbody)

    def forces(self):
        return O.system_forces(self.w.systems, self.w.nsys, self.sys_of, self.y_off, self.y, self.u_off, self.b_off)


def _one(w, inst, g, ys, us):
    return One(w, inst, g["y0"][ys]).with_nu(us.stop - us.start)


def _rel(a, b, scale=None):
    s = np.linalg.norm(b) if scale is None else scale
    return np.linalg.norm(a - b) / max(s, 1e-300)


def test_m_times_recorded_minv_is_identity(gold, workloads):
    for cfg, inst, w, d, ys, us in _records(gold, workloads):
        o = _one(w, inst, gold, ys, us)
        mf = o.op("mv", x=gold["minv_f"][us])
        assert _rel(mf, gold["f"][us]) <= 1e-11, (cfg, inst)


def test_residual_of_recorded_udot_is_zero(gold, workloads):
    checked = 0
    for cfg, inst, w, d, ys, us in _records(gold, workloads, loops=False):
        o = _one(w, inst, gold, ys, us)
        nq = (ys.stop - ys.start) - o.nu
        udot = gold["ydot"][ys][nq:]
        fm, fb = o.forces()
        res = o.op("residual", x=udot, fmob=fm, fbody=fb)
        scale = np.linalg.norm(o.op("mv", x=udot)) + np.linalg.norm(fm) + np.linalg.norm(o.op("jtf", fbody=fb))
        assert np.linalg.norm(res) / scale <= 1e-12, (cfg, inst)
        checked += 1
    assert checked >= 8


def test_residual_is_linear_in_udot_and_self_consistent(gold, workloads):
    rng = np.random.default_rng(5)
    for cfg, inst, w, d, ys, us in _records(gold, workloads):
        o = _one(w, inst, gold, ys, us)
        x, fm, fb = rng.standard_normal(o.nu), rng.standard_normal(o.nu), rng.standard_normal(6 * o.nb)
        r_x = o.op("residual", x=x, fmob=fm, fbody=fb)
        r_0 = o.op("residual", fmob=fm, fbody=fb)
        assert _rel(r_x - r_0, o.op("mv", x=x)) <= 1e-11, (cfg, inst)
        zero = o.op("residual", x=x, fmob=fm + r_x, fbody=fb)   # TestMassMatrix.cpp:772-778
        assert np.linalg.norm(zero) <= 1e-11 * max(np.linalg.norm(r_x), 1.0), (cfg, inst)


def test_jacobian_transpose_is_adjoint_and_matches_residual_at_rest(gold, workloads):
    rng = np.random.default_rng(6)
    for cfg, inst, w, d, ys, us in _records(gold, workloads):
        o = _one(w, inst, gold, ys, us)
        v, F = rng.standard_normal(o.nu), rng.standard_normal(6 * o.nb)
        jv, jtf = o.op("jv", x=v), o.op("jtf", fbody=F)
        assert abs(jv @ F - v @ jtf) <= 1e-12 * np.linalg.norm(jv) * np.linalg.norm(F), (cfg, inst)
        y_rest = o.y.copy()
        y_rest[len(y_rest) - o.nu:] = 0.0
        r = o.op("residual", fbody=F, y=y_rest)
        assert _rel(r, -o.op("jtf", fbody=F, y=y_rest)) <= 1e-13, (cfg, inst)


def test_composite_inertias_reproduce_the_mass_matrix_diagonal(gold, workloads):
    for cfg, inst, w, d, ys, us in _records(gold, workloads):
        o = _one(w, inst, gold, ys, us)
        R = o.op("composite").reshape(o.nb, 10)
        # the base bodies carry the mass of their whole subtree
        roots = [b for b in range(o.nb) if d.bodies[b].parent == 0]
        assert np.isclose(sum(R[b, 0] for b in roots), sum(d.bodies[b].mass for b in range(o.nb)), rtol=1e-13)
        owner = []
        for b in range(o.nb):
            owner += [b] * N.NU[d.bodies[b].mobilizer]
        for j in range(o.nu):
            e = np.zeros(o.nu)
            e[j] = 1.0
            mjj = o.op("mv", x=e)[j]
            V = o.op("jv", x=e).reshape(o.nb, 6)[owner[j]]
            m, p, g = R[owner[j], 0], R[owner[j], 1:4], R[owner[j], 4:10]
            G = np.array([[g[0], g[3], g[4]], [g[3], g[1], g[5]], [g[4], g[5], g[2]]])
            w_, v_ = V[:3], V[3:]
            ke2 = m * (w_ @ G @ w_ + 2.0 * w_ @ np.cross(p, v_) + v_ @ v_)
            assert abs(ke2 - mjj) <= 1e-12 * max(abs(mjj), 1e-300) * 10, (cfg, inst, j)
