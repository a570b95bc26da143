"""ctypes wrapper of oracle/_build/liboracle.so, the CPU restatement of
Simbody's articulated-body recursions and fixed-step RK-Merson driver
(sbg_oracle*.{hpp,cpp}). Test infrastructure only."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from simbody_gb300 import _native as N

_LIB = None
_HERE = Path(__file__).resolve().parent


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        path = _HERE / "_build" / "liboracle.so"
        if not path.exists():
            raise RuntimeError(f"oracle library missing: {path} (run python -m simbody_gb300.build)")
        L = C.CDLL(str(path))
        P = C.POINTER
        dp, ip, i64p = P(C.c_double), P(C.c_int32), P(C.c_int64)
        sd = P(N.SystemDesc)
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_system_sizes.argtypes = [sd, ip, ip, ip]
        L.oracle_realize_batch.argtypes = [sd, C.c_int32, ip, C.c_int32, i64p, dp, dp, ip, C.c_int32]
        L.oracle_minv_batch.argtypes = [sd, C.c_int32, ip, C.c_int32, i64p, dp, i64p, dp, dp, C.c_int32]
        L.oracle_rk_merson_batch.argtypes = [sd, C.c_int32, ip, C.c_int32, i64p, dp, dp, C.c_double, C.c_int32,
                                             C.c_double, C.c_double, C.c_int32, ip, i64p, C.c_int32]
        L.oracle_rk_merson_run_batch.argtypes = [sd, C.c_int32, ip, C.c_int32, i64p, dp, dp, C.c_double,
                                                 C.c_int32, C.c_double, C.c_int32, C.c_double, C.c_double,
                                                 C.c_int32, ip, C.c_int32]
        L.oracle_qdotdot_batch.argtypes = [sd, C.c_int32, ip, C.c_int32, i64p, dp, dp, i64p, dp]
        L.oracle_tree_op_batch.argtypes = [sd, C.c_int32, ip, C.c_int32, i64p, dp, i64p, i64p, C.c_int32, dp, dp,
                                           dp, dp, C.c_int32]
        L.oracle_system_forces_batch.argtypes = [sd, C.c_int32, ip, C.c_int32, i64p, dp, i64p, i64p, dp, dp,
                                                 C.c_int32]
        L.oracle_rk_merson_adaptive_batch.argtypes = [sd, C.c_int32, ip, C.c_int32, i64p, dp, dp, C.c_double,
                                                      C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                                      C.c_int32, C.c_int32, ip, i64p, C.c_int32]
        L.oracle_instance_invariants.argtypes = [C.POINTER(N.SystemDesc), dp, dp, dp, dp, dp]
        L.oracle_qtz_solve.argtypes = [C.c_int32, C.c_int32, dp, C.c_double, dp, dp]
        L.oracle_adjust_step_size.argtypes = [C.c_double, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double,
                                              dp]
        L.oracle_count_realize.argtypes = [sd, dp, i64p]
        L.oracle_time_realize.argtypes = [sd, C.c_int32, ip, C.c_int32, i64p, dp, dp, C.c_int32, C.c_int32]
        L.oracle_time_realize.restype = C.c_double
        L.oracle_hardware_threads.restype = C.c_int
        _LIB = L
    return _LIB


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def _l(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def _check(rc):
    if rc:
        raise RuntimeError(lib().oracle_last_error().decode())


def _systems_array(systems):
    if isinstance(systems, C.Array) or hasattr(systems, "contents"):
        return systems
    arr = (N.SystemDesc * len(systems))(*systems)
    return arr


def hardware_threads() -> int:
    return int(lib().oracle_hardware_threads())


def realize(systems, nsys, sys_of, y_off, y, nthreads=0):
    sys_of = np.ascontiguousarray(sys_of, dtype=np.int32)
    y_off = np.ascontiguousarray(y_off, dtype=np.int64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    ydot = np.empty_like(y)
    st = np.empty(len(sys_of), dtype=np.int32)
    _check(lib().oracle_realize_batch(systems, nsys, _i(sys_of), len(sys_of), _l(y_off), _d(y), _d(ydot), _i(st),
                                      nthreads))
    return ydot, st


def multiply_by_minv(systems, nsys, sys_of, y_off, y, u_off, f, nthreads=0):
    sys_of = np.ascontiguousarray(sys_of, dtype=np.int32)
    f = np.ascontiguousarray(f, dtype=np.float64)
    out = np.empty_like(f)
    _check(lib().oracle_minv_batch(systems, nsys, _i(sys_of), len(sys_of), _l(np.ascontiguousarray(y_off)),
                                   _d(np.ascontiguousarray(y)), _l(np.ascontiguousarray(u_off)), _d(f), _d(out),
                                   nthreads))
    return out


TREE_OPS = {"residual": 0, "mv": 1, "jv": 2, "jtf": 3, "composite": 4}


def tree_op(systems, nsys, sys_of, y_off, y, u_off, b_off, op, x=None, fmob=None, fbody=None, nthreads=0):
    """One of the O(n) tree operators (TREE_OPS) per instance. u-like arrays
    are packed at u_off; body arrays hold 6 values (10 for composite
    inertias) per body at b_off (bodies before each instance)."""
    sys_of = np.ascontiguousarray(sys_of, dtype=np.int32)
    u_off = np.ascontiguousarray(u_off, dtype=np.int64)
    b_off = np.ascontiguousarray(b_off, dtype=np.int64)
    k = TREE_OPS[op]
    n = len(sys_of)
    nout = {2: 6 * int(b_off[n]), 4: 10 * int(b_off[n])}.get(k, int(u_off[n]))
    out = np.empty(nout)
    keep = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None for a in (x, fmob, fbody)]
    ptr = [None if a is None else _d(a) for a in keep]
    _check(lib().oracle_tree_op_batch(systems, nsys, _i(sys_of), n, _l(np.ascontiguousarray(y_off)),
                                      _d(np.ascontiguousarray(y)), _l(u_off), _l(b_off), k, ptr[0], ptr[1], ptr[2],
                                      _d(out), nthreads))
    return out


def system_forces(systems, nsys, sys_of, y_off, y, u_off, b_off, nthreads=0):
    """(mobility forces, body forces) of the systems' own force elements."""
    sys_of = np.ascontiguousarray(sys_of, dtype=np.int32)
    u_off = np.ascontiguousarray(u_off, dtype=np.int64)
    b_off = np.ascontiguousarray(b_off, dtype=np.int64)
    n = len(sys_of)
    fm = np.empty(int(u_off[n]))
    fb = np.empty(6 * int(b_off[n]))
    _check(lib().oracle_system_forces_batch(systems, nsys, _i(sys_of), n, _l(np.ascontiguousarray(y_off)),
                                            _d(np.ascontiguousarray(y)), _l(u_off), _l(b_off), _d(fm), _d(fb),
                                            nthreads))
    return fm, fb


def rk_merson(systems, nsys, sys_of, y_off, y, h, nsteps, t=None, accuracy=0.0, cons_tol=0.0,
              project_every_step=False, nthreads=0):
    sys_of = np.ascontiguousarray(sys_of, dtype=np.int32)
    y = np.array(y, dtype=np.float64, copy=True)
    tt = np.zeros(len(sys_of)) if t is None else np.array(t, dtype=np.float64, copy=True)
    st = np.empty(len(sys_of), dtype=np.int32)
    npj = C.c_int64()
    _check(lib().oracle_rk_merson_batch(systems, nsys, _i(sys_of), len(sys_of), _l(np.ascontiguousarray(y_off)),
                                        _d(y), _d(tt), float(h), int(nsteps), accuracy, cons_tol,
                                        int(project_every_step), _i(st), C.byref(npj), nthreads))
    return y, tt, st, npj.value


def rk_merson_run(systems, nsys, sys_of, y_off, y, h, nsteps=-1, t_report=0.0, t=None, initialize=True,
                  accuracy=0.0, cons_tol=0.0, project_every_step=False, nthreads=0):
    """One call of the fixed-step integrator: nsteps >= 0 steps of h, or
    (nsteps < 0) stepTo(t_report) with interpolation off; initialize=False
    continues the integration (y, t) describe. Returns (y, t, status)."""
    sys_of = np.ascontiguousarray(sys_of, dtype=np.int32)
    y = np.array(y, dtype=np.float64, copy=True)
    tt = np.zeros(len(sys_of)) if t is None else np.array(t, dtype=np.float64, copy=True)
    st = np.empty(len(sys_of), dtype=np.int32)
    _check(lib().oracle_rk_merson_run_batch(systems, nsys, _i(sys_of), len(sys_of), _l(np.ascontiguousarray(y_off)),
                                            _d(y), _d(tt), float(h), int(nsteps), float(t_report), int(initialize),
                                            accuracy, cons_tol, int(project_every_step), _i(st), nthreads))
    return y, tt, st


def qdotdot(systems, nsys, sys_of, y_off, y, ydot, q_off):
    """State::getQDotDot() from a realized y and its ydot; nq values per
    instance at q_off[i]."""
    sys_of = np.ascontiguousarray(sys_of, dtype=np.int32)
    q_off = np.ascontiguousarray(q_off, dtype=np.int64)
    out = np.zeros(int(q_off[-1]))
    _check(lib().oracle_qdotdot_batch(systems, nsys, _i(sys_of), len(sys_of), _l(np.ascontiguousarray(y_off)),
                                      _d(np.ascontiguousarray(y)), _d(np.ascontiguousarray(ydot)), _l(q_off),
                                      _d(out)))
    return out


def rk_merson_adaptive(systems, nsys, sys_of, y_off, y, t_final, t=None, h_init=0.0, h_min=0.0, h_max=0.0,
                       accuracy=0.0, cons_tol=0.0, project_every_step=False, max_steps=1_000_000, nthreads=0):
    """Error-controlled RK-Merson to t_final (instances without constraints).
    Returns (y, t, status, stats) with stats[i] = (accepted, rejected)."""
    sys_of = np.ascontiguousarray(sys_of, dtype=np.int32)
    y = np.array(y, dtype=np.float64, copy=True)
    tt = np.zeros(len(sys_of)) if t is None else np.array(t, dtype=np.float64, copy=True)
    st = np.empty(len(sys_of), dtype=np.int32)
    stats = np.zeros((len(sys_of), 2), dtype=np.int64)
    _check(lib().oracle_rk_merson_adaptive_batch(systems, nsys, _i(sys_of), len(sys_of),
                                                 _l(np.ascontiguousarray(y_off)), _d(y), _d(tt), float(t_final),
                                                 float(h_init), float(h_min), float(h_max), float(accuracy),
                                                 float(cons_tol), int(project_every_step), int(max_steps), _i(st),
                                                 _l(stats), nthreads))
    return y, tt, st, stats


def adjust_step_size(err, h, accuracy=1e-3, err_order=4, limited=False, h_min=0.0, h_max=0.0):
    """The step-size controller alone: (success, new h)."""
    hh = C.c_double(h)
    ok = lib().oracle_adjust_step_size(float(err), int(err_order), int(limited), float(accuracy), float(h_min),
                                       float(h_max), C.byref(hh))
    return bool(ok), hh.value


def invariants(system, y):
    """Kinetic, gravity and spring energies and the Ball closures' position,
    velocity and acceleration errors (after the constrained realize) of one
    instance: dict(ke, pe_gravity, pe_springs, perr, verr, aerr, status)."""
    y = np.ascontiguousarray(y, dtype=np.float64)
    m = 3 * int(system.nconstraints)
    en = np.zeros(3)
    perr, verr, aerr = np.zeros(max(m, 1)), np.zeros(max(m, 1)), np.zeros(max(m, 1))
    st = lib().oracle_instance_invariants(C.byref(system), _d(y), _d(en), _d(perr), _d(verr), _d(aerr))
    if st < 0:
        raise RuntimeError(lib().oracle_last_error().decode())
    return dict(ke=en[0], pe_gravity=en[1], pe_springs=en[2], perr=perr[:m], verr=verr[:m], aerr=aerr[:m],
                status=st)


def qtz_solve(A, b, rcond):
    """The rank-revealing solve of the loop closures alone: (minimum-norm
    least-squares x of A x = b at conditioning tolerance rcond, rank)."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(A.shape[1])
    r = lib().oracle_qtz_solve(A.shape[0], A.shape[1], _d(A), float(rcond), _d(b), _d(x))
    return x, r


def count_realize(system_ptr, y):
    y = np.ascontiguousarray(y, dtype=np.float64)
    counts = np.zeros(6, dtype=np.int64)
    _check(lib().oracle_count_realize(system_ptr, _d(y), _l(counts)))
    return dict(zip(["add", "mul", "div", "sqrt", "trig", "cmp"], counts.tolist()))


def time_realize(systems, nsys, sys_of, y_off, y, nreps=1, nthreads=0) -> float:
    sys_of = np.ascontiguousarray(sys_of, dtype=np.int32)
    y = np.ascontiguousarray(y, dtype=np.float64)
    ydot = np.empty_like(y)
    return float(lib().oracle_time_realize(systems, nsys, _i(sys_of), len(sys_of),
                                           _l(np.ascontiguousarray(y_off)), _d(y), _d(ydot), int(nreps),
                                           int(nthreads)))


# ------------------------------------------------------ workload helpers
def realize_workload(w, instances=None, nthreads=0):
    idx = np.arange(w.ninst) if instances is None else np.asarray(instances)
    sys_of = w.instance_system[idx]
    y = np.concatenate([w.y0[w.instance_slice(int(i))] for i in idx])
    lens = np.array([w.y_offsets[i + 1] - w.y_offsets[i] for i in idx], dtype=np.int64)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    return realize(w.systems, w.nsys, sys_of, off, y, nthreads)


def rk_workload(w, h, nsteps, instances=None, nthreads=0, **kw):
    idx = np.arange(w.ninst) if instances is None else np.asarray(instances)
    sys_of = w.instance_system[idx]
    y = np.concatenate([w.y0[w.instance_slice(int(i))] for i in idx])
    lens = np.array([w.y_offsets[i + 1] - w.y_offsets[i] for i in idx], dtype=np.int64)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    return rk_merson(w.systems, w.nsys, sys_of, off, y, h, nsteps, nthreads=nthreads, **kw)
