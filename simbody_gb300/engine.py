"""Python face of the C ABI: topologies and device-resident batches of states.

A ``Batch`` holds the states of many instances on one GPU. Its methods map to
Simbody calls (paths relative to the Simbody source tree):

  set_state / get_state      State::updY / getY       (State.h:962-1034)
  realize_acceleration       System::realize(s, Stage::Acceleration) + getYDot
  multiply_by_minv           SimbodyMatterSubsystem::multiplyByMInv (.h:1343)
  calc_residual_force        ...::calcResidualForceIgnoringConstraints (.h:2234)
  multiply_by_m              ...::multiplyByM (.h:1262)
  multiply_by_system_jacobian / _transpose
                             ...::multiplyBySystemJacobian(Transpose) (.h:554, 646)
  calc_composite_body_inertias
                             ...::calcCompositeBodyInertias (.h:2323)
  rk_merson_fixed            RungeKuttaMersonIntegrator, setFixedStepSize(h),
                             initialize, stepTo(t0 + n h)
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _native as N


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Topology:
    """A realized topology (System::realizeTopology) owned by the engine."""

    def __init__(self, desc: N.SystemDesc, keepalive=None):
        lib = N.engine_lib()
        h = C.c_void_p()
        N.check(lib.sbg_topology_create(C.byref(desc), C.byref(h)))
        self._h = h
        self._keep = keepalive
        nq, nu, nb, nl, nqt, nc = (C.c_int32() for _ in range(6))
        N.check(lib.sbg_topology_info(h, C.byref(nq), C.byref(nu), C.byref(nb), C.byref(nl), C.byref(nqt),
                                      C.byref(nc)))
        self.nq, self.nu, self.nbodies = nq.value, nu.value, nb.value
        self.nlevels, self.nquaternions, self.nconstraint_equations = nl.value, nqt.value, nc.value

    @property
    def handle(self):
        return self._h

    def default_state(self) -> np.ndarray:
        y = np.zeros(self.nq + self.nu)
        N.check(N.engine_lib().sbg_topology_default_state(self._h, _dptr(y)))
        return y

    def __del__(self):
        if getattr(self, "_h", None) and N._engine is not None:
            N._engine.sbg_topology_destroy(self._h)
            self._h = None


class Batch:
    """A device-resident batch of instances; instance i uses
    ``topologies[instance_topology[i]]``."""

    def __init__(self, topologies: Sequence[Topology], instance_topology, precision: str = "fp64",
                 device: int = 0, device_budget_bytes: int = 0):
        lib = N.engine_lib()
        self.topologies = list(topologies)
        self.instance_topology = np.ascontiguousarray(instance_topology, dtype=np.int32)
        self.ninst = len(self.instance_topology)
        prec = {"fp64": N.PRECISION_FP64, "mixed": N.PRECISION_MIXED, "mixed_fast": N.PRECISION_MIXED_FAST}[precision]
        self.precision = precision
        cfg = N.BatchConfig(prec, device, int(device_budget_bytes))
        handles = (C.c_void_p * len(self.topologies))(*[t.handle for t in self.topologies])
        h = C.c_void_p()
        N.check(lib.sbg_batch_create(handles, len(self.topologies), _iptr(self.instance_topology), self.ninst,
                                     C.byref(cfg), C.byref(h)))
        self._h = h
        self.y_offsets = np.zeros(self.ninst + 1, dtype=np.int64)
        nyt = C.c_int64()
        N.check(lib.sbg_batch_layout(h, self.y_offsets.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(nyt)))
        self.ny_total = nyt.value
        nqs = np.array([self.topologies[k].nq for k in self.instance_topology], dtype=np.int64)
        nus = np.array([self.topologies[k].nu for k in self.instance_topology], dtype=np.int64)
        self.nq = nqs
        self.nu = nus
        self.u_offsets = np.concatenate([[0], np.cumsum(nus)]).astype(np.int64)
        nbs = np.array([self.topologies[k].nbodies for k in self.instance_topology], dtype=np.int64)
        self.body_offsets = np.concatenate([[0], np.cumsum(nbs)]).astype(np.int64)

    # -- state
    def set_state(self, y: np.ndarray, t: np.ndarray | None = None) -> None:
        y = np.ascontiguousarray(y, dtype=np.float64)
        assert y.size == self.ny_total
        tt = None if t is None else np.ascontiguousarray(t, dtype=np.float64)
        N.check(N.engine_lib().sbg_batch_set_state(self._h, None if tt is None else _dptr(tt), _dptr(y)))

    def get_state(self):
        y = np.empty(self.ny_total)
        t = np.empty(self.ninst)
        N.check(N.engine_lib().sbg_batch_get_state(self._h, _dptr(t), _dptr(y)))
        return y, t

    # -- operators
    def realize_acceleration(self, ydot: np.ndarray | None = None, status: np.ndarray | None = None):
        """System::realize(Stage::Acceleration) + getYDot for every instance.
        ``ydot`` / ``status`` may be caller-owned output arrays (float64,
        int32, C-contiguous); page-locked ones are written directly."""
        if ydot is None:
            ydot = np.empty(self.ny_total)
        if status is None:
            status = np.empty(self.ninst, dtype=np.int32)
        assert ydot.dtype == np.float64 and ydot.size == self.ny_total and ydot.flags.c_contiguous
        assert status.dtype == np.int32 and status.size == self.ninst and status.flags.c_contiguous
        N.check(N.engine_lib().sbg_realize_acceleration(self._h, _dptr(ydot), _iptr(status)))
        return ydot, status

    def realize_acceleration_from(self, y: np.ndarray, ydot: np.ndarray | None = None,
                                  status: np.ndarray | None = None):
        """set_state(y) + realize_acceleration() in one call, with the copies
        pipelined against the compute where the batch allows it."""
        y = np.ascontiguousarray(y, dtype=np.float64)
        assert y.size == self.ny_total
        if ydot is None:
            ydot = np.empty(self.ny_total)
        if status is None:
            status = np.empty(self.ninst, dtype=np.int32)
        assert ydot.dtype == np.float64 and ydot.size == self.ny_total and ydot.flags.c_contiguous
        assert status.dtype == np.int32 and status.size == self.ninst and status.flags.c_contiguous
        N.check(N.engine_lib().sbg_realize_acceleration_host(self._h, _dptr(y), _dptr(ydot), _iptr(status)))
        return ydot, status

    def multiply_by_minv(self, f: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(f, dtype=np.float64)
        assert f.size == self.u_offsets[-1]
        out = np.empty_like(f)
        N.check(N.engine_lib().sbg_multiply_by_minv(self._h, _dptr(f), _dptr(out)))
        return out

    # -- tree operators (FP64 whatever the precision; body arrays: one entry
    #    per mobilized body in description order, instances one after another)
    def _uvec(self, a, name):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.size == self.u_offsets[-1], f"{name}: {a.size} values for {self.u_offsets[-1]} mobilities"
        return a

    def _bvec(self, a, name):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.size == 6 * self.body_offsets[-1], f"{name}: {a.size} values for {self.body_offsets[-1]} bodies"
        return a

    @staticmethod
    def _opt(a):
        return None if a is None else _dptr(a)

    def calc_residual_force(self, mobility_forces=None, body_forces=None, known_udot=None):
        """Inverse dynamics: M udot + C(q,u) - f - ~J F per instance; any input
        may be None (zero). Returns (residual, status)."""
        f = self._uvec(mobility_forces, "mobility_forces")
        F = self._bvec(body_forces, "body_forces")
        x = self._uvec(known_udot, "known_udot")
        out = np.empty(self.u_offsets[-1])
        st = np.empty(self.ninst, dtype=np.int32)
        N.check(N.engine_lib().sbg_calc_residual_force(self._h, self._opt(f), self._opt(F), self._opt(x), _dptr(out),
                                                       _iptr(st)))
        return out, st

    def multiply_by_m(self, a):
        a = self._uvec(a, "a")
        out = np.empty(self.u_offsets[-1])
        st = np.empty(self.ninst, dtype=np.int32)
        N.check(N.engine_lib().sbg_multiply_by_m(self._h, _dptr(a), _dptr(out), _iptr(st)))
        return out, st

    def multiply_by_system_jacobian(self, u):
        u = self._uvec(u, "u")
        out = np.empty(6 * self.body_offsets[-1])
        st = np.empty(self.ninst, dtype=np.int32)
        N.check(N.engine_lib().sbg_multiply_by_system_jacobian(self._h, _dptr(u), _dptr(out), _iptr(st)))
        return out, st

    def multiply_by_system_jacobian_transpose(self, F_G):
        F = self._bvec(F_G, "F_G")
        out = np.empty(self.u_offsets[-1])
        st = np.empty(self.ninst, dtype=np.int32)
        N.check(N.engine_lib().sbg_multiply_by_system_jacobian_transpose(self._h, _dptr(F), _dptr(out), _iptr(st)))
        return out, st

    def calc_composite_body_inertias(self):
        out = np.empty(10 * self.body_offsets[-1])
        st = np.empty(self.ninst, dtype=np.int32)
        N.check(N.engine_lib().sbg_calc_composite_body_inertias(self._h, _dptr(out), _iptr(st)))
        return out, st

    def fallback_count(self) -> int:
        """Mixed batches: realizations recomputed in FP64 so far (an
        ill-conditioned M; SBG_INST_ILL_CONDITIONED)."""
        n = C.c_int64()
        N.check(N.engine_lib().sbg_batch_fallback_count(self._h, C.byref(n)))
        return n.value

    def fp64_steps(self) -> int:
        """Mixed batches: instance steps of the integrations so far taken in
        FP64 (an ill-conditioned M met by a mixed RHS)."""
        n = C.c_int64()
        N.check(N.engine_lib().sbg_batch_fp64_steps(self._h, C.byref(n)))
        return n.value

    def last_operator_ms(self) -> float:
        """Device time of the last tree operator's kernels (copies excluded)."""
        ms = C.c_double()
        N.check(N.engine_lib().sbg_batch_last_operator_ms(self._h, C.byref(ms)))
        return ms.value

    def rk_merson_fixed(self, h: float, nsteps: int, accuracy: float = 0.0, constraint_tolerance: float = 0.0,
                        project_every_step: bool = False, continue_integration: bool = False) -> np.ndarray:
        """nsteps fixed RK-Merson steps of h; Integrator::initialize first
        unless continue_integration."""
        opts = N.IntegOpts(accuracy, constraint_tolerance, int(project_every_step), int(continue_integration))
        st = np.empty(self.ninst, dtype=np.int32)
        N.check(N.engine_lib().sbg_rk_merson_fixed(self._h, float(h), int(nsteps), C.byref(opts), _iptr(st)))
        return st

    def rk_merson_step_to(self, h: float, t_report: float, accuracy: float = 0.0, constraint_tolerance: float = 0.0,
                          project_every_step: bool = False, continue_integration: bool = False) -> np.ndarray:
        """Integrator::stepTo(t_report) with a fixed step h and interpolation
        off (the last step shortened to land on t_report)."""
        opts = N.IntegOpts(accuracy, constraint_tolerance, int(project_every_step), int(continue_integration))
        st = np.empty(self.ninst, dtype=np.int32)
        N.check(N.engine_lib().sbg_rk_merson_step_to(self._h, float(h), float(t_report), C.byref(opts), _iptr(st)))
        return st

    def rk_merson_adaptive(self, t_final: float, accuracy: float = 0.0, constraint_tolerance: float = 0.0,
                           initial_step: float = 0.0, min_step: float = 0.0, max_step: float = 0.0,
                           project_every_step: bool = False, max_steps: int = 0):
        """Error-controlled RK-Merson to t_final (setFinalTime, initialize,
        stepTo), FP64 batches. Returns (status, stats) with stats[i] =
        (accepted, rejected) steps of instance i."""
        opts = N.AdaptiveOpts(accuracy, constraint_tolerance, initial_step, min_step, max_step,
                              int(project_every_step), int(max_steps))
        st = np.empty(self.ninst, dtype=np.int32)
        stats = np.zeros((self.ninst, 2), dtype=np.int64)
        N.check(N.engine_lib().sbg_rk_merson_adaptive(self._h, float(t_final), C.byref(opts), _iptr(st),
                                                      stats.ctypes.data_as(C.POINTER(C.c_int64))))
        return st, stats

    # -- device-resident timing path
    @property
    def stream(self) -> int:
        return N.engine_lib().sbg_batch_stream(self._h) or 0

    def realize_acceleration_async(self) -> None:
        N.check(N.engine_lib().sbg_realize_acceleration_async(self._h))

    def rk_merson_fixed_async(self, h: float, nsteps: int) -> None:
        N.check(N.engine_lib().sbg_rk_merson_fixed_async(self._h, float(h), int(nsteps), None))

    def get_ydot(self):
        ydot = np.empty(self.ny_total)
        st = np.empty(self.ninst, dtype=np.int32)
        N.check(N.engine_lib().sbg_batch_get_ydot(self._h, _dptr(ydot), _iptr(st)))
        return ydot, st

    def get_qdotdot(self) -> np.ndarray:
        """State::getQDotDot() of the last realize: nq values per instance."""
        out = np.empty(int(self.y_offsets[-1] - self.u_offsets[-1]))
        N.check(N.engine_lib().sbg_batch_get_qdotdot(self._h, _dptr(out)))
        return out

    def sync(self) -> None:
        N.check(N.engine_lib().sbg_batch_sync(self._h))

    @property
    def launch_count(self) -> int:
        return int(N.engine_lib().sbg_batch_launch_count(self._h))

    @property
    def kernel_variant(self) -> int:
        return int(N.engine_lib().sbg_batch_kernel_variant(self._h))

    @property
    def group_lanes_shift(self) -> int:
        return int(N.engine_lib().sbg_batch_group_lanes_shift(self._h))

    @property
    def device_bytes(self) -> int:
        b = C.c_int64()
        N.check(N.engine_lib().sbg_batch_device_bytes(self._h, C.byref(b)))
        return b.value

    def close(self) -> None:
        if getattr(self, "_h", None) and N._engine is not None:
            N._engine.sbg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def device_count() -> int:
    return int(N.engine_lib().sbg_device_count())
