"""Python face of the serving loop (sbg_server_* in include/simbody_gb300.h).

A ``Server`` admits rollout requests -- one State of any supported System,
Integrator::initialize and fixed-step RK-Merson stepTo(t0 + n h) -- and runs
them with continuous batching on one GPU. ``simulate`` runs the same
admission and chunk policy without a device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .engine import Topology

POOLS = ("rows", "forces", "state", "scratch", "loop_scratch")


class Server:
    def __init__(self, precision: str = "mixed", device: int = 0, device_budget_bytes: int = 1 << 30,
                 max_slots: int = 0, chunk_steps: int = 0):
        lib = N.engine_lib()
        prec = {"fp64": N.PRECISION_FP64, "mixed": N.PRECISION_MIXED, "mixed_fast": N.PRECISION_MIXED_FAST}[precision]
        cfg = N.ServerConfig(prec, device, int(device_budget_bytes), int(max_slots), int(chunk_steps))
        h = C.c_void_p()
        N.check(lib.sbg_server_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._ny = {}

    def submit(self, topology: Topology, y0: np.ndarray, h: float, nsteps: int, t0: float = 0.0,
               accuracy: float = 0.0, constraint_tolerance: float = 0.0, project_every_step: bool = False) -> int:
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        assert y0.size == topology.nq + topology.nu
        opts = N.IntegOpts(accuracy, constraint_tolerance, int(project_every_step), 0)
        rid = C.c_int64()
        N.check(N.engine_lib().sbg_server_submit(self._h, topology.handle, y0.ctypes.data_as(C.POINTER(C.c_double)),
                                                 float(t0), float(h), int(nsteps), C.byref(opts), C.byref(rid)))
        self._ny[rid.value] = topology.nq + topology.nu
        return rid.value

    def tick(self) -> int:
        n = C.c_int32()
        N.check(N.engine_lib().sbg_server_tick(self._h, C.byref(n)))
        return n.value

    def drain(self) -> None:
        N.check(N.engine_lib().sbg_server_drain(self._h))

    def info(self, rid: int) -> dict:
        inf = N.RequestInfo()
        N.check(N.engine_lib().sbg_server_result(self._h, int(rid), None, C.byref(inf)))
        return {k: getattr(inf, k) for k, _ in N.RequestInfo._fields_}

    def result(self, rid: int):
        """(y, info) of a finished request, None while it runs."""
        inf = N.RequestInfo()
        lib = N.engine_lib()
        N.check(lib.sbg_server_result(self._h, int(rid), None, C.byref(inf)))
        if not inf.done:
            return None
        y = np.empty(self._ny[rid])
        N.check(lib.sbg_server_result(self._h, int(rid), y.ctypes.data_as(C.POINTER(C.c_double)), C.byref(inf)))
        return y, {k: getattr(inf, k) for k, _ in N.RequestInfo._fields_}

    def stats(self) -> dict:
        st = N.ServerStats()
        N.check(N.engine_lib().sbg_server_get_stats(self._h, C.byref(st)))
        d = {k: getattr(st, k) for k, _ in N.ServerStats._fields_ if not k.startswith("pool_")}
        d["pool_capacity"] = dict(zip(POOLS, list(st.pool_capacity)))
        d["pool_in_use"] = dict(zip(POOLS, list(st.pool_in_use)))
        return d

    def lane_stats(self, lane: int) -> dict:
        """Stats of one lane: 0 = trees, 1 / 2 = the FP64 lanes (loop closures
        and reruns of failed mixed-precision requests; cheaper / costlier per
        step)."""
        st = N.ServerStats()
        N.check(N.engine_lib().sbg_server_get_lane_stats(self._h, int(lane), C.byref(st)))
        d = {k: getattr(st, k) for k, _ in N.ServerStats._fields_ if not k.startswith("pool_")}
        d["pool_capacity"] = dict(zip(POOLS, list(st.pool_capacity)))
        d["pool_in_use"] = dict(zip(POOLS, list(st.pool_in_use)))
        return d

    def clock(self) -> float:
        return float(N.engine_lib().sbg_server_clock(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None) and N._engine is not None:
            N._engine.sbg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def simulate(units, horizons, arrival_tick, capacity, max_slots: int, chunk_steps: int):
    """Run the server's admission and chunk policy without a device.
    Returns (admit_tick, done_tick, peak_resident)."""
    units = np.ascontiguousarray(units, dtype=np.int64).reshape(-1, 5)
    n = units.shape[0]
    hz = np.ascontiguousarray(horizons, dtype=np.int32)
    at = np.ascontiguousarray(arrival_tick, dtype=np.int64)
    cap = np.ascontiguousarray(capacity, dtype=np.int64)
    adm = np.full(n, -1, dtype=np.int64)
    done = np.full(n, -1, dtype=np.int64)
    peak = C.c_int64()
    i64 = C.POINTER(C.c_int64)
    N.check(N.engine_lib().sbg_serve_simulate(n, units.ctypes.data_as(i64), hz.ctypes.data_as(C.POINTER(C.c_int32)),
                                              at.ctypes.data_as(i64), cap.ctypes.data_as(i64), int(max_slots),
                                              int(chunk_steps), adm.ctypes.data_as(i64), done.ctypes.data_as(i64),
                                              C.byref(peak)))
    return adm, done, peak.value
