"""Seeded synthetic workloads shaped like the benchmark configurations (the
generator is C++: simbody_gb300/csrc/workloads.cpp, so the C++ drivers and the
Python harness see identical inputs).

  1  2-Pin double pendulum, 1024 instances, RK Merson h=1e-3, 1000 steps
  2  32-Ball chain, 65,536 instances, realize(Acceleration)
  3  random trees of 20-40 bodies (Free root; Pin/Slider/Universal/Ball),
     gravity + a MobilityLinearSpring and -Damper per mobility, 16,384
     instances, h=5e-4, 2000 steps
  4  10,000 trees with body count log-uniform in [4,256], 1000 steps
  5  serving requests: trees as 4, horizons log-uniform in [100,10000] steps,
     20% with 1-4 Ball loop closures
  6  trees as 3 over all twelve mobilizers (Free or Bushing root)
  7  trees as 3 with Euler-angle Ball and Free bodies
  8  trees as 3 with a contact sphere on every body over a ground half-space
  9  trees as 7 (Euler-angle mode), 20% with 1-4 Ball loop closures
 10  trees as 3 with redundant Ball closures: a repeated closure, a second
     pinned point of a closed body, or both (rank-deficient G M^-1 G^T)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

DEFAULT_INSTANCES = {1: 1024, 2: 65536, 3: 16384, 4: 10000, 5: 2000, 6: 16384, 7: 16384, 8: 16384, 9: 1000, 10: 300}


class Workload:
    def __init__(self, config: int, ninstances: int | None = None):
        lib = N.workload_lib()
        n = DEFAULT_INSTANCES[config] if ninstances is None else int(ninstances)
        h = C.c_void_p()
        rc = lib.sbg_workload_create(int(config), n, C.byref(h))
        if rc:
            raise RuntimeError(lib.sbg_workload_last_error().decode())
        self._h = h
        self.config = config
        self.ninst = lib.sbg_workload_num_instances(h)
        self.nsys = lib.sbg_workload_num_systems(h)
        self.systems = lib.sbg_workload_systems(h)  # POINTER(SystemDesc), nsys entries
        self.instance_system = np.ctypeslib.as_array(lib.sbg_workload_instance_system(h), (self.ninst,)).copy()
        self.y_offsets = np.ctypeslib.as_array(lib.sbg_workload_y_offsets(h), (self.ninst + 1,)).copy()
        self.y0 = np.ctypeslib.as_array(lib.sbg_workload_y0(h), (int(self.y_offsets[-1]),)).copy()
        self.h = lib.sbg_workload_h(h)
        self.nsteps = lib.sbg_workload_nsteps(h)
        hp = lib.sbg_workload_horizons(h)
        self.horizons = np.ctypeslib.as_array(hp, (self.ninst,)).copy() if hp else None
        ap = lib.sbg_workload_arrivals(h)
        self.arrivals = np.ctypeslib.as_array(ap, (self.ninst,)).copy() if ap else None

    def system(self, k: int) -> N.SystemDesc:
        return self.systems[k]

    def nbodies(self) -> np.ndarray:
        nb = np.array([self.systems[k].nbodies for k in range(self.nsys)])
        return nb[self.instance_system]

    def instance_slice(self, i: int) -> slice:
        return slice(int(self.y_offsets[i]), int(self.y_offsets[i + 1]))

    def close(self):
        if getattr(self, "_h", None) and N._workloads is not None:
            N._workloads.sbg_workload_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def engine_batch(w: Workload, precision: str = "fp64", instances=None, device_budget_bytes: int = 0):
    """Topologies + a device batch for (a subset of) a workload's instances."""
    from .engine import Batch, Topology

    idx = np.arange(w.ninst) if instances is None else np.asarray(instances)
    used = sorted(set(int(w.instance_system[i]) for i in idx))
    remap = {k: j for j, k in enumerate(used)}
    topos = [Topology(w.systems[k], keepalive=w) for k in used]
    inst_topo = np.array([remap[int(w.instance_system[i])] for i in idx], dtype=np.int32)
    b = Batch(topos, inst_topo, precision=precision, device_budget_bytes=device_budget_bytes)
    y0 = np.concatenate([w.y0[w.instance_slice(int(i))] for i in idx]) if len(idx) else np.zeros(0)
    return b, y0
