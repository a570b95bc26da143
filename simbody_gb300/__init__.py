"""simbody_gb300 -- a GB300-native batched forward-dynamics engine for
Simbody's O(n) articulated-body hot path (realize through Stage::Acceleration
and fixed-step Runge-Kutta-Merson integration of many States at once).

The compute path is the CUDA library simbody_gb300/_build/libsimbody_gb300.so
behind the C ABI in include/simbody_gb300.h; there is no CPU fallback.
"""
from . import _native  # noqa: F401
from .engine import Batch, Topology, device_count  # noqa: F401
from .serve import Server  # noqa: F401
from .workloads import Workload, engine_batch  # noqa: F401

__all__ = ["Batch", "Server", "Topology", "Workload", "engine_batch", "device_count"]
