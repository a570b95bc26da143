"""ctypes bindings of the C ABI (include/simbody_gb300.h) and of the workload
generator. The CUDA engine is the only compute path: if its shared library is
missing, importing the engine API raises instead of falling back to anything.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

PKG = Path(__file__).resolve().parent
BUILD = PKG / "_build"

# ----------------------------------------------------------------- structs
(SBG_PIN, SBG_SLIDER, SBG_UNIVERSAL, SBG_BALL, SBG_FREE, SBG_GIMBAL, SBG_TRANSLATION, SBG_CYLINDER, SBG_PLANAR,
 SBG_BUSHING, SBG_WELD, SBG_SCREW) = range(12)
NQ = {SBG_PIN: 1, SBG_SLIDER: 1, SBG_UNIVERSAL: 2, SBG_BALL: 4, SBG_FREE: 7, SBG_GIMBAL: 3, SBG_TRANSLATION: 3,
      SBG_CYLINDER: 2, SBG_PLANAR: 3, SBG_BUSHING: 6, SBG_WELD: 0, SBG_SCREW: 1}
NU = {SBG_PIN: 1, SBG_SLIDER: 1, SBG_UNIVERSAL: 2, SBG_BALL: 3, SBG_FREE: 6, SBG_GIMBAL: 3, SBG_TRANSLATION: 3,
      SBG_CYLINDER: 2, SBG_PLANAR: 3, SBG_BUSHING: 6, SBG_WELD: 0, SBG_SCREW: 1}
SYSTEM_EULER_ANGLES = 1
PRECISION_FP64, PRECISION_MIXED, PRECISION_MIXED_FAST = 0, 1, 2

INST_OK = 0
INST_NONFINITE = 1
INST_SINGULAR_D = 2
INST_PROJECTION_FAILED = 4
INST_CHOLESKY_FAIL = 8
INST_TIMEOUT = 16
INST_ILL_CONDITIONED = 32  # mixed form: the FP32 factorisation of M too poor for the refinement

STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "BUDGET", 5: "STATE", 6: "UNSUPPORTED",
                7: "NO_DEVICE"}


class BodyDesc(C.Structure):
    _fields_ = [("parent", C.c_int32), ("mobilizer", C.c_int32), ("mass", C.c_double),
                ("com", C.c_double * 3), ("unit_inertia", C.c_double * 6),
                ("X_PF", C.c_double * 12), ("X_BM", C.c_double * 12), ("pitch", C.c_double)]


class MobilityForceDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("body", C.c_int32), ("which", C.c_int32), ("reserved", C.c_int32),
                ("coef", C.c_double), ("q0", C.c_double)]


class BallConstraintDesc(C.Structure):
    _fields_ = [("body1", C.c_int32), ("body2", C.c_int32), ("station1", C.c_double * 3),
                ("station2", C.c_double * 3)]


class ContactDesc(C.Structure):
    _fields_ = [("body", C.c_int32), ("reserved", C.c_int32), ("station", C.c_double * 3), ("radius", C.c_double),
                ("halfspace", C.c_double * 12), ("stiffness", C.c_double), ("dissipation", C.c_double),
                ("static_friction", C.c_double), ("dynamic_friction", C.c_double),
                ("viscous_friction", C.c_double), ("transition_velocity", C.c_double), ("cf", C.c_double),
                ("bd", C.c_double), ("bv", C.c_double)]


class SystemDesc(C.Structure):
    _fields_ = [("nbodies", C.c_int32), ("nforces", C.c_int32), ("nconstraints", C.c_int32),
                ("flags", C.c_int32), ("gravity", C.c_double * 3),
                ("bodies", C.POINTER(BodyDesc)), ("forces", C.POINTER(MobilityForceDesc)),
                ("constraints", C.POINTER(BallConstraintDesc)), ("ncontacts", C.c_int32),
                ("reserved2", C.c_int32), ("contacts", C.POINTER(ContactDesc))]


class IntegOpts(C.Structure):
    _fields_ = [("accuracy", C.c_double), ("constraint_tolerance", C.c_double),
                ("project_every_step", C.c_int32), ("continue_integration", C.c_int32)]


class AdaptiveOpts(C.Structure):
    _fields_ = [("accuracy", C.c_double), ("constraint_tolerance", C.c_double), ("initial_step", C.c_double),
                ("min_step", C.c_double), ("max_step", C.c_double), ("project_every_step", C.c_int32),
                ("max_steps", C.c_int32)]


class BatchConfig(C.Structure):
    _fields_ = [("precision", C.c_int32), ("device", C.c_int32), ("device_budget_bytes", C.c_int64)]


class ServerConfig(C.Structure):
    _fields_ = [("precision", C.c_int32), ("device", C.c_int32), ("device_budget_bytes", C.c_int64),
                ("max_slots", C.c_int32), ("chunk_steps", C.c_int32)]


class RequestInfo(C.Structure):
    _fields_ = [("done", C.c_int32), ("status", C.c_int32), ("nbodies", C.c_int32), ("nsteps", C.c_int32),
                ("t", C.c_double), ("submit_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double),
                ("attempts", C.c_int32), ("fp64_steps", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("queued", C.c_int64),
                ("resident", C.c_int64), ("peak_resident", C.c_int64), ("ticks", C.c_int64),
                ("launches", C.c_int64), ("body_steps", C.c_int64), ("device_bytes", C.c_int64),
                ("max_slots", C.c_int32), ("chunk_steps", C.c_int32),
                ("pool_capacity", C.c_int64 * 5), ("pool_in_use", C.c_int64 * 5),
                ("gpu_seconds", C.c_double), ("host_seconds", C.c_double)]


assert C.sizeof(BodyDesc) == 288 and C.sizeof(MobilityForceDesc) == 32
assert C.sizeof(BallConstraintDesc) == 56 and C.sizeof(SystemDesc) == 80 and C.sizeof(ContactDesc) == 208

P = C.POINTER
dp, ip, i64p, vp = P(C.c_double), P(C.c_int32), P(C.c_int64), C.c_void_p

# name -> (restype, argtypes); every entry point of include/simbody_gb300.h
ENGINE_API = {
    "sbg_last_error": (C.c_char_p, []),
    "sbg_abi_version": (C.c_int, []),
    "sbg_device_count": (C.c_int, []),
    "sbg_topology_create": (C.c_int, [P(SystemDesc), P(vp)]),
    "sbg_topology_destroy": (C.c_int, [vp]),
    "sbg_topology_info": (C.c_int, [vp, ip, ip, ip, ip, ip, ip]),
    "sbg_topology_default_state": (C.c_int, [vp, dp]),
    "sbg_batch_create": (C.c_int, [P(vp), C.c_int32, ip, C.c_int32, P(BatchConfig), P(vp)]),
    "sbg_batch_destroy": (C.c_int, [vp]),
    "sbg_batch_layout": (C.c_int, [vp, i64p, i64p]),
    "sbg_batch_device_bytes": (C.c_int, [vp, i64p]),
    "sbg_batch_set_state": (C.c_int, [vp, dp, dp]),
    "sbg_batch_get_state": (C.c_int, [vp, dp, dp]),
    "sbg_realize_acceleration": (C.c_int, [vp, dp, ip]),
    "sbg_realize_acceleration_host": (C.c_int, [vp, dp, dp, ip]),
    "sbg_multiply_by_minv": (C.c_int, [vp, dp, dp]),
    "sbg_calc_residual_force": (C.c_int, [vp, dp, dp, dp, dp, ip]),
    "sbg_multiply_by_m": (C.c_int, [vp, dp, dp, ip]),
    "sbg_multiply_by_system_jacobian": (C.c_int, [vp, dp, dp, ip]),
    "sbg_multiply_by_system_jacobian_transpose": (C.c_int, [vp, dp, dp, ip]),
    "sbg_calc_composite_body_inertias": (C.c_int, [vp, dp, ip]),
    "sbg_batch_last_operator_ms": (C.c_int, [vp, dp]),
    "sbg_batch_fallback_count": (C.c_int, [vp, i64p]),
    "sbg_batch_fp64_steps": (C.c_int, [vp, i64p]),
    "sbg_rk_merson_fixed": (C.c_int, [vp, C.c_double, C.c_int32, P(IntegOpts), ip]),
    "sbg_batch_stream": (vp, [vp]),
    "sbg_realize_acceleration_async": (C.c_int, [vp]),
    "sbg_rk_merson_fixed_async": (C.c_int, [vp, C.c_double, C.c_int32, P(IntegOpts)]),
    "sbg_rk_merson_step_to": (C.c_int, [vp, C.c_double, C.c_double, P(IntegOpts), ip]),
    "sbg_rk_merson_step_to_async": (C.c_int, [vp, C.c_double, C.c_double, P(IntegOpts)]),
    "sbg_batch_get_ydot": (C.c_int, [vp, dp, ip]),
    "sbg_batch_sync": (C.c_int, [vp]),
    "sbg_rk_merson_adaptive": (C.c_int, [vp, C.c_double, P(AdaptiveOpts), ip, i64p]),
    "sbg_batch_get_qdotdot": (C.c_int, [vp, dp]),
    "sbg_batch_launch_count": (C.c_int64, [vp]),
    "sbg_batch_kernel_variant": (C.c_int, [vp]),
    "sbg_batch_group_lanes_shift": (C.c_int, [vp]),
    "sbg_server_create": (C.c_int, [P(ServerConfig), P(vp)]),
    "sbg_server_destroy": (C.c_int, [vp]),
    "sbg_server_submit": (C.c_int, [vp, vp, dp, C.c_double, C.c_double, C.c_int32, P(IntegOpts), i64p]),
    "sbg_server_tick": (C.c_int, [vp, ip]),
    "sbg_server_drain": (C.c_int, [vp]),
    "sbg_server_result": (C.c_int, [vp, C.c_int64, dp, P(RequestInfo)]),
    "sbg_server_get_stats": (C.c_int, [vp, P(ServerStats)]),
    "sbg_server_get_lane_stats": (C.c_int, [vp, C.c_int32, P(ServerStats)]),
    "sbg_server_clock": (C.c_double, [vp]),
    "sbg_serve_simulate": (C.c_int, [C.c_int32, i64p, ip, i64p, i64p, C.c_int32, C.c_int32, i64p, i64p, i64p]),
    "sbg_realize_acceleration_noalloc": (C.c_int, [vp, C.c_int32, vp, vp, vp, vp]),
    "sbg_noalloc_last_error": (C.c_char_p, []),
}

WORKLOAD_API = {
    "sbg_workload_last_error": (C.c_char_p, []),
    "sbg_workload_create": (C.c_int, [C.c_int32, C.c_int32, P(vp)]),
    "sbg_workload_destroy": (C.c_int, [vp]),
    "sbg_workload_num_systems": (C.c_int32, [vp]),
    "sbg_workload_num_instances": (C.c_int32, [vp]),
    "sbg_workload_systems": (P(SystemDesc), [vp]),
    "sbg_workload_instance_system": (ip, [vp]),
    "sbg_workload_y_offsets": (i64p, [vp]),
    "sbg_workload_y0": (dp, [vp]),
    "sbg_workload_h": (C.c_double, [vp]),
    "sbg_workload_nsteps": (C.c_int32, [vp]),
    "sbg_workload_horizons": (ip, [vp]),
    "sbg_workload_arrivals": (dp, [vp]),
}


def _bind(lib: C.CDLL, api: dict) -> C.CDLL:
    for name, (res, args) in api.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_engine = None
_workloads = None


def engine_lib() -> C.CDLL:
    """The CUDA engine library. Raises if it has not been built."""
    global _engine
    if _engine is None:
        path = BUILD / "libsimbody_gb300.so"
        if not path.exists():
            raise RuntimeError(f"CUDA engine library missing: {path} (run python -m simbody_gb300.build)")
        _engine = _bind(C.CDLL(str(path)), ENGINE_API)
    return _engine


def workload_lib() -> C.CDLL:
    global _workloads
    if _workloads is None:
        path = BUILD / "libsbg_workloads.so"
        if not path.exists():
            raise RuntimeError(f"workload library missing: {path} (run python -m simbody_gb300.build)")
        _workloads = _bind(C.CDLL(str(path)), WORKLOAD_API)
    return _workloads


class EngineError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def check(rc: int) -> None:
    if rc != 0:
        msg = engine_lib().sbg_last_error()
        raise EngineError(rc, msg.decode() if msg else "")
