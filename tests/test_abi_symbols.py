"""The C-ABI library loads on a machine without a GPU and exports every entry
point declared in include/simbody_gb300.h (no compute calls)."""
import ctypes as C
import re
from pathlib import Path

from simbody_gb300 import _native as N

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "simbody_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sbg_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    from simbody_gb300.build import build_engine

    build_engine()
    lib = N.engine_lib()
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # every declared symbol has a ctypes prototype in the Python binding
    assert set(names) <= set(N.ENGINE_API), set(names) - set(N.ENGINE_API)


def test_abi_version_and_no_device_here():
    lib = N.engine_lib()
    assert lib.sbg_abi_version() == 2
    assert lib.sbg_device_count() >= 0  # 0 on a machine without a driver; never raises


def test_struct_layouts_match_header():
    assert C.sizeof(N.BodyDesc) == 288
    assert C.sizeof(N.SystemDesc) == 80
    assert C.sizeof(N.ContactDesc) == 208


def test_batch_entry_points_refuse_a_null_batch_without_touching_the_device():
    """Argument checks come before any CUDA call, so they hold on a machine
    without a GPU: a null batch is SBG_ERR_INVALID with a message."""
    from simbody_gb300.build import build_engine

    build_engine()
    lib = N.engine_lib()
    d = (C.c_double * 4)()
    i32 = (C.c_int32 * 4)()
    i64 = C.c_int64()
    calls = {
        "sbg_calc_residual_force": (None, d, d, d, d, i32),
        "sbg_multiply_by_m": (None, d, d, i32),
        "sbg_multiply_by_system_jacobian": (None, d, d, i32),
        "sbg_multiply_by_system_jacobian_transpose": (None, d, d, i32),
        "sbg_calc_composite_body_inertias": (None, d, i32),
        "sbg_multiply_by_minv": (None, d, d),
        "sbg_batch_fallback_count": (None, C.byref(i64)),
        "sbg_batch_fp64_steps": (None, C.byref(i64)),
        "sbg_batch_get_qdotdot": (None, d),
        "sbg_rk_merson_step_to": (None, 1e-3, 1.0, None, i32),
        "sbg_rk_merson_adaptive": (None, 1.0, None, i32, C.byref(i64)),
        "sbg_batch_last_operator_ms": (None, d),
    }
    for name, args in calls.items():
        assert getattr(lib, name)(*args) == 1, name  # SBG_ERR_INVALID
        assert lib.sbg_last_error(), name


def test_header_is_plain_c_and_cxx(tmp_path):
    """The boundary header compiles as C99 (what a cgo / N-API / ctypes
    binding sees) and as C++ (the drop-in surface), warnings as errors."""
    import shutil
    import subprocess

    gcc, gxx = shutil.which("gcc"), shutil.which("g++")
    if not gcc or not gxx:
        import pytest
        pytest.skip("no host C/C++ compiler")
    src_c = tmp_path / "use.c"
    src_c.write_text('#include "simbody_gb300.h"\nint main(void) { return sbg_abi_version() == SBG_ABI_VERSION ? 0 : 1; }\n')
    src_cc = tmp_path / "use.cc"
    src_cc.write_text(src_c.read_text())
    inc = str(ROOT / "include")
    for cc, src, std in ((gcc, src_c, "-std=c99"), (gxx, src_cc, "-std=c++17")):
        r = subprocess.run([cc, std, "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only", "-I", inc, str(src)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_status_bits_match_the_header():
    text = (ROOT / "include" / "simbody_gb300.h").read_text()
    defines = dict(re.findall(r"#define SBG_(INST_[A-Z_]+)\s+(\d+)", text))
    assert len(defines) >= 7
    for name, value in defines.items():
        assert getattr(N, name) == int(value), name
