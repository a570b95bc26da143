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
    assert lib.sbg_abi_version() == 1
    assert lib.sbg_device_count() >= 0  # 0 on a machine without a driver; never raises


def test_struct_layouts_match_header():
    assert C.sizeof(N.BodyDesc) == 280
    assert C.sizeof(N.SystemDesc) == 64
