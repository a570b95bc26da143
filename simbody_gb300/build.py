"""Builds the native libraries in-tree (no cmake, no pip install).

  simbody_gb300/_build/libsimbody_gb300.so   CUDA engine + C ABI (sm_103a)
  simbody_gb300/_build/libsbg_workloads.so   seeded synthetic workloads (host)
  oracle/_build/liboracle.so                 CPU oracle (test infrastructure)

Translation units compile in parallel; a unit is rebuilt only when it is older
than one of its sources. Run ``python -m simbody_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
CU_UNITS = ["k_r64.cu", "k_r32c.cu", "k_r32cr.cu", "k_r32s.cu", "k_r32g.cu", "k_rk64.cu", "k_rk32c.cu", "k_rk32cr.cu", "k_rk32g.cu",
            "k_util.cu", "k_noalloc.cu", "k_loops.cu", "k_rkloops.cu", "k_rkloops1.cu", "k_ops.cu", "k_fallback.cu",
            "k_rkadapt.cu", "serve.cu"]
HOST_UNITS = ["capi.cpp"]
HEADERS = ["abi_device.cuh", "loops_device.cuh", "spatial.cuh", "engine.h", "kernels.h", "topology_internal.h",
           "serve_sched.h", "ops_device.cuh", "rk32c_launch.cuh",
           "r32c_launch.cuh"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA engine cannot be built")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_engine(verbose: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = [CSRC / h for h in HEADERS] + [ROOT / "include" / "simbody_gb300.h"]
    objs, jobs = [], []
    for unit in CU_UNITS + HOST_UNITS:
        src = CSRC / unit
        obj = OUT / (unit + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    lib = OUT / "libsimbody_gb300.so"
    if jobs or _stale(lib, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", str(lib)] + [str(o) for o in objs])
    return lib


def build_workloads() -> Path:
    OUT.mkdir(exist_ok=True)
    src = CSRC / "workloads.cpp"
    lib = OUT / "libsbg_workloads.so"
    if _stale(lib, [src, CSRC / "sbg_workloads.h", ROOT / "include" / "simbody_gb300.h"]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", str(lib), str(src)])
    return lib


def build_oracle() -> Path:
    """The CPU oracle is test infrastructure; it is built beside the engine so
    the tests and the CPU-baseline legs can load it."""
    out = ORACLE / "_build"
    out.mkdir(exist_ok=True)
    src = ORACLE / "sbg_oracle.cpp"
    lib = out / "liboracle.so"
    deps = [src, ORACLE / "sbg_oracle.hpp", ORACLE / "sbg_oracle_impl.hpp", ORACLE / "flopcount.hpp",
            ORACLE / "sbg_oracle_api.h", ROOT / "include" / "simbody_gb300.h"]
    if _stale(lib, deps):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-shared", "-o", str(lib), str(src),
              "-lpthread"])
    return lib


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_engine, verbose), ex.submit(build_workloads), ex.submit(build_oracle)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built:", *(str(p) for p in sorted(OUT.glob("*.so"))), str(ORACLE / "_build" / "liboracle.so"))
