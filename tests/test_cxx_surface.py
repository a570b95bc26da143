"""The header-only C++ surface (include/simbody_gb300.hpp) builds against the
C ABI library and behaves like SimTK on the host: a topology reports its
sizes and default state, an ill-formed system throws sbg::Error with
SBG_ERR_INVALID, and without a GPU a batch throws SBG_ERR_NO_DEVICE."""
import shutil
import subprocess

import pytest

from simbody_gb300.build import build_engine

from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

PROGRAM = r"""
#include <cstdio>
#include "simbody_gb300.hpp"

static sbg_body_desc pin(int parent) {
    sbg_body_desc b{};
    b.parent = parent; b.mobilizer = SBG_PIN; b.mass = 1.0;
    b.unit_inertia[0] = b.unit_inertia[1] = b.unit_inertia[2] = 1.0;
    b.X_PF[0] = b.X_PF[4] = b.X_PF[8] = 1.0;
    b.X_BM[0] = b.X_BM[4] = b.X_BM[8] = 1.0;
    b.X_BM[10] = 1.0;
    return b;
}

int main() {
    sbg_body_desc bodies[2] = {pin(0), pin(1)};
    sbg_system_desc d{};
    d.nbodies = 2; d.gravity[1] = -9.8; d.bodies = bodies;
    sbg::Topology topo(d);
    if (topo.getNQ() != 2 || topo.getNU() != 2 || topo.getNumBodies() != 2 || topo.getNumLevels() != 2) return 10;
    for (double v : topo.getDefaultY()) if (v != 0.0) return 11;
    bodies[1].parent = 2;  // a parent must precede its child
    try { sbg::Topology bad(d); return 12; } catch (const sbg::Error& e) { if (e.code() != SBG_ERR_INVALID) return 13; }
    bodies[1].parent = 1;
    if (sbg_device_count() == 0) {
        try {
            sbg::StateBatch b({&topo}, {0, 0, 0}, sbg::Precision::Mixed);
            return 14;
        } catch (const sbg::Error& e) {
            if (e.code() != SBG_ERR_NO_DEVICE) return 15;
        }
    }
    std::puts("ok");
    return 0;
}
"""


def test_cxx_surface_on_the_host(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no host C++ compiler")
    lib = build_engine()
    src = tmp_path / "surface.cc"
    src.write_text(PROGRAM)
    exe = tmp_path / "surface"
    r = subprocess.run([gxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"), str(src),
                        "-o", str(exe), str(lib), f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)


def test_simtk_adapter_round_trips_every_recorded_system():
    """include/simbody_gb300_simtk.hpp is compiled against Simbody by the
    golden-vector generator (tests/golden/make_golden.{py,cpp}), which builds
    each recorded system through its ForceLog, reads it back with describe()
    and stops unless every descriptor field equals the workload's bit for bit;
    gravity, kept by Force::Gravity as a direction and a magnitude, is
    recorded as a relative deviation. Every record carries one, and all are
    within rounding."""
    import numpy as np

    g = np.load(ROOT / "tests" / "golden" / "reference_vectors.npz")
    assert len(g["adapter_gdev"]) == len(g["cfg"]) > 0
    assert set(np.unique(g["cfg"])) == set(range(1, 11))
    assert g["adapter_gdev"].max() <= 1e-15
    # and it refused each of six systems with one element outside the GPU
    # path (a two-point spring, a spring created outside its log, gravity
    # excluding a body, a moving half-space, a Rod constraint, an Ellipsoid)
    assert int(g["adapter_refusals"]) == 6
