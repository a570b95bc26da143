"""The header-only C++ surface (include/simbody_gb300.hpp) on the GPU.

A C++ program written with the Simbody vocabulary builds one sbg::Topology per
system of the random-tree workload (Free base, Pin/Slider/Universal/Ball
children, springs and dampers), a StateBatch over 256 states, realizes them
through Stage::Acceleration and integrates them with
RungeKuttaMersonBatchIntegrator: stepTo(t1), stepTo(t2) (a continued
integration) and stepBy(0.3 h) (a shortened last step); it reads
getQDotDot() after the realize, and integrates a second batch of the same
states error-controlled (no fixed step size; accuracy 1e-3) to t = 0.03. Its
outputs are compared with the oracle: realize to 1e-12, qdotdot to 1e-12, the
states to 1e-10 (FP64), and the error-controlled run's accepted and attempted
step counts exactly.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from simbody_gb300 import Workload

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
N_INST = 256

PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "simbody_gb300.hpp"
#include "sbg_workloads.h"

int main(int argc, char** argv) {
    if (argc < 2) return 1;
    sbg_workload w;
    if (sbg_workload_create(3, NINST, &w)) return 2;
    const int nsys = sbg_workload_num_systems(w);
    const sbg_system_desc* sys = sbg_workload_systems(w);
    const int32_t* isys = sbg_workload_instance_system(w);
    const int64_t* yo = sbg_workload_y_offsets(w);
    const double h = sbg_workload_h(w);
    std::vector<sbg::Topology> topos;
    topos.reserve(nsys);
    for (int k = 0; k < nsys; ++k) topos.emplace_back(sys[k]);
    std::vector<const sbg::Topology*> tp;
    for (auto& t : topos) tp.push_back(&t);
    std::vector<int32_t> inst(isys, isys + NINST);
    sbg::StateBatch batch(tp, inst, sbg::Precision::FP64);
    std::vector<double> y0(sbg_workload_y0(w), sbg_workload_y0(w) + yo[NINST]);
    batch.setY(y0);
    std::vector<int32_t> st;
    const std::vector<double> ydot = batch.realizeAcceleration(&st);
    for (int32_t s : st) if (s) return 3;
    const std::vector<double> qdd = batch.getQDotDot();
    sbg::RungeKuttaMersonBatchIntegrator integ(batch);
    integ.setFixedStepSize(h);
    integ.initialize(0.0);
    int bad = 0;
    for (double tr : {7 * h, 15 * h}) for (int32_t s : integ.stepTo(tr)) bad |= s;
    for (int32_t s : integ.stepBy(0.3 * h)) bad |= s;
    if (bad & ~4) return 4;
    const std::vector<double> y = batch.getY();
    const std::vector<double> t = batch.getTime();
    // error-controlled: no fixed step size
    sbg::StateBatch batch2(tp, inst, sbg::Precision::FP64);
    batch2.setY(y0);
    sbg::RungeKuttaMersonBatchIntegrator ec(batch2);
    ec.setAccuracy(1e-3);
    for (int32_t s : ec.stepTo(0.03)) bad |= s;
    if (bad & ~4) return 6;
    const std::vector<double> ya = batch2.getY();
    std::vector<double> counts;
    for (size_t i = 0; i < inst.size(); ++i) {
        counts.push_back((double)ec.getNumStepsTaken()[i]);
        counts.push_back((double)ec.getNumStepsAttempted()[i]);
    }
    FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 5;
    std::fwrite(ydot.data(), sizeof(double), ydot.size(), f);
    std::fwrite(y.data(), sizeof(double), y.size(), f);
    std::fwrite(t.data(), sizeof(double), t.size(), f);
    std::fwrite(qdd.data(), sizeof(double), qdd.size(), f);
    std::fwrite(ya.data(), sizeof(double), ya.size(), f);
    std::fwrite(counts.data(), sizeof(double), counts.size(), f);
    std::fclose(f);
    std::printf("ok %d\n", (int)batch.getNumInstances());
    sbg_workload_destroy(w);
    return 0;
}
"""


def test_cxx_surface_realize_and_integrate_on_gpu(engine, tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no host C++ compiler")
    from simbody_gb300.build import build_engine, build_workloads

    lib, wl = build_engine(), build_workloads()
    src = tmp_path / "surface.cc"
    src.write_text(PROGRAM.replace("NINST", str(N_INST)))
    exe = tmp_path / "surface"
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
                        "-I", str(ROOT / "simbody_gb300" / "csrc"), str(src), "-o", str(exe), str(lib), str(wl),
                        f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == f"ok {N_INST}", (r.returncode, r.stdout, r.stderr)

    w = Workload(3, N_INST)
    off = w.y_offsets
    ny = int(off[-1])
    raw = np.fromfile(out, dtype=np.float64)
    from simbody_gb300 import _native as N

    def nq_of(i):
        d = w.systems[int(w.instance_system[i])]
        return sum(N.NQ[d.bodies[k].mobilizer] for k in range(d.nbodies))

    qoff = np.concatenate([[0], np.cumsum([nq_of(i) for i in range(N_INST)])]).astype(np.int64)
    nqt = int(qoff[-1])
    assert raw.size == 3 * ny + N_INST + nqt + 2 * N_INST
    ydot, y, t = raw[:ny], raw[ny:2 * ny], raw[2 * ny:2 * ny + N_INST]
    k = 2 * ny + N_INST
    qdd, ya, counts = raw[k:k + nqt], raw[k + nqt:k + nqt + ny], raw[k + nqt + ny:].reshape(N_INST, 2)
    ref, rst = O.realize_workload(w)
    assert (rst == 0).all()

    def worst(a, b):
        return max(np.linalg.norm(a[off[i]:off[i + 1]] - b[off[i]:off[i + 1]]) / np.linalg.norm(b[off[i]:off[i + 1]])
                   for i in range(N_INST))

    assert worst(ydot, ref) <= 1e-12
    h, so, y0 = w.h, w.instance_system[:N_INST], w.y0[:ny]
    ry, rt, _ = O.rk_merson_run(w.systems, w.nsys, so, off, y0, h, t_report=7 * h)
    ry, rt, _ = O.rk_merson_run(w.systems, w.nsys, so, off, ry, h, t_report=15 * h, t=rt, initialize=False)
    ry, rt, _ = O.rk_merson_run(w.systems, w.nsys, so, off, ry, h, t_report=15 * h + 0.3 * h, t=rt, initialize=False)
    np.testing.assert_array_equal(t, rt)
    assert worst(y, ry) <= 1e-10
    # getQDotDot after the realize
    rq = O.qdotdot(w.systems, w.nsys, so, off, y0, ydot, qoff)
    assert max(np.linalg.norm(qdd[qoff[i]:qoff[i + 1]] - rq[qoff[i]:qoff[i + 1]]) /
               max(np.linalg.norm(rq[qoff[i]:qoff[i + 1]]), 1e-300) for i in range(N_INST)) <= 1e-12
    # the error-controlled mode: same accepted / attempted steps, state to 1e-10
    ay, at, ast, astats = O.rk_merson_adaptive(w.systems, w.nsys, so, off, y0, 0.03, accuracy=1e-3)
    ok = ast == 0
    assert ok.mean() > 0.95
    np.testing.assert_array_equal(counts[ok, 0], astats[ok, 0])
    np.testing.assert_array_equal(counts[ok, 1], astats[ok, 0] + astats[ok, 1])
    assert max(np.linalg.norm(ya[off[i]:off[i + 1]] - ay[off[i]:off[i + 1]]) / np.linalg.norm(ay[off[i]:off[i + 1]])
               for i in np.nonzero(ok)[0]) <= 1e-10
