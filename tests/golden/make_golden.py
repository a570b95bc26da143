"""Regenerates tests/golden/reference_vectors.npz from a built Simbody.

  python tests/golden/make_golden.py --simbody-src SRC --simbody-lib LIBDIR

SRC is a Simbody source tree (its public headers are used) and LIBDIR holds
libSimTKcommon/libSimTKmath/libSimTKsimbody from a Release build of it. The
driver make_golden.cpp is compiled against them, run on the seeded workloads
(libsbg_workloads), and its records are packed into one .npz:

  cfg, inst, ny, nu, nsteps, status, h, t_rk,    one entry per record
  cons_tol (0 = the integrator's default)
  adapter_refusals (how many systems with one element outside the GPU path
                    -- a two-point spring, a spring created outside the
                    log, gravity excluding a body, a moving half-space, a
                    Rod constraint, an Ellipsoid mobilizer -- describe()
                    refused; the run stops if it takes one)
  adapter_gdev (include/simbody_gb300_simtk.hpp read the built system back
                into descriptors equal to the workload's; gravity's relative
                deviation, the only field not kept bit for bit)
  y_off, u_off, q_off                            offsets into the flat arrays
  y0, ydot, y_rk (by y_off); f, minv_f (by u_off); qdd (by q_off)

and the integrator continuation records (setAllowInterpolation(false)), one
per instance and mode (0: stepTo(t_mid); stepTo(t_end), 1: stepTo(t_end),
2: stepTo(t_end + 0.3 h)):

  c_cfg, c_inst, c_ny, c_mode, c_status, c_steps, c_h, c_t_mid, c_t_end,
  c_t_out, c_y_off; c_y0, c_y_out (by c_y_off)

and the error-controlled records (setAccuracy(acc), setFinalTime(t_final),
stepTo(t_final); steps taken and attempted):

  a_cfg, a_inst, a_ny, a_status, a_taken, a_attempted, a_accuracy, a_t_final,
  a_t_out, a_y_off; a_y0, a_y_out (by a_y_off)

The vectors are committed; the tests only read the .npz.
"""
from __future__ import annotations

import argparse
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]


def include_dirs(src: Path) -> list[str]:
    dirs = []
    for p in sorted(src.rglob("include")):
        rel = p.relative_to(src).parts
        if p.is_dir() and not any(x in ("tests", "examples", "doc", "src") for x in rel):
            dirs.append(str(p))
    return dirs


def read_records(path: Path) -> dict:
    raw = path.read_bytes()
    pos = 0
    recs = []
    while pos < len(raw):
        hdr = np.frombuffer(raw, dtype=np.int64, count=6, offset=pos)
        pos += 48
        h, t, ctol, gdev = np.frombuffer(raw, dtype=np.float64, count=4, offset=pos)
        pos += 32
        cfg, inst, ny, nu, nsteps, status = (int(v) for v in hdr)
        arrs = {}
        for name, n in (("y0", ny), ("ydot", ny), ("f", nu), ("minv_f", nu), ("y_rk", ny), ("qdd", ny - nu)):
            arrs[name] = np.frombuffer(raw, dtype=np.float64, count=n, offset=pos).copy()
            pos += 8 * n
        recs.append(dict(cfg=cfg, inst=inst, ny=ny, nu=nu, nsteps=nsteps, status=status, h=h, t_rk=t, cons_tol=ctol,
                         adapter_gdev=gdev, **arrs))
    out = {k: np.array([r[k] for r in recs]) for k in ("cfg", "inst", "ny", "nu", "nsteps", "status", "h", "t_rk",
                                                 "cons_tol", "adapter_gdev")}
    out["y_off"] = np.concatenate([[0], np.cumsum(out["ny"])]).astype(np.int64)
    out["u_off"] = np.concatenate([[0], np.cumsum(out["nu"])]).astype(np.int64)
    out["q_off"] = np.concatenate([[0], np.cumsum(out["ny"] - out["nu"])]).astype(np.int64)
    for k in ("y0", "ydot", "y_rk"):
        out[k] = np.concatenate([r[k] for r in recs])
    for k in ("f", "minv_f", "qdd"):
        out[k] = np.concatenate([r[k] for r in recs])
    return out


def read_continuation(path: Path) -> dict:
    raw = path.read_bytes()
    pos = 0
    recs = []
    while pos < len(raw):
        cfg, inst, ny, mode, status, steps = (int(v) for v in np.frombuffer(raw, dtype=np.int64, count=6, offset=pos))
        pos += 48
        h, tmid, tend, tout = np.frombuffer(raw, dtype=np.float64, count=4, offset=pos)
        pos += 32
        y0 = np.frombuffer(raw, dtype=np.float64, count=ny, offset=pos).copy()
        pos += 8 * ny
        yout = np.frombuffer(raw, dtype=np.float64, count=ny, offset=pos).copy()
        pos += 8 * ny
        recs.append(dict(cfg=cfg, inst=inst, ny=ny, mode=mode, status=status, steps=steps, h=h, t_mid=tmid,
                         t_end=tend, t_out=tout, y0=y0, y_out=yout))
    out = {"c_" + k: np.array([r[k] for r in recs])
           for k in ("cfg", "inst", "ny", "mode", "status", "steps", "h", "t_mid", "t_end", "t_out")}
    out["c_y_off"] = np.concatenate([[0], np.cumsum(out["c_ny"])]).astype(np.int64)
    out["c_y0"] = np.concatenate([r["y0"] for r in recs])
    out["c_y_out"] = np.concatenate([r["y_out"] for r in recs])
    return out


def read_adaptive(path: Path) -> dict:
    raw = path.read_bytes()
    pos = 0
    recs = []
    while pos < len(raw):
        cfg, inst, ny, status, taken, attempted = (int(v) for v in np.frombuffer(raw, dtype=np.int64, count=6,
                                                                                  offset=pos))
        pos += 48
        acc, tf, tout = np.frombuffer(raw, dtype=np.float64, count=3, offset=pos)
        pos += 24
        y0 = np.frombuffer(raw, dtype=np.float64, count=ny, offset=pos).copy()
        pos += 8 * ny
        yout = np.frombuffer(raw, dtype=np.float64, count=ny, offset=pos).copy()
        pos += 8 * ny
        recs.append(dict(cfg=cfg, inst=inst, ny=ny, status=status, taken=taken, attempted=attempted, accuracy=acc,
                         t_final=tf, t_out=tout, y0=y0, y_out=yout))
    out = {"a_" + k: np.array([r[k] for r in recs])
           for k in ("cfg", "inst", "ny", "status", "taken", "attempted", "accuracy", "t_final", "t_out")}
    out["a_y_off"] = np.concatenate([[0], np.cumsum(out["a_ny"])]).astype(np.int64)
    out["a_y0"] = np.concatenate([r["y0"] for r in recs])
    out["a_y_out"] = np.concatenate([r["y_out"] for r in recs])
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--simbody-src", required=True, type=Path)
    ap.add_argument("--simbody-lib", required=True, type=Path)
    ap.add_argument("--out", type=Path, default=HERE / "reference_vectors.npz")
    a = ap.parse_args()
    sys.path.insert(0, str(ROOT))
    from simbody_gb300.build import OUT, build_workloads

    wl = build_workloads()
    with tempfile.TemporaryDirectory() as td:
        exe = Path(td) / "make_golden"
        cmd = ["g++", "-O2", "-std=c++17", str(HERE / "make_golden.cpp"), "-o", str(exe),
               f"-I{ROOT / 'simbody_gb300' / 'csrc'}", f"-I{ROOT / 'include'}"]
        cmd += [f"-I{d}" for d in include_dirs(a.simbody_src)]
        cmd += [f"-L{a.simbody_lib}", "-lSimTKsimbody", "-lSimTKmath", "-lSimTKcommon",
                f"-Wl,-rpath,{a.simbody_lib}", str(wl), f"-Wl,-rpath,{OUT}"]
        subprocess.run(cmd, check=True)
        binf = Path(td) / "records.bin"
        conf = Path(td) / "cont.bin"
        adaf = Path(td) / "adapt.bin"
        reff = Path(td) / "refusals.txt"
        subprocess.run([str(exe), str(binf), str(conf), str(adaf), str(reff)], check=True,
                       env={"OPENBLAS_NUM_THREADS": "1"})
        data = read_records(binf)
        data.update(read_continuation(conf))
        data.update(read_adaptive(adaf))
        data["adapter_refusals"] = np.array(int(reff.read_text().strip()), dtype=np.int64)
    np.savez_compressed(a.out, **data)
    print(f"wrote {a.out}: {len(data['cfg'])} records")
    return 0


if __name__ == "__main__":
    sys.exit(main())
