"""Benchmark of the batched forward-dynamics hot path on one GB300.

Workload (default): the 32-Ball chain, 65,536 instances, realize(Stage::
Acceleration) of every instance per step ("body-steps" = body-RHS
evaluations). The headline value is the mixed-precision form (FP32 spatial
recursions + compensated refinement, FP64 state); the plain FP64 form is timed
on the same inputs and reported beside it with the relative udot error.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Timing: W untimed steps, then K steps bracketed by synchronisation, timed with
CUDA events recorded on the batch's own stream. The working set (state,
derivatives, per-body scratch) is larger than the 129 MB L2, so no flush is
needed between steps. ``e2e`` times the same metric through the public C-ABI
path with host buffers: per step a host->device state upload, the realize and
a device->host copy of [qdot, udot] and the status words.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
# DRAM bytes (read + write) of one launch of the mixed realize kernel (the
# staged chain driver, kernel variant 8) on the 65,536-instance 32-Ball
# workload, from an ncu capture of that launch
# (profiles/realize_32ball_65536_ncu.md): the per-body scratch records
# dominate it, against 235 MB of compulsory state I/O.
TRAFFIC_BYTES_PER_LAUNCH = 1.848917e9 + 0.893990e9
FP32_LANES = 152 * 128  # SMs x FP32 lanes per SM


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--instances", type=int, default=65536)
    p.add_argument("--cpu-seconds", type=float, default=10.0, help="target CPU-baseline sample duration")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--arm", default="all", choices=["all", "mixed", "fp64"],
                   help="profiling aid: time only this form's realize (no e2e, no CPU baseline)")
    p.add_argument("--no-trajectories", action="store_true")
    p.add_argument("--serve-seconds", type=float, default=1.0, help="arrival window of the serving stream (0 = skip)")
    p.add_argument("--serve-chunk", type=int, default=64)
    p.add_argument("--serve-sustained-rate", type=float, default=20.0,
                   help="arrival rate of the sustained serving run (requests/s)")
    p.add_argument("--serve-budget-gb", type=float, default=40.0)
    p.add_argument("--serve-deadline", type=float, default=90.0,
                   help="seconds after the first arrival at which unfinished requests are reported as censored")
    return p.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    return rank, world


def barrier() -> None:
    """All replicas line up (multi-GPU runs: one process per GPU)."""
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(x: float, device: str = "cuda") -> float:
    """The slowest replica's value: a timed region ends when every rank is done.
    Replicas run disjoint instances and exchange nothing else."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1):
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    try:
        d = json.loads(PEAKS_FILE.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# ------------------------------------------------------------ CPU baseline
def cpu_baseline(w, seconds: float, instances: int):
    """The oracle (the reference's CPU algorithm restated, compiled -O2) timed
    on this host's cores over a bounded sample of the same workload."""
    from oracle import oracle as O

    threads = O.hardware_threads()
    n = min(instances, w.ninst)
    sys_of = w.instance_system[:n]
    y = w.y0[: int(w.y_offsets[n])]
    off = w.y_offsets[: n + 1]
    t1 = O.time_realize(w.systems, w.nsys, sys_of, off, y, nreps=1, nthreads=threads)
    reps = max(1, int(seconds / max(t1, 1e-6)))
    t = O.time_realize(w.systems, w.nsys, sys_of, off, y, nreps=reps, nthreads=threads)
    nb = int(w.nbodies()[:n].sum())
    return {"value": nb * reps / t, "unit": "body-steps/s", "cores": threads, "kind": "port",
            "sample": f"{n} instances x {reps} realize(Acceleration) passes, {t:.1f} s wall"}


# ------------------------------------------------------------- tree operators
def tree_operators(b, w, y0, reps: int, cpu_instances: int):
    """The tree operators on the headline workload (FP64 in every batch
    precision): device time of the kernels (CUDA events on the batch stream,
    copies excluded), the same through the public API with host buffers, and
    the oracle port on the host cores for a sample of the instances."""
    from oracle import oracle as O

    nu, nb = int(b.u_offsets[-1]), int(b.body_offsets[-1])
    rng = np.random.default_rng(0)
    x, f, F = rng.standard_normal(nu), rng.standard_normal(nu), rng.standard_normal(6 * nb)
    calls = {"residual": (lambda: b.calc_residual_force(f, F, x), dict(x=x, fmob=f, fbody=F)),
             "mv": (lambda: b.multiply_by_m(x), dict(x=x)),
             "jv": (lambda: b.multiply_by_system_jacobian(x), dict(x=x)),
             "jtf": (lambda: b.multiply_by_system_jacobian_transpose(F), dict(fbody=F)),
             "composite": (lambda: b.calc_composite_body_inertias(), {})}
    n = min(cpu_instances, b.ninst)
    threads = O.hardware_threads()
    out = {"unit": "body-ops/s", "instances": b.ninst, "bodies": nb,
           "cpu_sample": f"oracle port, {n} instances, {threads} threads"}
    for name, (fn, kw) in calls.items():
        fn()
        dev, wall = [], []
        for _ in range(reps):
            t0 = time.perf_counter()
            _, st = fn()
            wall.append(time.perf_counter() - t0)
            dev.append(b.last_operator_ms())
        assert (st == 0).all()
        dev_ms, wall_ms = float(np.median(dev)), float(np.median(wall)) * 1e3
        sub = {k: (v[: int(b.u_offsets[n])] if k in ("x", "fmob") else v[: 6 * int(b.body_offsets[n])])
               for k, v in kw.items()}
        t0 = time.perf_counter()
        O.tree_op(w.systems, w.nsys, w.instance_system[:n], b.y_offsets[: n + 1], y0[: int(b.y_offsets[n])],
                  b.u_offsets[: n + 1], b.body_offsets[: n + 1], name, nthreads=threads, **sub)
        cpu_s = time.perf_counter() - t0
        nbs = int(b.body_offsets[n])
        out[name] = {"device_ms": dev_ms, "device_body_ops_per_s": nb / (dev_ms * 1e-3),
                     "api_ms": wall_ms, "api_body_ops_per_s": nb / (wall_ms * 1e-3),
                     "cpu_body_ops_per_s": nbs / cpu_s}
    return out


# ------------------------------------------------------------------ GPU arm
def time_resident(b, steps: int, warmup: int):
    import torch

    stream = torch.cuda.ExternalStream(b.stream)
    for _ in range(warmup):
        b.realize_acceleration_async()
    b.sync()
    torch.cuda.synchronize()
    barrier()
    n0 = b.launch_count
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        b.realize_acceleration_async()
    end.record(stream)
    end.synchronize()
    torch.cuda.synchronize()
    barrier()
    return start.elapsed_time(end) / steps, b.launch_count - n0


def pinned(shape, dtype):
    """A numpy array in page-locked host memory (a pinned torch tensor's
    storage), as a caller that streams states would hold them."""
    import torch

    tdt = {np.float64: torch.float64, np.int32: torch.int32}[dtype]
    return torch.empty(shape, dtype=tdt, pin_memory=True).numpy()


def time_e2e(b, y0, steps: int, warmup: int):
    """The public API with host buffers: per step one
    sbg_realize_acceleration_host call (State::updY + realize + getYDot:
    host -> device state, realize, device -> host [qdot, udot] and status,
    pipelined in chunks)."""
    yh = pinned(y0.shape, np.float64)
    yh[:] = y0
    ydot = pinned((b.ny_total,), np.float64)
    st = pinned((b.ninst,), np.int32)
    for _ in range(warmup):
        b.realize_acceleration_from(yh, ydot, st)
    t0 = time.perf_counter()
    n0 = b.launch_count
    for _ in range(steps):
        b.realize_acceleration_from(yh, ydot, st)
    dt = (time.perf_counter() - t0) / steps
    return dt * 1e3, b.launch_count - n0, ydot


def time_rk(b, h, nsteps):
    """One fixed-step RK-Merson integration of the batch's resident state,
    timed with CUDA events on the batch's stream."""
    import torch

    stream = torch.cuda.ExternalStream(b.stream)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = b.launch_count
    start.record(stream)
    b.rk_merson_fixed_async(h, nsteps)
    end.record(stream)
    end.synchronize()
    return start.elapsed_time(end), b.launch_count - n0


def cpu_trajectory_baseline(w, h, nsteps, seconds: float = 4.0, max_instances: int = 4096):
    """The oracle (the reference's CPU algorithm restated, -O2) integrating a
    bounded sample of the same instances on all host threads, for about
    `seconds`: body-steps/s."""
    from oracle import oracle as O

    threads = O.hardware_threads()
    n = min(threads, w.ninst)
    while True:
        idx = np.arange(n)
        t0 = time.perf_counter()
        O.rk_workload(w, h, nsteps, idx, nthreads=threads)
        dt = time.perf_counter() - t0
        if dt >= seconds / 4 or n >= min(max_instances, w.ninst):
            break
        n = min(min(max_instances, w.ninst), max(n + 1, int(n * seconds / max(dt, 1e-3) / 2)))
    return {"value": float(w.nbodies()[:n].sum()) * nsteps / dt, "unit": "body-steps/s", "cores": threads,
            "kind": "port", "sample": f"{n} instances x {nsteps} steps, {dt:.1f} s wall"}


def trajectories():
    """Fixed-step RK-Merson throughput (body-steps/s) on the trajectory
    workloads: the double pendulum (FP64), the random trees, the uneven
    batch, and the random trees with a contact sphere on every body over a
    ground half-space (FP64: the mixed form takes contact instances through
    FP64, the indentation being beyond FP32 kinematics). The trees run in
    both precisions: the mixed form (FP32 recursions,
    FP64 state; steps whose RHS meets an ill-conditioned M taken in FP64) over
    the full horizon, FP64 over a shorter one for its rate. Beside them: the
    mixed form's state error after all steps against the FP64 engine on a
    subset of instances, and the oracle port on the host cores."""
    from simbody_gb300 import Workload, engine_batch

    out = {}
    for cfg, n_inst, n_ref, fp64_steps in [(1, 1024, 0, 0), (3, 16384, 512, 400), (4, 10000, 256, 300),
                                           (8, 16384, 0, 400)]:
        w = Workload(cfg, n_inst)
        horizon = fp64_steps if cfg == 8 else w.nsteps
        rec = {"instances": w.ninst, "steps": horizon, "h": w.h}
        body = int(w.nbodies().sum())
        runs = (("fp64", w.nsteps),) if cfg == 1 else (("fp64", fp64_steps),) if cfg == 8 else \
            (("mixed", w.nsteps), ("fp64", fp64_steps))
        for prec, steps in runs:
            b, y0 = engine_batch(w, prec)
            b.set_state(y0)
            time_rk(b, w.h, 2)  # warm-up (the first call tunes the launch)
            b.set_state(y0)
            f0 = b.fp64_steps()
            ms, launches = time_rk(b, w.h, steps)
            y, _ = b.get_state()
            _, st = b.get_ydot()
            r = {"steps": steps, "ms": ms, "body_steps_per_s": body * steps / (ms * 1e-3), "gpu_launches": launches,
                 "status_nonzero": int((st != 0).sum())}
            if prec == "mixed":
                # instance steps taken in FP64 (a mixed RHS met an ill-conditioned M)
                r["fp64_instance_steps_frac"] = (b.fp64_steps() - f0) / float(w.ninst * steps)
                ymix = y
            rec[prec] = r
            b.close()
        if cfg in (3, 4):
            rec["mixed_over_fp64"] = rec["mixed"]["body_steps_per_s"] / rec["fp64"]["body_steps_per_s"]
        if n_ref:
            idx = np.arange(n_ref)
            r, yr0 = engine_batch(w, "fp64", instances=idx)
            r.set_state(yr0)
            r.rk_merson_fixed(w.h, w.nsteps)
            yr, _ = r.get_state()
            offs = w.y_offsets  # the batch's host packing is the workload's, instance order

            def rel(a, oa, c, oc):
                return np.array([np.linalg.norm(a[oa[i]:oa[i + 1]] - c[oc[i]:oc[i + 1]]) /
                                 np.linalg.norm(c[oc[i]:oc[i + 1]]) for i in idx])

            errs = rel(ymix, offs, yr, r.y_offsets)
            # the same FP64 run from a start perturbed by 1e-12 (relative):
            # how far rounding-sized differences grow over the horizon
            rng = np.random.default_rng(0)
            r.set_state(yr0 * (1 + 1e-12 * rng.standard_normal(yr0.size)))
            r.rk_merson_fixed(w.h, w.nsteps)
            yp, _ = r.get_state()
            pert = rel(yp, r.y_offsets, yr, r.y_offsets)
            rec["state_rel_err_vs_fp64"] = {"instances": n_ref, "median": float(np.median(errs)),
                                            "max": float(errs.max()),
                                            "fp64_from_1e-12_perturbed_start": {"median": float(np.median(pert)),
                                                                                "max": float(pert.max())}}
            r.close()
        rec["cpu_baseline"] = cpu_trajectory_baseline(w, w.h, horizon)
        out[{1: "double_pendulum", 3: "random_trees", 4: "uneven_batch", 8: "contact_trees"}[cfg]] = rec
    out["random_trees_error_controlled"] = error_controlled()
    return out


def error_controlled(t_final: float = 0.1, accuracy: float = 1e-3):
    """The error-controlled RK-Merson (FP64) on the random trees: accepted
    body-steps/s of the GPU kernel (every instance with its own step size)
    and of the oracle port on the host cores over a sample."""
    import torch
    from oracle import oracle as O
    from simbody_gb300 import Workload, engine_batch

    w = Workload(3, 16384)
    b, y0 = engine_batch(w, "fp64")
    b.set_state(y0)
    b.rk_merson_adaptive(0.002, accuracy=accuracy)  # warm-up
    b.set_state(y0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st, stats = b.rk_merson_adaptive(t_final, accuracy=accuracy)
    dt = time.perf_counter() - t0
    nb = w.nbodies()
    acc_body_steps = float((nb * stats[:, 0]).sum())
    threads = O.hardware_threads()
    n = 4 * threads
    t0 = time.perf_counter()
    _, _, _, cst = O.rk_merson_adaptive(w.systems, w.nsys, w.instance_system[:n], w.y_offsets[: n + 1],
                                        w.y0[: int(w.y_offsets[n])], t_final, accuracy=accuracy, nthreads=threads)
    cdt = time.perf_counter() - t0
    b.close()
    return {"instances": w.ninst, "t_final": t_final, "accuracy": accuracy, "s": dt,
            "accepted_body_steps_per_s": acc_body_steps / dt,
            "steps_per_instance": {"accepted_mean": float(stats[:, 0].mean()), "rejected_mean": float(stats[:, 1].mean()),
                                   "accepted_max": int(stats[:, 0].max())},
            "status_nonzero": int((st != 0).sum()),
            "cpu_baseline": {"value": float((nb[:n] * cst[:, 0]).sum()) / cdt, "unit": "body-steps/s",
                             "cores": threads, "kind": "port", "sample": f"{n} instances to t = {t_final}"}}


def serving(seconds: float, chunk: int, budget_gb: float, cpu_sample_body_steps: float, deadline_s: float,
            rate: float = 2000.0, trees_only: bool = False):
    """The serving stream: Poisson arrivals at `rate` requests/s (2,000 in
    the configuration) for `seconds`, trees from the uneven-batch
    distribution, horizons log-uniform in [100, 10000] steps, 20% with 1-4
    Ball loop closures (none with `trees_only`); continuous batching with a
    device budget. Latency = time the result reached the host - scheduled
    arrival. Requests still running `deadline_s` after the first arrival are
    reported as censored: their latency enters the percentiles as the time
    waited so far (a lower bound), and `censored` says how many there were."""
    from oracle import oracle as O
    from simbody_gb300 import Server, Topology, Workload

    want = int(round(rate * seconds))
    w = Workload(5, int(want * (1.3 if trees_only else 1.0)) + 8)
    keep = [i for i in range(w.ninst) if not (trees_only and w.systems[int(w.instance_system[i])].nconstraints)]
    keep = keep[:want]
    n = len(keep)
    # the workload's arrivals are a 2,000/s Poisson stream: rescaled to `rate`
    arrivals = np.array([w.arrivals[i] for i in keep]) * (2000.0 / rate)
    arrivals -= arrivals[0] - w.arrivals[0] * (2000.0 / rate)
    topos = [Topology(w.systems[int(w.instance_system[i])], keepalive=w) for i in keep]
    srv = Server("mixed", device_budget_bytes=int(budget_gb * (1 << 30)), chunk_steps=chunk)
    ids = np.zeros(n, dtype=np.int64)
    t_start = srv.clock()
    nxt, max_queue = 0, 0
    while nxt < n:
        now = srv.clock() - t_start
        while nxt < n and arrivals[nxt] <= now:
            i = keep[nxt]
            ids[nxt] = srv.submit(topos[nxt], w.y0[w.instance_slice(i)], w.h, int(w.horizons[i]))
            nxt += 1
        srv.tick()
        max_queue = max(max_queue, srv.stats()["queued"])
    while srv.stats()["completed"] < n and srv.clock() - t_start < deadline_s:
        srv.tick()
    t_end = srv.clock()
    lat, body_steps = np.empty(n), 0
    has_loops = np.array([w.systems[int(w.instance_system[i])].nconstraints > 0 for i in keep])
    status_bad = censored = fp64_steps = reruns = 0
    status_bits = {}
    for i in range(n):
        inf = srv.info(ids[i])
        if inf["done"]:
            lat[i] = inf["done_s"] - (t_start + arrivals[i])
            body_steps += inf["nbodies"] * inf["nsteps"]
            status_bad += inf["status"] != 0
            fp64_steps += inf["fp64_steps"]
            reruns += inf["attempts"] == 2
            for bit, name in [(1, "nonfinite"), (2, "singular_d"), (4, "projection_failed"), (8, "cholesky_fail")]:
                if inf["status"] & bit:
                    status_bits[name] = status_bits.get(name, 0) + 1
        else:
            lat[i] = t_end - (t_start + arrivals[i])
            censored += 1
    st = srv.stats()
    lanes = {name: {k: v for k, v in srv.lane_stats(li).items() if k in
                    ("submitted", "completed", "peak_resident", "ticks", "gpu_seconds", "device_bytes")}
             for li, name in [(0, "trees"), (1, "fp64_cheaper"), (2, "fp64_costlier")]}
    wall = t_end - t_start
    nbod = w.nbodies()
    offered = float(sum(int(nbod[i]) * int(w.horizons[i]) for i in keep)) / float(arrivals[-1])
    # CPU: requests run alone, one after another, on one core (the oracle)
    cpu_t, cpu_bs, k = 0.0, 0, 0
    while k < n and cpu_bs < cpu_sample_body_steps:
        i = keep[k]
        t0 = time.perf_counter()
        O.rk_workload(w, w.h, int(w.horizons[i]), instances=[i], nthreads=1)
        cpu_t += time.perf_counter() - t0
        cpu_bs += int(nbod[i]) * int(w.horizons[i])
        k += 1
    srv.close()
    return {"requests": n, "arrival_rate_per_s": rate, "arrival_window_s": float(arrivals[-1]),
            "requests_with_loop_closures": int(sum(w.systems[int(w.instance_system[i])].nconstraints > 0
                                                   for i in keep)),
            "precision": "mixed", "chunk_steps": chunk, "device_budget_bytes": st["device_bytes"],
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "mean": float(lat.mean()), "max": float(lat.max())},
            "latency_s_trees": {"p50": float(np.percentile(lat[~has_loops], 50)),
                                "p99": float(np.percentile(lat[~has_loops], 99))} if (~has_loops).any() else None,
            "latency_s_loop_closures": {"p50": float(np.percentile(lat[has_loops], 50)),
                                        "p99": float(np.percentile(lat[has_loops], 99))} if has_loops.any() else None,
            # every request finished and the queue stayed short: the server kept up with the arrivals
            "kept_up": bool(censored == 0 and max_queue <= max(8, n // 10)),
            "throughput_body_steps_per_s": body_steps / wall, "offered_body_steps_per_s": offered,
            "completed_requests_per_s": (n - censored) / wall, "wall_s": wall, "max_queued": int(max_queue),
            "peak_resident": st["peak_resident"], "ticks": st["ticks"], "gpu_launches": st["launches"],
            "host_tick_seconds": st["host_seconds"],
            "requests_with_status": int(status_bad), "status_bits": status_bits, "censored": int(censored),
            "requests_switched_to_fp64": int(fp64_steps), "requests_rerun_in_fp64": int(reruns),
            "deadline_s": deadline_s,
            "lanes": lanes,
            "cpu_alone_sequential": {"requests": k, "body_steps_per_s": cpu_bs / max(cpu_t, 1e-9), "cores": 1,
                                     "kind": "port"}}


def udot_rel_err(d_mixed, d_64, b):
    errs = np.empty(b.ninst)
    for i in range(b.ninst):
        s = slice(int(b.y_offsets[i] + b.nq[i]), int(b.y_offsets[i + 1]))
        x, y = d_mixed[s], d_64[s]
        errs[i] = np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300)
    return errs


def run_ours(args):
    import torch

    rank, world = _dist()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from simbody_gb300 import Workload, engine_batch
    from simbody_gb300.build import build_all

    build_all()
    w = Workload(2, args.instances)
    nb_total = int(w.nbodies().sum())
    if args.arm != "all":
        b, y0 = engine_batch(w, args.arm)
        b.set_state(y0)
        ms, launches = time_resident(b, args.steps, args.warmup)
        print(json.dumps({"arm": args.arm, "instances": w.ninst, "ms_per_step": ms,
                          "body_rhs_per_s": nb_total / (ms * 1e-3), "gpu_launches": launches}))
        return

    b64, y0 = engine_batch(w, "fp64")
    bmx, _ = engine_batch(w, "mixed")
    bft, _ = engine_batch(w, "mixed_fast")
    for b in (b64, bmx, bft):
        b.set_state(y0)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms_mx, launches = time_resident(bmx, args.steps, args.warmup)
        ms_64, _ = time_resident(b64, max(3, args.steps // 4), 1)
        ms_ft, _ = time_resident(bft, max(3, args.steps // 4), 1)
    d64, st64 = b64.realize_acceleration()
    dmx, stmx = bmx.realize_acceleration()
    dft, _ = bft.realize_acceleration()
    err = udot_rel_err(dmx, d64, bmx)
    err_ft = udot_rel_err(dft, d64, bft)
    bft.close()
    ms_e2e, e2e_launches, _ = time_e2e(bmx, y0, max(3, args.steps // 2), 1)

    ms_mx = max_over_ranks(ms_mx)
    value = nb_total * world / (ms_mx * 1e-3)
    value64 = nb_total / (ms_64 * 1e-3)
    ny_total = b64.ny_total
    alg_bytes = 2 * ny_total * 8  # read [q,u], write [qdot,udot]
    peak, peak_kind = _peaks()
    achieved = alg_bytes / (ms_mx * 1e-3) / 1e9
    from oracle import oracle as O

    flops_inst = sum(O.count_realize(w.systems, w.y0[w.instance_slice(0)]).values())
    result = {
        "metric": "body-steps/sec mixed vs FP64 on 1 GPU at <=1e-5 rel udot err",
        "value": value,
        "unit": "body-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_mx,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 recursions + f64 state",
        "data": "synthetic (seeded: std::mt19937_64(2<<32|i) states, body params from seed 2)",
        "config": {"workload": "32-Ball chain, 65,536 instances, realize(Stage::Acceleration) per step",
                   "instances": w.ninst, "bodies_per_instance": 32, "dof_per_instance": 96,
                   "l2": "working set (state 117 MB + derivatives + per-body scratch) larger than L2; no flush"},
        "fp64": {"value": value64, "ms_per_step": ms_64, "speedup_mixed_over_fp64": value / value64},
        "fp32_unrefined": {"value": nb_total / (ms_ft * 1e-3), "ms_per_step": ms_ft,
                           "udot_rel_err_max": float(err_ft.max())},
        "fp64_fallback_instances": bmx.fallback_count(),
        "udot_rel_err": {"max": float(err.max()), "p99": float(np.quantile(err, 0.99)), "mean": float(err.mean()),
                         "definition": "per instance ||udot_mixed - udot_fp64||_2 / ||udot_fp64||_2"},
        "status_nonzero": int((stmx != 0).sum() + (st64 != 0).sum()),
        "e2e": {"value": nb_total / (ms_e2e * 1e-3), "unit": "body-steps/s", "ms_per_step": ms_e2e,
                "h2d_bytes_per_step": ny_total * 8, "d2h_bytes_per_step": ny_total * 8 + 4 * w.ninst},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": TRAFFIC_BYTES_PER_LAUNCH if w.ninst == 65536 else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of this "
                                       "kernel on this workload (profiles/realize_32ball_65536_ncu.md)",
                     "dram_gbs_measured_traffic": (TRAFFIC_BYTES_PER_LAUNCH / (ms_mx * 1e-3) / 1e9
                                                  if w.ninst == 65536 else None),
                     "peak_kind": peak_kind,
                     "algorithmic_bytes": "16 B per state element: read [q,u] (f64), write [qdot,udot] (f64) = "
                                          f"{alg_bytes} B per launch"},
        "fp_work": {"flops_per_instance_fp64_algorithm": flops_inst,
                    "achieved_tflops": flops_inst * w.ninst / (ms_mx * 1e-3) / 1e12,
                    "fp32_peak_tflops_at_clock": FP32_LANES * 2 * (clk.summary()["sm_mhz"] or 2070.0) * 1e6 / 1e12,
                    "note": "the 6x6 spatial recursions are scalar FP32 FMA work (no tensor-core contraction); "
                            "the fraction of the FP32 peak is achieved / fp32_peak"},
        "gpu_launches": launches,
        "kernel_variant": bmx.kernel_variant,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(w, args.cpu_seconds, min(args.instances, 65536))
    try:
        result["tree_operators"] = tree_operators(bmx, w, y0, 5, 8192)
    except Exception as e:  # noqa: BLE001
        result["tree_operators"] = {"error": repr(e)}
    b64.close()
    bmx.close()
    # the extra sections never keep the headline line from being printed
    if not args.no_trajectories:
        try:
            result["trajectories"] = trajectories()
        except Exception as e:  # noqa: BLE001
            result["trajectories"] = {"error": repr(e)}
    if args.serve_seconds > 0:
        try:
            result["serving"] = serving(args.serve_seconds, args.serve_chunk, args.serve_budget_gb, 2e6,
                                        args.serve_deadline)
        except Exception as e:  # noqa: BLE001
            result["serving"] = {"error": repr(e)}
        # the same stream at a rate the server sustains (every request
        # finishes, the queue stays short): latency at sustained throughput
        try:
            result["serving_sustained"] = serving(args.serve_seconds * 4, args.serve_chunk, args.serve_budget_gb, 0,
                                                  args.serve_deadline, rate=args.serve_sustained_rate)
        except Exception as e:  # noqa: BLE001
            result["serving_sustained"] = {"error": repr(e)}
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_reference(args):
    rank, world = _dist()
    if rank != 0:
        return
    from simbody_gb300 import Workload
    from simbody_gb300.build import build_oracle, build_workloads

    build_workloads()
    build_oracle()
    from oracle import oracle as O

    w = Workload(2, args.instances)
    threads = O.hardware_threads()
    n = w.ninst
    nb = int(w.nbodies().sum())
    off = w.y_offsets
    for _ in range(args.warmup):
        O.time_realize(w.systems, w.nsys, w.instance_system, off, w.y0, nreps=1, nthreads=threads)
    times = []
    for _ in range(args.steps):
        times.append(O.time_realize(w.systems, w.nsys, w.instance_system, off, w.y0, nreps=1, nthreads=threads))
    t = float(np.mean(times))
    v = nb / t
    print(json.dumps({
        "impl": "reference",
        "metric": "body-steps/sec mixed vs FP64 on 1 GPU at <=1e-5 rel udot err",
        "value": v, "unit": "body-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (same seeded inputs as the GPU arm)",
        "config": {"workload": "32-Ball chain, 65,536 instances, realize(Stage::Acceleration) per step",
                   "instances": n},
        "cpu_baseline": {"value": v, "unit": "body-steps/s", "cores": threads, "kind": "port",
                         "sample": f"the full {n}-instance batch per step, {args.steps} steps"},
        "e2e": {"value": v, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


if __name__ == "__main__":
    a = _args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
