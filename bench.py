#!/usr/bin/env python3
"""Benchmark of the MHFEM time step on GB300.

Workload: the 3D heterogeneous-diffusion problem on the unit cube as a 64^3
grid of cubes split into 6 tetrahedra each (1,572,864 cells, 3,170,304 faces,
interior vertices jittered by +-0.15h, D = exp(g) with g a seeded Gaussian
field, f = 1, Dirichlet 0 on x=0,1 and zero flux elsewhere, dt = 1e-3,
BiCGStab to a relative residual of 1e-10).  A "step" is one backward-Euler
time step: coefficient / mass-matrix update, condensation, assembly, Krylov
solve and reconstruction (control.h:83-98).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Rank 0 prints one JSON line.  `value` is time steps/s of the plain FP64 form
summed over all replicas (each GPU runs an independent copy of the
workload: the path is not sharded, "replicas only").  `e2e` is the same
metric through the public C ABI with host buffers: every step uploads the
source field from pinned host memory and reads Z_iK back.  Beside it:
  forms.mixed             the mixed form on the same workload and steps;
  forms.learned_protocol  the learned-form protocol (200 training + 800 used
                          steps of the time-varying source) for four forms;
  other_configs           the 128^2 heat equation (100 steps), the 512^2
                          two-component ADR (200 steps) and the mixed form on
                          the 128^3 cube (20 steps);
every one with the relative error of each step's face traces against the
FP64 form solved to 1e-13 in lockstep.  `--impl reference` times the CPU
restatement of the reference algorithm (the reference itself cannot be
built: its TNL dependency is absent) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
PKG = REPO / "tnl-mhfem_gb300"
for _p in (str(PKG), str(REPO)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "time steps/s & face-DOF/s: FP64 vs mixed/learned at 1e-8 rel err; HBM GB/s"
UNIT = "time steps/s"


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--grid", type=int, default=64, help="cubes per axis (64 = the benchmark workload)")
    ap.add_argument("--cpu-steps", type=int, default=3, help="timed time steps of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-form protocol leg")
    ap.add_argument("--no-box", action="store_true", help="skip the cuboid (box cell) leg")
    ap.add_argument("--no-gmres", action="store_true", help="skip the GMRES leg")
    ap.add_argument("--configs", default="heat2d,adr2d,mixed128",
                    help="comma-separated other workloads to run: heat2d (128^2 heat equation, 100 steps), "
                         "adr2d (512^2 two-component ADR, 200 steps), mixed128 (mixed form on the 128^3 cube, "
                         "20 steps); 'none' skips them")
    ap.add_argument("--learned-train", type=int, default=200, help="online training steps of the learned protocol")
    ap.add_argument("--learned-used", type=int, default=800, help="steps after training in the learned protocol")
    ap.add_argument("--learned-iters", type=int, default=2, help="Adam iterations per training step")
    ap.add_argument("--learned-order", type=int, default=3,
                    help="polynomial extrapolation order of the base the network corrects (0-3)")
    ap.add_argument("--profile-run", action="store_true",
                    help="only the warm-up and timed steps (for an ncu launch list)")
    ap.add_argument("--profile-form", choices=["fp64", "mixed", "learned", "box", "gmres", "heat2d"], default="fp64",
                    help="form used by --profile-run (learned: --learned-train training steps first; heat2d: "
                         "the FP64 form on the 128^2 heat-equation workload, a small-system solve)")
    return ap.parse_args()


def allowed_cpus() -> int:
    """Host threads this process may run on (its CPU affinity)."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def workload_config(grid, C, F, rows, tol, dt, n=1, nf=4):
    """The `config` object of both arms: the same keys and values for the same workload."""
    W = (2 * nf - 1) * n - 1
    return {"workload": f"diffusion3d_{grid}", "cells": C, "faces": F, "rows": rows, "tol": tol, "dt": dt,
            "l2": f"working set larger than L2 (ELL values+columns {rows * W * 12 / 1e6:.0f} MB, cell records "
                  f"{8 * (n * nf + 1) * n * nf * C / 1e6:.0f} MB)"}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value: float, world: int) -> float:
    """Max of a per-rank timing over all ranks (the slowest replica sets the pace)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_value(steps: int, world: int, el_ms_max: float) -> float:
    """Whole-job steps/s: every replica ran `steps` steps; the slowest took el_ms_max."""
    return world * steps / (el_ms_max / 1e3)


def measured_peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples taken during the timed region."""

    def __init__(self, device: int):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.file.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.file.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def step_bytes(n, nf, S, C, F, V, W, iters, d_full=True):
    """Algorithmic bytes of one time step (each array once at its size)."""
    R = n * F
    rec = nf * n * (n * nf + 1) * C * 8
    cell = 4 * nf * C + 8 * 3 * V + (8 * n * n * C if d_full else 0) + 8 * n * C + 4 * nf * C + C \
        + 8 * n * n * S * C + 8 * n * n * nf * C + 8 * n * C + rec
    assemble = 15 * F + rec + 8 * W * R + 8 * R
    init = R * (12 * W + 8 + 8 + 8 + 24)
    per_iter = R * (24 * W + 152)  # SpMVs 12W + 24 and 12W + 16, updates 24 + 56 + 32
    recon = 4 * nf * C + 8 * n * F + 8 * n * n * nf * C + 16 * n * C
    return cell + assemble + init + iters * per_iter + recon


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    from mhfem import problems
    from oracle.oracle import OracleModel, load

    lib = load()
    threads = allowed_cpus()
    lib.orc_set_threads(threads)
    p = problems.diffusion3d(N=args.grid)
    m = OracleModel.from_problem(p)
    t = 0.0
    for _ in range(args.warmup):
        m.step(t, p.dt, p.tol)
        t += p.dt
    iters = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        it, _ = m.step(t, p.dt, p.tol)
        iters.append(it)
        t += p.dt
    el = time.perf_counter() - t0
    value = args.steps / el
    sample = (f"{args.steps} time steps of the {args.grid}^3 tetrahedral workload after {args.warmup} warm-up steps "
              f"(CPU restatement of the reference algorithm, C + OpenMP, -O3 as the reference's release build, FP64)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": f"synthetic: seeded jittered {args.grid}^3 cube grid split into 6 tetrahedra, D = exp(Gaussian field)",
            "form": "fp64 (CPU restatement, OpenMP)",
            "config": workload_config(args.grid, m.C, m.F, m.F * p.n, p.tol, p.dt),
            "face_dof_per_s": value * m.F * p.n, "iterations_per_step": statistics.mean(iters),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def kernel_table(s, L, hbm_peak):
    """CUDA-event times of the step's kernels (algorithmic bytes / FLOPs from the library)."""
    out = {}
    for name, kid, reps in [("cell_local", L.KERNEL_CELL_LOCAL, 20), ("assemble", L.KERNEL_ASSEMBLE, 20),
                            ("reconstruct", L.KERNEL_RECONSTRUCT, 20), ("spmv_fp64", L.KERNEL_SPMV_FP64, 50)]:
        r = s.time_kernel(kid, reps=reps)
        gbs = r["bytes"] / (r["ms"] * 1e-3) / 1e9
        out[name] = {"ms": r["ms"], "gbs": gbs, "hbm_frac": gbs / hbm_peak,
                     "fp64_tflops": r["flops"] / (r["ms"] * 1e-3) / 1e12}
    return out


# The five kernels of one FP64 BiCGStab iteration (one launch each; every
# check_every-th iteration the second SpMV and the x / r update also form the
# norms): name, kernel id, kernel symbol.
ITERATION_KERNELS = [
    ("spmv_dot", "KERNEL_SPMV_FP64", "k_spmv_dot<double,6,1> (v = A p, (rh, v))"),
    ("update_s", "KERNEL_UPDATE_S_FP64", "k_update_s<double,2> (s = r - alpha v)"),
    ("spmv_dots2", "KERNEL_SPMV2_FP64", "k_spmv_dots2<double,6,1,0> (t = A s, (t, s), (t, t))"),
    ("update_xr", "KERNEL_UPDATE_XR_FP64", "k_update_xr<double,2,0> (x, r updates, (rh, r))"),
    ("update_p", "KERNEL_UPDATE_P_FP64", "k_update_p<double,2> (p = r + beta (p - omega v))"),
]


def iteration_table(s, L, hbm_peak, reps=50):
    """CUDA-event time, algorithmic bytes and share of the iteration of each
    FP64 BiCGStab kernel, timed alone (back-to-back launches on the
    library's stream); the roofline names the one with the largest share."""
    out = {}
    for name, kid, sym in ITERATION_KERNELS:
        r = s.time_kernel(getattr(L, kid), reps=reps)
        gbs = r["bytes"] / (r["ms"] * 1e-3) / 1e9
        out[name] = {"kernel": sym, "ms": r["ms"], "bytes": r["bytes"], "gbs": gbs, "hbm_frac": gbs / hbm_peak,
                     "fp64_tflops": r["flops"] / (r["ms"] * 1e-3) / 1e12}
    total = sum(v["ms"] for v in out.values())
    for v in out.values():
        v["share_of_iteration"] = v["ms"] / total
    return out, total


def box_leg(args, dev, world):
    """The heterogeneous-diffusion model on (2 grid)^3 graded cuboids (box
    cells: closed-form RT0 inverse, 6 faces per cell, ELL width 10), FP64
    form, the same warm-up and timed steps as the headline."""
    import torch

    from mhfem import _lib as L
    from mhfem import problems

    N = 2 * args.grid
    p = problems.diffusion3d_box(N=N)
    p.config.device = dev
    s = problems.make_solver(p, check_every=8)
    ext = torch.cuda.ExternalStream(s.stream(), device=dev)
    t = 0.0
    for _ in range(args.warmup):
        s.step(t, p.dt)
        t += p.dt
    it0, _, _ = s.totals()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(ext)
    for _ in range(args.steps):
        s.step(t, p.dt)
        t += p.dt
    e1.record(ext)
    e1.synchronize()
    el = max_over_ranks(e0.elapsed_time(e1), world)
    it1, _, _ = s.totals()
    hbm_peak, _ = measured_peaks()
    out = {"workload": f"diffusion3d_box_{N}", "cells": s.C, "faces": s.F, "tol": p.tol, "dt": p.dt,
           "value": world * args.steps / (el / 1e3), "unit": UNIT, "ms_per_step": el / args.steps,
           "iterations_per_step": (it1 - it0) / args.steps, "kernels": kernel_table(s, L, hbm_peak)}
    s.close()
    return out


def gmres_leg(args, dev, world):
    """The FP64 form with restarted GMRES on the same workload, warm-up and
    timed steps: the reference example's solver keys (CGS, restart length
    varying between 3 and 30 in steps of 2 to 4), and the fixed restart
    length 30 beside them."""
    import torch

    from mhfem import problems

    def run(**restart):
        p = problems.diffusion3d(N=args.grid)
        p.config.device = dev
        s = problems.make_solver(p, check_every=8)
        s.setup(tol=p.tol, max_iter=100000, check_every=8, linear_solver="gmres", gmres_restart=30,
                gmres_variant="cgs", **restart)
        ext = torch.cuda.ExternalStream(s.stream(), device=dev)
        t = 0.0
        for _ in range(args.warmup):
            s.step(t, p.dt)
            t += p.dt
        it0, _, _ = s.totals()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(ext)
        for _ in range(args.steps):
            s.step(t, p.dt)
            t += p.dt
        e1.record(ext)
        e1.synchronize()
        el = max_over_ranks(e0.elapsed_time(e1), world)
        it1, _, _ = s.totals()
        s.close()
        return {"value": world * args.steps / (el / 1e3), "unit": UNIT, "ms_per_step": el / args.steps,
                "iterations_per_step": (it1 - it0) / args.steps}

    out = {"solver": "GMRES, classical Gram-Schmidt, restart length 3..30 (steps 2..4: "
                     "examples/HeatEquation/config.ini)"}
    out.update(run(gmres_restart_min=3, gmres_restart_step_min=2, gmres_restart_step_max=4))
    out["fixed_restart_30"] = run()
    return out


class Arm:
    """One solver of a lockstep run: every step is timed with CUDA events on
    the library's stream (synchronized after the step, so other solvers' work
    between the steps is not counted), and its face traces are compared on
    the device with the reference solver's after every step."""

    def __init__(self, name, sol, dev):
        import torch

        self.name, self.sol, self.dev = name, sol, dev
        self.ext = torch.cuda.ExternalStream(sol.stream(), device=dev)
        self.e0 = torch.cuda.Event(enable_timing=True)
        self.e1 = torch.cuda.Event(enable_timing=True)
        self.ms, self.stats, self.err_f, self.err_k = [], [], [], []
        self.zf = torch.as_tensor(sol.array_device("Z_iF"), device=f"cuda:{dev}")
        self.zk = torch.as_tensor(sol.array_device("Z_iK"), device=f"cuda:{dev}")

    def step(self, t, dt):
        self.e0.record(self.ext)
        st = self.sol.step(t, dt)
        self.e1.record(self.ext)
        self.e1.synchronize()
        self.ms.append(self.e0.elapsed_time(self.e1))
        self.stats.append(st)
        return st

    def close(self):
        self.sol.close()


def _rel_dev(a, b) -> float:
    """max |a - b| / max |b| on the device (FP64)."""
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))


def lockstep(arms, exact, dt, steps, t0=0.0):
    """Advances every arm and the reference solver `exact` (FP64 solved to
    1e-13, the exact discrete solution up to rounding) from the same state in
    lockstep; after each step every arm's face traces and cell values are
    compared with the reference's."""
    t = t0
    for _ in range(steps):
        for a in arms:
            a.step(t, dt)
        if exact is not None:
            exact.step(t, dt)
            for a in arms:
                a.err_f.append(_rel_dev(a.zf, exact.zf))
                a.err_k.append(_rel_dev(a.zk, exact.zk))
        t += dt
    return t


def arm_summary(a, world=1, lo=0, hi=None, err_bound=1e-8, full_errors=True):
    """Steps/s, iterations and errors of an arm over steps [lo, hi)."""
    import numpy as np

    hi = len(a.ms) if hi is None else hi
    ms = float(np.sum(a.ms[lo:hi]))
    n = hi - lo
    its = [st["iterations"] for st in a.stats[lo:hi]]
    out = {"value": world * n / (ms / 1e3), "ms_per_step": ms / n, "steps": n,
           "iterations_per_step": float(np.mean(its))}
    sw = [st["sweeps"] for st in a.stats[lo:hi]]
    if max(sw) > 1:
        out["sweeps_per_step"] = float(np.mean(sw))
    if a.err_f:
        ef, ek = a.err_f[lo:hi], a.err_k[lo:hi]
        out["rel_err_vs_fp64_1e-13_max"] = {"face_traces": max(ef), "cell_values": max(ek)}
        out["steps_over_1e-8"] = int(sum(1 for e in ef if e > err_bound))
        if full_errors:
            out["rel_err_vs_fp64_1e-13_per_step"] = [float(f"{e:.3e}") for e in ef]
        else:
            out["rel_err_vs_fp64_1e-13_every_10th_step"] = [float(f"{e:.3e}") for e in ef[::10]]
    return out


def _solver(p, dev, check_every=8, tol=None):
    from mhfem import problems

    p.config.device = dev
    if tol is not None:
        p.tol = tol
    return problems.make_solver(p, check_every=check_every)


def mixed_leg(args, dev, world, el_fp64_ms):
    """The mixed form on the headline workload: the same warm-up and timed
    steps as the FP64 form, in lockstep with the FP64 form solved to 1e-13
    (per-step errors of every step, warm-up included), and the FP32 SpMV."""
    from mhfem import _lib as L
    from mhfem import problems

    pm = problems.diffusion3d(N=args.grid, form=L.FORM_MIXED)
    mixed = Arm("mixed", _solver(pm, dev), dev)
    exact = Arm("exact", _solver(problems.diffusion3d(N=args.grid), dev, tol=1e-13), dev)
    lockstep([mixed], exact, pm.dt, args.warmup + args.steps)
    out = arm_summary(mixed, world, lo=args.warmup)
    out["speedup_vs_fp64"] = (out["value"] / world) / (args.steps / (el_fp64_ms / 1e3))
    errs = arm_summary(mixed, world)
    out["rel_err_vs_fp64_1e-13_per_step"] = errs["rel_err_vs_fp64_1e-13_per_step"]
    out["rel_err_vs_fp64_1e-13_max"] = errs["rel_err_vs_fp64_1e-13_max"]
    out["steps_over_1e-8"] = errs["steps_over_1e-8"]
    out["error_steps"] = "every step from the initial state, warm-up steps included"
    sp32 = mixed.sol.time_kernel(L.KERNEL_SPMV_FP32, reps=50)
    out["spmv_fp32_gbs"] = sp32["bytes"] / (sp32["ms"] * 1e-3) / 1e9
    mixed.close()
    exact.close()
    return out


def heat2d_leg(args, dev, world):
    """The plain FP64 heat equation on the 128^2 triangle
    mesh (49,408 faces), 100 steps of dt = 1e-4 from the Gaussian bump, tol
    1e-12; every step timed, in lockstep with the FP64 form at 1e-13; the CPU
    oracle over the same 100 steps beside it."""
    from mhfem import problems

    p = problems.heat2d(N=128)
    a = Arm("fp64", _solver(p, dev), dev)
    exact = Arm("exact", _solver(problems.heat2d(N=128), dev, tol=1e-13), dev)
    lockstep([a], exact, p.dt, p.steps)
    out = {"workload": "heat2d_128", "cells": a.sol.C, "faces": a.sol.F, "tol": p.tol,
           "dt": p.dt, "steps_from_initial_condition": p.steps, "fp64": arm_summary(a, world, full_errors=False)}
    out["fp64"]["face_dof_per_s"] = out["fp64"]["value"] * a.sol.F
    a.close()
    exact.close()
    if not args.no_cpu_baseline and world == 1:
        out["cpu_baseline"] = cpu_baseline(problems.heat2d(N=128), p.steps, warmup=0,
                                           what=f"all {p.steps} time steps of the 128^2 heat-equation workload")
    return out


def adr2d_leg(args, dev, world):
    """Coupled two-component advection-diffusion-reaction on
    the 512^2 triangle mesh (n = 2, 1,574,912 rows), 200 steps of dt = 5e-4,
    tol 1e-10; every step timed, in lockstep with the FP64 form at 1e-13."""
    from mhfem import problems

    p = problems.adr2d(N=512)
    a = Arm("fp64", _solver(p, dev), dev)
    exact = Arm("exact", _solver(problems.adr2d(N=512), dev, tol=1e-13), dev)
    lockstep([a], exact, p.dt, p.steps)
    out = {"workload": "adr2d_512", "cells": a.sol.C, "faces": a.sol.F, "rows": 2 * a.sol.F,
           "tol": p.tol, "dt": p.dt, "steps_from_initial_condition": p.steps,
           "fp64": arm_summary(a, world, full_errors=False)}
    out["fp64"]["face_dof_per_s"] = out["fp64"]["value"] * 2 * a.sol.F
    a.close()
    exact.close()
    if not args.no_cpu_baseline and world == 1:
        out["cpu_baseline"] = cpu_baseline(problems.adr2d(N=512), args.cpu_steps, warmup=1,
                                           what=f"{args.cpu_steps} time steps of the 512^2 ADR workload after 1 "
                                                "warm-up step")
    return out


def mixed128_leg(args, dev, world):
    """The mixed form on the 128^3 cube (12,582,912
    tetrahedra, 25,264,128 faces), 20 steps from the initial state, with the
    plain FP64 form on the same steps, both in lockstep with the FP64 form
    solved to 1e-13; the assembly kernel timed at this size."""
    from mhfem import _lib as L
    from mhfem import problems

    hbm_peak, _ = measured_peaks()
    steps = 20
    fp = Arm("fp64", _solver(problems.diffusion3d(N=128), dev), dev)
    mx = Arm("mixed", _solver(problems.diffusion3d(N=128, form=L.FORM_MIXED), dev), dev)
    exact = Arm("exact", _solver(problems.diffusion3d(N=128), dev, tol=1e-13), dev)
    p = problems.diffusion3d(N=2)
    lockstep([fp, mx], exact, p.dt, steps)
    out = {"workload": "diffusion3d_128", "cells": fp.sol.C, "faces": fp.sol.F, "tol": p.tol,
           "dt": p.dt, "inner_tol": 1e-4, "steps_from_initial_condition": steps,
           "fp64": arm_summary(fp, world), "mixed": arm_summary(mx, world)}
    out["mixed"]["speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["iterations_per_step_fp64"] = [st["iterations"] for st in fp.stats]
    out["inner_iterations_per_step_mixed"] = [st["iterations"] for st in mx.stats]
    out["sweeps_per_step_mixed"] = [st["sweeps"] for st in mx.stats]
    kern = {}
    for name, sol in (("assemble_fp64", fp.sol), ("assemble_mixed", mx.sol)):
        r = sol.time_kernel(L.KERNEL_ASSEMBLE, reps=10)
        gbs = r["bytes"] / (r["ms"] * 1e-3) / 1e9
        kern[name] = {"ms": r["ms"], "gbs": gbs, "hbm_frac": gbs / hbm_peak}
    r = fp.sol.time_kernel(L.KERNEL_SPMV_FP64, reps=20)
    kern["spmv_fp64"] = {"ms": r["ms"], "gbs": r["bytes"] / (r["ms"] * 1e-3) / 1e9}
    kern["spmv_fp64"]["hbm_frac"] = kern["spmv_fp64"]["gbs"] / hbm_peak
    out["kernels"] = kern
    for a in (fp, mx, exact):
        a.close()
    return out


def learned_protocol_leg(args, dev, world):
    """The learned form's whole protocol: the time-varying source
    f = 1 + 0.5 sin(2 pi t / T) psi(x) on the 64^3 workload (T = the
    protocol's span), the network trained online on the first
    `learned_train` steps and used for the next `learned_used`.  Four forms
    run it from the initial state, each timed over every step (training
    included): plain FP64, mixed, learned (FP64 BiCGStab from the gated
    guess: the protocol's form) and learned with the mixed-precision solve;
    all in lockstep with the FP64 form solved to 1e-13 for per-step errors."""
    import numpy as np

    from mhfem import _lib as L
    from mhfem import problems

    total = args.learned_train + args.learned_used
    mk = lambda form: problems.diffusion3d_source(N=args.grid, steps=total, form=form)
    fp = Arm("fp64", _solver(mk(L.FORM_FP64), dev), dev)
    mx = Arm("mixed", _solver(mk(L.FORM_MIXED), dev), dev)
    ln = Arm("learned", _solver(mk(L.FORM_LEARNED), dev), dev)
    lm = Arm("learned_mixed", _solver(mk(L.FORM_LEARNED), dev), dev)
    # ablations: the same form with the network never consulted (the gate
    # chooses between the warm start and the extrapolated base only), and the
    # network on the linear base 2 Zn - Zn1 (the previous two traces), with
    # and without the network
    bo = Arm("extrapolation_only", _solver(mk(L.FORM_LEARNED), dev), dev)
    l1 = Arm("learned_linear_base", _solver(mk(L.FORM_LEARNED), dev), dev)
    b1 = Arm("extrapolation_only_linear", _solver(mk(L.FORM_LEARNED), dev), dev)
    for a, mixed_solve, order in ((ln, False, args.learned_order), (lm, True, args.learned_order), (l1, False, 1)):
        a.sol.learned_options(train_steps=args.learned_train, train_iters=args.learned_iters, learning_rate=3e-3,
                              use_during_training=True, mixed_solve=mixed_solve, extrapolation_order=order)
    bo.sol.learned_options(train_steps=0, extrapolation_order=args.learned_order)
    b1.sol.learned_options(train_steps=0, extrapolation_order=1)
    # the FP64 solution to 1e-13 in lockstep (started from the extrapolated
    # base when that is closer: the initial guess changes its iteration
    # count, not its solution)
    exact = Arm("exact", _solver(mk(L.FORM_LEARNED), dev, tol=1e-13), dev)
    exact.sol.learned_options(train_steps=0, extrapolation_order=3)
    p = mk(L.FORM_FP64)
    arms = [fp, mx, ln, lm, bo, l1, b1]
    lockstep(arms, exact, p.dt, total)
    nt = args.learned_train
    out = {"workload": f"diffusion3d_source_{args.grid} (f = 1 + 0.5 sin(2 pi t/T) psi, "
                       f"T = {total} dt)",
           "train_steps": nt, "used_steps": args.learned_used, "adam_iterations_per_training_step": args.learned_iters,
           "extrapolation_order": args.learned_order,
           "timing": "every step of the protocol from the initial state, training included"}
    for a in arms:
        d = {"protocol": arm_summary(a, world, full_errors=False),
             "training_phase": arm_summary(a, world, 0, nt, full_errors=False),
             "used_phase": arm_summary(a, world, nt, total, full_errors=False)}
        for ph in ("training_phase", "used_phase"):
            for k in list(d[ph]):
                if k.startswith("rel_err") or k == "steps_over_1e-8":
                    del d[ph][k]
        if a in (ln, lm, bo, l1, b1):
            used = [st for st in a.stats[nt:]]
            d["used_phase"]["guess_accepted_steps"] = int(sum(st["guess_used"] for st in used))
            for ph, lo, hi in (("training_phase", 0, nt), ("used_phase", nt, total)):
                src = [st["guess_source"] for st in a.stats[lo:hi]]
                d[ph]["initial_guess_steps"] = {"warm_start": src.count(0), "network": src.count(1),
                                                "extrapolated_base": src.count(2)}
            rb = [st["base_residual"] for st in used if st["base_residual"] > 0]
            if rb:
                d["used_phase"]["base_rel_residual_geomean"] = float(np.exp(np.mean(np.log(rb))))
            rg = [st["guess_residual"] for st in used if st["guess_residual"] > 0]
            rw = [st["warm_residual"] for st in used if st["warm_residual"] > 0]
            if rg:
                d["used_phase"]["guess_rel_residual_geomean"] = float(np.exp(np.mean(np.log(rg))))
                d["used_phase"]["warm_start_rel_residual_geomean"] = float(np.exp(np.mean(np.log(rw))))
            d["used_phase"]["iterations_per_100_steps"] = [
                float(np.mean([st["iterations"] for st in a.stats[k:k + 100]])) for k in range(nt, total, 100)]
            if a not in (bo, b1):
                d["final_training_loss"] = a.sol.learned_status()["last_loss"]
        out[a.name] = d
    out["network_gain_over_extrapolation_only"] = {
        base: {ph: out[net][ph]["value"] / out[ext][ph]["value"] for ph in ("protocol", "used_phase")}
        for base, net, ext in (("cubic_base", "learned", "extrapolation_only"),
                               ("linear_base", "learned_linear_base", "extrapolation_only_linear"))}
    base = out["fp64"]
    for a in arms[1:]:
        out[a.name]["speedup_vs_fp64"] = {
            ph: out[a.name][ph]["value"] / base[ph]["value"] for ph in ("protocol", "training_phase", "used_phase")}
    out["learned_mixed"]["speedup_vs_mixed"] = {
        ph: out["learned_mixed"][ph]["value"] / out["mixed"][ph]["value"] for ph in ("protocol", "used_phase")}
    for a in arms + [exact]:
        a.close()
    return out


def profile_other_form(args, dev):
    """Warm-up + timed steps of the mixed or learned form, of the FP64 form on
    (2 grid)^3 cuboids ("box"), with GMRES ("gmres"), or on the 128^2
    heat-equation workload ("heat2d"), only (for ncu launch lists)."""
    import torch

    from mhfem import _lib as L
    from mhfem import problems

    if args.profile_form == "mixed":
        p = problems.diffusion3d(N=args.grid, form=L.FORM_MIXED)
    elif args.profile_form == "box":
        p = problems.diffusion3d_box(N=2 * args.grid)
    elif args.profile_form == "gmres":
        p = problems.diffusion3d(N=args.grid)
    elif args.profile_form == "heat2d":
        p = problems.heat2d(N=128)
    else:
        p = problems.diffusion3d_source(N=args.grid, steps=1000, form=L.FORM_LEARNED)
    p.config.device = dev
    s = problems.make_solver(p, check_every=8)
    if args.profile_form == "gmres":
        s.setup(tol=p.tol, max_iter=100000, check_every=8, linear_solver="gmres", gmres_restart=30,
                gmres_variant="cgs")
    t = 0.0
    if args.profile_form == "learned":
        s.learned_options(train_steps=args.learned_train, train_iters=args.learned_iters, learning_rate=3e-3)
        for _ in range(args.learned_train):
            s.step(t, p.dt)
            t += p.dt
    for _ in range(args.warmup):
        s.step(t, p.dt)
        t += p.dt
    it0, _, _ = s.totals()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.step(t, p.dt)
        t += p.dt
    torch.cuda.synchronize()
    it1, _, _ = s.totals()
    print(json.dumps({"profile_run": True, "form": args.profile_form,
                      "ms_per_step": 1e3 * (time.perf_counter() - t0) / args.steps,
                      "iterations_per_step": (it1 - it0) / args.steps}))
    s.close()


def cpu_baseline(p, steps, warmup=1, what=None):
    """The CPU oracle (the restatement of the reference's algorithm, C +
    OpenMP on the threads this process may use) over `steps` time steps after
    `warmup` untimed ones: a bounded sample of the workload."""
    from oracle.oracle import OracleModel, load

    lib = load()
    threads = allowed_cpus()
    lib.orc_set_threads(threads)
    m = OracleModel.from_problem(p)
    t = 0.0
    for _ in range(warmup):
        m.step(t, p.dt, p.tol)
        t += p.dt
    t0 = time.perf_counter()
    for _ in range(steps):
        m.step(t, p.dt, p.tol)
        t += p.dt
    el = time.perf_counter() - t0
    what = what or f"{steps} time steps of the same workload after {warmup} warm-up step(s)"
    return {"value": steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{what} (CPU restatement of the reference algorithm, C + OpenMP, -O3 as the reference's "
                      "release build, FP64, same tolerance)"}


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        return

    import numpy as np
    import torch

    from mhfem import _lib as L
    from mhfem import problems

    torch.cuda.set_device(local)
    dev = local
    if args.profile_run and args.profile_form != "fp64":
        profile_other_form(args, dev)
        return
    p = problems.diffusion3d(N=args.grid)
    p.config.device = dev
    s = problems.make_solver(p, check_every=8)
    ext = torch.cuda.ExternalStream(s.stream(), device=dev)
    n, nf, S = p.n, 4, 14
    C, F, V = s.C, s.F, s.V
    rows = n * F
    W = (2 * nf - 1) * n - 1

    t = 0.0
    for _ in range(args.warmup):
        s.step(t, p.dt)
        t += p.dt
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    it0, _, kl0 = s.totals()
    clocks = ClockSampler(dev)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    stats = []
    torch.cuda.synchronize()
    ev0.record(ext)
    for _ in range(args.steps):
        stats.append(s.step(t, p.dt))
        t += p.dt
    ev1.record(ext)
    ev1.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    el_ms = ev0.elapsed_time(ev1)
    it1, _, kl1 = s.totals()
    el_ms = max_over_ranks(el_ms, world)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    iters = (it1 - it0) / args.steps
    if args.profile_run:
        if rank == 0:
            print(json.dumps({"profile_run": True, "ms_per_step": el_ms / args.steps, "iterations_per_step": iters}))
        s.close()
        return
    ms_step = el_ms / args.steps
    value = replicas_value(args.steps, world, el_ms)
    bytes_step = step_bytes(n, nf, S, C, F, V, W, iters)

    # the iteration kernels, each timed alone; the roofline names the one with the largest share
    hbm_peak, peak_kind = measured_peaks()
    iteration, iter_kernel_ms = iteration_table(s, L, hbm_peak)
    top = max(iteration, key=lambda k: iteration[k]["share_of_iteration"])
    # the two SpMVs take nearly equal shares (the launch list ranks them within
    # 0.1%): the roofline carries the other one beside the leader
    other = "spmv_dot" if top == "spmv_dots2" else "spmv_dots2"
    kernels = kernel_table(s, L, hbm_peak)
    traffic, traffic_src = ncu_traffic(top, args.grid)
    traffic_o, _ = ncu_traffic(other, args.grid)
    gpu_launches = kl1 - kl0

    forms = {}
    if not args.no_mixed:
        forms["mixed"] = mixed_leg(args, dev, world, el_ms)
    if not args.no_gmres:
        forms["fp64_gmres"] = gmres_leg(args, dev, world)
    other_cells = None
    if not args.no_box:
        other_cells = {"cuboids": box_leg(args, dev, world)}
    configs = {}
    wanted = [c for c in args.configs.split(",") if c and c != "none"]
    for name, leg in (("heat2d", heat2d_leg), ("adr2d", adr2d_leg), ("mixed128", mixed128_leg)):
        if name in wanted:
            configs[name] = leg(args, dev, world)
    if not args.no_learned:
        forms["learned_protocol"] = learned_protocol_leg(args, dev, world)

    e2e = None
    if not args.no_e2e:
        # the same warm-up and timed steps, on a fresh solver, through the public C ABI with host buffers
        import ctypes as ct
        pe = problems.diffusion3d(N=args.grid)
        pe.config.device = dev
        se = problems.make_solver(pe, check_every=8)
        f_host = torch.ones(C, dtype=torch.float64).pin_memory().numpy()
        zk_host = torch.empty(C, dtype=torch.float64).pin_memory().numpy()
        zk_ptr = zk_host.ctypes.data_as(ct.POINTER(ct.c_double))
        te = 0.0
        for _ in range(args.warmup):
            se.step(te, pe.dt, stats=False)
            te += pe.dt
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            se.set_coeff("f", f_host)                         # host -> device: this step's source field
            se.step(te, pe.dt, stats=False)
            se._ck(se.lib.mhfem_get_state(se._h, None, zk_ptr))  # device -> host: Z_iK
            te += pe.dt
        torch.cuda.synchronize()
        e_el = time.perf_counter() - t0
        se.close()
        e_el = max_over_ranks(e_el, world)
        e2e = {"value": world * args.steps / e_el, "unit": UNIT, "h2d_bytes_per_step": 8 * C,
               "d2h_bytes_per_step": 8 * C, "path": "mhfem_set_coeff + mhfem_step + mhfem_get_state (ctypes)",
               "steps": "the same warm-up and timed steps as `value`, on a fresh solver"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(problems.diffusion3d(N=args.grid), args.cpu_steps, warmup=1,
                           what=f"{args.cpu_steps} time steps of the same {args.grid}^3 workload after 1 warm-up step")

    s.close()
    if rank != 0:
        return
    tk = iteration[top]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic: seeded jittered {args.grid}^3 cube grid split into 6 tetrahedra, D = exp(Gaussian field)",
        "form": "fp64", "parallelism": "replicas" if world > 1 else "single GPU",
        "config": workload_config(args.grid, C, F, rows, p.tol, p.dt, n, nf),
        "face_dof_per_s": value * F * n, "iterations_per_step": iters,
        "hbm_gbs_step": bytes_step / (ms_step * 1e-3) / 1e9,
        "hbm_frac_step": bytes_step / (ms_step * 1e-3) / 1e9 / hbm_peak,
        "roofline": {"bound": "hbm", "kernel": tk["kernel"], "achieved": tk["gbs"], "peak": hbm_peak, "unit": "GB/s",
                     "frac": tk["hbm_frac"], "traffic": traffic, "traffic_source": traffic_src,
                     "peak_kind": peak_kind, "bytes_per_launch": tk["bytes"], "ms_per_launch": tk["ms"],
                     "share_of_iteration": tk["share_of_iteration"],
                     "selection": "largest share of the FP64 BiCGStab iteration's kernel time (each kernel timed "
                                  "alone with CUDA events on the library's stream)",
                     "other_spmv": {"kernel": iteration[other]["kernel"], "achieved": iteration[other]["gbs"],
                                    "frac": iteration[other]["hbm_frac"], "traffic": traffic_o,
                                    "bytes_per_launch": iteration[other]["bytes"],
                                    "ms_per_launch": iteration[other]["ms"],
                                    "share_of_iteration": iteration[other]["share_of_iteration"]}},
        "iteration_kernels": iteration,
        "iteration_kernel_ms": iter_kernel_ms,
        "iteration_ms_in_step": ms_step / max(iters, 1),
        "kernels": kernels,
        "forms": forms,
        "other_cells": other_cells,
        "other_configs": configs,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": gpu_launches,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def ncu_traffic(kernel_name, grid):
    """DRAM bytes per launch of a kernel from the committed ncu summary of the
    iteration kernels (`traffic <name> <bytes> <commit>` lines; captured on
    the 64^3 workload), with the file and commit it came from."""
    f = REPO / "profiles" / "iteration_kernels_fp64_diffusion3d64.txt"
    if grid != 64 or not f.exists():
        return None, None
    for line in f.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 4 and parts[0] == "traffic" and parts[1] == kernel_name:
            try:
                return float(parts[2]), f"profiles/{f.name}, ncu capture of commit {parts[3]}"
            except ValueError:
                return None, None
    return None, None


if __name__ == "__main__":
    main()
