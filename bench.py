"""Benchmark of the projection step: cell-updates per second on one GB300.

Workload (the single-cavity configuration the headline metric is quoted on):
a 512 x 512 lid-driven cavity on the unit square, Re = 1000, lid velocity 1.0,
zero initial fields, QUICK advection, CFL target 0.5 / growth 1.05, pressure
CG with rtol 1e-8 and lin_maxiter 300, Jacobi preconditioner.  A step is one
full projection step (predictor, pressure PCG, correction, reductions).  The
arithmetic is binary64 throughout (the plain path).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

* ``value``: cell-updates/s with the state resident in HBM, K steps timed with
  CUDA events on the launching stream; L2 is flushed (a 256 MiB write) between
  timed steps, outside the timed intervals.
* ``e2e``: the same metric through the public API (``step`` on a State whose
  fields are host NumPy arrays): every step copies u, v, p host->device and
  back, inside the timed region (wall clock).
* ``roofline``: the dominant kernel (k_cg_matvec: p = z + beta p; q = A p; p.q)
  timed per launch with CUDA events; algorithmic bytes per launch = 4 words
  (read r, p_old; write p_new, q) x 8 B x cells.
* ``cpu_baseline``: the oracle port (NumPy restatement with the reference's own
  reductions) on a bounded sample of the same workload, on this host.
* ``--impl reference``: the oracle port timed as the reference arm.
With torchrun (N > 1) every rank runs an independent replica (a single cavity
does not shard): value = all cells updated / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NX = NY = 512
RE = 1000.0
MAXITER = 300
WORKLOAD = "lid-driven cavity 512x512, Re=1000, lid 1.0, unit square, QUICK, CG rtol 1e-8 maxiter 300, Jacobi"


def make_cfg(precision="fp64"):
    from types import SimpleNamespace
    return SimpleNamespace(nx=NX, ny=NY, lx=1.0, ly=1.0, Re=RE, lid_velocity=1.0, advection_scheme="quick",
                           cfl_target=0.5, cfl_growth=1.05, lin_tol=1e-8, lin_maxiter=MAXITER,
                           enable_jacobi_pc=True, diagnostics=False, precision=precision)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, flag in zip(names, parts[3:7]):
                if flag.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_oracle_rate(steps: int, threads_note: int):
    """cell-updates/s of the oracle port (reference reductions) on a bounded sample."""
    from oracle import step as ost
    cfg = make_cfg()
    st = ost.allocate_state(NX, NY)
    tr = ost.ResidualManager()
    ost.step(cfg, st, tr, 0, red="numpy")              # step 0: zero RHS, not timed
    t0 = time.perf_counter()
    for it in range(1, steps + 1):
        ost.step(cfg, st, tr, it, red="numpy")
    dt = time.perf_counter() - t0
    return NX * NY * steps / dt, {"steps_timed": steps, "seconds": dt, "threads": threads_note}


def run_reference_arm(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup if args.warmup < 1 else 1):
        pass
    steps = max(1, min(args.steps, 6))
    v, info = cpu_oracle_rate(steps, cores)
    vals.append(v)
    line = {
        "impl": "reference", "metric": "cell-updates/s", "value": v, "unit": "cell-updates/s",
        "n_gpus": args.gpus, "steps": steps, "warmup": 1, "ms_per_step": 1e3 * NX * NY / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "nx": NX, "ny": NY, "Re": RE, "lin_maxiter": MAXITER},
        "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": cores, "kind": "port",
                         "sample": f"steps 1..{steps} after an untimed step 0 of the same 512x512 cavity "
                                   "(oracle port: NumPy restatement with the reference's np.dot/np.mean "
                                   "reductions and scipy's CG sequence)"},
        "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--no-roofline", action="store_true")
    ap.add_argument("--no-graph", action="store_true", help="individual launches instead of one graph per step")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference_arm(args)
        return
    if args.warmup < 3:
        args.warmup = 3

    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from pyflow_solver_gb300 import ResidualManager, allocate_state, step
    from pyflow_solver_gb300 import _capi
    from pyflow_solver_gb300.solvers import _handle
    _handle.GRAPH_MODE = not args.no_graph
    lib = _capi.load()

    cfg = make_cfg(args.precision)
    st = allocate_state(NX, NY)
    tr = ResidualManager()
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    it = 0
    for _ in range(args.warmup):
        step(cfg, st, tr, it)
        it += 1
    # timed steps: events around each step, L2 flushed in between (outside the intervals)
    step_ms = []
    cg_iters = []
    passes = []
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.fill_(float(it))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _, res, diag = step(cfg, st, tr, it)
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            cg_iters.append(diag["cg_iterations"])
            passes.append(diag.get("refine_passes"))
            it += 1
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    total_ms = sum(step_ms)
    if dist is not None:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    cells = NX * NY * args.steps * world
    value = cells / (total_ms / 1e3)

    # roofline of the dominant kernel: per-launch CUDA-event timing of k_cg_matvec
    roof = None if (args.no_roofline or args.precision == "mixed") else kernel_roofline(lib, st, cfg, it, tr)
    it += 1

    # end to end through the public API with host buffers
    e2e = e2e_rate(cfg, args.e2e_steps) if args.e2e_steps > 0 else None

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            v, info = cpu_oracle_rate(6, 1)
            cpu = {"value": v, "unit": "cell-updates/s", "cores": 1, "kind": "port",
                   "sample": "steps 1..6 after an untimed step 0 of the same 512x512 cavity, one thread "
                             "(oracle port: NumPy restatement with the reference's reductions)"}
        launches_per_step = 9 + 2 * MAXITER
        line = {
            "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "nx": NX, "ny": NY, "Re": RE, "lin_maxiter": MAXITER,
                       "precision": "binary64 plain path (exactly rounded reductions)",
                       "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "cg_iterations_per_step": cg_iters, "refine_passes_per_step": passes},
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def kernel_roofline(lib, st, cfg, it, tr):
    """Per-launch CUDA-event timing of k_cg_matvec during one more step of the same run."""
    import ctypes

    import torch

    from pyflow_solver_gb300 import _capi, step
    from pyflow_solver_gb300.solvers._handle import instance_for
    from pyflow_solver_gb300.solvers.solver import step_params
    P, *_ = step_params(cfg, NX, NY)
    inst = instance_for(st, P)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    src = "measured" if "hbm_gbs" in peaks else "fallback"
    _capi.check(lib.pfgb_set_profiling(inst.handle, 1), "set_profiling")
    step(cfg, st, tr, it)
    ms = ctypes.c_double()
    n = ctypes.c_int()
    _capi.check(lib.pfgb_profile_result(inst.handle, ctypes.byref(ms), ctypes.byref(n)), "profile_result")
    _capi.check(lib.pfgb_set_profiling(inst.handle, 0), "set_profiling")
    tops = ctypes.c_double()
    _capi.check(lib.pfgb_probe_fp64(torch.cuda.current_stream().cuda_stream, ctypes.byref(tops)), "probe_fp64")
    per_launch_s = ms.value / 1e3 / max(n.value, 1)
    bytes_per_launch = 4 * 8 * NX * NY
    achieved = bytes_per_launch / per_launch_s / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": None, "kernel": "k_cg_matvec", "peak_source": src, "launches_timed": n.value,
            "per_launch_us": per_launch_s * 1e6, "algorithmic_bytes_per_launch": bytes_per_launch,
            "fp64_fma_peak_tinst_s": tops.value,
            "note": "binary64 stencil kernel: issue-bound on the FP64 pipe of GB300, not on HBM"}


def e2e_rate(cfg, steps):
    """Through the public step() on a State with host NumPy fields (copies in the timed region)."""
    import numpy as np

    from pyflow_solver_gb300 import ResidualManager
    from pyflow_solver_gb300.core.ghost_fields import State
    from pyflow_solver_gb300.solvers.solver import step
    if steps <= 0:
        return None
    host = State(NX, NY, {k: np.zeros((NY + 2, NX + 2)) for k in "uvp"})
    tr = ResidualManager()
    step(cfg, host, tr, 0)
    step(cfg, host, tr, 1)
    t0 = time.perf_counter()
    for it in range(2, 2 + steps):
        step(cfg, host, tr, it)
    dt = time.perf_counter() - t0
    nbytes = 3 * (NY + 2) * (NX + 2) * 8
    return {"value": NX * NY * steps / dt, "unit": "cell-updates/s", "h2d_bytes_per_step": nbytes,
            "d2h_bytes_per_step": nbytes, "steps": steps}


if __name__ == "__main__":
    main()
