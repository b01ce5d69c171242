"""Benchmark of the projection step on one GB300: cell-updates per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload cavity512|cavity2048|batched256|serving] [--precision mixed|fp64]

Workloads (zero initial fields, unit square, CFL target 0.5 / growth 1.05,
QUICK advection, Jacobi preconditioner, pressure tolerance 1e-8; seeded
synthetic draws stand in for any dataset):

* ``cavity512`` (default): one 512 x 512 cavity, Re 1000, lid 1.0.  A step is
  one projection step.  Default precision ``mixed``: binary32
  multigrid-preconditioned CG (rel tol 1e-5) inside a binary64 refinement of
  the pressure solve to 1e-8, everything else binary64.  The same run also
  times the plain binary64 path (the reference's algorithm, CG with
  lin_maxiter 300) on the same cavity: ``plain_fp64`` and the ratio
  ``speedup_vs_plain_fp64``.
* ``cavity2048``: one 2048 x 2048 cavity, Re 3200, lid 1.0 (both precisions).
* ``batched256``: 256 cavities from seed 0 (nx, ny in {32..128}, Re
  log-uniform in [100, 5000], lid uniform in [0.5, 2]) advanced together: a
  step advances every instance once (one graph launch).
* ``serving``: the Poisson request trace (200 req/s for 60 s, seed 1) served
  by continuous batching; reports latency percentiles beside throughput.

Line contents:
* ``value``: cell-updates/s with the state resident in HBM, K steps timed
  with CUDA events on the launching stream after W warm-up steps (K defaults
  to the workload's own step count: 2000 for the 512^2 cavity, 1000 for
  2048^2, 500 for the batch); L2 (129 MB) is flushed by a 256 MiB write
  between timed steps, outside the timed intervals.
* ``e2e``: the same metric through the public API with the fields in host
  memory: every step copies u, v, p host->device and back inside the timed
  (wall-clock) region.
* ``roofline``: the pressure matvec (``k_mx_matvec`` in the mixed form,
  ``k_cg_matvec`` in the binary64 form), timed per launch with CUDA events
  during one more step (4 words per cell: read z or r, p_old; write p_new, q).
* ``cpu_baseline``: the oracle port (NumPy restatement of the reference with
  its own reductions and CG sequence) on a bounded sample of the workload.
* ``--impl reference``: that CPU port timed as the reference arm.
With torchrun (N > 1) every rank runs an independent replica (a cavity does
not shard; replicas only): value = all cells updated / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

CAVITIES = {
    "cavity512": dict(n=512, Re=1000.0, lid=1.0, maxiter=300, steps=2000),
    "cavity2048": dict(n=2048, Re=3200.0, lid=1.0, maxiter=300, steps=1000),
}
BATCH_STEPS = 500                 # steps of each batched instance
L2_FLUSH_BYTES = 256 * 1024 * 1024
PRECISION_NOTE = {
    "mixed": "binary32 multigrid-PCG inner solves (rel tol 1e-5; every pass also stops a quarter below the outer "
             "target, and the first pass of an instance whose first passes have been reaching the outer target "
             "aims there, down to rel 3e-7) inside binary64 refinement to rel 1e-8, warm-started from the previous "
             "pressure; predictor, correction, pressure residual and all norms binary64",
    "fp64": "binary64 plain path (the reference's Jacobi-PCG, lin_maxiter 300, exactly rounded reductions)",
}


def cavity_cfg(name, precision):
    from pyflow_solver_gb300.workloads import cavity_config
    c = CAVITIES[name]
    return cavity_config(c["n"], c["n"], c["Re"], c["lid"], precision, lin_tol=1e-8, lin_maxiter=c["maxiter"])


def describe(name):
    c = CAVITIES[name]
    return (f"lid-driven cavity {c['n']}x{c['n']}, Re={c['Re']:g}, lid {c['lid']:g}, unit square, QUICK, "
            f"pressure rel tol 1e-8")


def dist_env():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


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
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            # the timed region starts once the sampler is producing (nvidia-smi takes a moment to start)
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 5.0:
                time.sleep(0.01)
            self.first = len(self.lines)
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
        # the samples taken while the timed work ran (plus the one just before it)
        lines = self.lines[max(0, getattr(self, "first", 1) - 1):]
        for ln in lines:
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


# ---- kernel-launch accounting ------------------------------------------------

def mg_levels(nx, ny, dx=None, dy=None):
    """Global multigrid levels of the mixed solve (the last one is the coarse CTA's):
    halve both axes, or only the strongly coupled one, while above 4096 cells."""
    import numpy as np
    dx = 1.0 / max(nx - 1, 1) if dx is None else dx
    dy = 1.0 / max(ny - 1, 1) if dy is None else dy
    cx, cy = float(np.float32(1.0 / (dx * dx))), float(np.float32(1.0 / (dy * dy)))
    n, lx, ly = 1, nx, ny
    while n < 16 and lx * ly > 4096:
        fx, fy = lx % 2 == 0 and lx // 2 >= 8, ly % 2 == 0 and ly // 2 >= 8
        px, py = (2, 1) if cx > 2 * cy else ((1, 2) if cy > 2 * cx else (2, 2))
        if not ((px == 1 or fx) and (py == 1 or fy)):
            px, py = (2, 2) if (fx and fy) else ((2, 1) if fx else ((1, 2) if fy else (0, 0)))
        if px == 0:
            break
        lx, ly = lx // px, ly // py
        cx, cy = cx * py / px, cy * px / py
        n += 1
    return n


def series_summary(xs):
    """A per-step series as its mean, range and first and last ten entries."""
    if not xs:
        return {}
    return {"mean": sum(xs) / len(xs), "min": min(xs), "max": max(xs), "first": list(xs[:10]), "last": list(xs[-10:])}


def launches_per_step(precision, cg_iters, passes, nlev, persistent=True):
    """Kernel launches of one step from its loop trip counts."""
    if precision == "fp64":
        return 11 + 3 * cg_iters
    if persistent:                    # prestep, predictor, RHS, loop reset, the solve, correction, diagnostics
        return 7
    v = 2 * nlev - 1                  # a V-cycle: down-sweeps, the coarse CTA, up-sweeps
    # an iteration: the V-cycle after level 0's down-sweep (which the update before it
    # fuses), the matvec and the update; a pass: loop reset, prep, level 0's first
    # down-sweep, loop arm, correction, residual (the loop guards run in the last CTA
    # of the update and of the residual kernels)
    per_iter = (v - 1 if nlev >= 2 else v) + 2
    per_pass = 5 + (1 if nlev >= 2 else 0)
    # a step: prestep (with dt), predictor, RHS, loop reset, init, loop arm, correction,
    # diagnostics (with the solve summary and the step record)
    return 8 + passes * per_pass + cg_iters * per_iter


# ---- CPU arm -----------------------------------------------------------------

def cpu_port_rate(name, steps):
    """cell-updates/s of the oracle port (reference reductions, scipy CG sequence), one thread."""
    from oracle import step as ost
    cfg = cavity_cfg(name, "fp64")
    n = CAVITIES[name]["n"]
    st = ost.allocate_state(n, n)
    tr = ost.ResidualManager()
    ost.step(cfg, st, tr, 0, red="numpy")              # step 0: zero RHS, not timed
    t0 = time.perf_counter()
    for it in range(1, steps + 1):
        ost.step(cfg, st, tr, it, red="numpy")
    dt = time.perf_counter() - t0
    return n * n * steps / dt, dt


def _port_instance(args):
    nx, ny, Re, U, steps = args
    from oracle import step as ost
    from pyflow_solver_gb300.workloads import cavity_config
    cfg = cavity_config(nx, ny, Re, U, "fp64")
    st = ost.allocate_state(nx, ny)
    tr = ost.ResidualManager()
    for it in range(steps):
        ost.step(cfg, st, tr, it, red="numpy")
    return nx * ny * steps


def cpu_port_batched_rate(n_inst, steps, procs):
    """The oracle port over the batched instances, one process per host core."""
    import multiprocessing as mp

    from pyflow_solver_gb300.workloads import batched_instances
    work = [(nx, ny, Re, U, steps) for nx, ny, Re, U in batched_instances(256, 0)[:n_inst]]
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        pool.map(_port_instance, work[:procs])           # start-up, not timed
        t0 = time.perf_counter()
        cells = sum(pool.map(_port_instance, work))
        dt = time.perf_counter() - t0
    return cells / dt, dt


def run_reference_arm(args):
    _, rank, _ = dist_env()
    if rank != 0:
        return
    wl = args.workload
    if wl in CAVITIES:
        steps = max(1, min(args.steps, 6 if wl == "cavity512" else 1))
        v, dt = cpu_port_rate(wl, steps)
        cores = 1
        sample = (f"steps 1..{steps} after an untimed step 0 of the same {CAVITIES[wl]['n']}^2 cavity "
                  "(oracle port: NumPy restatement with the reference's np.dot/np.mean reductions and "
                  "scipy's CG sequence; one thread)")
        cfg = {"workload": describe(wl)}
    else:
        cores = os.cpu_count() or 1
        n_inst = min(256, 4 * cores)
        v, dt = cpu_port_batched_rate(n_inst, 5, cores)
        sample = f"5 steps of each of the first {n_inst} batched instances, one process per core"
        cfg = {"workload": "256 batched cavities, seed 0" if wl == "batched256" else "serving trace mix"}
    line = {
        "impl": "reference", "metric": "cell-updates/s", "value": v, "unit": "cell-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * CAVITIES[wl]["n"] ** 2 / v if wl in CAVITIES else None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": cfg,
        "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": cores, "kind": "port", "sample": sample,
                         "seconds": dt},
        "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---- GPU arm -------------------------------------------------------------------

def timed_steps(fn, steps, stream, flush, dist):
    """CUDA-event time of each call of fn (L2 flushed before each, outside the interval)."""
    import torch
    ms, outs = [], []
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(steps):
        flush.fill_(float(k))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        outs.append(fn())
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    return ms, outs


def pct(ms):
    """p50/p95/p99 of per-step times (ms)."""
    v = sorted(ms)
    pick = lambda q: v[min(len(v) - 1, int(q * (len(v) - 1) + 0.5))]  # noqa: E731
    return {"p50": pick(0.50), "p95": pick(0.95), "p99": pick(0.99)} if v else None


def max_over_ranks(x, dist):
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the roofline
# kernel, from the ncu captures summarised in profiles/ (two launches each, averaged).
TRAFFIC = {
    ("cavity512", "mixed::k_mx_matvec"): 1.60e6,
    ("cavity2048", "mixed::k_mx_matvec"): 34.11e6,
    ("cavity2048", "mixed::k_mx_matvec_tma"): 33.74e6,
    ("cavity2048", "pfgb::k_cg_matvec"): 94.64e6,
    ("cavity512", "pfgb::k_cg_matvec"): 4.27e6,
}


def mixed_solve_bytes(cells, inner, passes):
    """Compulsory bytes of one persistent mixed solve (binary32 levels, binary64 refinement):
    per inner iteration 16 (matvec) + 24 (update) + 22 (level-0 down- and up-sweep) + 7
    (coarser levels) bytes per cell; per refinement pass 16 (prep) + 29 (its V-cycle) + 20
    (correction) + 24 (binary64 residual); 32 for the start (mean removal, x = 0, r = b)."""
    return cells * (32 + 89 * passes + 69 * inner)


def kernel_roofline(lib, cfg, st, tr, it, cells, precision, workload=None):
    """Live CUDA-event timing of the dominant kernel during one more step: the
    persistent solve (mixed) or the CG matvec (binary64)."""
    import ctypes

    import torch

    from pyflow_solver_gb300 import _capi, step
    from pyflow_solver_gb300.solvers._handle import instance_for
    from pyflow_solver_gb300.solvers.solver import step_params
    P, *_ = step_params(cfg, st.nx, st.ny)
    inst = instance_for(st, P)
    hbm, src = peaks()
    _capi.check(lib.pfgb_set_profiling(inst.handle, 1), "set_profiling")
    _, _, diag = step(cfg, st, tr, it)
    ms, n = ctypes.c_double(), ctypes.c_int()
    _capi.check(lib.pfgb_profile_result(inst.handle, ctypes.byref(ms), ctypes.byref(n)), "profile_result")
    _capi.check(lib.pfgb_set_profiling(inst.handle, 0), "set_profiling")
    torch.cuda.synchronize()
    per_launch_s = ms.value / 1e3 / max(n.value, 1)
    from pyflow_solver_gb300.solvers import _handle
    if precision == "mixed" and _handle.PERSISTENT:
        nbytes = mixed_solve_bytes(cells, diag["cg_iterations"], diag.get("refine_passes", 0))
        kern, model = "mixed::k_mx_persist", "mixed_solve_bytes (bench.py)"
    elif precision == "mixed":
        nbytes = 4 * 4 * cells
        tma = ctypes.c_int()
        _capi.check(lib.pfgb_matvec_form(inst.handle, ctypes.byref(tma)), "matvec_form")
        kern = "mixed::k_mx_matvec_tma" if tma.value else "mixed::k_mx_matvec"
        model = "4 binary32 words per cell"
    else:
        nbytes = 4 * 8 * cells
        kern, model = "pfgb::k_cg_matvec", "4 binary64 words per cell"
    achieved = nbytes / per_launch_s / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": TRAFFIC.get((workload, kern)), "kernel": kern, "peak_source": f"{src} (copy bandwidth)",
            "launches_timed": n.value, "per_launch_us": per_launch_s * 1e6,
            "algorithmic_bytes_per_launch": nbytes, "bytes_model": model}


def e2e_cavity(cfg, n, steps, warmup=2):
    """Through the public step() on a State whose fields are host NumPy arrays: `warmup`
    untimed steps, then `steps` timed ones (the same step range as the device-timed run)."""
    import numpy as np

    from pyflow_solver_gb300 import ResidualManager
    from pyflow_solver_gb300.core.ghost_fields import State
    from pyflow_solver_gb300.solvers.solver import step
    if steps <= 0:
        return None
    host = State(n, n, {k: np.zeros((n + 2, n + 2)) for k in "uvp"})
    tr = ResidualManager()
    for it in range(warmup):
        step(cfg, host, tr, it)
    t0 = time.perf_counter()
    for it in range(warmup, warmup + steps):
        step(cfg, host, tr, it)
    dt = time.perf_counter() - t0
    nbytes = 3 * (n + 2) ** 2 * 8
    return {"value": n * n * steps / dt, "unit": "cell-updates/s", "h2d_bytes_per_step": nbytes,
            "d2h_bytes_per_step": nbytes, "steps": steps}


def bench_cavity(args, dist, world, rank, local):
    import torch

    from pyflow_solver_gb300 import ResidualManager, _capi, allocate_state, step
    lib = _capi.load()
    wl = args.workload
    n = CAVITIES[wl]["n"]
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def run(precision, steps, warmup):
        cfg = cavity_cfg(wl, precision)
        st = allocate_state(n, n)
        tr = ResidualManager()
        box = {"it": 0}

        def one():
            r = step(cfg, st, tr, box["it"])
            box["it"] += 1
            return r[2]
        for _ in range(warmup):
            one()
        ms, diags = timed_steps(one, steps, stream, flush, dist)
        return cfg, st, tr, box["it"], ms, diags

    with ClockSampler(local) as clocks:
        cfg, st, tr, it, ms, diags = run(args.precision, args.steps, args.warmup)
    total = max_over_ranks(sum(ms), dist)
    value = n * n * args.steps * world / (total / 1e3)
    cg = [d["cg_iterations"] for d in diags]
    passes = [d.get("refine_passes", 0) for d in diags]
    nlev = mg_levels(n, n)
    launches = sum(launches_per_step(args.precision, c, p, nlev, args.persistent) for c, p in zip(cg, passes))
    roof = None if args.no_roofline else kernel_roofline(lib, cfg, st, tr, it, n * n, args.precision, wl)
    extra = {}
    if args.precision == "mixed" and not args.no_plain:
        _, _, _, _, pms, pd = run("fp64", args.plain_steps, 1)
        ptot = max_over_ranks(sum(pms), dist)
        pval = n * n * args.plain_steps * world / (ptot / 1e3)
        extra["plain_fp64"] = {"value": pval, "unit": "cell-updates/s", "ms_per_step": ptot / args.plain_steps,
                               "steps": args.plain_steps, "cg_iterations_per_step": [d["cg_iterations"] for d in pd]}
        extra["speedup_vs_plain_fp64"] = value / pval
    e2e_steps = args.steps if args.e2e_steps is None else args.e2e_steps
    e2e = e2e_cavity(cfg, n, e2e_steps, args.warmup) if e2e_steps > 0 else None
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        steps = 6 if wl == "cavity512" else 1
        v, dt = cpu_port_rate(wl, steps)
        cpu = {"value": v, "unit": "cell-updates/s", "cores": 1, "kind": "port", "seconds": dt,
               "sample": f"steps 1..{steps} after an untimed step 0 of the same cavity, one thread (oracle port: "
                         "NumPy restatement with the reference's reductions and CG sequence, lin_maxiter 300)"}
    line = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+f32" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": describe(wl), "nx": n, "ny": n, "Re": CAVITIES[wl]["Re"],
                   "precision": PRECISION_NOTE[args.precision],
                   "l2": "flushed between timed steps (256 MiB write)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "timed_steps": f"steps {args.warmup}..{args.warmup + args.steps - 1} of a run from zero fields",
                   "cg_iterations_per_step": series_summary(cg), "refine_passes_per_step": series_summary(passes),
                   "steps_not_converged": sum(1 for d in diags if not d.get("Rp_converged", True))},
        **extra,
        "step_latency_ms": pct(ms),
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": launches, "clocks": clocks.summary(),
    }
    return line


def bench_batched(args, dist, world, rank, local):
    import numpy as np
    import torch

    from pyflow_solver_gb300.batch import BatchedCavities
    from pyflow_solver_gb300.core.ghost_fields import State
    from pyflow_solver_gb300.workloads import batched_instances, cavity_config
    inst = batched_instances(256, 0)
    # one device arena for all fields (and its pinned host mirror for the end-to-end run)
    sizes = [3 * (ny + 2) * (nx + 2) for nx, ny, _, _ in inst]
    arena = torch.zeros(sum(sizes), dtype=torch.float64, device="cuda")
    states, off = [], 0
    for (nx, ny, _, _), sz in zip(inst, sizes):
        f = arena[off:off + sz].view(3, ny + 2, nx + 2)
        states.append(State(nx, ny, {"u": f[0], "v": f[1], "p": f[2]}))
        off += sz
    cfgs = [cavity_config(nx, ny, Re, U, args.precision) for nx, ny, Re, U in inst]
    B = BatchedCavities(cfgs, states)
    cells = int(B.cells.sum())
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        B.step_arrays()
    with ClockSampler(local) as clocks:
        ms, outs = timed_steps(B.step_arrays, args.steps, stream, flush, dist)
    total = max_over_ranks(sum(ms), dist)
    value = cells * args.steps * world / (total / 1e3)
    maxit = [int(o["cg_iterations"].max()) for o in outs]
    maxpass = [int(o["refine_passes"].max()) for o in outs]
    nlev = max(mg_levels(nx, ny) for nx, ny, _, _ in inst)
    launches = sum(launches_per_step(args.precision, c, p, nlev, args.persistent) for c, p in zip(maxit, maxpass))
    # end to end: the fields of all instances copied in (pinned host -> device) and out every step
    host = torch.empty(arena.numel(), dtype=torch.float64, pin_memory=True)
    host.copy_(arena)
    e2e_steps = max(1, args.steps if args.e2e_steps is None else args.e2e_steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        arena.copy_(host, non_blocking=True)
        B.step_arrays()
        host.copy_(arena, non_blocking=True)
        torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    nbytes = arena.numel() * 8
    e2e = {"value": cells * e2e_steps / dt, "unit": "cell-updates/s", "h2d_bytes_per_step": nbytes,
           "d2h_bytes_per_step": nbytes, "steps": e2e_steps}
    line = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+f32" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": "256 lid-driven cavities from seed 0: nx, ny in {32,48,64,96,128}, Re log-uniform "
                               "[100,5000], lid uniform [0.5,2]; one graph launch per step for all instances",
                   "instances": len(inst), "cells_per_step": cells, "precision": PRECISION_NOTE[args.precision],
                   "l2": "flushed between timed steps (256 MiB write)",
                   "max_cg_iterations_per_step": series_summary(maxit),
                   "max_refine_passes_per_step": series_summary(maxpass),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "step_latency_ms": pct(ms),
        "roofline": None, "cpu_baseline": None, "e2e": e2e, "gpu_launches": launches,
        "gpu_launches_note": "from the largest loop trip counts of each step", "clocks": clocks.summary(),
    }
    B.close()
    return line


def bench_serving(args, dist, world, rank, local):
    import torch

    from pyflow_solver_gb300.serving import ServingEngine
    from pyflow_solver_gb300.workloads import SIDES_SERVE, serving_trace
    trace = serving_trace(200.0, args.serve_seconds, 1)
    # slots in proportion to each side's share of the offered cell-updates, within the memory budget
    slots = {32: 96, 64: 96, 128: 64, 256: 32, 512: 8, 1024: 4}
    eng = ServingEngine({s: slots[s] for s in SIDES_SERVE}, precision=args.precision,
                        memory_budget_bytes=60e9)
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        rep = eng.run(trace, max_wall=args.serve_seconds * 1.5)
    pct = rep.latency_percentiles()
    line = {
        "metric": "cell-updates/s", "value": rep.cell_updates / rep.wall_s, "unit": "cell-updates/s",
        "n_gpus": world, "steps": rep.engine_steps, "warmup": 0, "ms_per_step": 1e3 * rep.wall_s / max(1, rep.engine_steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+f32" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": f"Poisson arrivals 200 req/s for {args.serve_seconds:g} s, seed 1; sides "
                               "{32..1024}, Re log-uniform [100,3200], lid [0.5,2], 100-2000 steps, continuity "
                               "tol 1e-6, 60 GB device budget", "slots": slots, "device_bytes": rep.device_bytes,
                   "requests": len(trace), "completed": len(rep.completed), "in_flight_at_end": rep.in_flight,
                   "queued_at_end": rep.queued, "wall_s": rep.wall_s},
        "latency_s": pct,
        "roofline": None, "cpu_baseline": None,
        "e2e": {"value": rep.cell_updates / rep.wall_s, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0, "note": "wall clock of the request loop; state resident on the device"},
        "gpu_launches": None, "clocks": clocks.summary(),
    }
    eng.close()
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: the workload's own step count, 2000 / 1000 / 500)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--workload", default="cavity512", choices=["cavity512", "cavity2048", "batched256", "serving"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-roofline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain binary64 comparison run")
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=None,
                    help="timed steps of the end-to-end run (default: --steps; 0 skips it)")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--no-graph", action="store_true", help="individual launches instead of one graph per step")
    ap.add_argument("--persistent", action="store_true",
                    help="mixed form: the pressure solve as one persistent cooperative launch, not a kernel graph")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = CAVITIES[args.workload]["steps"] if args.workload in CAVITIES else BATCH_STEPS
    if args.impl == "reference":
        run_reference_arm(args)
        return
    args.warmup = max(args.warmup, 3)

    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from pyflow_solver_gb300.solvers import _handle
    _handle.GRAPH_MODE = not args.no_graph
    _handle.PERSISTENT = args.persistent
    if args.workload in CAVITIES:
        line = bench_cavity(args, dist, world, rank, local)
    elif args.workload == "batched256":
        line = bench_batched(args, dist, world, rank, local)
    else:
        line = bench_serving(args, dist, world, rank, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
