"""Benchmark of the projection step on one GB300: cell-updates per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload batched256|cavity512|cavity2048|serving] [--precision mixed|fp64]

Workloads (zero initial fields, unit square, CFL target 0.5 / growth 1.05,
QUICK advection, Jacobi preconditioner, pressure tolerance 1e-8; seeded
synthetic draws stand in for any dataset):

* ``batched256`` (default): 256 cavities from seed 0 (nx, ny in {32..128}, Re
  log-uniform in [100, 5000], lid uniform in [0.5, 2]) advanced together: a
  step advances every instance once (one graph launch).  Default precision
  ``mixed``: binary32 multigrid-preconditioned CG (rel tol 1e-5) inside a
  binary64 refinement of the pressure solve to 1e-8, everything else binary64.
  The same run times the plain binary64 path (the reference's algorithm, CG
  with lin_maxiter 300) on the same 256 cavities: ``plain_fp64`` and the ratio
  ``speedup_vs_plain_fp64``.
* ``cavity512``: one 512 x 512 cavity, Re 1000, lid 1.0 (with the same plain
  comparison).
* ``cavity2048``: one 2048 x 2048 cavity, Re 3200, lid 1.0 (both precisions).
* ``serving``: the Poisson request trace (200 req/s for 60 s, seed 1) served
  by continuous batching; reports latency percentiles beside throughput.

Line contents:
* ``value``: cell-updates/s with the state resident in HBM, K steps timed
  with CUDA events on the launching stream after W warm-up steps (K defaults
  to the workload's own step count: 500 for the batch, 2000 for the 512^2
  cavity, 1000 for 2048^2); L2 (129 MB) is flushed by a 256 MiB write between
  timed steps, outside the timed intervals.
* ``e2e``: the same metric through the public API with the fields in host
  memory: every step copies u, v, p host->device and back inside the timed
  (wall-clock) region.
* ``kernels`` / ``roofline``: one more step run kernel by kernel with CUDA
  events around every launch: per kernel its launches, device time, share of
  the step, algorithmic bytes per launch (per-cell words of each kernel times
  the cells of its level) and the fraction of the measured HBM copy bandwidth
  that implies.  ``roofline`` is the kernel with the largest share;
  ``step_roofline`` is the whole step's algorithmic bytes over its time.
* ``cpu_baseline``: the oracle port (NumPy restatement of the reference with
  its own reductions and CG sequence) on a bounded sample of the workload.
* ``--impl reference``: that CPU port timed as the reference arm (all host
  cores for the batch, one process per core; one thread for a single cavity).
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


PRECISION_REFERENCE = ("binary64, the reference's algorithm: Jacobi-PCG with lin_maxiter 300 and the reference's "
                       "own NumPy reductions (oracle port)")
L2_NOTE = "GPU arm: L2 flushed between timed steps (256 MiB write)"


def cavity_config_line(name):
    """The `config` of a single-cavity line (the same in both arms)."""
    c = CAVITIES[name]
    return {"workload": describe(name), "nx": c["n"], "ny": c["n"], "Re": c["Re"], "l2": L2_NOTE}


def batch_config():
    """The `config` of a batched line (the same in both arms)."""
    from pyflow_solver_gb300.workloads import batched_instances
    inst = batched_instances(256, 0)
    return {"workload": BATCH_WORKLOAD, "instances": len(inst), "cells_per_step": sum(nx * ny for nx, ny, _, _ in inst),
            "l2": L2_NOTE}


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

def mg_shapes(nx, ny, dx=None, dy=None):
    """Global multigrid levels (nx_l, ny_l) of the mixed solve (the last one is the
    coarse CTA's finest): halve both axes, or only the strongly coupled one, while
    above 4096 cells -- the plan the library builds."""
    import numpy as np
    dx = 1.0 / max(nx - 1, 1) if dx is None else dx
    dy = 1.0 / max(ny - 1, 1) if dy is None else dy
    cx, cy = float(np.float32(1.0 / (dx * dx))), float(np.float32(1.0 / (dy * dy)))
    lx, ly = nx, ny
    out = [(lx, ly)]
    while len(out) < 16 and lx * ly > 4096:
        fx, fy = lx % 2 == 0 and lx // 2 >= 8, ly % 2 == 0 and ly // 2 >= 8
        px, py = (2, 1) if cx > 2 * cy else ((1, 2) if cy > 2 * cx else (2, 2))
        if not ((px == 1 or fx) and (py == 1 or fy)):
            px, py = (2, 2) if (fx and fy) else ((2, 1) if fx else ((1, 2) if fy else (0, 0)))
        if px == 0:
            break
        lx, ly = lx // px, ly // py
        cx, cy = cx * py / px, cy * px / py
        out.append((lx, ly))
    return out


def mg_levels(nx, ny, dx=None, dy=None):
    return len(mg_shapes(nx, ny, dx, dy))


def series_summary(xs):
    """A per-step series as its mean, range and first and last ten entries."""
    if not xs:
        return {}
    return {"mean": sum(xs) / len(xs), "min": min(xs), "max": max(xs), "first": list(xs[:10]), "last": list(xs[-10:])}


def launches_per_step(precision, cg_iters, passes, nlev, persistent=False):
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


# Compulsory DRAM bytes per cell of each kernel at the level it works on (binary64
# words 8 B, binary32 words 4 B): what it must read and write once.
KERNEL_BYTES = {
    # binary64 plain path
    "k_prestep": 16,        # u, v
    "k_predict": 32,        # u, v -> u*, v*
    "k_rhs": 24,            # u*, v* -> b
    "k_cg_init": 40,        # b -> b, r, x, M r
    "k_cg_matvec": 32,      # M r, p_old -> p, q
    "k_cg_update": 56,      # x, p, r, q -> x, r, M r
    "k_post_resid": 16,     # b, x
    "k_pin_correct": 80,    # x, u*, v*, u, v -> u*, v*, u, v, p
    "k_post_diag": 48,      # u*, v*, p, b, u, v
    # mixed form: binary64 stages
    "k_prestep_m": 16,
    "k_predict_m": 32,
    "k_rhs_m": 24,
    "k_mx_init": 40,        # b, p_prev -> b, x, r64
    "k_mx_prep": 16,        # r64 -> f0 (binary32), e
    "k_mx_correct": 20,     # x, e -> x
    "k_mx_resid": 24,       # x, b -> r64
    "k_correct_diag_m": 64,  # x, u*, v*, u, v -> u, v, p (the divergences from the same pass)
    # mixed form: binary32 PCG and V-cycle (per cell of the kernel's level)
    "k_mx_matvec": 16,      # z, p_old -> p, q
    "k_mx_matvec_tma": 16,
    "k_mx_update_down": 33,  # e, p, r, q -> e, r (24) + level-0 down-sweep: t, coarse f (9)
    "k_mg_down": 9,         # f -> t, coarse f (a quarter of the cells on full coarsening)
    "k_mg_post": 13,        # t, f, coarse u -> u
    "k_mg_coarse": 8,       # f -> u of its finest level (everything else stays in shared memory)
}


def level_cells(shape_lists):
    """Cells of the levels that have a coarser global level below them (the tiles of
    the down- and up-sweeps of level l), and of every instance's last global level
    (where its coarse CTA starts)."""
    pre, coarse = {}, 0
    for shapes in shape_lists:
        for l, (a, b) in enumerate(shapes):
            if l + 1 < len(shapes):
                pre[l] = pre.get(l, 0) + a * b
        coarse += shapes[-1][0] * shapes[-1][1]
    return pre, coarse


def kernel_table(prof, cells, shape_lists, step_ms, hbm):
    """Rows {kernel, launches, total_us, us_per_launch, share, bytes_per_launch,
    gbs, frac} of a profiled step, largest share first; plus the step-level
    figures (all kernels' algorithmic bytes over the timed step's mean)."""
    pre, coarse = level_cells(shape_lists)
    all_ms = sum(ms for _, _, ms in prof)
    rows, step_bytes = [], 0.0
    for name, n, ms in prof:
        base, _, lvl = name.partition("@")
        per_cell = KERNEL_BYTES.get(base)
        if base in ("k_mg_down", "k_mg_post"):
            c = pre.get(int(lvl), 0)
        elif base == "k_mg_coarse":
            c = coarse
        elif base in ("k_dt", "k_gather", "k_mx_persist"):
            c = 0
        else:
            c = cells
        b = per_cell * c if per_cell is not None else None
        us = 1e3 * ms / max(n, 1)
        row = {"kernel": name, "launches": n, "total_us": 1e3 * ms, "us_per_launch": us,
               "share": ms / all_ms if all_ms > 0 else None, "bytes_per_launch": b}
        if b:
            row["gbs"] = b / (us * 1e-6) / 1e9
            row["frac"] = row["gbs"] / hbm
            step_bytes += b * n
        rows.append(row)
    rows.sort(key=lambda r: -(r["share"] or 0.0))
    step = {"bytes": step_bytes, "profiled_ms": all_ms, "timed_ms": step_ms,
            "achieved": step_bytes / (step_ms * 1e-3) / 1e9 if step_ms else None}
    if step["achieved"] is not None:
        step["frac"] = step["achieved"] / hbm
    return rows, step


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from ncu
# captures of the same kernel and workload, with the file that records the capture.
TRAFFIC = {
    ("batched256", "k_mg_coarse"): (6.54e6, "profiles/k_mg_coarse_batched256.md"),
    ("batched256", "k_mx_update_down"): (26.90e6, "profiles/k_mg_coarse_batched256.md (other batch kernels)"),
    ("batched256", "k_mg_post@0"): (10.68e6, "profiles/k_mg_coarse_batched256.md (other batch kernels)"),
    ("cavity512", "k_mg_coarse"): (7.94e4, "profiles/k_mg_coarse_512.md"),
    ("cavity2048", "k_mx_update_down"): (80.8e6, "profiles/k_mx_update_down_2048.md"),
    ("cavity512", "k_mx_matvec"): (1.60e6, "profiles/k_mx_matvec_2048.md (512^2 capture)"),
    ("cavity2048", "k_mx_matvec"): (34.11e6, "profiles/k_mx_matvec_2048.md"),
    ("cavity2048", "k_mx_matvec_tma"): (33.74e6, "profiles/k_mx_matvec_tma_2048.md"),
    ("cavity2048", "k_cg_matvec"): (92.91e6, "profiles/k_cg_pair_fp64_2048.md"),
    ("cavity2048", "k_cg_update"): (194.53e6, "profiles/k_cg_pair_fp64_2048.md"),
    ("cavity512", "k_cg_matvec"): (4.27e6, "profiles/k_cg_matvec_fp64_512.md"),
}


def profile_step(handle, run_one):
    """One more step run kernel by kernel with events around every launch."""
    import torch

    from pyflow_solver_gb300 import _capi
    lib = _capi.load()
    _capi.check(lib.pfgb_set_profiling(handle, 1), "set_profiling")
    try:
        out = run_one()
        torch.cuda.synchronize()
        prof = _capi.profile_kernels(handle)
    finally:
        _capi.check(lib.pfgb_set_profiling(handle, 0), "set_profiling")
    return prof, out


def roofline_of(rows, step, workload, hbm, src):
    top = rows[0]
    tr = TRAFFIC.get((workload, top["kernel"]))
    return {"bound": "hbm", "achieved": top.get("gbs"), "peak": hbm, "unit": "GB/s", "frac": top.get("frac"),
            "traffic": tr[0] if tr else None, "traffic_source": tr[1] if tr else None,
            "kernel": top["kernel"], "share_of_step": top["share"], "per_launch_us": top["us_per_launch"],
            "launches_timed": top["launches"], "algorithmic_bytes_per_launch": top["bytes_per_launch"],
            "peak_source": f"{src} (copy bandwidth)",
            "bytes_model": "KERNEL_BYTES per cell of the kernel's level (bench.py)"}


# ---- CPU arm -----------------------------------------------------------------

def cpu_port_rate(name, steps, warm=1):
    """cell-updates/s of the oracle port (reference reductions, scipy CG sequence), one thread:
    `warm` untimed steps from zero fields (step 0 has a zero right-hand side), then `steps`."""
    from oracle import step as ost
    cfg = cavity_cfg(name, "fp64")
    n = CAVITIES[name]["n"]
    st = ost.allocate_state(n, n)
    tr = ost.ResidualManager()
    for it in range(warm):
        ost.step(cfg, st, tr, it, red="numpy")
    t0 = time.perf_counter()
    for it in range(warm, warm + steps):
        ost.step(cfg, st, tr, it, red="numpy")
    dt = time.perf_counter() - t0
    return n * n * steps / dt, dt


def _port_group(args):
    """One worker's share of the batch: its instances stepped `warm` times untimed, then
    `steps` times timed (the instances are independent: no step-by-step hand-off)."""
    group, warm, steps = args
    from oracle import step as ost
    from pyflow_solver_gb300.workloads import cavity_config
    sims = []
    for nx, ny, Re, U in group:
        sims.append((cavity_config(nx, ny, Re, U, "fp64"), ost.allocate_state(nx, ny), ost.ResidualManager()))
    for it in range(warm):
        for cfg, st, tr in sims:
            ost.step(cfg, st, tr, it, red="numpy")
    t0 = time.perf_counter()
    for it in range(warm, warm + steps):
        for cfg, st, tr in sims:
            ost.step(cfg, st, tr, it, red="numpy")
    return time.perf_counter() - t0, sum(nx * ny for nx, ny, _, _ in group) * steps


BLAS_THREAD_VARS = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")


def cpu_port_batched_rate(steps, warm, procs):
    """The oracle port over all 256 batched instances, split by cells over `procs`
    processes (one per host core): cell-updates/s = all cells x steps / slowest worker."""
    import multiprocessing as mp

    from pyflow_solver_gb300.workloads import batched_instances
    inst = sorted(batched_instances(256, 0), key=lambda t: -t[0] * t[1])
    groups, load = [[] for _ in range(procs)], [0] * procs
    for t in inst:                                     # largest first onto the least loaded worker
        k = load.index(min(load))
        groups[k].append(t)
        load[k] += t[0] * t[1]
    groups = [g for g in groups if g]
    ctx = mp.get_context("spawn")
    # one BLAS thread per worker: the workers already take every core (the children
    # inherit this environment before they import NumPy)
    saved = {k: os.environ.get(k) for k in BLAS_THREAD_VARS}
    os.environ.update({k: "1" for k in BLAS_THREAD_VARS})
    try:
        with ctx.Pool(len(groups)) as pool:
            res = pool.map(_port_group, [(g, warm, steps) for g in groups])
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    wall = max(r[0] for r in res)
    cells = sum(r[1] for r in res)
    return cells / wall, wall


REF_CAP = {"cavity512": 20, "cavity2048": 3, "batched256": 40, "serving": 40}


def run_reference_arm(args):
    _, rank, _ = dist_env()
    if rank != 0:
        return
    wl = args.workload
    # the port's steps are seconds long: K and W are capped so that the run ends in a few minutes
    steps = max(1, min(args.steps, REF_CAP[wl]))
    if wl in CAVITIES:
        warm = max(1, min(args.warmup, 3))
        v, dt = cpu_port_rate(wl, steps, warm)
        cores = 1
        n = CAVITIES[wl]["n"]
        sample = (f"steps {warm}..{warm + steps - 1} of the {n}^2 cavity from zero fields after {warm} untimed "
                  "(oracle port: NumPy restatement with the reference's np.dot/np.mean reductions and scipy's CG "
                  "sequence; one thread -- the reference steps one cavity at a time)")
        cfg = cavity_config_line(wl)
        ms = 1e3 * dt / steps
    else:
        warm = max(1, min(args.warmup, 5))
        cores = os.cpu_count() or 1
        v, dt = cpu_port_batched_rate(steps, warm, cores)
        sample = (f"all 256 batched instances, steps {warm}..{warm + steps - 1} after {warm} untimed, split by cells "
                  f"over {cores} processes (one per host core; oracle port, lin_maxiter 300)")
        cfg = batch_config() if wl == "batched256" else {"workload": "serving trace mix (the batched instances "
                                                                     "stand in on the CPU)"}
        ms = 1e3 * dt / steps
    line = {
        "impl": "reference", "metric": "cell-updates/s", "value": v, "unit": "cell-updates/s",
        "n_gpus": args.gpus, "steps": steps, "warmup": warm, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": cfg,
        "run": {"precision": PRECISION_REFERENCE},
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

    from pyflow_solver_gb300 import ResidualManager, allocate_state, step
    from pyflow_solver_gb300.solvers._handle import instance_for
    from pyflow_solver_gb300.solvers.solver import step_params
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
        return cfg, st, one, ms, diags

    with ClockSampler(local) as clocks:
        cfg, st, one, ms, diags = run(args.precision, args.steps, args.warmup)
    total = max_over_ranks(sum(ms), dist)
    value = n * n * args.steps * world / (total / 1e3)
    cg = [d["cg_iterations"] for d in diags]
    passes = [d.get("refine_passes", 0) for d in diags]
    shapes = mg_shapes(n, n)
    launches = sum(launches_per_step(args.precision, c, p, len(shapes), args.persistent) for c, p in zip(cg, passes))
    kernels = roof = step_roof = None
    if not args.no_roofline:
        hbm, src = peaks()
        P, *_ = step_params(cfg, st.nx, st.ny)
        prof, _ = profile_step(instance_for(st, P).handle, one)
        rows, step_roof = kernel_table(prof, n * n, [shapes] if args.precision == "mixed" else [], total / args.steps,
                                       hbm)
        kernels = rows
        roof = roofline_of(rows, step_roof, wl, hbm, src)
    extra = {}
    if args.precision == "mixed" and not args.no_plain:
        _, _, _, pms, pd = run("fp64", args.plain_steps, 1)
        ptot = max_over_ranks(sum(pms), dist)
        pval = n * n * args.plain_steps * world / (ptot / 1e3)
        extra["plain_fp64"] = {"value": pval, "unit": "cell-updates/s", "ms_per_step": ptot / args.plain_steps,
                               "steps": args.plain_steps, "cg_iterations_per_step": [d["cg_iterations"] for d in pd]}
        extra["speedup_vs_plain_fp64"] = value / pval
    e2e_steps = args.steps if args.e2e_steps is None else args.e2e_steps
    e2e = e2e_cavity(cfg, n, e2e_steps, args.warmup) if e2e_steps > 0 else None
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
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
        "config": cavity_config_line(wl),
        "run": {"precision": PRECISION_NOTE[args.precision],
                "parallelism": "replicas" if world > 1 else "single GPU",
                "timed_steps": f"steps {args.warmup}..{args.warmup + args.steps - 1} of a run from zero fields",
                "cg_iterations_per_step": series_summary(cg), "refine_passes_per_step": series_summary(passes),
                "steps_not_converged": sum(1 for d in diags if not d.get("Rp_converged", True))},
        **extra,
        "step_latency_ms": pct(ms),
        "roofline": roof, "step_roofline": step_roof, "kernels": kernels, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": launches, "clocks": clocks.summary(),
    }
    return line


BATCH_WORKLOAD = ("256 lid-driven cavities from seed 0: nx, ny in {32,48,64,96,128}, Re log-uniform [100,5000], "
                  "lid uniform [0.5,2]; one graph launch per step for all instances")


def make_batch(inst, precision):
    """The 256 instances over one device arena of fields (u, v, p of every instance)."""
    import torch

    from pyflow_solver_gb300.batch import BatchedCavities
    from pyflow_solver_gb300.core.ghost_fields import State
    from pyflow_solver_gb300.workloads import cavity_config
    sizes = [3 * (ny + 2) * (nx + 2) for nx, ny, _, _ in inst]
    arena = torch.zeros(sum(sizes), dtype=torch.float64, device="cuda")
    states, off = [], 0
    for (nx, ny, _, _), sz in zip(inst, sizes):
        f = arena[off:off + sz].view(3, ny + 2, nx + 2)
        states.append(State(nx, ny, {"u": f[0], "v": f[1], "p": f[2]}))
        off += sz
    cfgs = [cavity_config(nx, ny, Re, U, precision) for nx, ny, Re, U in inst]
    return BatchedCavities(cfgs, states), arena


def bench_batched(args, dist, world, rank, local):
    import torch

    from pyflow_solver_gb300.workloads import batched_instances
    inst = batched_instances(256, 0)
    B, arena = make_batch(inst, args.precision)
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
    shapes = [mg_shapes(nx, ny) for nx, ny, _, _ in inst]
    nlev = max(len(s) for s in shapes)
    launches = sum(launches_per_step(args.precision, c, p, nlev, args.persistent) for c, p in zip(maxit, maxpass))
    kernels = roof = step_roof = None
    if not args.no_roofline:
        hbm, src = peaks()
        prof, _ = profile_step(B._h, B.step_arrays)
        kernels, step_roof = kernel_table(prof, cells, shapes if args.precision == "mixed" else [],
                                          total / args.steps, hbm)
        roof = roofline_of(kernels, step_roof, "batched256", hbm, src)
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
    B.close()
    del arena
    extra = {}
    if args.precision == "mixed" and not args.no_plain:
        # the same 256 cavities through the plain binary64 path (the reference's CG, lin_maxiter 300)
        P, parena = make_batch(inst, "fp64")
        P.step_arrays()                                # step 0: zero right-hand side
        pms, pouts = timed_steps(P.step_arrays, args.plain_steps, stream, flush, dist)
        ptot = max_over_ranks(sum(pms), dist)
        pval = cells * args.plain_steps * world / (ptot / 1e3)
        extra["plain_fp64"] = {"value": pval, "unit": "cell-updates/s", "ms_per_step": ptot / args.plain_steps,
                               "steps": args.plain_steps, "timed_steps": f"steps 1..{args.plain_steps}",
                               "max_cg_iterations_per_step": [int(o["cg_iterations"].max()) for o in pouts]}
        extra["speedup_vs_plain_fp64"] = value / pval
        P.close()
        del parena
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        v, wall = cpu_port_batched_rate(2, 1, cores)
        cpu = {"value": v, "unit": "cell-updates/s", "cores": cores, "kind": "port", "seconds": wall,
               "sample": f"all 256 instances, steps 1..2 after step 0, split by cells over {cores} processes "
                         "(oracle port: NumPy restatement with the reference's reductions and CG sequence, "
                         "lin_maxiter 300)"}
    line = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+f32" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": batch_config(),
        "run": {"precision": PRECISION_NOTE[args.precision],
                "timed_steps": f"steps {args.warmup}..{args.warmup + args.steps - 1} of a run from zero fields",
                "max_cg_iterations_per_step": series_summary(maxit),
                "max_refine_passes_per_step": series_summary(maxpass),
                "parallelism": "replicas" if world > 1 else "single GPU"},
        **extra,
        "step_latency_ms": pct(ms),
        "roofline": roof, "step_roofline": step_roof, "kernels": kernels, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": launches, "gpu_launches_note": "from the largest loop trip counts of each step",
        "clocks": clocks.summary(),
    }
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
    ap.add_argument("--workload", default="batched256", choices=["batched256", "cavity512", "cavity2048", "serving"])
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
