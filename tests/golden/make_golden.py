"""Generate the golden fixtures of this directory by running the reference.

Run from the repository root on a machine that has the reference checkout:

    python tests/golden/make_golden.py --ref PATH_TO_REFERENCE_CHECKOUT [--only NAME]

(or with the checkout's path in the environment variable PYFLOW_REFERENCE).

The script imports the reference package (``src/pyflow``) read-only, runs its
own ``SimulationDriver.run`` / ``step`` / ``solve_pressure_poisson`` and numerics
functions, and writes compressed ``.npz`` fixtures.  It counts the true CG
iterations by wrapping ``scipy.sparse.linalg.cg`` with an iteration callback
(the reference only reports 0/maxiter).  Nothing in the test suite, the
package or the benchmark reads the reference at run time: only these files.

Every fixture records the BLAS/NumPy/SciPy versions and the machine it was made
on, because the reference's dot products round in an order that depends on the
BLAS kernel of that machine.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _import_reference(ref_root):
    src = os.path.join(ref_root, "src")
    if src not in sys.path:
        sys.path.insert(0, src)
    import scipy.sparse.linalg as spla

    import pyflow.core.ghost_fields as gf
    import pyflow.drivers.simulation_driver as drv
    import pyflow.numerics.core_ops_coherent as coh
    import pyflow.numerics.fluid_ops as fops
    import pyflow.numerics.operators.advection as adv
    import pyflow.residuals.manager as rm
    import pyflow.solvers.pressure_solver as ps
    import pyflow.solvers.solver as sol

    counter = {"calls": [], "cur": 0}
    orig_cg = spla.cg

    def counting_cg(A, b, *args, **kw):
        user_cb = kw.pop("callback", None)
        counter["cur"] = 0

        def cb(xk):
            counter["cur"] += 1
            if user_cb is not None:
                user_cb(xk)

        out = orig_cg(A, b, *args, callback=cb, **kw)
        counter["calls"].append(counter["cur"])
        return out

    spla.cg = counting_cg
    return dict(gf=gf, drv=drv, coh=coh, fops=fops, adv=adv, rm=rm, ps=ps, sol=sol, counter=counter)


def _meta():
    import scipy
    try:
        blas = np.show_config(mode="dicts")["Build Dependencies"]["blas"]["name"]
    except Exception:  # pragma: no cover
        blas = "unknown"
    return json.dumps({
        "machine": platform.machine(), "python": platform.python_version(),
        "numpy": np.__version__, "scipy": scipy.__version__, "blas": blas,
        "generated": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
    })


class Cfg:
    """Duck-typed config, read by the reference through getattr."""

    def __init__(self, **kw):
        self.diagnostics = False
        self.force_quiet = True
        for k, v in kw.items():
            setattr(self, k, v)

    def as_dict(self):
        return {k: v for k, v in vars(self).items()}


SCALARS = ("dt", "CFL", "Ru", "Rv", "continuity", "Rp_iterations", "Rp_residual",
           "divergence_norm", "max_residual", "residual_drop_Ru_orders", "nu")


def run_trajectory(R, cfg, nx, ny, steps, save_fields_at, init=None):
    gf = R["gf"]
    state = gf.allocate_state(nx, ny)
    if init is not None:
        for k, arr in init.items():
            gf.interior_view(state.fields[k])[:] = arr
    drv = R["drv"].SimulationDriver(cfg, state, R["rm"].ResidualManager())
    R["counter"]["calls"].clear()
    out = {k: [] for k in SCALARS}
    out.update({"Rp_converged": [], "nan_detected": [], "dt_prev": [], "div_hist": [], "centerline": []})
    fields = {}
    t0 = time.time()
    for st, res, diag in drv.run(max_steps=steps):
        it = diag["iteration"]
        for k in SCALARS:
            out[k].append(float(res[k]) if k in res else float(diag[k]))
        out["Rp_converged"].append(bool(diag["Rp_converged"]))
        out["nan_detected"].append(bool(diag["nan_detected"]))
        out["dt_prev"].append(float(st.meta["dt_prev"]))
        h = list(st.meta["divergence_history"])
        out["div_hist"].append(h + [np.nan] * (5 - len(h)))
        out["centerline"].append(np.asarray(diag["u_centerline"][1]))
        if it in save_fields_at:
            for k in ("u", "v", "p"):
                fields[f"{k}_{it}"] = gf.interior_view(st.fields[k]).copy()
    wall = time.time() - t0
    arrays = {k: np.asarray(v) for k, v in out.items()}
    arrays["cg_true_iterations"] = np.asarray(R["counter"]["calls"])
    arrays["wall_s"] = np.asarray(wall)
    arrays.update(fields)
    arrays["saved_steps"] = np.asarray(sorted(save_fields_at))
    return arrays


def make_ops(R):
    coh, fops, adv = R["coh"], R["fops"], R["adv"]
    out = {}
    for (nx, ny) in [(8, 8), (16, 12), (5, 9), (33, 17), (2, 2), (3, 2), (2, 5)]:
        rng = np.random.default_rng(1000 + 37 * nx + ny)
        dx = 1.0 / (nx - 1)
        dy = 1.0 / (ny - 1)
        u = rng.standard_normal((ny, nx))
        v = rng.standard_normal((ny, nx))
        p = rng.standard_normal((ny, nx))
        # zero some velocities so that the sign branches at 0 are exercised
        u[rng.random((ny, nx)) < 0.1] = 0.0
        v[rng.random((ny, nx)) < 0.1] = -0.0
        key = f"{nx}x{ny}"
        out[f"{key}_u"], out[f"{key}_v"], out[f"{key}_p"] = u, v, p
        out[f"{key}_dxdy"] = np.asarray([dx, dy])
        gx, gy = coh.gradient_coherent(p, dx, dy)
        out[f"{key}_gx"], out[f"{key}_gy"] = gx, gy
        out[f"{key}_divc"] = coh.divergence_coherent(u, v, dx, dy)
        out[f"{key}_lap"] = coh.laplacian_coherent(p, dx, dy)
        out[f"{key}_divcentral"] = fops.divergence(u, v, 1.0, 1.0)
        out[f"{key}_divcentral_h"] = fops.divergence(u, v, dx, dy)
        out[f"{key}_quick_u"] = adv.advect_quick(u, v, u, dx, dy)
        out[f"{key}_quick_v"] = adv.advect_quick(u, v, v, dx, dy)
        out[f"{key}_upwind_u"] = adv.advect_upwind(u, v, u, dx, dy)
        out[f"{key}_upwind_v"] = adv.advect_upwind(u, v, v, dx, dy)
    return out


def make_manufactured(R):
    gf, ps = R["gf"], R["ps"]
    out = {}
    nx = ny = 8
    dx = dy = 1.0 / (nx - 1)
    x = np.linspace(0.0, 1.0, nx)
    X, Y = np.meshgrid(x, x)
    p_an = np.sin(np.pi * X) * np.sin(np.pi * Y)
    rhs_grid = np.zeros((ny, nx))
    rhs_grid[1:-1, 1:-1] = (-2.0 * np.pi**2) * p_an[1:-1, 1:-1]
    rhs = rhs_grid.reshape(-1)
    rhs[0] = 0.0
    state = gf.allocate_state(nx, ny)
    cfg = Cfg(lin_tol=1e-10, lin_maxiter=500)
    R["counter"]["calls"].clear()
    p, diag = ps.solve_pressure_poisson(state, 1.0, dx, dy, cfg, rhs_override=rhs.copy())
    out["rhs"] = rhs
    out["p"] = gf.interior_view(state.fields["p"]).copy()
    out["cg_true_iterations"] = np.asarray(R["counter"]["calls"])
    for k in ("Rp_iterations", "Rp_residual", "divergence_norm", "lin_residual_norm", "lin_residual_rel"):
        out[k] = np.asarray(float(diag[k]))
    # one normal-mode projection from a bump (preconditioner on and off)
    for pc in (True, False):
        nx, ny = 24, 20
        state = gf.allocate_state(nx, ny)
        gf.interior_view(state.fields["u"])[ny // 3, nx // 3] = 1.0
        cfg = Cfg(lin_tol=1e-10, lin_maxiter=300, enable_jacobi_pc=pc)
        R["counter"]["calls"].clear()
        p, diag = ps.solve_pressure_poisson(state, 0.01, 1.0, 1.0, cfg)
        tag = "pc" if pc else "nopc"
        for k in ("u", "v", "p"):
            out[f"bump_{tag}_{k}"] = gf.interior_view(state.fields[k]).copy()
        out[f"bump_{tag}_iters"] = np.asarray(R["counter"]["calls"])
        for k in ("Rp_iterations", "Rp_residual", "divergence_norm", "lin_residual_norm",
                  "lin_residual_rel", "divergence_norm_initial"):
            out[f"bump_{tag}_{k}"] = np.asarray(float(diag[k]))
    return out


def cavity_cfg(nx, ny, Re, lid, unit_square, scheme="quick", maxiter=300, tol=1e-8, **extra):
    kw = dict(nx=nx, ny=ny, Re=Re, lid_velocity=lid, advection_scheme=scheme, cfl_target=0.5,
              cfl_growth=1.05, lin_tol=tol, lin_maxiter=maxiter, enable_jacobi_pc=True,
              disable_advection=False)
    if unit_square:
        kw.update(lx=1.0, ly=1.0)
    kw.update(extra)
    return Cfg(**kw)


def batched_instances(n=256, seed=0):
    """The 256 uneven cavities of the batched workload (seeded draw order)."""
    rng = np.random.default_rng(seed)
    sides = [32, 48, 64, 96, 128]
    out = []
    for _ in range(n):
        nx = int(rng.choice(sides))
        ny = int(rng.choice(sides))
        Re = float(np.exp(rng.uniform(np.log(100.0), np.log(5000.0))))
        U = float(rng.uniform(0.5, 2.0))
        out.append((nx, ny, Re, U))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("PYFLOW_REFERENCE"),
                    help="root of the reference checkout (default: $PYFLOW_REFERENCE)")
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    if not args.ref:
        ap.error("the reference checkout is needed: pass --ref or set PYFLOW_REFERENCE")
    R = _import_reference(args.ref)
    meta = _meta()

    def want(name):
        return args.only is None or args.only == name

    def save(name, arrays, cfg=None):
        arrays = dict(arrays)
        arrays["meta"] = np.asarray(meta)
        if cfg is not None:
            arrays["config"] = np.asarray(json.dumps(cfg.as_dict()))
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **arrays)
        print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")

    if want("ops"):
        save("ops", make_ops(R))
    if want("manufactured"):
        save("manufactured", make_manufactured(R))
    if want("cavity64_unit"):
        cfg = cavity_cfg(64, 64, 100.0, 1.0, True)
        save("cavity64_unit", run_trajectory(R, cfg, 64, 64, 50, {0, 1, 2, 9, 10, 49}), cfg)
    if want("cavity64_cli"):
        cfg = cavity_cfg(64, 64, 100.0, 1.0, False)
        save("cavity64_cli", run_trajectory(R, cfg, 64, 64, 20, {0, 1, 19}), cfg)
    if want("small"):
        cases = {
            "s8_upwind": (cavity_cfg(8, 8, 100.0, 1.0, True, scheme="upwind", maxiter=50, tol=1e-10), 8, 8, 12),
            "s16x12_quick": (cavity_cfg(16, 12, 400.0, 1.5, True, maxiter=120), 16, 12, 12),
            "s5x9_quick": (cavity_cfg(5, 9, 100.0, 1.0, False, maxiter=40), 5, 9, 10),
            "s12x10_nopc": (cavity_cfg(12, 10, 100.0, 1.0, True, maxiter=60, enable_jacobi_pc=False), 12, 10, 8),
            "s9x7_noadv": (cavity_cfg(9, 7, 100.0, 1.0, True, maxiter=60, disable_advection=True), 9, 7, 6),
            "s6x6_nolid": (cavity_cfg(6, 6, 100.0, None, True, maxiter=60), 6, 6, 4),
            "s3x4_tiny": (cavity_cfg(3, 4, 50.0, 1.0, True, maxiter=30), 3, 4, 6),
            "s2x2_min": (cavity_cfg(2, 2, 50.0, 1.0, True, maxiter=30), 2, 2, 4),
        }
        for name, (cfg, nx, ny, steps) in cases.items():
            save(name, run_trajectory(R, cfg, nx, ny, steps, set(range(steps))), cfg)
        # a non-zero initial field (localized patch, cf. the reference's multi-step test)
        cfg = cavity_cfg(16, 16, 100.0, 1.0, False, maxiter=300, tol=1e-10, cfl_growth=1.1)
        u0 = np.zeros((16, 16))
        u0[4:10, 4:10] = 1.0
        save("s16_patch", run_trajectory(R, cfg, 16, 16, 8, set(range(8)), init={"u": u0}), cfg)
    if want("cavity512"):
        cfg = cavity_cfg(512, 512, 1000.0, 1.0, True)
        arr = run_trajectory(R, cfg, 512, 512, 4, {1, 3})
        save("cavity512", arr, cfg)
    if want("config_hashes"):
        from pyflow.config.model import SimulationConfig
        cases = [dict(nx=64, ny=64), dict(nx=32, ny=32, Re=400.0, lid_velocity=1.5, advection_scheme="quick",
                                          lin_tol=1e-8, lin_maxiter=300, diagnostics=False, seed=7),
                 dict(nx=512, ny=512, Re=1000.0, cfl_growth=1.1, checkpoint_interval=10, disable_advection=True)]
        out = [{"kwargs": c, "hash": SimulationConfig(**c).config_hash} for c in cases]
        path = os.path.join(HERE, "config_hashes.json")
        with open(path, "w") as f:
            json.dump({"meta": json.loads(meta), "cases": out}, f, indent=1)
        print(f"wrote {path}")
    if want("batched16"):
        inst = batched_instances()
        pick = list(range(0, 256, 16))
        out = {"picked": np.asarray(pick), "instances": np.asarray(inst)}
        for i in pick:
            nx, ny, Re, U = inst[i]
            cfg = cavity_cfg(nx, ny, Re, U, True)
            # fields only for the smaller instances (fixture size); scalars for all
            arr = run_trajectory(R, cfg, nx, ny, 5, {4} if nx * ny <= 64 * 64 else set())
            for k, v in arr.items():
                out[f"i{i}_{k}"] = v
        save("batched16", out)


if __name__ == "__main__":
    main()
