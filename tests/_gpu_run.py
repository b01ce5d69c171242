"""Run the GPU driver and the oracle twin side by side (test helper)."""
from __future__ import annotations

import numpy as np

from oracle import step as ost

SCALARS = ("dt", "CFL", "Ru", "Rv", "continuity", "Rp_residual", "divergence_norm", "Rp_iterations",
           "Rp_converged", "max_residual", "residual_drop_Ru_orders", "nu", "nan_detected")


def gpu_trajectory(cfg, nx, ny, steps, u0=None, v0=None, keep=None):
    import torch

    from pyflow_solver_gb300 import SimulationDriver, allocate_state, interior_view
    st = allocate_state(nx, ny)
    if u0 is not None:
        interior_view(st.fields["u"]).copy_(torch.from_numpy(u0))
    if v0 is not None:
        interior_view(st.fields["v"]).copy_(torch.from_numpy(v0))
    out = []
    for s, res, diag in SimulationDriver(cfg, st).run(max_steps=steps):
        rec = {k: (res[k] if k in res else diag[k]) for k in SCALARS}
        rec["cg_iterations"] = diag["cg_iterations"]
        rec["centerline"] = np.asarray(diag["u_centerline"][1])
        if keep is None or diag["iteration"] in keep:
            rec["fields"] = {k: interior_view(s.fields[k]).cpu().numpy().copy() for k in "uvp"}
        rec["meta"] = {"dt_prev": s.meta["dt_prev"], "hist": list(s.meta["divergence_history"])}
        out.append(rec)
    return out


def twin_trajectory(cfg, nx, ny, steps, u0=None, v0=None, keep=None, red="exact"):
    st = ost.allocate_state(nx, ny)
    if u0 is not None:
        ost.interior(st.fields["u"])[:] = u0
    if v0 is not None:
        ost.interior(st.fields["v"])[:] = v0
    out, extras = [], []
    for s, res, diag in ost.run(cfg, st, max_steps=steps, red=red, extras=extras):
        rec = {k: (res[k] if k in res else diag[k]) for k in SCALARS}
        rec["centerline"] = np.asarray(diag["u_centerline"][1])
        if keep is None or diag["iteration"] in keep:
            rec["fields"] = {k: ost.interior(s.fields[k]).copy() for k in "uvp"}
        rec["meta"] = {"dt_prev": s.meta["dt_prev"], "hist": list(s.meta["divergence_history"])}
        out.append(rec)
    for rec, ex in zip(out, extras):
        rec["cg_iterations"] = ex["cg_true_iterations"]
    return out


def same(a, b):
    if isinstance(a, float) and isinstance(b, float) and np.isnan(a) and np.isnan(b):
        return True
    return a == b


def rel_err(a, b):
    den = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / den)
