"""Oracle work for the large parity cases, run in worker processes (test helper).

The twin (exactly rounded reductions) and the converged binary64 oracle take
seconds to minutes per step at the benchmark sizes, so the parity tests hand
them to a process pool started with ``spawn`` (never ``fork`` after CUDA is
initialised) and run the GPU side meanwhile.  Every function here is plain
NumPy/SciPy on the CPU and returns plain arrays and dicts.
"""
from __future__ import annotations

import multiprocessing as mp
import os
from concurrent.futures import ProcessPoolExecutor
from types import SimpleNamespace

import numpy as np


def pool(max_workers=None):
    n = max_workers or max(1, min(16, (os.cpu_count() or 2) - 1))
    return ProcessPoolExecutor(max_workers=n, mp_context=mp.get_context("spawn"))


def twin(cfg_kw, nx, ny, steps, keep, red="exact"):
    """A trajectory of the oracle from zero fields (records as tests._gpu_run.twin_trajectory)."""
    from tests._gpu_run import twin_trajectory
    return twin_trajectory(SimpleNamespace(**cfg_kw), nx, ny, steps, keep=set(keep), red=red)


def converged_chain(cfg_kw, nx, ny, steps, start=None, start_iteration=0):
    """States S_0 .. S_steps of the converged binary64 oracle (the CG replaced by a sparse
    direct solve), from zero fields or from ``start`` = {"u", "v", "p" interiors, "meta"}.
    Each entry: interiors of u, v, p, the state's meta, and the step's dt (None for S_0)."""
    from oracle import step as ost
    cfg = SimpleNamespace(**cfg_kw, oracle_pressure="converged")
    st = ost.allocate_state(nx, ny)
    if start is not None:
        for k in "uvp":
            ost.interior(st.fields[k])[:] = start[k]
        st.meta = dict(start["meta"])
    tr = ost.ResidualManager()

    def snap(dt):
        return {"u": ost.interior(st.fields["u"]).copy(), "v": ost.interior(st.fields["v"]).copy(),
                "p": ost.interior(st.fields["p"]).copy(),
                "meta": {"dt_prev": st.meta.get("dt_prev", 1e-2),
                         "divergence_history": list(st.meta.get("divergence_history", []))}, "dt": dt}
    chain = [snap(None)]
    for it in range(start_iteration, start_iteration + steps):
        _, _, diag = ost.step(cfg, st, tr, it, red="exact")
        chain.append(snap(diag["dt"]))
    return chain
