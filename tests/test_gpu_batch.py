"""Batched cavities: every instance gets exactly what it gets alone.

A batch of uneven cavities (sizes, Re, lid velocity, scheme) advances with one
graph launch per step; each instance's fields, dicts and state.meta must equal
bit for bit the single-instance GPU path and the oracle twin, including when
instances sit steps out (continuous batching).
"""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import step as ost

pytestmark = pytest.mark.gpu

CASES = [(64, 64, 100.0, 1.0, "quick"), (48, 96, 400.0, 1.5, "quick"), (32, 32, 250.0, 1.0, "upwind"),
         (96, 48, 1000.0, 0.7, "quick"), (37, 21, 200.0, 1.2, "quick"), (128, 64, 3000.0, 2.0, "quick")]


def cfg_of(nx, ny, Re, U, scheme, maxiter=120):
    return SimpleNamespace(nx=nx, ny=ny, lx=1.0, ly=1.0, Re=Re, lid_velocity=U, advection_scheme=scheme,
                           cfl_target=0.5, cfl_growth=1.05, lin_tol=1e-8, lin_maxiter=maxiter, diagnostics=False)


def fields(st):
    from pyflow_solver_gb300 import interior_view
    return [interior_view(st.fields[k]).cpu().numpy().copy() for k in "uvp"]


def test_batch_equals_single_instances_and_twin():
    from pyflow_solver_gb300 import ResidualManager, allocate_state, step
    from pyflow_solver_gb300.batch import BatchedCavities
    cfgs = [cfg_of(*c) for c in CASES]
    states = [allocate_state(c.nx, c.ny) for c in cfgs]
    B = BatchedCavities(cfgs, states)
    batch_out = [B.step() for _ in range(4)]
    for k, cfg in enumerate(cfgs):
        st = allocate_state(cfg.nx, cfg.ny)
        tr = ResidualManager()
        tw = ost.allocate_state(cfg.nx, cfg.ny)
        ttr = ost.ResidualManager()
        for it in range(4):
            _, res, diag = step(cfg, st, tr, it)
            bres, bdiag = batch_out[it][k]
            assert res == bres, (k, it)
            assert {kk: diag[kk] for kk in diag} == bdiag, (k, it)
            _, tres, _ = ost.step(cfg, tw, ttr, it, red="exact")
            assert res == tres, (k, it)
        for a, b, c in zip(fields(st), fields(states[k]), [ost.interior(tw.fields[q]) for q in "uvp"]):
            np.testing.assert_array_equal(a, b)
            np.testing.assert_array_equal(a, c)
        assert st.meta["dt_prev"] == states[k].meta["dt_prev"]


def test_batch_instances_can_sit_out_steps():
    from pyflow_solver_gb300 import ResidualManager, allocate_state, step
    from pyflow_solver_gb300.batch import BatchedCavities
    cfgs = [cfg_of(*c, maxiter=60) for c in CASES[:4]]
    states = [allocate_state(c.nx, c.ny) for c in cfgs]
    B = BatchedCavities(cfgs, states)
    masks = [[1, 1, 1, 1], [1, 0, 1, 0], [0, 0, 1, 1], [1, 1, 1, 1], [1, 1, 0, 1]]
    for m in masks:
        before = [fields(s) for s in states]
        out = B.step(active=[bool(x) for x in m])
        for k, a in enumerate(m):
            if not a:
                assert out[k] is None
                for x, y in zip(before[k], fields(states[k])):
                    np.testing.assert_array_equal(x, y)
    # each instance equals its own single-instance run of the same number of steps
    for k, cfg in enumerate(cfgs):
        n = sum(m[k] for m in masks)
        assert B.iterations[k] == n
        st = allocate_state(cfg.nx, cfg.ny)
        tr = ResidualManager()
        for it in range(n):
            step(cfg, st, tr, it)
        for a, b in zip(fields(st), fields(states[k])):
            np.testing.assert_array_equal(a, b)


def test_mixed_batch_equals_single_instances():
    """Mixed-precision batch of uneven cavities: bit for bit the single-instance mixed path."""
    from pyflow_solver_gb300 import ResidualManager, allocate_state, step
    from pyflow_solver_gb300.batch import BatchedCavities
    cases = [(64, 64, 100.0, 1.0, "quick"), (48, 96, 400.0, 1.5, "quick"), (128, 32, 2500.0, 0.6, "quick"),
             (32, 32, 150.0, 1.0, "upwind"), (96, 96, 5000.0, 2.0, "quick")]
    cfgs = []
    for c in cases:
        cfg = cfg_of(*c)
        cfg.precision = "mixed"
        cfgs.append(cfg)
    states = [allocate_state(c.nx, c.ny) for c in cfgs]
    B = BatchedCavities(cfgs, states)
    outs = [B.step(active=m) for m in ([1] * 5, [1, 0, 1, 1, 0], [1] * 5)]
    for k, cfg in enumerate(cfgs):
        n = sum(1 for m in ([1] * 5, [1, 0, 1, 1, 0], [1] * 5) if m[k])
        st = allocate_state(cfg.nx, cfg.ny)
        tr = ResidualManager()
        single = [step(cfg, st, tr, it)[1:] for it in range(n)]
        mine = [o[k] for o in outs if o[k] is not None]
        for (r1, d1), (r2, d2) in zip(single, mine):
            assert r1 == r2 and d1 == d2, k
        for a, b in zip(fields(st), fields(states[k])):
            np.testing.assert_array_equal(a, b)
        assert all(d["Rp_converged"] for _, d in mine[1:])


def test_wide_mixed_batch_equals_single_instances():
    """A mixed batch with more instances than the GPU has SMs runs its coarse cycles as
    512-thread CTAs, two to an SM; every sum there is taken in the 1024-thread order, so
    instances still get the bits of their single-instance runs (1024-thread CTAs)."""
    import torch

    from pyflow_solver_gb300 import ResidualManager, allocate_state, step
    from pyflow_solver_gb300.batch import BatchedCavities
    n = torch.cuda.get_device_properties(0).multi_processor_count + 8
    rng = np.random.default_rng(5)
    sizes = [(16, 16), (32, 32), (64, 32), (48, 64), (64, 64), (8, 8), (24, 40)]
    cfgs = []
    for k in range(n):
        nx, ny = sizes[k % len(sizes)]
        cfg = cfg_of(nx, ny, float(rng.uniform(100, 3000)), float(rng.uniform(0.5, 2.0)), "quick")
        cfg.precision = "mixed"
        cfgs.append(cfg)
    states = [allocate_state(c.nx, c.ny) for c in cfgs]
    B = BatchedCavities(cfgs, states)
    outs = [B.step() for _ in range(3)]
    for k in list(range(len(sizes))) + [n - 1]:
        cfg = cfgs[k]
        st = allocate_state(cfg.nx, cfg.ny)
        tr = ResidualManager()
        for it in range(3):
            assert step(cfg, st, tr, it)[1:] == outs[it][k], (k, it)
        for a, b in zip(fields(st), fields(states[k])):
            np.testing.assert_array_equal(a, b)


def test_step_arrays_and_slot_reuse():
    """The array host path gives the same fields and records as step(); a slot
    reused with new parameters equals a fresh run of the new request."""
    from pyflow_solver_gb300 import ResidualManager, allocate_state, step
    from pyflow_solver_gb300.batch import BatchedCavities
    cases = [(64, 64, 100.0, 1.0, "quick"), (48, 32, 700.0, 1.4, "quick"), (32, 32, 250.0, 0.8, "upwind")]
    for prec in ("fp64", "mixed"):
        cfgs = []
        for c in cases:
            cfg = cfg_of(*c, maxiter=80)
            cfg.precision = prec
            cfgs.append(cfg)
        sa = [allocate_state(c.nx, c.ny) for c in cfgs]
        sb = [allocate_state(c.nx, c.ny) for c in cfgs]
        A = BatchedCavities(cfgs, sa)
        Bc = BatchedCavities(cfgs, sb)
        for it in range(3):
            ra = A.step()
            ob = Bc.step_arrays()
            cont = Bc.continuity(ob)
            for k in range(len(cases)):
                assert ra[k][0]["continuity"] == cont[k]
                assert ra[k][1]["dt"] == ob["dt"][k]
                assert ra[k][1]["cg_iterations"] == ob["cg_iterations"][k]
        Bc.sync_meta()
        for k in range(len(cases)):
            for a, b in zip(fields(sa[k]), fields(sb[k])):
                np.testing.assert_array_equal(a, b)
            assert sa[k].meta["dt_prev"] == sb[k].meta["dt_prev"]
            assert sa[k].meta["divergence_history"] == sb[k].meta["divergence_history"]
        # slot 1 takes a new request (same grid, new Re and lid velocity)
        new = cfg_of(48, 32, 2200.0, 0.6, "quick", maxiter=80)
        new.precision = prec
        Bc.set_params(1, new)
        for _ in range(4):
            Bc.step_arrays(active=[False, True, True])
        Bc.sync_meta(1)
        st = allocate_state(48, 32)
        tr = ResidualManager()
        for it in range(4):
            step(new, st, tr, it)
        for a, b in zip(fields(st), fields(sb[1])):
            np.testing.assert_array_equal(a, b)
        assert st.meta["dt_prev"] == sb[1].meta["dt_prev"]
        A.close()
        Bc.close()
