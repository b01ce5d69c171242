"""Parity at the benchmark sizes.

* 512 x 512, Re 1000 (the single-cavity workload), plain binary64: P1 bit for bit
  against the oracle twin for 4 steps (every scalar, the true CG counts, the
  fields at steps 1 and 3) and P2 against the reference's own fields at those
  steps (the committed ``cavity512.npz``): within 2x the summation-order floor.
* The batched workload's real draws: the 16 instances of ``batched16.npz`` (every
  16th of the 256 seed-0 cavities) stepped together through ``BatchedCavities``:
  plain binary64 bit for bit against the twin and within the floor of the
  reference's fields and CG counts; mixed precision per step against the
  converged binary64 oracle at 1e-6.
* Mixed precision from a developed flow (P3 per step, 1e-6): 512 x 512 after 1000
  steps and 1024 x 1024 after 500 steps, where the warm start and the
  outer-target aim of the refinement are active.
* 2048 x 2048, Re 3200, plain binary64: P1 bit for bit against the twin for three
  steps with lin_maxiter 20 (the twin's exactly rounded dot products cost about
  2 s per CG iteration at this size on one host core; every kernel, tile and
  reduction of the step still runs at full size).

The oracle side runs in a ``spawn`` process pool while the GPU works.
"""
from types import SimpleNamespace

import numpy as np
import pytest

from tests import _golden as G
from tests import _oracle_jobs as J
from tests._gpu_run import SCALARS, gpu_trajectory, rel_err, same

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

TOL = 1e-6


def cavity_kw(nx, ny, Re, lid, maxiter=300):
    return dict(nx=nx, ny=ny, lx=1.0, ly=1.0, Re=float(Re), lid_velocity=float(lid), advection_scheme="quick",
                cfl_target=0.5, cfl_growth=1.05, lin_tol=1e-8, lin_maxiter=maxiter, enable_jacobi_pc=True,
                disable_advection=False, diagnostics=False)


def b16_instances():
    g = G.load("batched16")
    inst = g["instances"]
    return g, [(int(i), int(inst[i][0]), int(inst[i][1]), float(inst[i][2]), float(inst[i][3])) for i in g["picked"]]


@pytest.fixture(scope="module")
def oracle_work():
    """Submit every oracle job that needs no GPU result up front."""
    ex = J.pool()
    futs = {}
    g512 = G.load("cavity512")
    futs["c512"] = ex.submit(J.twin, vars(G.config_of(g512)), 512, 512, 4, [1, 3])
    futs["c2048"] = ex.submit(J.twin, cavity_kw(2048, 2048, 3200.0, 1.0, maxiter=20), 2048, 2048, 3, [1, 2])
    _, inst = b16_instances()
    for i, nx, ny, Re, U in inst:
        futs[("b16", i)] = ex.submit(J.twin, cavity_kw(nx, ny, Re, U), nx, ny, 5, [4])
        futs[("b16c", i)] = ex.submit(J.converged_chain, cavity_kw(nx, ny, Re, U), nx, ny, 5)
    yield ex, futs
    ex.shutdown(wait=False, cancel_futures=True)


def check_records(got, ref, name):
    assert len(got) == len(ref)
    for it, (a, b) in enumerate(zip(got, ref)):
        for k in SCALARS:
            assert same(a[k], b[k]), f"{name} step {it} {k}: gpu {a[k]!r} twin {b[k]!r}"
        assert a["cg_iterations"] == b["cg_iterations"], f"{name} step {it} CG iterations"
        assert a["meta"]["dt_prev"] == b["meta"]["dt_prev"]
        assert a["meta"]["hist"] == b["meta"]["hist"]
        if "fields" in a and "fields" in b:
            for k in "uvp":
                np.testing.assert_array_equal(a["fields"][k], b["fields"][k], err_msg=f"{name} step {it} {k}")


def test_cavity512_plain_p1_and_p2(oracle_work):
    _, futs = oracle_work
    g = G.load("cavity512")
    cfg = G.config_of(g)
    got = gpu_trajectory(cfg, 512, 512, 4, keep={1, 3})
    twin = futs["c512"].result()
    check_records(got, twin, "cavity512")
    # the reference never converges here: 300 true CG iterations at every step after step 0
    assert [r["cg_iterations"] for r in got] == list(g["cg_true_iterations"])
    for it in (1, 3):
        for k in "uvp":
            ref = g[f"{k}_{it}"]
            floor = rel_err(twin[it]["fields"][k], ref)
            err = rel_err(got[it]["fields"][k], ref)
            assert err <= 2.0 * floor + 1e-15, f"step {it} {k}: gpu {err:.3e} floor {floor:.3e}"


def _batch_records(B, steps, keep):
    from pyflow_solver_gb300 import interior_view
    recs = [[] for _ in range(len(B))]
    for it in range(steps):
        out = B.step()
        for k, (res, diag) in enumerate(out):
            rec = {q: (res[q] if q in res else diag[q]) for q in SCALARS}
            rec["cg_iterations"] = diag["cg_iterations"]
            st = B.states[k]
            rec["meta"] = {"dt_prev": st.meta["dt_prev"], "hist": list(st.meta["divergence_history"])}
            if it in keep:
                rec["fields"] = {q: interior_view(st.fields[q]).cpu().numpy().copy() for q in "uvp"}
            recs[k].append(rec)
    return recs


def test_batched16_plain_p1_p2(oracle_work):
    from pyflow_solver_gb300 import allocate_state
    from pyflow_solver_gb300.batch import BatchedCavities
    _, futs = oracle_work
    g, inst = b16_instances()
    cfgs = [SimpleNamespace(**cavity_kw(nx, ny, Re, U)) for _, nx, ny, Re, U in inst]
    B = BatchedCavities(cfgs, [allocate_state(c.nx, c.ny) for c in cfgs])
    try:
        recs = _batch_records(B, 5, {4})
    finally:
        B.close()
    for k, (i, nx, ny, Re, U) in enumerate(inst):
        twin = futs[("b16", i)].result()
        check_records(recs[k], twin, f"instance {i} ({nx}x{ny})")
        # the reference's own true CG counts (a counting callback around scipy's CG)
        ref_counts = [int(c) for c in g[f"i{i}_cg_true_iterations"]]
        assert all(abs(a["cg_iterations"] - c) <= 1 for a, c in zip(recs[k], ref_counts)), (i, ref_counts)
        if f"i{i}_u_4" in g.files:
            for q in "uvp":
                ref = g[f"i{i}_{q}_4"]
                floor = rel_err(twin[4]["fields"][q], ref)
                err = rel_err(recs[k][4]["fields"][q], ref)
                assert err <= 2.0 * floor + 1e-15, f"instance {i} {q}: gpu {err:.3e} floor {floor:.3e}"


def _load(st, snap):
    import torch

    from pyflow_solver_gb300 import interior_view
    for q in "uvp":
        interior_view(st.fields[q]).copy_(torch.from_numpy(snap[q]))
    st.meta = {"dt_prev": snap["meta"]["dt_prev"], "divergence_history": list(snap["meta"]["divergence_history"])}


def _errors(st, snap):
    from pyflow_solver_gb300 import interior_view
    out = {}
    for q in "uvp":
        ref = snap[q]
        if np.max(np.abs(ref)) > 0:
            out[q] = rel_err(interior_view(st.fields[q]).cpu().numpy(), ref)
    nx = snap["u"].shape[1]
    got_c = interior_view(st.fields["u"])[:, nx // 2].cpu().numpy()
    out["u_centerline"] = rel_err(got_c, snap["u"][:, nx // 2])
    return out


def test_batched16_mixed_p3_per_step(oracle_work):
    """The 16 real draws, mixed precision, one batch launch per step; before every step each
    instance is reset to the converged oracle's state, after it compared with the oracle's next."""
    from pyflow_solver_gb300 import allocate_state
    from pyflow_solver_gb300.batch import BatchedCavities
    _, futs = oracle_work
    _, inst = b16_instances()
    cfgs = [SimpleNamespace(**cavity_kw(nx, ny, Re, U), precision="mixed") for _, nx, ny, Re, U in inst]
    states = [allocate_state(c.nx, c.ny) for c in cfgs]
    B = BatchedCavities(cfgs, states)
    chains = [futs[("b16c", i)].result() for i, *_ in inst]
    worst = {}
    try:
        for s in range(5):
            for k in range(len(inst)):
                _load(states[k], chains[k][s])
            B.reload_meta()
            out = B.step()
            for k, (i, *_rest) in enumerate(inst):
                assert out[k][1]["dt"] == chains[k][s + 1]["dt"], (i, s)
                if s > 0:
                    assert out[k][1]["Rp_converged"], (i, s)
                for q, e in _errors(states[k], chains[k][s + 1]).items():
                    worst[q] = max(worst.get(q, 0.0), e)
    finally:
        B.close()
    print(f"\nbatched16 mixed vs converged binary64 (worst over 16 instances x 5 steps): "
          + ", ".join(f"{q} {e:.2e}" for q, e in worst.items()))
    assert max(worst.values()) <= TOL, worst


@pytest.mark.parametrize("n,Re,develop", [(512, 1000.0, 1000), (1024, 3200.0, 500)])
def test_mixed_p3_from_developed_flow(oracle_work, n, Re, develop):
    """P3 per step after the flow has developed: the GPU runs `develop` mixed steps from zero,
    its state seeds the converged oracle, and three steps are compared each from the oracle's
    state (the same GPU state object keeps its refinement history)."""
    from pyflow_solver_gb300 import ResidualManager, allocate_state, interior_view, step
    ex, _ = oracle_work
    kw = cavity_kw(n, n, Re, 1.0)
    cfg = SimpleNamespace(**kw, precision="mixed")
    st = allocate_state(n, n)
    tr = ResidualManager()
    for it in range(develop):
        step(cfg, st, tr, it)
    start = {q: interior_view(st.fields[q]).cpu().numpy().copy() for q in "uvp"}
    start["meta"] = {"dt_prev": st.meta["dt_prev"], "divergence_history": list(st.meta["divergence_history"])}
    chain = ex.submit(J.converged_chain, kw, n, n, 3, start, develop).result()
    worst = {}
    for s in range(3):
        _load(st, chain[s])
        _, _, diag = step(cfg, st, tr, develop + s)
        assert diag["dt"] == chain[s + 1]["dt"]
        assert diag["Rp_converged"]
        for q, e in _errors(st, chain[s + 1]).items():
            worst[q] = max(worst.get(q, 0.0), e)
    print(f"\nmixed vs converged binary64, {n}x{n} Re {Re:g} after {develop} steps: "
          + ", ".join(f"{q} {e:.2e}" for q, e in worst.items()))
    assert max(worst.values()) <= TOL, worst


def test_cavity2048_plain_p1(oracle_work):
    _, futs = oracle_work
    cfg = SimpleNamespace(**cavity_kw(2048, 2048, 3200.0, 1.0, maxiter=20))
    got = gpu_trajectory(cfg, 2048, 2048, 3, keep={1, 2})
    check_records(got, futs["c2048"].result(), "cavity2048")
    assert [r["cg_iterations"] for r in got] == [0, 20, 20]
