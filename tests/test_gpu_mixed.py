"""Mixed-precision step (P3): binary32 multigrid-PCG inside binary64 refinement.

The reference's own CG stops at lin_maxiter far from the solution of its
pressure system (relative residual ~0.3 at 512x512 after 300 iterations), so
the mixed form is checked against the *converged* binary64 solution of the same
system: the oracle step with the CG replaced by a sparse direct solve.  The
bar is 1e-6 relative error (max |gpu - oracle| / max |oracle|) in u, v and p,
step by step from the same state and along short trajectories.
"""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import step as ost

pytestmark = pytest.mark.gpu

TOL = 1e-6


def cavity(nx, ny, Re, lid, **kw):
    c = SimpleNamespace(nx=nx, ny=ny, lx=1.0, ly=1.0, Re=Re, lid_velocity=lid, advection_scheme="quick",
                        cfl_target=0.5, cfl_growth=1.05, lin_tol=1e-8, lin_maxiter=300, diagnostics=False)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def run_pair(cfg, steps):
    import torch

    from pyflow_solver_gb300 import ResidualManager, allocate_state, interior_view, step
    gcfg = SimpleNamespace(**vars(cfg), precision="mixed")
    ocfg = SimpleNamespace(**vars(cfg), oracle_pressure="converged")
    st = allocate_state(cfg.nx, cfg.ny)
    tw = ost.allocate_state(cfg.nx, cfg.ny)
    tr, otr = ResidualManager(), ost.ResidualManager()
    worst = {"u": 0.0, "v": 0.0, "p": 0.0}
    diags = []
    for it in range(steps):
        # per-step parity: start the GPU step from the oracle's state
        for k in "uvp":
            interior_view(st.fields[k]).copy_(torch.from_numpy(ost.interior(tw.fields[k])))
        st.meta = {"dt_prev": tw.meta.get("dt_prev", 1e-2), "divergence_history": list(tw.meta.get("divergence_history", []))}
        _, res, diag = step(gcfg, st, tr, it)
        _, ores, odiag = ost.step(ocfg, tw, otr, it, red="exact")
        assert diag["dt"] == odiag["dt"]
        for k in "uvp":
            got = interior_view(st.fields[k]).cpu().numpy()
            ref = ost.interior(tw.fields[k])
            if np.max(np.abs(ref)) > 0:
                worst[k] = max(worst[k], rel(got, ref))
        diags.append(diag)
    return worst, diags


@pytest.mark.parametrize("nx,ny,Re,lid,steps,scheme", [(64, 64, 100.0, 1.0, 12, "quick"), (96, 48, 800.0, 1.5, 6, "quick"),
                                                      (128, 128, 1000.0, 1.0, 4, "quick"),
                                                      (80, 64, 300.0, 1.2, 6, "upwind")])
def test_mixed_step_matches_converged_fp64(nx, ny, Re, lid, steps, scheme):
    worst, diags = run_pair(cavity(nx, ny, Re, lid, advection_scheme=scheme), steps)
    assert max(worst.values()) <= TOL, worst
    for d in diags[1:]:
        assert d["Rp_converged"], d
        assert d["cg_iterations"] > 0


@pytest.mark.slow
def test_mixed_step_512_matches_converged_fp64():
    worst, diags = run_pair(cavity(512, 512, 1000.0, 1.0), 3)
    assert max(worst.values()) <= TOL, worst


def test_mixed_trajectory_stays_close():
    """Free-running trajectories (no resynchronisation) of GPU mixed and converged oracle:
    u, v and p after 20 steps within the 1e-6 bar."""
    from pyflow_solver_gb300 import ResidualManager, SimulationDriver, allocate_state, interior_view
    cfg = cavity(64, 64, 100.0, 1.0)
    gcfg = SimpleNamespace(**vars(cfg), precision="mixed")
    ocfg = SimpleNamespace(**vars(cfg), oracle_pressure="converged")
    st = allocate_state(64, 64)
    for _ in SimulationDriver(gcfg, st, ResidualManager()).run(max_steps=20):
        pass
    tw = ost.allocate_state(64, 64)
    for _ in ost.run(ocfg, tw, max_steps=20, red="exact"):
        pass
    errs = {k: rel(interior_view(st.fields[k]).cpu().numpy(), ost.interior(tw.fields[k])) for k in "uvp"}
    print("\nfree-running 20 steps, 64x64 Re 100, mixed vs converged binary64: "
          + ", ".join(f"{k} {e:.2e}" for k, e in errs.items()))
    assert max(errs.values()) <= TOL, errs


def test_mixed_warm_start_and_fallback():
    """The refinement starts from the state's pressure.  A guess worse than zero (noise, or a
    NaN) falls back to the cold start and gives its bits exactly; a good guess (the pressure
    of the previous step) gives the cold start's fields within the mixed tolerance."""
    import torch

    from pyflow_solver_gb300 import ResidualManager, SimulationDriver, allocate_state, interior_view, step
    nx, ny = 96, 64
    base = cavity(nx, ny, 600.0, 1.0, precision="mixed")
    st0 = allocate_state(nx, ny)
    for _ in SimulationDriver(base, st0, ResidualManager()).run(max_steps=6):
        pass

    def run(p_fill, warm):
        st = allocate_state(nx, ny)
        for k in "uvp":
            st.fields[k].copy_(st0.fields[k])
        if p_fill is not None:
            p_fill(interior_view(st.fields["p"]))
        st.meta = {"dt_prev": st0.meta["dt_prev"], "divergence_history": list(st0.meta["divergence_history"])}
        cfg = SimpleNamespace(**vars(base), mixed_warm_start=warm)
        _, res, diag = step(cfg, st, ResidualManager(), 6)
        return [interior_view(st.fields[k]).cpu().numpy() for k in "uvp"], res, diag

    g = torch.Generator(device="cpu").manual_seed(3)
    noise = (1e3 * torch.randn(ny, nx, generator=g, dtype=torch.float64))

    def fill_noise(pi):
        pi.copy_(noise.to(pi.device))

    def fill_nan(pi):
        pi[ny // 2, nx // 3] = float("nan")

    cold = run(None, False)
    for fill in (fill_noise, fill_nan):
        fb = run(fill, True)
        for a, b in zip(cold[0], fb[0]):
            np.testing.assert_array_equal(a, b)
        assert fb[1] == cold[1] and fb[2] == cold[2]
    warm = run(None, True)
    assert warm[2]["Rp_converged"]
    assert warm[2]["cg_iterations"] <= cold[2]["cg_iterations"]
    for a, b in zip(warm[0], cold[0]):
        assert rel(a, b) <= TOL


@pytest.mark.parametrize("nx,ny,Re", [(512, 512, 1000.0), (320, 448, 400.0)])
def test_interior_tile_forms_same_bits(nx, ny, Re, monkeypatch):
    """Tiles away from the walls run the interior forms of the phases (no per-cell wall
    logic); with those turned off (every tile through the general forms) the bits are the
    same."""
    from pyflow_solver_gb300 import ResidualManager, allocate_state, interior_view, step
    cfg = cavity(nx, ny, Re, 1.0, precision="mixed")
    runs = []
    for flag in ("1", "0"):
        monkeypatch.setenv("PFGB_TILE_INTERIOR", flag)
        st = allocate_state(nx, ny)
        tr = ResidualManager()
        diags = [step(cfg, st, tr, it)[2] for it in range(3)]
        runs.append(([interior_view(st.fields[k]).cpu().numpy() for k in "uvp"], diags))
    for a, b in zip(runs[0][0], runs[1][0]):
        np.testing.assert_array_equal(a, b)
    assert runs[0][1] == runs[1][1]


@pytest.mark.parametrize("nx,ny,Re", [(512, 512, 1000.0), (200, 136, 400.0)])
def test_tma_matvec_same_bits(nx, ny, Re, monkeypatch, capfd):
    """The TMA form of the kernel graph's matvec (PFGB_MATVEC_TMA=1: persistent over the
    tiles, each tile's halo copied by TMA in a box widened to start on a 16-byte boundary,
    zeros outside the grid) gives the bits of the default one-tile-per-CTA matvec, on a
    grid whose edge tiles are ragged as well."""
    from pyflow_solver_gb300 import ResidualManager, allocate_state, interior_view, step
    cfg = cavity(nx, ny, Re, 1.0, precision="mixed")
    monkeypatch.setenv("PFGB_GRAPH_DEBUG", "1")
    runs = []
    for flag in ("1", "0"):
        monkeypatch.setenv("PFGB_MATVEC_TMA", flag)
        st = allocate_state(nx, ny)
        tr = ResidualManager()
        diags = [step(cfg, st, tr, it)[2] for it in range(4)]
        runs.append(([interior_view(st.fields[k]).cpu().numpy() for k in "uvp"], diags))
    err = capfd.readouterr().err
    assert err.index("TMA matvec on") < err.index("TMA matvec off"), err
    assert all(d["Rp_converged"] for d in runs[0][1][1:])
    for a, b in zip(runs[0][0], runs[1][0]):
        np.testing.assert_array_equal(a, b)
    assert runs[0][1] == runs[1][1]


def test_tma_matvec_chosen_by_batch_shape(monkeypatch, capfd):
    """Without PFGB_MATVEC_TMA the TMA matvec is taken where a CTA gets several tiles of one
    instance (a 2048 x 2048 cavity: 4096 tiles) and not where it gets about one (512 x 512:
    256 tiles)."""
    from pyflow_solver_gb300 import ResidualManager, allocate_state, step
    monkeypatch.delenv("PFGB_MATVEC_TMA", raising=False)
    monkeypatch.setenv("PFGB_GRAPH_DEBUG", "1")
    seen = {}
    for n in (2048, 512):
        capfd.readouterr()
        st = allocate_state(n, n)
        step(cavity(n, n, 1000.0, 1.0, precision="mixed"), st, ResidualManager(), 0)
        err = capfd.readouterr().err
        seen[n] = "TMA matvec on" in err
        del st
    assert seen == {2048: True, 512: False}


def test_loop_guard_stops_the_inner_loop_at_its_bound(monkeypatch):
    """The guard run by the last CTA of each loop body's last kernel stops a loop at its trip
    bound and the step reports it.  The bound is set below what the solve needs on the host
    (a test setting); nothing faults on the device, and a new instance steps normally."""
    from pyflow_solver_gb300 import ResidualManager, _capi, allocate_state, step
    cfg = cavity(64, 64, 400.0, 1.0, precision="mixed")
    monkeypatch.setenv("PFGB_TEST_LOOP_BOUND", "2")
    st = allocate_state(64, 64)
    tr = ResidualManager()
    step(cfg, st, tr, 0)                        # zero right-hand side: no loop runs
    with pytest.raises(_capi.PFGBError, match="loop guard"):
        step(cfg, st, tr, 1)
    monkeypatch.delenv("PFGB_TEST_LOOP_BOUND")
    st2 = allocate_state(64, 64)
    tr2 = ResidualManager()
    diags = [step(cfg, st2, tr2, it)[2] for it in range(3)]
    assert all(d["Rp_converged"] for d in diags[1:])


def test_mixed_graph_and_direct_launches_agree():
    """The graph (device-side loop control) and the host-driven direct form give the same bits."""
    from pyflow_solver_gb300 import ResidualManager, SimulationDriver, allocate_state, interior_view
    from pyflow_solver_gb300.solvers import _handle
    cfg = SimpleNamespace(**vars(cavity(64, 48, 400.0, 1.0)), precision="mixed")
    out = []
    for mode in (True, False, 2):          # graph with programmatic edges, direct, plain graph
        _handle.GRAPH_MODE = mode
        try:
            st = allocate_state(64, 48)
            diags = [d for _, _, d in SimulationDriver(cfg, st, ResidualManager()).run(max_steps=4)]
        finally:
            _handle.GRAPH_MODE = True
        out.append(([interior_view(st.fields[k]).cpu().numpy() for k in "uvp"],
                    [(d["cg_iterations"], d["refine_passes"], d["dt"]) for d in diags]))
    for o in out[1:]:
        for a, b in zip(out[0][0], o[0]):
            np.testing.assert_array_equal(a, b)
    assert out[0][1] == out[1][1]


def test_persistent_solve_equals_kernel_graph():
    """The persistent cooperative solve and the graph of per-phase kernels give the same bits."""
    from pyflow_solver_gb300 import ResidualManager, _capi, allocate_state, interior_view, step
    from pyflow_solver_gb300.solvers._handle import instance_for
    from pyflow_solver_gb300.solvers.solver import step_params
    lib = _capi.load()
    for nx, ny in ((96, 64), (128, 128), (48, 40)):
        cfg = cavity(nx, ny, 700.0, 1.3, precision="mixed")
        runs = []
        for persistent in (1, 0):
            st = allocate_state(nx, ny)
            P, *_ = step_params(cfg, nx, ny)
            _capi.check(lib.pfgb_set_persistent(instance_for(st, P).handle, persistent), "set_persistent")
            tr = ResidualManager()
            diags = [step(cfg, st, tr, it)[2] for it in range(4)]
            runs.append(([interior_view(st.fields[k]).cpu().numpy() for k in "uvp"], diags))
        for a, b in zip(runs[0][0], runs[1][0]):
            np.testing.assert_array_equal(a, b)
        assert runs[0][1] == runs[1][1]


def test_persistent_groups_taking_several_tiles():
    """At 2048 x 2048 the persistent solve's four groups per CTA take several tiles of level 0
    and of level 1 in turn (more tiles than groups); the bits equal the kernel graph's."""
    from pyflow_solver_gb300 import ResidualManager, _capi, allocate_state, interior_view, step
    from pyflow_solver_gb300.solvers._handle import instance_for
    from pyflow_solver_gb300.solvers.solver import step_params
    lib = _capi.load()
    cfg = cavity(2048, 2048, 1000.0, 1.0, precision="mixed")
    runs = []
    for persistent in (1, 0):
        st = allocate_state(2048, 2048)
        P, *_ = step_params(cfg, 2048, 2048)
        _capi.check(lib.pfgb_set_persistent(instance_for(st, P).handle, persistent), "set_persistent")
        tr = ResidualManager()
        diags = [step(cfg, st, tr, it)[2] for it in range(3)]
        runs.append(([interior_view(st.fields[k]).cpu().numpy() for k in "uvp"], diags))
    for a, b in zip(runs[0][0], runs[1][0]):
        np.testing.assert_array_equal(a, b)
    assert runs[0][1] == runs[1][1]


def test_mixed_error_report_fields_and_centerline(capsys):
    """Worst relative error of the mixed step against the converged binary64 oracle, per
    field and for the u centerline (u[:, nx // 2], the driver's u_centerline), step by step
    from the same state."""
    import torch

    from pyflow_solver_gb300 import ResidualManager, allocate_state, interior_view, step
    report = {}
    for nx, ny, Re in ((64, 64, 100.0), (128, 128, 1000.0)):
        cfg = cavity(nx, ny, Re, 1.0)
        gcfg = SimpleNamespace(**vars(cfg), precision="mixed")
        ocfg = SimpleNamespace(**vars(cfg), oracle_pressure="converged")
        st = allocate_state(nx, ny)
        tw = ost.allocate_state(nx, ny)
        tr, otr = ResidualManager(), ost.ResidualManager()
        worst = {"u": 0.0, "v": 0.0, "p": 0.0, "u_centerline": 0.0}
        for it in range(6):
            for k in "uvp":
                interior_view(st.fields[k]).copy_(torch.from_numpy(ost.interior(tw.fields[k])))
            st.meta = {"dt_prev": tw.meta.get("dt_prev", 1e-2),
                       "divergence_history": list(tw.meta.get("divergence_history", []))}
            step(gcfg, st, tr, it)
            ost.step(ocfg, tw, otr, it, red="exact")
            for k in "uvp":
                got, ref = interior_view(st.fields[k]).cpu().numpy(), ost.interior(tw.fields[k])
                if np.max(np.abs(ref)) > 0:
                    worst[k] = max(worst[k], rel(got, ref))
            gu, ou = interior_view(st.fields["u"]).cpu().numpy()[:, nx // 2], ost.interior(tw.fields["u"])[:, nx // 2]
            if np.max(np.abs(ou)) > 0:
                worst["u_centerline"] = max(worst["u_centerline"], rel(gu, ou))
        report[f"{nx}x{ny} Re {Re:g}"] = worst
    with capsys.disabled():
        for k, w in report.items():
            print(f"\nmixed vs converged binary64, {k}: " + ", ".join(f"{f} {e:.2e}" for f, e in w.items()))
    assert all(e <= TOL for w in report.values() for e in w.values()), report
