"""Steady-state driver and benchmark harness over the GPU step.

The steady-state driver (src/pyflow/driver/simulation_driver.py) must yield the
reference's payload keys, detect the steady state at the step where the
least-squares slope of log10(Ru) over the window falls below the tolerance
(the same test run on the oracle's Ru series), and stop there.  The harness
(src/pyflow/benchmark/harness.py) keeps the reference's JSON shape.
"""
import numpy as np
import pytest

from oracle import step as ost

pytestmark = pytest.mark.gpu


def test_steady_driver_detects_and_stops_like_the_oracle_series():
    from pyflow_solver_gb300.driver import DriverConfig, PhysicsConfig, SimulationDriver
    phys = PhysicsConfig(Re=100.0, lid_velocity=1.0, lin_tol=1e-8, lin_maxiter=200)
    dcfg = DriverConfig(nx=17, ny=17, max_steps=40, report_interval=1000, steady_window=6, steady_slope_tol=0.08)
    drv = SimulationDriver(dcfg, phys)
    payloads = list(drv.run())
    keys = {"iteration", "state", "residuals", "diagnostics", "divergence_mean", "divergence_mean_free_norm",
            "steady", "steady_slope", "elapsed"}
    assert all(set(p) == keys for p in payloads)
    assert all(p["state"] is drv.state for p in payloads)
    # the same slope test on the oracle twin's Ru series
    tw = ost.allocate_state(17, 17)
    tr = ost.ResidualManager()
    expect = None
    for it in range(40):
        ost.step(phys, tw, tr, it, red="exact")
        ru = tr.ru
        if len(ru) >= 6:
            rec = np.array(ru[-6:])
            if np.all(rec > 0) and abs(float(np.polyfit(np.arange(6), np.log10(rec), 1)[0])) < 0.08:
                expect = it
                break
    assert expect is not None
    assert drv.steady_detected and drv.steady_iteration == expect
    # the device's slope (formed in the step's last kernel) against NumPy's polyfit on the
    # host tracker's series, at every step where the window is full
    ru = drv.tracker.series["Ru"].values
    for p in payloads:
        n = p["iteration"] + 2                      # series entries after this step (seed included)
        if n < 6:
            assert p["steady_slope"] is None
            continue
        rec = np.array(ru[n - 6:n])
        host = float(np.polyfit(np.arange(6), np.log10(rec), 1)[0])
        assert p["steady_slope"] == pytest.approx(host, rel=1e-9, abs=1e-12)
    assert payloads[-1]["steady"] and payloads[-1]["iteration"] == expect and len(payloads) == expect + 1
    # divergence statistics of the last step: central divergence, mean and mean-free norm
    from oracle import ops as oops
    d = oops.divergence_central(ost.interior(tw.fields["u"]), ost.interior(tw.fields["v"]), tw.meta["dx"], tw.meta["dy"])
    assert payloads[-1]["divergence_mean"] == pytest.approx(float(d.mean()), rel=1e-9, abs=1e-15)
    assert payloads[-1]["divergence_mean_free_norm"] == pytest.approx(float(np.linalg.norm(d - d.mean())), rel=1e-9)


def test_harness_json_shape_and_work():
    from pyflow_solver_gb300.benchmark.harness import benchmark
    res = benchmark([16, 24], 3, precision="mixed")
    assert res["benchmark"] == "lid_driven_cavity" and res["steps_requested"] == 3
    for r in res["runs"]:
        assert {"nx", "ny", "steps", "total_time_s", "avg_time_per_step_s", "avg_cg_iterations"} <= set(r)
        assert r["steps"] == 3 and r["avg_true_cg_iterations"] > 0
        assert 0 < r["device_time_s"] <= r["total_time_s"]
    deg = benchmark([16], 2, reference_defaults=True)
    assert deg["runs"][0]["avg_true_cg_iterations"] == 0
