"""Continuous batching: every request's result is the same alone and in the mix.

A small trace with more requests than slots makes requests wait, enter slots
that others left (the slot's parameters replaced in place) and overlap on the
device with requests admitted earlier; each completed request's final fields
and step count must equal, bit for bit, the same request run alone through the
single-instance step.
"""
import json

import numpy as np
import pytest

from pyflow_solver_gb300.workloads import Request

pytestmark = pytest.mark.gpu

TRACE = [Request(0, 0.0, 32, 150.0, 1.0, 6), Request(1, 0.0, 48, 900.0, 1.6, 4),
         Request(2, 0.0, 32, 2400.0, 0.7, 9), Request(3, 0.0, 32, 400.0, 1.2, 3),
         Request(4, 0.0, 48, 120.0, 0.5, 7), Request(5, 0.0, 32, 3100.0, 1.9, 5)]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_each_request_same_alone_and_in_the_mix(precision):
    from pyflow_solver_gb300.serving import ServingEngine, run_alone
    eng = ServingEngine({32: 2, 48: 1}, precision=precision, lin_maxiter=120)
    rep = eng.run(TRACE, realtime=False, keep_fields=True)
    assert len(rep.completed) == len(TRACE) and rep.in_flight == 0 and rep.queued == 0
    # slots were reused: more requests than slots, all completed
    assert rep.slots == 3
    for s in rep.completed:
        req = TRACE[s.rid]
        st, n = run_alone(req, precision=precision, lin_maxiter=120)
        assert s.steps_done == n == req.steps and s.stop == "steps"
        for f in "uvp":
            np.testing.assert_array_equal(st.fields[f].cpu().numpy(), s.fields[f].cpu().numpy())
    assert rep.cell_updates == sum(r.side ** 2 * r.steps for r in TRACE)
    eng.close()


def test_continuity_early_stop_and_streamed_records():
    from pyflow_solver_gb300.serving import ServingEngine, run_alone
    # tol between the 32x32 continuity after steps 1 and 3 of these requests
    tol = 8e-4
    trace = [Request(0, 0.0, 32, 100.0, 1.0, 40), Request(1, 0.0, 32, 200.0, 1.0, 40)]
    lines = []
    eng = ServingEngine({32: 1}, precision="mixed", continuity_tol=tol, lin_maxiter=120)
    rep = eng.run(trace, realtime=False, sink=lines.append, keep_fields=True)
    assert len(rep.completed) == 2
    for s in rep.completed:
        st, n = run_alone(trace[s.rid], precision="mixed", continuity_tol=tol, lin_maxiter=120)
        assert s.stop == "continuity" and s.steps_done == n < 40
        np.testing.assert_array_equal(st.fields["u"].cpu().numpy(), s.fields["u"].cpu().numpy())
    recs = [json.loads(x) for x in lines]
    assert len(recs) == sum(s.steps_done for s in rep.completed)
    assert all(r["type"] == "step" and "continuity" in r["residuals"] for r in recs)
    assert [r["iteration"] for r in recs if r["request"] == 0] == list(range(rep.completed[0].steps_done))
    eng.close()


def test_requests_retire_on_the_device_steady_test():
    """With a steady window the engine ends a request when the device-side slope test fires
    for its slot; the same request alone, stopped by the reference's host-side test (NumPy
    polyfit of the tracker's Ru series), runs the same number of steps to the same fields."""
    from pyflow_solver_gb300.serving import ServingEngine, run_alone
    W, tol = 6, 0.08
    trace = [Request(0, 0.0, 32, 100.0, 1.0, 80), Request(1, 0.0, 32, 150.0, 0.8, 80),
             Request(2, 0.0, 32, 120.0, 1.2, 80)]
    eng = ServingEngine({32: 2}, precision="fp64", continuity_tol=0.0, lin_maxiter=120, steady_window=W,
                        steady_slope_tol=tol)
    rep = eng.run(trace, realtime=False, keep_fields=True)
    assert len(rep.completed) == 3
    for s in rep.completed:
        st, n = run_alone(trace[s.rid], precision="fp64", continuity_tol=0.0, lin_maxiter=120, steady_window=W,
                          steady_slope_tol=tol)
        assert s.stop == "steady" and s.steps_done == n < 80
        for f in "uvp":
            np.testing.assert_array_equal(st.fields[f].cpu().numpy(), s.fields[f].cpu().numpy())
    eng.close()