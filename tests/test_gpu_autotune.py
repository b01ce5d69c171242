"""The launch-shape autotuner: every shape gives the same bits.

The binary64 CG kernel pair comes in three tile shapes (32 x 8, 32 x 16 and
32 x 32 cells per CTA).  Its dot products are exactly rounded, so the tuner may
pick any of them: a step on each shape must equal the oracle twin bit for bit,
and the tuner must report a valid choice with a time for every shape.

The mixed solve comes in up to four launch variants (the TMA or the tile matvec,
1024- or 512-thread coarse CTAs); each must give the bits of the others, and
tuning in the middle of a run must leave the run's results unchanged.
"""
import ctypes
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import step as ost

pytestmark = pytest.mark.gpu


def cfg():
    return SimpleNamespace(nx=70, ny=45, lx=1.0, ly=1.0, Re=400.0, lid_velocity=1.0, advection_scheme="quick",
                           cfl_target=0.5, cfl_growth=1.05, lin_tol=1e-8, lin_maxiter=150, diagnostics=False)


def test_every_tile_shape_matches_the_twin():
    import torch

    from pyflow_solver_gb300 import ResidualManager, _capi, allocate_state, interior_view, step
    from pyflow_solver_gb300.solvers._handle import instance_for
    from pyflow_solver_gb300.solvers.solver import step_params
    c = cfg()
    tw = ost.allocate_state(c.nx, c.ny)
    ttr = ost.ResidualManager()
    for it in range(3):
        ost.step(c, tw, ttr, it, red="exact")
    ref = [ost.interior(tw.fields[k]) for k in "uvp"]
    lib = _capi.load()
    for v in range(3):
        st = allocate_state(c.nx, c.ny)
        P, *_ = step_params(c, c.nx, c.ny)
        inst = instance_for(st, P)
        _capi.check(lib.pfgb_set_cg_variant(inst.handle, v), "set_cg_variant")
        tr = ResidualManager()
        for it in range(3):
            step(c, st, tr, it)
        for k, r in zip("uvp", ref):
            np.testing.assert_array_equal(interior_view(st.fields[k]).cpu().numpy(), r)
    torch.cuda.synchronize()


def test_autotune_reports_a_choice():
    from pyflow_solver_gb300 import _capi
    from pyflow_solver_gb300._device import stream_handle
    from pyflow_solver_gb300.solvers.solver import step_params
    c = cfg()
    P, *_ = step_params(c, c.nx, c.ny)
    lib = _capi.load()
    h = ctypes.c_void_p()
    _capi.check(lib.pfgb_create(ctypes.byref(P), ctypes.byref(h)), "create")
    v = ctypes.c_int(-1)
    us = (ctypes.c_double * 4)()
    _capi.check(lib.pfgb_autotune(h, stream_handle(), ctypes.byref(v), us), "autotune")
    assert v.value in (0, 1, 2)
    assert all(x > 0 for x in us[:3]) and us[v.value] == min(us[:3])
    lib.pfgb_destroy(h)


MIXED = [(128, 96, 700.0, 1.2), (64, 64, 150.0, 1.0), (96, 48, 2500.0, 0.8), (256, 128, 1200.0, 1.5)]


def _mixed_batch():
    from pyflow_solver_gb300 import allocate_state
    from pyflow_solver_gb300.batch import BatchedCavities
    cfgs = []
    for nx, ny, Re, U in MIXED:
        c = cfg()
        c.nx, c.ny, c.Re, c.lid_velocity, c.precision = nx, ny, Re, U, "mixed"
        cfgs.append(c)
    return BatchedCavities(cfgs, [allocate_state(c.nx, c.ny) for c in cfgs])


def _same_records(a, b, what):
    for name in a.dtype.names:          # field by field (the records' padding bytes are not data)
        np.testing.assert_array_equal(a[name], b[name], err_msg=f"{what}: {name}")


def _run(B, steps):
    from pyflow_solver_gb300 import interior_view
    recs = [B.step_arrays().copy() for _ in range(steps)]
    return recs, [[interior_view(st.fields[k]).cpu().numpy().copy() for k in "uvp"] for st in B.states]


def test_mixed_launch_variants_same_bits_and_tuning_keeps_the_run():
    from pyflow_solver_gb300 import _capi
    from pyflow_solver_gb300._device import stream_handle
    from pyflow_solver_gb300.solvers import _handle
    lib = _capi.load()
    _handle.AUTOTUNE = False
    try:
        ref_B = _mixed_batch()
        ref_recs, ref_fields = _run(ref_B, 6)
        ref_B.close()
        ran = []
        for v in range(4):
            B = _mixed_batch()
            if lib.pfgb_set_mixed_variant(B._h, v) != 0:      # not runnable for this batch
                B.close()
                continue
            ran.append(v)
            recs, fields = _run(B, 6)
            for a, b in zip(recs, ref_recs):
                _same_records(a, b, f"variant {v}")
            for fa, fb in zip(fields, ref_fields):
                for x, y in zip(fa, fb):
                    np.testing.assert_array_equal(x, y)
            B.close()
        assert 0 in ran and len(ran) >= 2
        # tuning after three steps: the next three steps are those of the untuned run
        B = _mixed_batch()
        recs = [B.step_arrays().copy() for _ in range(3)]
        v = ctypes.c_int(-1)
        us = (ctypes.c_double * 4)()
        _capi.check(lib.pfgb_autotune(B._h, stream_handle(), ctypes.byref(v), us), "autotune")
        assert v.value in ran and us[v.value] > 0 and all((us[k] > 0) == (k in ran) for k in range(4))
        recs += [B.step_arrays().copy() for _ in range(3)]
        for a, b in zip(recs, ref_recs):
            _same_records(a, b, "tuned mid-run")
        B.close()
    finally:
        _handle.AUTOTUNE = True
