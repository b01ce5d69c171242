"""The CG tile autotuner: every tile shape gives the same bits.

The binary64 CG kernel pair comes in three tile shapes (32 x 8, 32 x 16 and
32 x 32 cells per CTA).  Its dot products are exactly rounded, so the tuner may
pick any of them: a step on each shape must equal the oracle twin bit for bit,
and the tuner must report a valid choice with a time for every shape.
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
    us = (ctypes.c_double * 3)()
    _capi.check(lib.pfgb_autotune(h, stream_handle(), ctypes.byref(v), us), "autotune")
    assert v.value in (0, 1, 2)
    assert all(x > 0 for x in us) and us[v.value] == min(us)
    lib.pfgb_destroy(h)
