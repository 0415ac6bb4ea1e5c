"""Host-side checks of the 1-D C-ABI (include/lss_heat1d.h) that need no GPU: invalid problems
are rejected with the documented codes before any device work."""
import ctypes

import numpy as np
import pytest


def _tables(L, n=8, nt=4, **over):
    c = L.LssHeat1DTables()
    c.n, c.nt, c.t_lo, c.t_hi = n, nt, 0.0, 1.0
    c.theta_scheme, c.forward, c.lo_kind, c.hi_kind = L.THETAS["cn"], 1, 0, 0
    keep = [np.zeros((3, n)), np.zeros(n), np.zeros((nt - 1, 4))]
    c.coef, c.initial, c.boundary = (a.ctypes.data for a in keep)
    for k, v in over.items():
        setattr(c, k, v)
    return c, keep


@pytest.mark.parametrize("over,code", [
    (dict(n=3), 1), (dict(nt=1), 1), (dict(theta_scheme=1), 1), (dict(theta_scheme=3), 1), (dict(lo_kind=3), 1),
    (dict(hi_kind=-1), 1), (dict(t_hi=0.0), 1), (dict(coef=None), 1),
])
def test_heat1d_create_rejects_invalid_tables(lss, over, code):
    from linear_system_solvers_gb300 import _lib as L

    c, keep = _tables(L, **over)
    h = ctypes.c_void_p()
    assert L.load().lss_heat1d_batch_create(ctypes.byref(c), 1, L.FP64, L.ARITH_FAST, 0, ctypes.byref(h)) == code
    assert h.value is None
    assert L.load().lss_adi_last_error().decode().startswith("heat1d:")


def test_heat1d_time_dependent_robin_linear_is_unsupported(lss):
    from linear_system_solvers_gb300 import _lib as L

    c, keep = _tables(L, lo_kind=2)
    keep[2][:, 1] = np.linspace(0.1, 0.4, 3)  # linear value changes from step to step
    c.boundary = keep[2].ctypes.data
    h = ctypes.c_void_p()
    rc = L.load().lss_heat1d_batch_create(ctypes.byref(c), 1, L.FP64, L.ARITH_REFERENCE, 0, ctypes.byref(h))
    assert rc == L.EUNSUPPORTED
    assert "Robin" in L.load().lss_adi_last_error().decode()


@pytest.mark.parametrize("prec,arith,opts,count", [(5, 0, 0, 1), (0, 4, 0, 1), (0, 0, 8, 1), (0, 0, 0, 0)])
def test_heat1d_create_rejects_invalid_batch_arguments(lss, prec, arith, opts, count):
    from linear_system_solvers_gb300 import _lib as L

    q = lss.BlackScholesProblem().to_c()
    h = ctypes.c_void_p()
    assert L.load().lss_heat1d_batch_create_bs(ctypes.byref(q), count, prec, arith, opts, ctypes.byref(h)) == 1
    assert h.value is None


@pytest.mark.parametrize("field,value", [("n", 3), ("nt", 1), ("sigma", 0.0), ("maturity", -1.0), ("s_hi", -1.0)])
def test_black_scholes_create_rejects_invalid_problem(lss, field, value):
    from linear_system_solvers_gb300 import _lib as L

    q = lss.BlackScholesProblem().to_c()
    setattr(q, field, value)
    h = ctypes.c_void_p()
    assert L.load().lss_heat1d_batch_create_bs(ctypes.byref(q), 1, L.FP64, L.ARITH_FAST, 0, ctypes.byref(h)) == 1


def test_python_front_end_validates_before_the_device(lss):
    with pytest.raises(ValueError):
        lss.GeneralHeatEquation1D(a=lambda t, x: 1.0, b=lambda t, x: 0.0, c=lambda t, x: 0.0, initial=lambda x: x,
                                  boundary=(lss.Dirichlet(lambda t: 0.0), lss.Dirichlet(lambda t: 0.0)),
                                  space=(0.0, 1.0), n=3, time=(0.0, 1.0), nt=10)
    with pytest.raises(ValueError, match="time-invariant"):
        lss.GeneralHeatEquation1D(a=lambda t, x: 1.0 + t, b=lambda t, x: 0.0, c=lambda t, x: 0.0,
                                  initial=lambda x: x,
                                  boundary=(lss.Dirichlet(lambda t: 0.0), lss.Dirichlet(lambda t: 0.0)),
                                  space=(0.0, 1.0), n=10, time=(0.0, 1.0), nt=10)
    with pytest.raises(ValueError):
        lss.BlackScholesProblem(theta_scheme="theta30").to_c()


def test_draw_black_scholes_is_seeded(lss):
    a = lss.draw_black_scholes(16, seed=1)
    b = lss.draw_black_scholes(16, seed=1)
    assert a == b
    assert {q.n for q in lss.draw_black_scholes(200)} <= {128, 256, 384, 512}
