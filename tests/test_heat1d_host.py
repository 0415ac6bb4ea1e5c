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


def test_python_front_end_tables_are_the_reference_tables(lss, oracle):
    """GeneralHeatEquation1D samples the user's callables as the reference does (grid map,
    coefficient and boundary transforms, time sequence of the loop): its tables equal the
    oracle's bit for bit in FP64, so a device run from them is the reference's run."""
    import math

    from cases_1d import SMALL_1D

    # the reference's Black-Scholes test problem
    sig, r, K, T = 0.25, 0.2, 10.0, 1.0
    eq = lss.GeneralHeatEquation1D(
        a=lambda t, x: 0.5 * sig * sig * x * x, b=lambda t, x: r * x, c=lambda t, x: -r,
        initial=lambda x: max(0.0, x - K),
        boundary=(lss.Dirichlet(lambda t: 0.0), lss.Dirichlet(lambda t: 20.0 - K * math.exp(-r * (T - t)))),
        space=(0.0, 20.0), n=100, time=(0.0, T), nt=100, theta_scheme="cn", forward=False)
    want = oracle.tables_1d(oracle.Heat1DProblem())
    got = eq._tables
    assert np.array_equal(got["coef"], want["coef"])
    assert np.array_equal(got["initial"], want["init"])
    assert np.array_equal(got["boundary"], want["bnd"])
    np.testing.assert_array_equal(eq.grid(), oracle.grid_1d(oracle.Heat1DProblem()))
    # Neumann / Robin ends, a heat source, a sinh grid, backward stepping
    for key in ("heat_source_neumann_robin_ds_f64", "advdiff_source_nonuniform_bwd_f64", "heat_robin_robin_cn_f64"):
        kw, _ = SMALL_1D[key]
        p = oracle.Heat1DProblem(**kw)
        kinds = {"dirichlet": lambda v, l: lss.Dirichlet(lambda t: v), "neumann": lambda v, l: lss.Neumann(lambda t: v),
                 "robin": lambda v, l: lss.Robin(lambda t: l, lambda t: v)}
        eq = lss.GeneralHeatEquation1D(
            a=lambda t, x: p.diff, b=lambda t, x: p.conv, c=lambda t, x: p.react,
            initial=lambda x: p.init0 + p.init1 * x,
            source=(lambda t, x: p.src0 + p.src1 * x) if p.has_source else None,
            boundary=(kinds[p.lo_kind](p.lo_value, p.lo_linear), kinds[p.hi_kind](p.hi_value, p.hi_linear)),
            space=(p.x_lo, p.x_hi), n=p.n, time=(p.t_lo, p.t_hi), nt=p.nt, theta_scheme=p.theta_scheme,
            forward=p.forward, nonuniform=p.nonuniform, acc_point=p.acc_point, alpha_scale=p.alpha_scale)
        want = oracle.tables_1d(p)
        got = eq._tables
        assert np.array_equal(got["coef"], want["coef"]), key
        assert np.array_equal(got["initial"], want["init"]), key
        assert np.array_equal(got["boundary"], want["bnd"]), key
        if p.has_source:
            assert np.array_equal(got["source"], want["src"]), key
