"""Pins the 1-D implicit heat oracle (oracle/lss_oracle_1d_impl.h) to the reference (CPU only).

* against the reference's own printed 1-D outputs outputs/*_approx_*.txt (6 significant
  digits; tests/golden/reference_outputs_1d.npz);
* against full-precision solutions of the compiled reference (tests/golden/small_reference_1d.npz,
  made by tests/golden/make_golden_1d.py), every time level;
* against the compiled reference itself (oracle/_ref/ref_driver_1d), bit for bit, where it was built.
"""
import os

import numpy as np
import pytest

from cases_1d import GOLDEN_1D, SMALL_1D
from conftest import rel_err

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "reference_outputs_1d.npz"))
SMALLREF = np.load(os.path.join(HERE, "golden", "small_reference_1d.npz"))
REF_1D = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "ref_driver_1d")


@pytest.mark.parametrize("fp", ["f64", "f32"])
@pytest.mark.parametrize("name", sorted(GOLDEN_1D))
def test_heat1d_oracle_matches_reference_golden(oracle, name, fp):
    kw, every_level = GOLDEN_1D[name]
    p = oracle.Heat1DProblem(**kw)
    v = oracle.solve_1d(p, fp, all_steps=every_level)
    g = GOLD[f"{name}|{fp}|values"]
    assert v.shape == g.shape
    # 6 printed significant digits: half a unit of the 6th digit is 5e-6 relative; the FP32
    # files come from the reference's MSVC build (its float sinh/cosh round differently)
    assert rel_err(v, g) < (6e-6 if fp == "f64" else 2e-5)
    np.testing.assert_allclose(oracle.grid_1d(p, fp), GOLD[f"{name}|{fp}|x"], rtol=6e-6, atol=1e-12)
    if every_level:
        k = (p.t_hi - p.t_lo) / (p.nt - 1)
        np.testing.assert_allclose(p.t_lo + k * np.arange(p.nt), GOLD[f"{name}|{fp}|t"], rtol=6e-6, atol=1e-12)


@pytest.mark.parametrize("key", sorted(SMALL_1D))
def test_heat1d_oracle_matches_compiled_reference_fixtures(oracle, key):
    kw, fp = SMALL_1D[key]
    v = oracle.solve_1d(oracle.Heat1DProblem(**kw), fp, all_steps=True)
    ref = SMALLREF[key]
    assert v.shape == ref.shape
    # identical operation order; only the host libm (sinh/cosh/asinh/exp on x86 vs aarch64)
    # may differ in the last bit
    assert rel_err(v, ref) < (1e-12 if fp == "f64" else 1e-5)


@pytest.mark.skipif(not os.path.exists(REF_1D), reason="compiled reference (oracle/_ref) not built here")
@pytest.mark.parametrize("key", ["bs_put_euler_nonuniform_f32", "heat_robin_robin_cn_f64",
                                 "heat_source_neumann_robin_ds_f64", "advdiff_source_nonuniform_bwd_f64"])
def test_heat1d_oracle_bitwise_vs_live_reference(oracle, key):
    kw, fp = SMALL_1D[key]
    p = oracle.Heat1DProblem(**kw)
    ref, _ = oracle.run_reference_1d(p, fp, all_steps=True)
    assert np.array_equal(oracle.solve_1d(p, fp, all_steps=True), ref)


def test_heat1d_oracle_tables_are_the_solver_inputs(oracle):
    # the tables a tabulated device problem takes: initial condition on the grid, A_ + D_ =
    # 2 lambda a (non-negative diffusion) and time-ordered boundary data
    kw, _ = SMALL_1D["bs_call_cn_bwd_f64"]
    p = oracle.Heat1DProblem(**kw)
    t = oracle.tables_1d(p)
    A, B, D = t["coef"]
    x = oracle.grid_1d(p)
    np.testing.assert_array_equal(t["init"], np.maximum(0.0, x - p.strike))
    assert np.all(A + D >= 0.0) and np.all((A + D)[1:] > 0.0)
    # backward stepping: boundary data at t_hi - k, t_hi - 2k, ...: the discounted upper value
    # V(x_hi) = x_hi - K e^{-r (T - t)} grows towards t = 0
    hi = t["bnd"][:, 2]
    assert np.all(np.diff(hi) > 0)
    assert hi[0] == np.float64(p.x_hi - p.strike * np.exp(-p.rate * (p.t_hi - (p.t_hi - (p.t_hi - p.t_lo) / (p.nt - 1)))))
    assert np.all(t["bnd"][:, 0] == 0.0)
