"""Seeded random sweep over the problem space of the single-instance path: scheme, theta
scheme, weight zeta, Heston or SABR (with r = 0 or r != 0), time direction, line solver, grid
map and odd or even sizes.  Each problem is solved in reference arithmetic (bit-identical to
the oracle, FP64 and FP32) and in fast arithmetic (FP64 within 1e-10 of the oracle, 1e-6 where
the reference scheme itself blows up).  The oracle is the C restatement pinned to the compiled
reference."""
import numpy as np
import pytest

from conftest import fp64_tol, problem_pair, rel_err

pytestmark = pytest.mark.gpu

SCHEMES = ("dr", "cs", "mcs", "hv")
THETAS = ("cn", "euler", "theta30", "theta80")


def draw(seed):
    r = np.random.default_rng(seed)
    sabr = r.random() < 0.35
    kw = dict(scheme=str(r.choice(SCHEMES)), theta_scheme=str(r.choice(THETAS)),
              zeta=float(r.choice([0.5, 1.0 / 3.0, 0.8])), nx=int(r.integers(4, 70)), ny=int(r.integers(4, 40)),
              nt=int(r.integers(2, 26)), forward=bool(r.random() < 0.3), solver=str(r.choice(["tlu", "ds"])))
    if sabr:
        kw.update(model="sabr", sigma=float(r.uniform(0.2, 0.6)), rho=float(r.uniform(-0.6, 0.3)),
                  sabr_beta=float(r.choice([0.3, 0.5, 0.7])), rate=float(r.choice([0.0, 0.03])), strike=0.05,
                  maturity=float(r.uniform(0.5, 2.0)), s_lo=0.0, s_hi=0.2, v_lo=0.0, v_hi=1.0)
        if r.random() < 0.6:
            kw.update(nonuniform=True, acc_point=0.05, alpha_scale=10.0, beta_scale=24.0)
    else:
        kw.update(model="heston", kappa=float(r.uniform(0.5, 5.0)), theta_v=float(r.uniform(0.01, 0.1)),
                  sigma=float(r.uniform(0.1, 1.0)), rho=float(r.uniform(-0.95, 0.0)), rate=float(r.uniform(0.0, 0.05)),
                  strike=float(r.uniform(80.0, 120.0)), maturity=float(r.uniform(0.25, 2.0)), s_lo=0.0, s_hi=200.0,
                  v_lo=0.0, v_hi=1.2)
        if r.random() < 0.6:
            kw.update(nonuniform=True, acc_point=100.0, alpha_scale=10.0, beta_scale=24.0)
    return kw


@pytest.mark.parametrize("seed", range(64))
def test_random_problem_parity(lss, oracle, seed):
    kw = draw(1000 + seed)
    op, pp = problem_pair(kw)
    want64 = oracle.solve(op, "f64")
    for fp in ("f64", "f32"):
        want = want64 if fp == "f64" else oracle.solve(op, "f32")
        got, _ = lss.ImplicitHestonSolver(pp, precision=fp, arith="reference").solve()
        assert np.array_equal(got, want, equal_nan=True), (kw, fp, rel_err(got, want))
    if np.all(np.isfinite(want64)):
        got, _ = lss.ImplicitHestonSolver(pp, precision="f64", arith="fast").solve()
        assert rel_err(got, want64) < fp64_tol(want64, op.s_hi), (kw, rel_err(got, want64))
