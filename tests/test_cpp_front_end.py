"""The C++17 front end (linear_system_solvers_gb300/cpp/lss_gb300_heston.hpp): the reference's
own test set-up (general_heston_equation / general_heston_equation_builder with the Heston
lambdas) run on the device policy, compared with the CPU oracle."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from cases import CONFIG1
from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "heston_front_end_t.cpp")
LIBDIR = os.path.join(ROOT, "linear_system_solvers_gb300", "_build")


@pytest.fixture(scope="module")
def front_end_binary(lss):
    out = os.path.join(tempfile.mkdtemp(), "heston_front_end_t")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "linear_system_solvers_gb300", "cpp"), SRC, "-L", LIBDIR, "-llss_adi",
           f"-Wl,-rpath,{LIBDIR}", "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_front_end_compiles_against_the_c_abi(front_end_binary):
    assert os.access(front_end_binary, os.X_OK)
    # wrong argument count is reported, not crashed on
    res = subprocess.run([front_end_binary], capture_output=True, text=True)
    assert res.returncode == 2 and "expected 26 arguments" in res.stderr


def run_front_end(binary, kw, fp, arith, builder, method="tlu", model=None):
    thetas = {"euler": 0, "theta30": 1, "cn": 2, "theta80": 3}
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "v.bin")
        args = [binary, fp, kw["scheme"], str(kw["nx"]), str(kw["ny"]), str(kw["nt"])]
        args += [repr(float(kw[k])) for k in ("kappa", "theta_v", "sigma", "rho", "rate", "strike", "maturity", "s_lo",
                                               "s_hi", "v_lo", "v_hi")]
        args += [repr(float(kw.get("zeta", 0.5))), str(thetas[kw.get("theta_scheme", "cn")]),
                 str(int(kw.get("nonuniform", False))), repr(float(kw.get("acc_point", 0.0))),
                 repr(float(kw.get("alpha_scale", 3.0))), repr(float(kw.get("beta_scale", 50.0))), str(arith),
                 str(builder), method, out]
        if model:
            args.append(model)
        res = subprocess.run(args, capture_output=True, text=True)
        assert res.returncode == 0, res.stderr
        dt = np.float32 if fp == "f32" else np.float64
        return np.fromfile(out, dtype=dt).reshape(kw["nx"], kw["ny"])


NU = dict(nonuniform=True, acc_point=100.0, alpha_scale=10.0, beta_scale=24.0)


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,fp,builder", [("dr", "f64", 0), ("dr", "f32", 1), ("mcs", "f64", 1),
                                                ("cs", "f32", 0), ("hv", "f64", 0)])
def test_front_end_reference_arith_bitwise(front_end_binary, oracle, scheme, fp, builder):
    kw = dict(CONFIG1, scheme=scheme, nx=60, ny=30, nt=41, **(NU if scheme != "dr" else {}))
    got = run_front_end(front_end_binary, kw, fp, arith=1, builder=builder)
    want = oracle.solve(oracle.Problem(**kw), fp)
    assert np.array_equal(got, want, equal_nan=True)


@pytest.mark.gpu
def test_front_end_config1_fast(front_end_binary, oracle):
    from conftest import rel_err

    got = run_front_end(front_end_binary, dict(CONFIG1), "f64", arith=0, builder=0)
    want = oracle.solve(oracle.Problem(**CONFIG1), "f64")
    assert rel_err(got, want) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,fp", [("dr", "f64"), ("mcs", "f32"), ("hv", "f64")])
def test_front_end_double_sweep_policy_bitwise(front_end_binary, oracle, scheme, fp):
    # tridiagonal_method_enum::GB300DoubleSweepSolver against the reference's DoubleSweepSolver
    kw = dict(CONFIG1, scheme=scheme, nx=50, ny=26, nt=31, **(NU if scheme != "dr" else {}))
    got = run_front_end(front_end_binary, kw, fp, arith=1, builder=0, method="ds")
    want = oracle.solve(oracle.Problem(**kw, solver="ds"), fp)
    assert np.array_equal(got, want, equal_nan=True)


@pytest.mark.gpu
@pytest.mark.parametrize("fp", ["f64", "f32"])
def test_front_end_explicit_euler_bitwise(front_end_binary, oracle, fp):
    # explicit_solvers::general_heston_equation with the device explicit Euler scheme
    kw = dict(CONFIG1, scheme="euler", rho=-0.5, nx=30, ny=20, nt=401, maturity=0.25)
    got = run_front_end(front_end_binary, kw, fp, arith=1, builder=0, method="euler")
    want = oracle.solve(oracle.Problem(**kw), fp)
    assert np.array_equal(got, want, equal_nan=True)


SABR_T = dict(model="sabr", kappa=0.0, theta_v=0.0, sigma=0.4, rho=-0.3, sabr_beta=0.5, rate=0.03, strike=0.05,
              maturity=1.0, s_lo=0.0, s_hi=0.2, v_lo=0.0, v_hi=1.0, nonuniform=True, acc_point=0.05, alpha_scale=10.0,
              beta_scale=24.0)


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,fp,arith", [("dr", "f64", 1), ("mcs", "f64", 1), ("hv", "f32", 1), ("cs", "f64", 0)])
def test_front_end_time_dependent_user_lambdas(front_end_binary, oracle, scheme, fp, arith):
    """Coefficient lambdas that change with t (SABR with r != 0: D(t) = exp(-r (T - t)) inside a and
    c) through the reference's general_heston_equation interface: the front end samples them at
    every step's time and the device runs one block of tables per step.  Reference arithmetic is
    bit-identical to the oracle (the reference's own SABR path); the FMA arithmetic within 1e-10."""
    from conftest import rel_err

    kw = dict(SABR_T, scheme=scheme, nx=40, ny=22, nt=26)
    got = run_front_end(front_end_binary, kw, fp, arith=arith, builder=0, model=f"sabr:{kw['sabr_beta']}")
    want = oracle.solve(oracle.Problem(**kw), fp)
    if arith == 1:
        assert np.array_equal(got, want, equal_nan=True), rel_err(got, want)
    else:
        assert rel_err(got, want) < 1e-10
