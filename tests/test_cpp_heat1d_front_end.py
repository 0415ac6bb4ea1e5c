"""The C++17 1-D front end (linear_system_solvers_gb300/cpp/lss_gb300_heat1d.hpp): the reference's
own 1-D test set-ups (general_heat_equation with Black-Scholes / heat lambdas) run on the device
policy, compared with the CPU oracle."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, rel_err

SRC = os.path.join(ROOT, "tests", "cpp", "heat1d_front_end_t.cpp")
LIBDIR = os.path.join(ROOT, "linear_system_solvers_gb300", "_build")


@pytest.fixture(scope="module")
def heat1d_binary(lss):
    out = os.path.join(tempfile.mkdtemp(), "heat1d_front_end_t")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "linear_system_solvers_gb300", "cpp"), SRC, "-L", LIBDIR, "-llss_adi",
           f"-Wl,-rpath,{LIBDIR}", "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_heat1d_front_end_compiles_against_the_c_abi(heat1d_binary):
    res = subprocess.run([heat1d_binary], capture_output=True, text=True)
    assert res.returncode == 2 and "expected 13 arguments" in res.stderr


def run(binary, model, fp, n, nt, theta, fwd, nonuniform, acc, alpha, arith, method, all_steps):
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "v.bin")
        args = [binary, fp, model, str(n), str(nt), theta, str(int(fwd)), str(int(nonuniform)), repr(float(acc)),
                repr(float(alpha)), str(arith), method, str(int(all_steps)), out]
        res = subprocess.run(args, capture_output=True, text=True)
        assert res.returncode == 0, res.stderr
        v = np.fromfile(out, dtype=np.float32 if fp == "f32" else np.float64)
        return v.reshape(nt, n) if all_steps else v


def oracle_problem(oracle, model, n, nt, theta, fwd, nonuniform, acc, alpha, method):
    if model == "bs":
        return oracle.Heat1DProblem(model="bs", n=n, nt=nt, theta_scheme=theta, forward=fwd, nonuniform=nonuniform,
                                    acc_point=acc, alpha_scale=alpha, solver=method)
    return oracle.Heat1DProblem(model="const", diff=1.0, conv=-0.5, react=-0.25, init0=0.3, init1=1.0,
                                lo_kind="neumann", lo_value=0.2, hi_kind="robin", hi_linear=0.4, hi_value=-0.1,
                                has_source=True, src0=0.0, src1=1.0, x_lo=0.0, x_hi=1.0, t_lo=0.0, t_hi=0.1, n=n,
                                nt=nt, theta_scheme=theta, forward=fwd, nonuniform=nonuniform, acc_point=acc,
                                alpha_scale=alpha, solver=method)


CASES = [("bs", "f64", 100, 100, "cn", False, False, 0.0, 3.0, "tlu", True),
         ("bs", "f32", 100, 100, "euler", False, True, 10.0, 3.0, "tlu", False),
         ("bs", "f64", 60, 40, "cn", False, True, 10.0, 3.0, "ds", False),
         ("heat", "f64", 40, 30, "cn", True, True, 0.5, 3.0, "tlu", True),
         ("heat", "f32", 40, 30, "euler", True, False, 0.0, 3.0, "ds", False)]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_heat1d_front_end_reference_arith_bitwise(heat1d_binary, oracle, case):
    model, fp, n, nt, theta, fwd, nu, acc, alpha, method, all_steps = case
    got = run(heat1d_binary, model, fp, n, nt, theta, fwd, nu, acc, alpha, 1, method, all_steps)
    p = oracle_problem(oracle, model, n, nt, theta, fwd, nu, acc, alpha, method)
    want = oracle.solve_1d(p, fp, all_steps=all_steps)
    assert np.array_equal(got, want), rel_err(got, want)


@pytest.mark.gpu
def test_heat1d_front_end_fast(heat1d_binary, oracle):
    got = run(heat1d_binary, "bs", "f64", 100, 100, "cn", False, False, 0.0, 3.0, 0, "tlu", False)
    want = oracle.solve_1d(oracle_problem(oracle, "bs", 100, 100, "cn", False, False, 0.0, 3.0, "tlu"), "f64")
    assert rel_err(got, want) < 1e-10
