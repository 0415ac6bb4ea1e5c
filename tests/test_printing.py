"""The surface writer reproduces the reference's print format: writing the oracle's surface
(bit-exact with the reference) and parsing it back gives exactly the numbers of the
reference's own outputs/*.txt golden files."""
import os

import numpy as np
import pytest

from cases import GOLDEN

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "reference_outputs.npz"))


def _parse(text):
    lines = [ln for ln in text.splitlines() if ln]
    i = lines.index("SPACE_POINTS_X")
    x = np.array([float(v) for v in lines[i + 1].split(",")])
    j = lines.index("SPACE_POINTS_Y")
    y = np.array([float(v) for v in lines[j + 1].split(",")])
    k = lines.index("VALUES")
    return x, y, np.array([[float(v) for v in ln.split(",")] for ln in lines[k + 1:]])


@pytest.mark.parametrize("name", ["ImplHestonEquationThomasLUSolverCrankNicolson",
                                  "ImplHestonEquationThomasLUSolverHundsdorferVerwerCrankNicolson",
                                  "ImplSABREquationDoubleSweepSolverCrankNicolson"])
def test_writer_round_trips_to_the_reference_golden_text(oracle, name):
    from linear_system_solvers_gb300.printing import format_surface

    p = oracle.Problem(**GOLDEN[name])
    v = oracle.solve(p, "f64")
    x, y = oracle.grid(p, "f64")
    px, py, pv = _parse(format_surface(x, y, v))
    assert np.array_equal(px, GOLD[f"{name}|f64|x"])
    assert np.array_equal(py, GOLD[f"{name}|f64|y"])
    # 6 significant digits: a last-digit flip only where MSVC's and glibc's libm differ in
    # the last bit right at a rounding boundary
    assert np.mean(pv == GOLD[f"{name}|f64|values"]) > 0.999


def test_format_matches_cpp_stream_defaults():
    from linear_system_solvers_gb300.printing import _fmt

    assert [_fmt(v) for v in (0.0, 1.0, 100.0, 123456.0, 1234567.0, 0.0001, 0.00001, -2.5e-7, 200.001, 3.14159265)] == \
        ["0", "1", "100", "123456", "1.23457e+06", "0.0001", "1e-05", "-2.5e-07", "200.001", "3.14159"]
