import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def lss():
    import linear_system_solvers_gb300 as lss

    lss.load()
    return lss


def problem_pair(kw):
    """Same problem for the oracle and the product (field names are shared)."""
    from oracle import oracle as O
    import linear_system_solvers_gb300 as lss

    okw = dict(kw)
    pkw = {k: v for k, v in kw.items() if k != "solver"}
    return O.Problem(**okw), lss.HestonProblem(**pkw)


def rel_err(a, ref):
    """max |a - ref| / max(|ref|, 1e-3 max|ref|) (denominator floor near V = 0)."""
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    return float(np.max(np.abs(a - ref) / den))
