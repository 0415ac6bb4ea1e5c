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

    return O.Problem(**kw), lss.HestonProblem(**kw)


def rel_err(a, ref):
    """max |a - ref| / max(|ref|, 1e-3 max|ref|) (denominator floor near V = 0)."""
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    return float(np.max(np.abs(a - ref) / den))


def oracle_unstable(ref, s_hi):
    """The reference's CS/MCS schemes blow up on some grids (|V| >> S_max); such runs are
    flagged "oracle unstable" and compared with a looser, stated tolerance."""
    import numpy as np

    ref = np.asarray(ref, dtype=np.float64)
    return (not np.all(np.isfinite(ref))) or float(np.abs(ref).max()) > 10.0 * s_hi


def fp64_tol(ref, s_hi):
    return 1e-6 if oracle_unstable(ref, s_hi) else 1e-10


def fp32_ok(dev32, ref32, ref64):
    """FP32 parity: the device FP32 surface must be about as close to the FP64 oracle as the
    reference's own FP32 run is.  Two FP32 evaluations of the same scheme with different
    rounding sequences differ from each other about as much as each differs from FP64, so the
    bound is 3x the reference's own FP32 error (or 1e-4)."""
    e_dev = rel_err(dev32, ref64)
    e_ref = rel_err(ref32, ref64)
    return e_dev <= max(3.0 * e_ref, 1e-4), e_dev, e_ref
