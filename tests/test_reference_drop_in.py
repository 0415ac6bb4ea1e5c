"""The device path as one more solver policy of the reference itself: the reference's own
implicit_solvers::general_heston_equation (and its builder), compiled from a build-time copy of its
sources with the enumerator tridiagonal_method_enum::GB300ThomasLUSolver and one Device dispatch
branch added (tests/cpp/build_reference_drop_in.sh), solves each case once with its Host
ThomasLUSolver policy and once with the GB300 kernel specialisation
(linear_system_solvers_gb300/cpp/lss_gb300_reference_kernel.hpp): the surfaces must be identical
bit for bit, FP64 and FP32, every splitting, backward and forward, time-dependent SABR coefficients
included (where the reference's scheme itself overflows, a NaN matches any NaN: host and GPU
arithmetic give NaNs of different payload)."""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SCRIPT = os.path.join(ROOT, "tests", "cpp", "build_reference_drop_in.sh")
BIN = os.path.join(ROOT, "oracle", "_ref", "dropin", "reference_drop_in_t")


def test_gb300_policy_inside_the_reference_is_bitwise_its_host_thomas_lu(lss):
    res = subprocess.run(["bash", SCRIPT], capture_output=True, text=True)
    if res.returncode == 3:
        pytest.skip("no build-time copy of the reference sources here: " + res.stderr.strip())
    assert res.returncode == 0, res.stderr[-2000:]
    run = subprocess.run([BIN], capture_output=True, text=True)
    lines = [ln.split() for ln in run.stdout.splitlines() if ln.strip()]
    assert len(lines) == 12, run.stdout + run.stderr
    assert all(flag == "1" for _, flag, _, _ in lines), run.stdout
    assert run.returncode == 0, run.stdout + run.stderr
