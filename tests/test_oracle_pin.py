"""Pins the CPU oracle (oracle/lss_oracle.c) to the reference (CPU, no GPU needed).

* against the reference's own golden surfaces outputs/*.txt (6 significant digits);
* against full-precision surfaces of the compiled reference (tests/golden/small_reference.npz,
  made by tests/golden/make_golden.py);
* against the compiled reference itself (oracle/_ref), bit for bit, where it was built.
"""
import os

import numpy as np
import pytest

from cases import CONFIG1, GOLDEN, SMALL
from conftest import rel_err

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "reference_outputs.npz"))
SMALLREF = np.load(os.path.join(HERE, "golden", "small_reference.npz"))

GOLDEN_FP64 = [n for n in GOLDEN if f"{n}|f64|values" in GOLD.files]
GOLDEN_FP32 = [n for n in GOLDEN if f"{n}|f32|values" in GOLD.files]


@pytest.mark.parametrize("name", GOLDEN_FP64)
def test_oracle_matches_reference_golden_fp64(oracle, name):
    p = oracle.Problem(**GOLDEN[name])
    v = oracle.solve(p, "f64")
    g = GOLD[f"{name}|f64|values"]
    assert v.shape == g.shape
    # the files hold 6 significant digits: half a unit of the 6th digit is 5e-6 relative
    assert rel_err(v, g) < 6e-6
    x, y = oracle.grid(p, "f64")
    np.testing.assert_allclose(x, GOLD[f"{name}|f64|x"], rtol=6e-6, atol=1e-12)
    np.testing.assert_allclose(y, GOLD[f"{name}|f64|y"], rtol=6e-6, atol=1e-12)


@pytest.mark.parametrize("name", GOLDEN_FP32)
def test_oracle_matches_reference_golden_fp32(oracle, name):
    # The FP32 files were written by the reference's MSVC build, whose float sinhf/coshf/
    # asinhf round differently from glibc's; the Thomas sweeps amplify those last-bit
    # differences to ~5e-4 relative (same denominator floor as everywhere).
    p = oracle.Problem(**GOLDEN[name])
    v = oracle.solve(p, "f32")
    assert rel_err(v, GOLD[f"{name}|f32|values"]) < 1e-3


@pytest.mark.parametrize("key", sorted(SMALL))
def test_oracle_matches_compiled_reference_fixtures(oracle, key):
    kw, fp = SMALL[key]
    v = oracle.solve(oracle.Problem(**kw), fp)
    ref = SMALLREF[key]
    # identical operation order; only the host libm (x86 vs aarch64 sinh/cosh/asinh) may
    # differ in the last bit
    tol = 1e-12 if fp == "f64" else 1e-4
    assert rel_err(v, ref) < tol


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref", "ref_driver")),
                    reason="compiled reference (oracle/_ref) not built here")
@pytest.mark.parametrize("scheme,fp", [("dr", "f64"), ("mcs", "f32"), ("hv", "f64")])
def test_oracle_bitwise_vs_live_reference(oracle, scheme, fp):
    kw = dict(CONFIG1, scheme=scheme, nx=40, ny=24, nt=21, nonuniform=True, acc_point=100.0, alpha_scale=10.0,
              beta_scale=24.0)
    p = oracle.Problem(**kw)
    ref, _ = oracle.run_reference(p, fp)
    assert np.array_equal(oracle.solve(p, fp), ref)


def test_index_of_remaps_match_reference_quirk(oracle):
    # grid_config::index_of truncates (step*j)/step: 4 of 100 S indices and 2 of 50 v indices
    # map to j-1 in FP64 (and 8 / 3 in FP32)
    p = oracle.Problem(**CONFIG1)
    im, jm = oracle.index_maps(p, "f64")
    assert np.count_nonzero(im != np.arange(p.nx)) == 4
    assert np.count_nonzero(jm != np.arange(p.ny)) == 2
    assert np.all((im == np.arange(p.nx)) | (im == np.arange(p.nx) - 1))
    im32, jm32 = oracle.index_maps(p, "f32")
    assert np.count_nonzero(im32 != np.arange(p.nx)) == 8
    assert np.count_nonzero(jm32 != np.arange(p.ny)) == 3


def test_mcs_equals_cs_when_zeta_equals_theta(oracle):
    kw = dict(CONFIG1, nx=30, ny=20, nt=21, nonuniform=True, acc_point=100.0, alpha_scale=10.0, beta_scale=24.0)
    cs = oracle.solve(oracle.Problem(**dict(kw, scheme="cs")))
    mcs = oracle.solve(oracle.Problem(**dict(kw, scheme="mcs")))
    assert np.array_equal(cs, mcs)


def test_oracle_rejects_invalid(oracle):
    for bad in (dict(nx=3), dict(ny=2), dict(nt=1), dict(s_hi=-1.0)):
        with pytest.raises(ValueError):
            oracle.solve(oracle.Problem(**dict(CONFIG1, **bad)))
