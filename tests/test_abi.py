"""C-ABI library checks that need no GPU: it builds, loads, exports every declared symbol
and rejects invalid problems before touching the device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for header in ("lss_adi.h", "lss_heat1d.h"):
        src = open(os.path.join(ROOT, "include", header)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(lss_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_library_exports_every_declared_symbol(lss):
    from linear_system_solvers_gb300 import _lib

    lib = ctypes.CDLL(_lib.lib_path())
    names = declared_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)
    assert lib.lss_adi_abi_version() == 1


@pytest.mark.parametrize("bad,code", [
    (dict(nx=3), 1), (dict(ny=3), 1), (dict(nt=1), 1), (dict(scheme_id=7), 1), (dict(theta_id=9), 1),
    (dict(s_hi=-5.0), 1), (dict(maturity=0.0), 1), (dict(precision_id=5), 1), (dict(model_id=3), 1),
    (dict(kappa=float("nan")), 1), (dict(options=64), 1),
])
def test_create_rejects_invalid_problem_without_device(lss, bad, code):
    from linear_system_solvers_gb300 import _lib as L

    p = lss.HestonProblem()
    c = p.to_c()
    for k, v in bad.items():
        if k == "scheme_id":
            c.scheme = v
        elif k == "theta_id":
            c.theta_scheme = v
        elif k == "precision_id":
            c.precision = v
        elif k == "model_id":
            c.model = v
        else:
            setattr(c, k, v)
    h = ctypes.c_void_p()
    rc = L.load().lss_adi_create(ctypes.byref(c), ctypes.byref(h))
    assert rc == code
    assert h.value is None
    assert L.load().lss_adi_last_error().decode().startswith("lss_adi_create:")


def test_time_dependent_sabr_is_single_instance_only(lss):
    # SABR with r != 0 carries D(t) = exp(-r (T - t)) in its coefficients: lss_adi_create runs
    # it (tables re-evaluated every step); the batch and the adjoint refuse it before any
    # device work
    from linear_system_solvers_gb300 import _lib as L

    p = lss.HestonProblem(model="sabr", rate=0.03, sigma=0.4, rho=-0.3, strike=0.05, s_hi=0.2, v_hi=1.0, nx=16, ny=8, nt=5)
    arr = (L.LssAdiProblem * 2)(p.to_c(), p.to_c())
    b = ctypes.c_void_p()
    assert L.load().lss_adi_batch_create(arr, 2, ctypes.byref(b)) == L.EUNSUPPORTED
    assert b.value is None
    assert "time-dependent" in L.load().lss_adi_last_error().decode()


def test_null_arguments_are_rejected(lss):
    from linear_system_solvers_gb300 import _lib as L

    lib = L.load()
    assert lib.lss_adi_create(None, None) == L.EINVAL
    assert lib.lss_adi_forward(None, None, None, None, 0, None) == L.EINVAL
    assert lib.lss_tridiag_thomas_lu(0, 3, 1, None, None, None, None, None, None, None, None) == L.EINVAL
    assert lib.lss_tridiag_thomas_lu(0, 8, 0, None, None, None, None, None, None, None, None) == L.OK
    lib.lss_adi_destroy(None)


def test_batch_generator_is_deterministic(lss):
    from linear_system_solvers_gb300.batch import draw_batch, grid_point_steps

    a = draw_batch(64)
    b = draw_batch(64)
    assert [x.kappa for x in a] == [x.kappa for x in b]
    assert all(x.nx in (64, 96, 128, 192, 256) and x.ny in (32, 48, 64, 96, 128) for x in a)
    assert all(100 <= x.nt - 1 <= 400 for x in a)
    assert all(0.5 <= x.kappa <= 5 and -0.95 <= x.rho <= 0 for x in a)
    assert grid_point_steps(a) == sum(x.nx * x.ny * (x.nt - 1) for x in a)
