"""ctypes binding of the C-ABI in include/lss_adi.h and include/lss_heat1d.h (liblss_adi.so).

The library is the only compute path: if it cannot be loaded the import fails loudly;
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

c_int, c_double, c_void_p = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
P = ctypes.POINTER

# return codes
OK, EINVAL, EUNSUPPORTED, ECUDA, ENOMEM, ENONFINITE = 0, 1, 2, -1, -2, -3
DEVICE_POINTERS = 1
FP64, FP32 = 0, 1
ARITH_FAST, ARITH_REFERENCE = 0, 1
OPT_FP64_TABLES = 1
OPT_DOUBLE_SWEEP = 2
OPT_LINE_PER_THREAD = 4
OPT_WIDE_ADJOINT = 8
OPT_STEP_TABLES = 16
HESTON, SABR = 0, 1
SCHEMES = {"dr": 0, "cs": 1, "mcs": 2, "hv": 3, "euler": 4}
THETAS = {"euler": 0, "theta30": 1, "cn": 2, "theta80": 3}


class LssAdiProblem(ctypes.Structure):
    """Mirror of ``lss_adi_problem``."""

    _fields_ = [
        ("model", c_int),
        ("kappa", c_double), ("theta_v", c_double), ("sigma", c_double), ("rho", c_double), ("rate", c_double),
        ("sabr_beta", c_double), ("strike", c_double), ("maturity", c_double),
        ("s_lo", c_double), ("s_hi", c_double), ("v_lo", c_double), ("v_hi", c_double),
        ("nx", c_int), ("ny", c_int), ("nt", c_int),
        ("scheme", c_int), ("zeta", c_double), ("theta_scheme", c_int),
        ("nonuniform", c_int), ("acc_point", c_double), ("alpha_scale", c_double), ("beta_scale", c_double),
        ("neumann_value", c_double), ("forward", c_int), ("precision", c_int), ("arith", c_int),
        ("eval_s", c_double), ("eval_v", c_double), ("options", c_int),
    ]


class LssAdiTables(ctypes.Structure):
    """Mirror of ``lss_adi_tables``."""

    _fields_ = [
        ("nx", c_int), ("ny", c_int), ("nt", c_int), ("t_lo", c_double), ("t_hi", c_double),
        ("scheme", c_int), ("theta_scheme", c_int), ("forward", c_int), ("precision", c_int), ("arith", c_int),
        ("zeta", c_double),
        ("coef", c_void_p), ("coef_v0", c_void_p), ("s_lo_dirichlet", c_void_p), ("s_hi_neumann", c_void_p),
        ("v_hi_dirichlet", c_void_p), ("payoff", c_void_p), ("options", c_int),
    ]


class LssHeat1DTables(ctypes.Structure):
    """Mirror of ``lss_heat1d_tables``."""

    _fields_ = [
        ("n", c_int), ("nt", c_int), ("t_lo", c_double), ("t_hi", c_double), ("theta_scheme", c_int),
        ("forward", c_int), ("lo_kind", c_int), ("hi_kind", c_int),
        ("coef", c_void_p), ("initial", c_void_p), ("boundary", c_void_p), ("source", c_void_p),
    ]


class LssHeat1DBs(ctypes.Structure):
    """Mirror of ``lss_heat1d_bs``."""

    _fields_ = [
        ("sigma", c_double), ("rate", c_double), ("strike", c_double), ("maturity", c_double), ("put", c_int),
        ("s_lo", c_double), ("s_hi", c_double), ("n", c_int), ("nt", c_int), ("theta_scheme", c_int),
        ("nonuniform", c_int), ("acc_point", c_double), ("alpha_scale", c_double), ("eval_s", c_double),
    ]


HEAT1D_DIRICHLET, HEAT1D_NEUMANN, HEAT1D_ROBIN = 0, 1, 2
HEAT1D_OPT_ALL_STEPS, HEAT1D_OPT_DOUBLE_SWEEP = 1, 2

# name -> (restype, argtypes); every symbol declared in include/lss_adi.h and include/lss_heat1d.h
SIGNATURES = {
    "lss_adi_abi_version": (c_int, []),
    "lss_adi_last_error": (ctypes.c_char_p, []),
    "lss_adi_create": (c_int, [P(LssAdiProblem), P(c_void_p)]),
    "lss_adi_create_tabulated": (c_int, [P(LssAdiTables), P(c_void_p)]),
    "lss_adi_forward": (c_int, [c_void_p, c_void_p, c_void_p, P(c_double), c_int, c_void_p]),
    "lss_adi_forward_graph": (c_int, [c_void_p, c_void_p, c_void_p, P(c_double), c_int, c_void_p]),
    "lss_adi_adjoint": (c_int, [c_void_p, c_void_p, P(c_double), P(c_double), c_void_p, c_int, c_int, c_void_p]),
    "lss_adi_grid": (c_int, [c_void_p, c_void_p, c_void_p]),
    "lss_adi_line_chunks": (c_int, [c_void_p, c_int, c_int, P(c_int), P(c_int), c_void_p]),
    "lss_adi_destroy": (None, [c_void_p]),
    "lss_adi_batch_create": (c_int, [P(LssAdiProblem), c_int, P(c_void_p)]),
    "lss_adi_batch_run": (c_int, [c_void_p, c_int, c_void_p]),
    "lss_adi_batch_graph_launch": (c_int, [c_void_p, c_int, c_void_p]),
    "lss_adi_batch_run_host": (c_int, [c_void_p, c_int, c_void_p, P(c_double), P(c_double), c_void_p]),
    "lss_adi_batch_results": (c_int, [c_void_p, P(c_double), P(c_double), P(c_int)]),
    "lss_adi_batch_surface": (c_int, [c_void_p, c_int, c_void_p]),
    "lss_adi_batch_payoff_gradient": (c_int, [c_void_p, c_int, c_void_p]),
    "lss_adi_batch_autotune": (c_int, [c_void_p, c_int, P(c_int), c_void_p]),
    "lss_adi_batch_launch_count": (c_int, [c_void_p]),
    "lss_adi_batch_checkpoints": (c_int, [c_void_p, P(c_int)]),
    "lss_adi_batch_set_workspace": (c_int, [c_void_p, c_double, c_int]),
    "lss_adi_batch_workspace_bytes": (c_double, [c_void_p]),
    "lss_adi_batch_destroy": (None, [c_void_p]),
    "lss_tridiag_thomas_lu": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_void_p]),
    "lss_tridiag_thomas_lu_noalloc": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                              c_void_p, c_void_p, c_void_p, c_void_p]),
    "lss_diag_fp64_rate": (c_int, [P(c_double), c_void_p]),
    "lss_heat1d_batch_create": (c_int, [P(LssHeat1DTables), c_int, c_int, c_int, c_int, P(c_void_p)]),
    "lss_heat1d_batch_create_bs": (c_int, [P(LssHeat1DBs), c_int, c_int, c_int, c_int, P(c_void_p)]),
    "lss_heat1d_batch_run": (c_int, [c_void_p, c_void_p]),
    "lss_heat1d_batch_run_host": (c_int, [c_void_p, c_void_p, P(c_double), P(c_int), c_void_p]),
    "lss_heat1d_batch_results": (c_int, [c_void_p, P(c_double), P(c_int)]),
    "lss_heat1d_batch_solution": (c_int, [c_void_p, c_int, c_void_p]),
    "lss_heat1d_batch_grid": (c_int, [c_void_p, c_int, c_void_p]),
    "lss_heat1d_batch_launch_count": (c_int, [c_void_p]),
    "lss_heat1d_batch_point_steps": (c_double, [c_void_p]),
    "lss_heat1d_batch_destroy": (None, [c_void_p]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load liblss_adi.so (building it in-tree with nvcc when missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise ImportError(f"liblss_adi.so not found at {path}; run linear_system_solvers_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.lss_adi_abi_version() != 1:
        raise ImportError("liblss_adi.so ABI version mismatch")
    _lib = lib
    return lib


class LssError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def check(rc: int):
    if rc != OK:
        msg = _lib.lss_adi_last_error().decode() if _lib is not None else ""
        raise LssError(rc, msg)
