"""CPU oracle bindings (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module, and only as the checker.  The product (``linear_system_solvers_gb300``) never
imports it.

* ``solve(problem, fp)`` runs the plain-C restatement in ``lss_oracle.c`` (reference:
  the host Thomas-LU / double-sweep ADI path of MichalSara99/linear_system_solvers).
* ``run_reference(problem, fp)`` runs the reference itself, compiled by
  ``build_ref.sh`` into ``oracle/_ref/ref_driver`` (only where it was built).
* ``solve_1d`` / ``tables_1d`` / ``run_reference_1d``: the same for the 1-D implicit heat path
  (``lss_oracle_1d_impl.h``, ``oracle/_ref/ref_driver_1d``).
"""
from __future__ import annotations

import ctypes
import dataclasses
import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblss_oracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")

SCHEMES = {"dr": 0, "cs": 1, "mcs": 2, "hv": 3, "euler": 4}
THETAS = {"euler": 0, "theta30": 1, "cn": 2, "theta80": 3}


@dataclasses.dataclass
class Problem:
    """One 2-D Heston/SABR pricing problem in the reference's vocabulary."""

    model: str = "heston"  # "heston" | "sabr"
    kappa: float = 1.5
    theta_v: float = 0.04
    sigma: float = 0.3
    rho: float = -0.9
    rate: float = 0.02
    sabr_beta: float = 0.5
    strike: float = 100.0
    maturity: float = 1.0
    s_lo: float = 0.0
    s_hi: float = 200.0
    v_lo: float = 0.0
    v_hi: float = 1.2
    nx: int = 100
    ny: int = 50
    nt: int = 201  # time points (steps = nt - 1)
    scheme: str = "dr"
    zeta: float = 0.5
    theta_scheme: str = "cn"
    nonuniform: bool = False
    acc_point: float = 0.0
    alpha_scale: float = 3.0
    beta_scale: float = 50.0
    neumann_value: float = -1.0
    solver: str = "tlu"  # "tlu" | "ds"
    forward: bool = False


class _CProblem(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int),
        ("kappa", ctypes.c_double), ("theta_v", ctypes.c_double), ("sigma", ctypes.c_double),
        ("rho", ctypes.c_double), ("rate", ctypes.c_double), ("sabr_beta", ctypes.c_double),
        ("strike", ctypes.c_double), ("maturity", ctypes.c_double),
        ("s_lo", ctypes.c_double), ("s_hi", ctypes.c_double),
        ("v_lo", ctypes.c_double), ("v_hi", ctypes.c_double),
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nt", ctypes.c_int),
        ("scheme", ctypes.c_int), ("zeta", ctypes.c_double), ("theta_scheme", ctypes.c_int),
        ("nonuniform", ctypes.c_int),
        ("acc_point", ctypes.c_double), ("alpha_scale", ctypes.c_double), ("beta_scale", ctypes.c_double),
        ("neumann_value", ctypes.c_double),
        ("solver", ctypes.c_int), ("forward", ctypes.c_int),
    ]


_lib = None


def build() -> str:
    """Compile the oracle library (gcc, seconds) and return its path."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        for fn, t in (("lsso_solve_f64", ctypes.c_double), ("lsso_solve_f32", ctypes.c_float)):
            getattr(_lib, fn).argtypes = [ctypes.POINTER(_CProblem), ctypes.c_void_p, ctypes.c_void_p]
            getattr(_lib, fn).restype = ctypes.c_int
        for fn in ("lsso_grid_f64", "lsso_grid_f32", "lsso_index_maps_f64", "lsso_index_maps_f32"):
            getattr(_lib, fn).argtypes = [ctypes.POINTER(_CProblem), ctypes.c_void_p, ctypes.c_void_p]
            getattr(_lib, fn).restype = ctypes.c_int
        _lib.lsso_coefficients_f64.argtypes = [ctypes.POINTER(_CProblem), ctypes.c_double, ctypes.c_void_p]
        _lib.lsso_coefficients_f64.restype = ctypes.c_int
    return _lib


def to_c(p: Problem) -> _CProblem:
    c = _CProblem()
    c.model = 1 if p.model == "sabr" else 0
    for name in ("kappa", "theta_v", "sigma", "rho", "rate", "sabr_beta", "strike", "maturity",
                 "s_lo", "s_hi", "v_lo", "v_hi", "zeta", "acc_point", "alpha_scale", "beta_scale",
                 "neumann_value"):
        setattr(c, name, float(getattr(p, name)))
    c.nx, c.ny, c.nt = int(p.nx), int(p.ny), int(p.nt)
    c.scheme = SCHEMES[p.scheme]
    c.theta_scheme = THETAS[p.theta_scheme]
    c.nonuniform = int(bool(p.nonuniform))
    c.solver = 1 if p.solver == "ds" else 0
    c.forward = int(bool(p.forward))
    return c


def _dtype(fp: str):
    return np.float32 if fp == "f32" else np.float64


def solve(p: Problem, fp: str = "f64", payoff: np.ndarray | None = None) -> np.ndarray:
    """Final surface V[i, j] (i = S index, j = v index) from the C restatement."""
    dt = _dtype(fp)
    out = np.empty((p.nx, p.ny), dtype=dt)
    pay = None
    if payoff is not None:
        pay = np.ascontiguousarray(payoff, dtype=dt)
    fn = lib().lsso_solve_f32 if fp == "f32" else lib().lsso_solve_f64
    rc = fn(ctypes.byref(to_c(p)), None if pay is None else pay.ctypes.data, out.ctypes.data)
    if rc != 0:
        raise ValueError(f"oracle rejected the problem (code {rc})")
    return out


def grid(p: Problem, fp: str = "f64"):
    dt = _dtype(fp)
    x = np.empty(p.nx, dtype=dt)
    y = np.empty(p.ny, dtype=dt)
    fn = lib().lsso_grid_f32 if fp == "f32" else lib().lsso_grid_f64
    rc = fn(ctypes.byref(to_c(p)), x.ctypes.data, y.ctypes.data)
    if rc != 0:
        raise ValueError(f"oracle rejected the problem (code {rc})")
    return x, y


def index_maps(p: Problem, fp: str = "f64"):
    imap = np.empty(p.nx, dtype=np.int32)
    jmap = np.empty(p.ny, dtype=np.int32)
    fn = lib().lsso_index_maps_f32 if fp == "f32" else lib().lsso_index_maps_f64
    rc = fn(ctypes.byref(to_c(p)), imap.ctypes.data, jmap.ctypes.data)
    if rc != 0:
        raise ValueError(f"oracle rejected the problem (code {rc})")
    return imap, jmap


def coefficients(p: Problem, t: float) -> dict:
    out = np.empty((10, p.nx, p.ny), dtype=np.float64)
    rc = lib().lsso_coefficients_f64(ctypes.byref(to_c(p)), float(t), out.ctypes.data)
    if rc != 0:
        raise ValueError(f"oracle rejected the problem (code {rc})")
    return dict(zip(("M", "P", "Z", "Mt", "Pt", "W", "C", "D", "E", "F"), out))


def reference_available() -> bool:
    return os.path.exists(REF_DRIVER) and os.access(REF_DRIVER, os.X_OK)


def run_reference(p: Problem, fp: str = "f64", repeat: int = 1):
    """Run the compiled reference; returns (surface, seconds for `repeat` solves)."""
    if not reference_available():
        raise FileNotFoundError(REF_DRIVER)
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "out.bin")
        args = [REF_DRIVER, fp, p.model, p.scheme, p.solver, str(p.nx), str(p.ny), str(p.nt)]
        args += [repr(float(v)) for v in (p.kappa, p.theta_v, p.sigma, p.rho, p.rate, p.sabr_beta,
                                          p.strike, p.maturity, p.s_lo, p.s_hi, p.v_lo, p.v_hi, p.zeta)]
        args += [str(THETAS[p.theta_scheme]), str(int(bool(p.nonuniform)))]
        args += [repr(float(v)) for v in (p.acc_point, p.alpha_scale, p.beta_scale, p.neumann_value)]
        args += [str(int(bool(p.forward))), str(int(repeat)), out]
        res = subprocess.run(args, check=True, capture_output=True, text=True)
        meta = json.loads(res.stdout.strip().splitlines()[-1])
        surf = np.fromfile(out, dtype=_dtype(fp)).reshape(p.nx, p.ny)
    return surf, meta["seconds"]


# ---------------------------------------------------------------------------------------------
# 1-D implicit heat / Black-Scholes (lss_oracle_1d_impl.h; reference:
# implicit_solvers::general_heat_equation with the host Thomas-LU / double-sweep policies)
# ---------------------------------------------------------------------------------------------
BC_KINDS = {"dirichlet": 0, "neumann": 1, "robin": 2}


@dataclasses.dataclass
class Heat1DProblem:
    """One 1-D problem u_t = a u_xx + b u_x + c u + F in the reference's vocabulary.

    model "bs": a = 0.5 sigma^2 x^2, b = rate x, c = -rate, terminal max(0, x - K) (put:
    max(0, K - x)), Dirichlet data of the reference's Black-Scholes tests.  model "const":
    constant a, b, c (diff, conv, react), initial init0 + init1 x, boundary kinds with constant
    data (Robin: lin * u + value), optional source F = src0 + src1 x."""

    model: str = "bs"
    sigma: float = 0.25
    rate: float = 0.2
    strike: float = 10.0
    put: bool = False
    diff: float = 1.0
    conv: float = 0.0
    react: float = 0.0
    init0: float = 0.0
    init1: float = 1.0
    lo_kind: str = "dirichlet"
    hi_kind: str = "dirichlet"
    lo_value: float = 0.0
    lo_linear: float = 0.0
    hi_value: float = 0.0
    hi_linear: float = 0.0
    has_source: bool = False
    src0: float = 0.0
    src1: float = 0.0
    x_lo: float = 0.0
    x_hi: float = 20.0
    t_lo: float = 0.0
    t_hi: float = 1.0
    n: int = 100
    nt: int = 100
    theta_scheme: str = "cn"  # "euler" | "cn"
    nonuniform: bool = False
    acc_point: float = 0.0
    alpha_scale: float = 3.0
    solver: str = "tlu"
    forward: bool = False


class _CHeat1D(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int),
        ("sigma", ctypes.c_double), ("rate", ctypes.c_double), ("strike", ctypes.c_double),
        ("put", ctypes.c_int),
        ("diff", ctypes.c_double), ("conv", ctypes.c_double), ("react", ctypes.c_double),
        ("init0", ctypes.c_double), ("init1", ctypes.c_double),
        ("lo_kind", ctypes.c_int), ("hi_kind", ctypes.c_int),
        ("lo_value", ctypes.c_double), ("lo_linear", ctypes.c_double),
        ("hi_value", ctypes.c_double), ("hi_linear", ctypes.c_double),
        ("has_source", ctypes.c_int), ("src0", ctypes.c_double), ("src1", ctypes.c_double),
        ("x_lo", ctypes.c_double), ("x_hi", ctypes.c_double), ("t_lo", ctypes.c_double), ("t_hi", ctypes.c_double),
        ("n", ctypes.c_int), ("nt", ctypes.c_int), ("theta_scheme", ctypes.c_int), ("nonuniform", ctypes.c_int),
        ("acc_point", ctypes.c_double), ("alpha_scale", ctypes.c_double),
        ("solver", ctypes.c_int), ("forward", ctypes.c_int),
    ]


REF_DRIVER_1D = os.path.join(HERE, "_ref", "ref_driver_1d")
_lib1d_ready = False


def lib1d():
    global _lib1d_ready
    L = lib()
    if not _lib1d_ready:
        for fn in ("lsso_heat1d_solve_f64", "lsso_heat1d_solve_f32"):
            getattr(L, fn).argtypes = [ctypes.POINTER(_CHeat1D), ctypes.c_void_p, ctypes.c_void_p]
            getattr(L, fn).restype = ctypes.c_int
        for fn in ("lsso_heat1d_grid_f64", "lsso_heat1d_grid_f32"):
            getattr(L, fn).argtypes = [ctypes.POINTER(_CHeat1D), ctypes.c_void_p]
            getattr(L, fn).restype = ctypes.c_int
        for fn in ("lsso_heat1d_tables_f64", "lsso_heat1d_tables_f32"):
            getattr(L, fn).argtypes = [ctypes.POINTER(_CHeat1D)] + [ctypes.c_void_p] * 4
            getattr(L, fn).restype = ctypes.c_int
        _lib1d_ready = True
    return L


def to_c_1d(p: Heat1DProblem) -> _CHeat1D:
    c = _CHeat1D()
    c.model = 0 if p.model == "bs" else 1
    for name in ("sigma", "rate", "strike", "diff", "conv", "react", "init0", "init1", "lo_value", "lo_linear",
                 "hi_value", "hi_linear", "src0", "src1", "x_lo", "x_hi", "t_lo", "t_hi", "acc_point",
                 "alpha_scale"):
        setattr(c, name, float(getattr(p, name)))
    c.put = int(bool(p.put))
    c.lo_kind, c.hi_kind = BC_KINDS[p.lo_kind], BC_KINDS[p.hi_kind]
    c.has_source = int(bool(p.has_source))
    c.n, c.nt = int(p.n), int(p.nt)
    c.theta_scheme = THETAS[p.theta_scheme]
    c.nonuniform = int(bool(p.nonuniform))
    c.solver = 1 if p.solver == "ds" else 0
    c.forward = int(bool(p.forward))
    return c


def solve_1d(p: Heat1DProblem, fp: str = "f64", all_steps: bool = False) -> np.ndarray:
    """Final solution (n,) or, with all_steps, every time level (nt, n) by time index."""
    dt = _dtype(fp)
    out = np.empty(p.n, dtype=dt)
    allv = np.empty((p.nt, p.n), dtype=dt) if all_steps else None
    fn = lib1d().lsso_heat1d_solve_f32 if fp == "f32" else lib1d().lsso_heat1d_solve_f64
    rc = fn(ctypes.byref(to_c_1d(p)), out.ctypes.data, None if allv is None else allv.ctypes.data)
    if rc != 0:
        raise ValueError(f"oracle rejected the problem (code {rc})")
    return allv if all_steps else out


def grid_1d(p: Heat1DProblem, fp: str = "f64") -> np.ndarray:
    x = np.empty(p.n, dtype=_dtype(fp))
    fn = lib1d().lsso_heat1d_grid_f32 if fp == "f32" else lib1d().lsso_heat1d_grid_f64
    rc = fn(ctypes.byref(to_c_1d(p)), x.ctypes.data)
    if rc != 0:
        raise ValueError(f"oracle rejected the problem (code {rc})")
    return x


def tables_1d(p: Heat1DProblem, fp: str = "f64") -> dict:
    """The tables a tabulated device problem takes, in the reference's arithmetic."""
    dt = _dtype(fp)
    coef = np.empty((3, p.n), dtype=dt)
    init = np.empty(p.n, dtype=dt)
    bnd = np.empty((p.nt - 1, 4), dtype=dt)
    src = np.empty((p.nt, p.n), dtype=dt) if p.has_source else None
    fn = lib1d().lsso_heat1d_tables_f32 if fp == "f32" else lib1d().lsso_heat1d_tables_f64
    rc = fn(ctypes.byref(to_c_1d(p)), coef.ctypes.data, init.ctypes.data, bnd.ctypes.data,
            None if src is None else src.ctypes.data)
    if rc != 0:
        raise ValueError(f"oracle rejected the problem (code {rc})")
    return {"coef": coef, "init": init, "bnd": bnd, "src": src}


def reference_1d_available() -> bool:
    return os.path.exists(REF_DRIVER_1D) and os.access(REF_DRIVER_1D, os.X_OK)


def run_reference_1d(p: Heat1DProblem, fp: str = "f64", all_steps: bool = False, repeat: int = 1):
    """Run the compiled reference 1-D solver; returns (solution, seconds for `repeat` solves)."""
    if not reference_1d_available():
        raise FileNotFoundError(REF_DRIVER_1D)
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "out.bin")
        args = [REF_DRIVER_1D, fp, "bs" if p.model == "bs" else "const", p.solver, str(p.n), str(p.nt)]
        args += [repr(float(v)) for v in (p.sigma, p.rate, p.strike)] + [str(int(bool(p.put)))]
        args += [repr(float(v)) for v in (p.diff, p.conv, p.react, p.init0, p.init1)]
        args += [str(BC_KINDS[p.lo_kind]), str(BC_KINDS[p.hi_kind])]
        args += [repr(float(v)) for v in (p.lo_value, p.lo_linear, p.hi_value, p.hi_linear)]
        args += [str(int(bool(p.has_source)))] + [repr(float(v)) for v in (p.src0, p.src1)]
        args += [repr(float(v)) for v in (p.x_lo, p.x_hi, p.t_lo, p.t_hi)]
        args += [str(THETAS[p.theta_scheme]), str(int(bool(p.nonuniform)))]
        args += [repr(float(v)) for v in (p.acc_point, p.alpha_scale)]
        args += [str(int(bool(p.forward))), str(int(bool(all_steps))), str(int(repeat)), out]
        res = subprocess.run(args, check=True, capture_output=True, text=True)
        meta = json.loads(res.stdout.strip().splitlines()[-1])
        vals = np.fromfile(out, dtype=_dtype(fp))
        vals = vals.reshape(p.nt, p.n) if all_steps else vals
    return vals, meta["seconds"]
