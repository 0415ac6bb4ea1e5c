"""Python front end of the GB300 ADI solver (thin layer over the C-ABI).

Vocabulary follows the reference (MichalSara99/linear_system_solvers):
``HestonProblem`` carries what the reference spreads over pde_discretization_config_2d,
splitting_method_config, heat_implicit_solver_config, grid_config_hints_2d and the model
lambdas of its tests; ``ImplicitHestonSolver.solve()`` plays
``implicit_solvers::general_heston_equation::solve`` with the device policy.
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np

from . import _lib as L


@dataclasses.dataclass
class HestonProblem:
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
    scheme: str = "dr"  # dr | cs | mcs | hv (splittings) | euler (explicit Euler)
    zeta: float = 0.5
    theta_scheme: str = "cn"  # euler | theta30 | cn | theta80
    nonuniform: bool = False
    acc_point: float = 0.0
    alpha_scale: float = 3.0
    beta_scale: float = 50.0
    neumann_value: float = -1.0
    forward: bool = False
    eval_s: float = 100.0
    eval_v: float = 0.04
    fp64_tables: bool = False  # FP32 only: tables and index_of remaps built in double
    solver: str = "tlu"  # tridiagonal_method_enum: "tlu" ThomasLUSolver | "ds" DoubleSweepSolver
    line_per_thread: bool = False  # fast single instance: no partitioned line solves (batched-kernel bits)
    wide_adjoint: bool = False  # adjoint(): whole-GPU kernel-per-stage path at any size (not one CTA)

    # fields that choose how the device runs a problem, not which PDE it is
    EXECUTION_FIELDS = ("eval_s", "eval_v", "fp64_tables", "line_per_thread", "wide_adjoint")

    @property
    def steps(self) -> int:
        return self.nt - 1

    def pde_fields(self) -> dict:
        """The fields that define the PDE problem (model, grid, scheme, boundaries)."""
        return {k: v for k, v in dataclasses.asdict(self).items() if k not in self.EXECUTION_FIELDS}

    def to_c(self, precision: str = "f64", arith: str = "fast") -> L.LssAdiProblem:
        c = L.LssAdiProblem()
        c.model = L.SABR if self.model == "sabr" else L.HESTON
        for name in ("kappa", "theta_v", "sigma", "rho", "rate", "sabr_beta", "strike", "maturity", "s_lo", "s_hi",
                     "v_lo", "v_hi", "zeta", "acc_point", "alpha_scale", "beta_scale", "neumann_value", "eval_s",
                     "eval_v"):
            setattr(c, name, float(getattr(self, name)))
        c.nx, c.ny, c.nt = int(self.nx), int(self.ny), int(self.nt)
        c.scheme = L.SCHEMES[self.scheme]
        c.theta_scheme = L.THETAS[self.theta_scheme]
        c.nonuniform = int(bool(self.nonuniform))
        c.forward = int(bool(self.forward))
        c.precision = L.FP32 if precision == "f32" else L.FP64
        c.arith = L.ARITH_REFERENCE if arith == "reference" else L.ARITH_FAST
        if self.solver not in ("tlu", "ds"):
            raise ValueError(f"solver must be 'tlu' or 'ds', not {self.solver!r}")
        c.options = ((L.OPT_FP64_TABLES if self.fp64_tables else 0) | (L.OPT_DOUBLE_SWEEP if self.solver == "ds" else 0)
                     | (L.OPT_LINE_PER_THREAD if self.line_per_thread else 0)
                     | (L.OPT_WIDE_ADJOINT if self.wide_adjoint else 0))
        return c


def _dtype(precision: str):
    return np.float32 if precision == "f32" else np.float64


class ImplicitHestonSolver:
    """One problem on the GPU (``lss_adi_handle``)."""

    def __init__(self, problem: HestonProblem, precision: str = "f64", arith: str = "fast"):
        self.lib = L.load()
        self.problem = problem
        self.precision = precision
        self.dtype = _dtype(precision)
        self._c = problem.to_c(precision, arith)
        h = ctypes.c_void_p()
        L.check(self.lib.lss_adi_create(ctypes.byref(self._c), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.lss_adi_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def line_chunks(self, s_chunks: int = 0, v_chunks: int = 0, stream: int = 0):
        """Chunks per S line / v line of the partitioned solves (0 = autotune); returns those in use."""
        a, b = ctypes.c_int(), ctypes.c_int()
        L.check(self.lib.lss_adi_line_chunks(self._h, int(s_chunks), int(v_chunks), ctypes.byref(a), ctypes.byref(b),
                                             ctypes.c_void_p(stream)))
        return a.value, b.value

    def grid(self):
        x = np.empty(self.problem.nx, dtype=self.dtype)
        y = np.empty(self.problem.ny, dtype=self.dtype)
        L.check(self.lib.lss_adi_grid(self._h, x.ctypes.data, y.ctypes.data))
        return x, y

    def solve(self, payoff: np.ndarray | None = None, graph: bool = False, stream: int = 0):
        """Final surface V[i, j] and the bilinear value V(eval_s, eval_v)."""
        out = np.empty((self.problem.nx, self.problem.ny), dtype=self.dtype)
        val = ctypes.c_double()
        pay = None if payoff is None else np.ascontiguousarray(payoff, dtype=self.dtype)
        fn = self.lib.lss_adi_forward_graph if graph else self.lib.lss_adi_forward
        L.check(fn(self._h, None if pay is None else pay.ctypes.data, out.ctypes.data, ctypes.byref(val), 0,
                   ctypes.c_void_p(stream)))
        return out, val.value

    def adjoint(self, payoff: np.ndarray | None = None, checkpoint_every: int = 0, want_payoff_grad: bool = True,
                stream: int = 0):
        """V(eval_s, eval_v), dV/d(kappa, theta, sigma, rho, r) and dV/d(payoff grid)."""
        val = ctypes.c_double()
        g = (ctypes.c_double * 5)()
        dpay = np.empty((self.problem.nx, self.problem.ny), dtype=self.dtype) if want_payoff_grad else None
        pay = None if payoff is None else np.ascontiguousarray(payoff, dtype=self.dtype)
        L.check(self.lib.lss_adi_adjoint(self._h, None if pay is None else pay.ctypes.data, ctypes.byref(val), g,
                                         None if dpay is None else dpay.ctypes.data, int(checkpoint_every), 0,
                                         ctypes.c_void_p(stream)))
        return val.value, np.array(list(g)), dpay


class TabulatedHestonSolver(ImplicitHestonSolver):
    """Time-invariant coefficients sampled on the grid by the caller (``lss_adi_create_tabulated``):
    the device drop-in for arbitrary coefficient functions of the reference's
    heat_coefficient_data_config_2d.

    coef: (7, nx, ny) M, P, Z, M~, P~, W, C; coef_v0: (3, nx) D, E, F on the v = v_lo line;
    s_lo: (ny,) Dirichlet values at S_lo; s_hi_neumann: (ny,) transformed Neumann data at S_hi;
    v_hi: (nx,) Dirichlet values at v_hi; payoff: (nx, ny).
    Time-dependent coefficients or boundaries: coef (nt - 1, 7, nx, ny), coef_v0 (nt - 1, 3, nx),
    s_lo / s_hi_neumann (nt - 1, ny), v_hi (nt - 1, nx), step s sampled at the time of step s
    (t_hi - k, t_hi - 2k, ... backward; LSS_ADI_OPT_STEP_TABLES).
    """

    def __init__(self, nt, t_lo, t_hi, scheme, theta_scheme, coef, coef_v0, s_lo, s_hi_neumann, v_hi, payoff,
                 zeta=0.5, forward=False, precision="f64", arith="fast", solver="tlu"):
        self.lib = L.load()
        self.precision = precision
        self.dtype = _dtype(precision)
        arrs = [np.ascontiguousarray(a, dtype=self.dtype) for a in (coef, coef_v0, s_lo, s_hi_neumann, v_hi, payoff)]
        self._keep = arrs
        nx, ny = arrs[5].shape
        step_tables = arrs[0].ndim == 4
        if step_tables and arrs[0].shape[0] != nt - 1:
            raise ValueError("per-step coefficient tables need nt - 1 blocks")
        self.problem = HestonProblem(nx=nx, ny=ny, nt=nt)
        t = L.LssAdiTables()
        t.nx, t.ny, t.nt = nx, ny, int(nt)
        t.t_lo, t.t_hi = float(t_lo), float(t_hi)
        t.scheme = L.SCHEMES[scheme]
        t.theta_scheme = L.THETAS[theta_scheme]
        t.forward = int(bool(forward))
        t.precision = L.FP32 if precision == "f32" else L.FP64
        t.arith = L.ARITH_REFERENCE if arith == "reference" else L.ARITH_FAST
        t.zeta = float(zeta)
        t.options = (L.OPT_DOUBLE_SWEEP if solver == "ds" else 0) | (L.OPT_STEP_TABLES if step_tables else 0)
        t.coef, t.coef_v0, t.s_lo_dirichlet, t.s_hi_neumann, t.v_hi_dirichlet, t.payoff = [a.ctypes.data for a in arrs]
        h = ctypes.c_void_p()
        L.check(self.lib.lss_adi_create_tabulated(ctypes.byref(t), ctypes.byref(h)))
        self._h = h


def thomas_lu_lines(lo, diag, up, rhs, bnd_lo, bnd_hi, precision: str = "f64"):
    """Batched Thomas LU through lss_tridiag_thomas_lu (arrays (n, lines), host numpy).

    Uses torch only as device-memory plumbing for the device pointers the C-ABI takes.
    """
    import torch

    lib = L.load()
    dt = torch.float32 if precision == "f32" else torch.float64
    dev = [torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda") for a in (lo, diag, up, rhs)]
    blo = torch.as_tensor(np.ascontiguousarray(bnd_lo), dtype=dt, device="cuda")
    bhi = torch.as_tensor(np.ascontiguousarray(bnd_hi), dtype=dt, device="cuda")
    x = torch.empty_like(dev[3])
    n, lines = dev[0].shape
    stream = torch.cuda.current_stream().cuda_stream
    L.check(lib.lss_tridiag_thomas_lu(L.FP32 if precision == "f32" else L.FP64, n, lines, dev[0].data_ptr(),
                                      dev[1].data_ptr(), dev[2].data_ptr(), dev[3].data_ptr(), blo.data_ptr(),
                                      bhi.data_ptr(), x.data_ptr(), ctypes.c_void_p(stream)))
    torch.cuda.synchronize()
    return x.cpu().numpy()
