"""1-D implicit heat / Black-Scholes solver on the GPU (include/lss_heat1d.h).

Mirrors the reference's 1-D implicit front end
(pde_solvers/one_dimensional/heat_type/lss_1d_general_heat_equation.hpp:60-250):

* ``GeneralHeatEquation1D`` takes what ``implicit_solvers::general_heat_equation`` takes --
  coefficient callables a(t, x), b(t, x), c(t, x), an initial condition, an optional heat source
  F(t, x), a boundary pair (``Dirichlet`` / ``Neumann`` / ``Robin``), the discretisation
  (space range, n, time range, nt), grid hints and the solver configuration (theta scheme,
  traverse direction, Thomas LU or double sweep) -- samples them on the grid in the reference's
  arithmetic (user callables in double; FP32 problems get the double tables rounded once)
  and solves on the device.  ``solve()`` returns the final values, ``solve_all()`` every time
  level (the reference's solve(container_2d&)).
* ``BlackScholesBatch`` runs many parametric Black-Scholes problems (the model of the
  reference's 1-D tests) in one launch.

The CUDA library is the only compute path; a missing library fails the import.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import Callable, Sequence

import numpy as np

from . import _lib as L


@dataclasses.dataclass
class Dirichlet:
    """dirichlet_boundary_1d: u = value(t)."""

    value: Callable[[float], float]
    kind: int = L.HEAT1D_DIRICHLET


@dataclasses.dataclass
class Neumann:
    """neumann_boundary_1d: u_x = value(t) (reference sign convention)."""

    value: Callable[[float], float]
    kind: int = L.HEAT1D_NEUMANN


@dataclasses.dataclass
class Robin:
    """robin_boundary_1d: u_x = linear(t) u + value(t)."""

    linear: Callable[[float], float]
    value: Callable[[float], float]
    kind: int = L.HEAT1D_ROBIN


def _prec(precision: str) -> tuple[int, type]:
    if precision not in ("f64", "f32"):
        raise ValueError("precision must be 'f64' or 'f32'")
    return (L.FP64, np.float64) if precision == "f64" else (L.FP32, np.float32)


def _arith(arith: str) -> int:
    if arith not in ("fast", "reference"):
        raise ValueError("arith must be 'fast' or 'reference'")
    return L.ARITH_FAST if arith == "fast" else L.ARITH_REFERENCE


def _theta(theta_scheme: str) -> int:
    if theta_scheme not in ("euler", "cn"):
        raise ValueError("the implicit 1-D kernel accepts theta_scheme 'euler' or 'cn'")
    return L.THETAS[theta_scheme]


class _Batch:
    """Owner of one lss_heat1d_batch handle."""

    def __init__(self, handle: ctypes.c_void_p, count: int, sizes: Sequence[int], nts: Sequence[int], dtype,
                 all_steps: bool, keep: list):
        self._h = handle
        self.count = count
        self.sizes = list(sizes)
        self.nts = list(nts)
        self.dtype = dtype
        self.all_steps = all_steps
        self._keep = keep

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            L.load().lss_heat1d_batch_destroy(h)
            self._h = None

    def run(self, stream: int | None = None):
        L.check(L.load().lss_heat1d_batch_run(self._h, stream))

    def run_host(self, initials: np.ndarray | None = None, stream: int | None = None):
        vals = np.empty(self.count, dtype=np.float64)
        st = np.empty(self.count, dtype=np.int32)
        ptr = None
        if initials is not None:
            initials = np.ascontiguousarray(initials, dtype=self.dtype)
            if initials.size != sum(self.sizes):
                raise ValueError("initials must hold n values per instance")
            ptr = initials.ctypes.data
        L.check(L.load().lss_heat1d_batch_run_host(self._h, ptr, vals.ctypes.data_as(L.P(L.c_double)),
                                                   st.ctypes.data_as(L.P(L.c_int)), stream))
        return vals, st

    def results(self):
        vals = np.empty(self.count, dtype=np.float64)
        st = np.empty(self.count, dtype=np.int32)
        L.check(L.load().lss_heat1d_batch_results(self._h, vals.ctypes.data_as(L.P(L.c_double)),
                                                  st.ctypes.data_as(L.P(L.c_int))))
        return vals, st

    def solution(self, index: int) -> np.ndarray:
        n, nt = self.sizes[index], self.nts[index]
        out = np.empty((nt, n) if self.all_steps else n, dtype=self.dtype)
        L.check(L.load().lss_heat1d_batch_solution(self._h, int(index), out.ctypes.data))
        return out

    def grid(self, index: int) -> np.ndarray:
        out = np.empty(self.sizes[index], dtype=self.dtype)
        L.check(L.load().lss_heat1d_batch_grid(self._h, int(index), out.ctypes.data))
        return out

    def point_steps(self) -> float:
        return float(L.load().lss_heat1d_batch_point_steps(self._h))

    def launch_count(self) -> int:
        return int(L.load().lss_heat1d_batch_launch_count(self._h))


def tabulated_batch(problems: Sequence[dict], precision: str = "f64", arith: str = "fast", all_steps: bool = False,
                    double_sweep: bool = False) -> _Batch:
    """Batch of tabulated problems: dicts with n, nt, t_lo, t_hi, theta_scheme ('euler'|'cn'),
    forward, lo_kind, hi_kind (0 Dirichlet, 1 Neumann, 2 Robin), coef (3, n), initial (n),
    boundary (nt-1, 4) and optional source (nt, n), all in the solver type (the layout of
    lss_heat1d_tables)."""
    prec, dt = _prec(precision)
    lib = L.load()
    arr = (L.LssHeat1DTables * len(problems))()
    keep = []
    for i, q in enumerate(problems):
        c = arr[i]
        c.n, c.nt = int(q["n"]), int(q["nt"])
        c.t_lo, c.t_hi = float(q["t_lo"]), float(q["t_hi"])
        c.theta_scheme = _theta(q.get("theta_scheme", "cn"))
        c.forward = int(bool(q.get("forward", False)))
        c.lo_kind, c.hi_kind = int(q.get("lo_kind", 0)), int(q.get("hi_kind", 0))
        for name, shape in (("coef", (3, c.n)), ("initial", (c.n,)), ("boundary", (c.nt - 1, 4))):
            a = np.ascontiguousarray(q[name], dtype=dt)
            if a.shape != shape:
                raise ValueError(f"{name} must have shape {shape}")
            keep.append(a)
            setattr(c, name, a.ctypes.data)
        if q.get("source") is not None:
            a = np.ascontiguousarray(q["source"], dtype=dt)
            if a.shape != (c.nt, c.n):
                raise ValueError(f"source must have shape {(c.nt, c.n)}")
            keep.append(a)
            c.source = a.ctypes.data
    opts = (L.HEAT1D_OPT_ALL_STEPS if all_steps else 0) | (L.HEAT1D_OPT_DOUBLE_SWEEP if double_sweep else 0)
    h = ctypes.c_void_p()
    L.check(lib.lss_heat1d_batch_create(arr, len(problems), prec, _arith(arith), opts, ctypes.byref(h)))
    return _Batch(h, len(problems), [q["n"] for q in problems], [q["nt"] for q in problems], dt, all_steps, [])


@dataclasses.dataclass
class BlackScholesProblem:
    """lss_heat1d_bs: the reference tests' Black-Scholes problem (call unless put)."""

    sigma: float = 0.25
    rate: float = 0.2
    strike: float = 10.0
    maturity: float = 1.0
    put: bool = False
    s_lo: float = 0.0
    s_hi: float = 20.0
    n: int = 100
    nt: int = 100
    theta_scheme: str = "cn"
    nonuniform: bool = False
    acc_point: float = 0.0
    alpha_scale: float = 3.0
    eval_s: float = 10.0

    def to_c(self) -> L.LssHeat1DBs:
        c = L.LssHeat1DBs()
        for name in ("sigma", "rate", "strike", "maturity", "s_lo", "s_hi", "acc_point", "alpha_scale", "eval_s"):
            setattr(c, name, float(getattr(self, name)))
        c.put = int(bool(self.put))
        c.n, c.nt = int(self.n), int(self.nt)
        c.theta_scheme = _theta(self.theta_scheme)
        c.nonuniform = int(bool(self.nonuniform))
        return c


def black_scholes_batch(problems: Sequence[BlackScholesProblem], precision: str = "f64", arith: str = "fast",
                        all_steps: bool = False, double_sweep: bool = False) -> _Batch:
    prec, dt = _prec(precision)
    arr = (L.LssHeat1DBs * len(problems))()
    for i, q in enumerate(problems):
        arr[i] = q.to_c()
    opts = (L.HEAT1D_OPT_ALL_STEPS if all_steps else 0) | (L.HEAT1D_OPT_DOUBLE_SWEEP if double_sweep else 0)
    h = ctypes.c_void_p()
    L.check(L.load().lss_heat1d_batch_create_bs(arr, len(problems), prec, _arith(arith), opts, ctypes.byref(h)))
    return _Batch(h, len(problems), [q.n for q in problems], [q.nt for q in problems], dt, all_steps, [])


def draw_black_scholes(count: int, seed: int = 20261205) -> list[BlackScholesProblem]:
    """Seeded batch of uneven Black-Scholes calls: sigma~U[0.1,0.6], r~U[0,0.1], T~U[0.25,2],
    K~U[80,120], S in [0, 4K], n from {128, 256, 384, 512}, 100-1000 time points, Crank-Nicolson,
    grid concentrated at K (alpha_scale 3), value at S = K."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(count):
        sigma = rng.uniform(0.1, 0.6)
        rate = rng.uniform(0.0, 0.1)
        mat = rng.uniform(0.25, 2.0)
        strike = rng.uniform(80.0, 120.0)
        n = int(rng.choice([128, 256, 384, 512]))
        nt = int(rng.integers(100, 1001))
        out.append(BlackScholesProblem(sigma=sigma, rate=rate, strike=strike, maturity=mat, s_lo=0.0,
                                       s_hi=4.0 * strike, n=n, nt=nt, theta_scheme="cn", nonuniform=True,
                                       acc_point=strike, alpha_scale=3.0, eval_s=strike))
    return out


class GeneralHeatEquation1D:
    """implicit_solvers::general_heat_equation on the device.

    a, b, c: callables (t, x) -> float; initial: x -> float; source: (t, x) -> float or None;
    boundary: (lower, upper) of Dirichlet / Neumann / Robin; space (x_lo, x_hi), n points;
    time (t_lo, t_hi), nt points; hints: accumulation point, alpha_scale, nonuniform
    (grid_config_hints_1d); theta_scheme 'euler' | 'cn'; forward (host_fwd_* configs) or
    backward; double_sweep picks tridiagonal_method_enum::DoubleSweepSolver.

    The coefficients must not depend on t (the device policy factorises once); this is
    checked at the first and last time of the loop, as the 2-D tabulated front end does."""

    def __init__(self, a, b, c, initial, boundary, space, n, time, nt, source=None, acc_point=0.0, alpha_scale=3.0,
                 nonuniform=False, theta_scheme="cn", forward=False, double_sweep=False, precision="f64",
                 arith="fast"):
        self.a, self.b, self.c, self.initial, self.source = a, b, c, initial, source
        self.lower, self.upper = boundary
        self.x_lo, self.x_hi = float(space[0]), float(space[1])
        self.t_lo, self.t_hi = float(time[0]), float(time[1])
        self.n, self.nt = int(n), int(nt)
        self.acc_point, self.alpha_scale, self.nonuniform = float(acc_point), float(alpha_scale), bool(nonuniform)
        self.theta_scheme, self.forward, self.double_sweep = theta_scheme, bool(forward), bool(double_sweep)
        self.precision, self.arith = precision, arith
        if self.n < 4 or self.nt < 2:
            raise ValueError("n must be >= 4 and nt >= 2")
        self._tables = self._tabulate()

    # grid_transform_config<One> (discretization/lss_grid_transform_config.hpp:32-87)
    def _map(self):
        low, high, point = self.x_lo, self.x_hi, self.acc_point
        alpha = high - low
        if self.nonuniform:
            alpha = (point - low) / self.alpha_scale
        c0 = math.asinh((high - point) / alpha)
        c1 = math.asinh((low - point) / alpha)
        cd = c0 - c1

        def arg(z):
            return c0 * z + c1 * (1.0 - z)

        return (lambda z: point + alpha * math.sinh(arg(z)), lambda z: alpha * cd * math.cosh(arg(z)),
                lambda z: alpha * cd * cd * math.sinh(arg(z)))

    def grid(self) -> np.ndarray:
        xv, _, _ = self._map()
        step = 1.0 / (self.n - 1)
        return np.array([xv(step * i) for i in range(self.n)])

    def _coefficients(self, t, xv, ad, bd, step, lam, gam, dlt):
        out = np.empty((3, self.n))
        for i in range(self.n):
            z = step * i
            x = xv(z)
            av = ad(z)
            ta = self.a(t, x) / (ad(z) * ad(z))
            tb = self.b(t, x) / av - (self.a(t, x) * bd(z)) / (av * av * av)
            tc = self.c(t, x)
            out[0, i] = lam * ta - gam * tb
            out[1, i] = lam * ta - dlt * tc
            out[2, i] = lam * ta + gam * tb
        return out

    def _times(self, k):
        t = self.t_lo + k if self.forward else self.t_hi - k
        out = []
        for _ in range(self.nt - 1):
            out.append(t)
            t = t + k if self.forward else t - k
        return out, t

    def _tabulate(self) -> dict:
        xv, ad, bd = self._map()
        step = 1.0 / (self.n - 1)
        k = (self.t_hi - self.t_lo) / (self.nt - 1)
        h = 1.0 / (self.n - 1)
        lam, gam, dlt = k / (h * h), k / (2.0 * h), 0.5 * k
        times, t_after = self._times(k)
        coef = self._coefficients(times[0], xv, ad, bd, step, lam, gam, dlt)
        if not np.array_equal(coef, self._coefficients(times[-1], xv, ad, bd, step, lam, gam, dlt)):
            raise ValueError("the device policy needs time-invariant coefficients")
        init = np.array([self.initial(xv(step * i)) for i in range(self.n)])
        bnd = np.zeros((self.nt - 1, 4))
        a0, a1 = ad(0.0), ad(1.0)
        for s, t in enumerate(times):
            for side, bc, aval in ((0, self.lower, a0), (2, self.upper, a1)):
                v = bc.value(t)
                if bc.kind == L.HEAT1D_DIRICHLET:
                    bnd[s, side] = v
                else:  # boundary_transform<One>: value * A(zeta), linear * A(zeta)
                    bnd[s, side] = v * aval
                    if bc.kind == L.HEAT1D_ROBIN:
                        bnd[s, side + 1] = bc.linear(t) * aval
        src = None
        if self.source is not None:
            rows = list(times) + [t_after]
            src = np.array([[self.source(t, xv(step * i)) for i in range(self.n)] for t in rows])
        return dict(n=self.n, nt=self.nt, t_lo=self.t_lo, t_hi=self.t_hi, theta_scheme=self.theta_scheme,
                    forward=self.forward, lo_kind=self.lower.kind, hi_kind=self.upper.kind, coef=coef, initial=init,
                    boundary=bnd, source=src)

    def solve(self) -> np.ndarray:
        b = tabulated_batch([self._tables], self.precision, self.arith, False, self.double_sweep)
        b.run()
        return b.solution(0)

    def solve_all(self) -> np.ndarray:
        b = tabulated_batch([self._tables], self.precision, self.arith, True, self.double_sweep)
        b.run()
        return b.solution(0)
