"""Batched uneven instances (``lss_adi_batch``) and the synthetic batch generator."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from .solver import HestonProblem

NX_CHOICES = (64, 96, 128, 192, 256)
NY_CHOICES = (32, 48, 64, 96, 128)


def draw_batch(count: int, seed: int = 20261203, scheme: str = "mcs") -> list[HestonProblem]:
    """Uneven Heston call batch.

    Per instance, in this order, from numpy PCG64(seed): kappa~U[0.5,5], theta~U[0.01,0.1],
    sigma~U[0.1,1], rho~U[-0.95,0], r~U[0,0.05], T~U[0.25,2], K~U[80,120],
    Nx in {64,96,128,192,256}, Ny in {32,48,64,96,128}, steps~U{100..400}.
    S in [0,200], v in [0,1.2]; sinh grid concentrated at K (alpha_scale 10) and at v=0
    (beta_scale 24, i.e. scale 0.05); value read at (S0, v0) = (100, 0.04).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(count):
        kappa = rng.uniform(0.5, 5.0)
        theta = rng.uniform(0.01, 0.1)
        sigma = rng.uniform(0.1, 1.0)
        rho = rng.uniform(-0.95, 0.0)
        rate = rng.uniform(0.0, 0.05)
        mat = rng.uniform(0.25, 2.0)
        strike = rng.uniform(80.0, 120.0)
        nx = NX_CHOICES[int(rng.integers(0, len(NX_CHOICES)))]
        ny = NY_CHOICES[int(rng.integers(0, len(NY_CHOICES)))]
        steps = int(rng.integers(100, 401))
        out.append(HestonProblem(kappa=kappa, theta_v=theta, sigma=sigma, rho=rho, rate=rate, maturity=mat,
                                 strike=strike, s_lo=0.0, s_hi=200.0, v_lo=0.0, v_hi=1.2, nx=nx, ny=ny,
                                 nt=steps + 1, scheme=scheme, zeta=0.5, theta_scheme="cn", nonuniform=True,
                                 acc_point=strike, alpha_scale=10.0, beta_scale=24.0, eval_s=100.0, eval_v=0.04))
    return out


def grid_point_steps(problems) -> int:
    return int(sum(p.nx * p.ny * (p.nt - 1) for p in problems))


class BatchSolver:
    """Many problems advanced by one persistent kernel (``lss_adi_batch``)."""

    def __init__(self, problems: list[HestonProblem], precision: str = "f64"):
        self.lib = L.load()
        self.problems = list(problems)
        self.precision = precision
        self.dtype = np.float32 if precision == "f32" else np.float64
        arr = (L.LssAdiProblem * len(self.problems))()
        for k, p in enumerate(self.problems):
            arr[k] = p.to_c(precision, "fast")
        self._arr = arr
        b = ctypes.c_void_p()
        L.check(self.lib.lss_adi_batch_create(arr, len(self.problems), ctypes.byref(b)))
        self._b = b

    def close(self):
        if getattr(self, "_b", None) and self._b.value:
            self.lib.lss_adi_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, mode: int = 0, stream: int = 0, graph: bool = False):
        fn = self.lib.lss_adi_batch_graph_launch if graph else self.lib.lss_adi_batch_run
        L.check(fn(self._b, int(mode), ctypes.c_void_p(stream)))

    def run_host(self, mode: int, values: np.ndarray, grads: np.ndarray | None = None, payoffs=None, stream: int = 0):
        gp = None if grads is None else grads.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        pp = None if payoffs is None else payoffs.ctypes.data
        L.check(self.lib.lss_adi_batch_run_host(self._b, int(mode), pp,
                                                values.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), gp,
                                                ctypes.c_void_p(stream)))

    def results(self):
        n = len(self.problems)
        v = np.empty(n, dtype=np.float64)
        g = np.empty((n, 5), dtype=np.float64)
        s = np.empty(n, dtype=np.int32)
        L.check(self.lib.lss_adi_batch_results(self._b, v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                               g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                               s.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return v, g, s

    def surface(self, index: int) -> np.ndarray:
        p = self.problems[index]
        out = np.empty((p.nx, p.ny), dtype=self.dtype)
        L.check(self.lib.lss_adi_batch_surface(self._b, int(index), out.ctypes.data))
        return out

    def payoff_gradient(self, index: int) -> np.ndarray:
        p = self.problems[index]
        out = np.empty((p.nx, p.ny), dtype=np.float64)
        L.check(self.lib.lss_adi_batch_payoff_gradient(self._b, int(index), out.ctypes.data))
        return out

    def autotune(self, mode: int = 0, threads: int = 0, stream: int = 0) -> int:
        """Pick the CTA size (threads per instance) for `mode` by timing, or set `threads`."""
        t = ctypes.c_int(int(threads))
        L.check(self.lib.lss_adi_batch_autotune(self._b, int(mode), ctypes.byref(t), ctypes.c_void_p(stream)))
        return t.value

    def launch_count(self) -> int:
        return int(self.lib.lss_adi_batch_launch_count(self._b))

    def set_workspace(self, max_bytes: float = 0.0, checkpoint_every: int = 0):
        """Cap the forward + adjoint workspace (bytes; 0 = a quarter of the device memory) and
        optionally fix the checkpoint interval (0 = planned from the cap)."""
        L.check(self.lib.lss_adi_batch_set_workspace(self._b, float(max_bytes), int(checkpoint_every)))

    def workspace_bytes(self) -> float:
        return float(self.lib.lss_adi_batch_workspace_bytes(self._b))

    def checkpoints(self) -> np.ndarray:
        """Checkpoint interval of every instance planned by the last adjoint run / autotune."""
        out = np.zeros(len(self.problems), dtype=np.int32)
        L.check(self.lib.lss_adi_batch_checkpoints(self._b, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return out
