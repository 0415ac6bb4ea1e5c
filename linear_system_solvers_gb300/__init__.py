"""GB300-native (sm_103a) 2-D Heston/SABR ADI solver and batched 1-D implicit heat solver.

A from-scratch device implementation of the implicit ADI time-stepping path of
MichalSara99/linear_system_solvers (Douglas-Rachford, Craig-Sneyd, modified Craig-Sneyd,
Hundsdorfer-Verwer splitting with Thomas-LU line solves), exposed through the C-ABI in
``include/lss_adi.h`` (``_build/liblss_adi.so``) and this thin Python layer.
"""
from ._lib import LssError, load  # noqa: F401
from .solver import HestonProblem, ImplicitHestonSolver, TabulatedHestonSolver, thomas_lu_lines  # noqa: F401
from .batch import BatchSolver, draw_batch  # noqa: F401
from .heat1d import (BlackScholesProblem, Dirichlet, GeneralHeatEquation1D, Neumann, Robin,  # noqa: F401
                     black_scholes_batch, draw_black_scholes, tabulated_batch)

__all__ = ["HestonProblem", "ImplicitHestonSolver", "TabulatedHestonSolver", "BatchSolver", "draw_batch", "thomas_lu_lines", "LssError",
           "load", "BlackScholesProblem", "GeneralHeatEquation1D", "Dirichlet", "Neumann", "Robin", "black_scholes_batch",
           "draw_black_scholes", "tabulated_batch"]
