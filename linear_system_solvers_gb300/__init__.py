"""GB300-native (sm_103a) 2-D Heston/SABR ADI solver.

A from-scratch device implementation of the implicit ADI time-stepping path of
MichalSara99/linear_system_solvers (Douglas-Rachford, Craig-Sneyd, modified Craig-Sneyd,
Hundsdorfer-Verwer splitting with Thomas-LU line solves), exposed through the C-ABI in
``include/lss_adi.h`` (``_build/liblss_adi.so``) and this thin Python layer.
"""
from ._lib import LssError, load  # noqa: F401
from .solver import HestonProblem, ImplicitHestonSolver, TabulatedHestonSolver, thomas_lu_lines  # noqa: F401
from .batch import BatchSolver, draw_batch  # noqa: F401

__all__ = ["HestonProblem", "ImplicitHestonSolver", "TabulatedHestonSolver", "BatchSolver", "draw_batch", "thomas_lu_lines", "LssError",
           "load"]
