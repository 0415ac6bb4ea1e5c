"""Surface writer in the reference's text format (common/lss_print.hpp:119-160).

    SPACE_POINTS_X
    x0,x1,...                (physical S grid: the sinh map of the computational grid)
    SPACE_POINTS_Y
    y0,y1,...
    VALUES
    V(0,0),V(0,1),...        (one line per S index)

Numbers use the C++ stream default (6 significant digits, shortest of fixed/scientific),
so a surface written here can be diffed against the reference's outputs/*.txt.
"""
from __future__ import annotations

import io

import numpy as np


def _fmt(v: float) -> str:
    """operator<<(std::ostream&, double) with default flags and precision 6."""
    v = float(v)
    if v != v:
        return "nan" if not np.signbit(v) else "-nan"
    if v in (float("inf"), float("-inf")):
        return "inf" if v > 0 else "-inf"
    return "%g" % v


def format_surface(x, y, values) -> str:
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    values = np.asarray(values, dtype=np.float64)
    if values.shape != (len(x), len(y)):
        raise ValueError("The input cont container must have the correct size")
    out = io.StringIO()
    out.write("SPACE_POINTS_X\n")
    out.write(",".join(_fmt(v) for v in x))
    out.write("\nSPACE_POINTS_Y\n")
    out.write(",".join(_fmt(v) for v in y))
    out.write("\nVALUES\n")
    for r in range(values.shape[0]):
        out.write(",".join(_fmt(v) for v in values[r]))
        out.write("\n")
    return out.getvalue()


def print_surface(solver, values, stream=None) -> str:
    """Write `values` (from solver.solve()) with the solver's grid; returns the text."""
    x, y = solver.grid()
    text = format_surface(x, y, values)
    if stream is not None:
        stream.write(text)
    return text
