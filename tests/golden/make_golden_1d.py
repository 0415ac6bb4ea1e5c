"""Regenerates the 1-D fixtures of tests/golden/ (run in a checkout that has the reference at
LSS_REFERENCE_DIR, default: a `reference` folder beside the repository's folder, and oracle/_ref/ref_driver_1d built):

* reference_outputs_1d.npz: the reference's own printed 1-D outputs
  outputs/<name>_approx_{double,float}.txt (6 significant digits; lss_print::print,
  common/lss_print.hpp:82-109 final values, :170-225 every time level) parsed into x, [t,] values;
* small_reference_1d.npz: full-precision solutions of tests/golden/cases_1d.py:SMALL_1D computed
  by the compiled reference (every time level).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from cases_1d import GOLDEN_1D, SMALL_1D  # noqa: E402
from oracle import oracle as O  # noqa: E402

REF = os.environ.get("LSS_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")


def parse_curve(path):
    """SPACE_POINTS / [TIME_POINTS /] VALUES text of lss_print::print (1-D)."""
    with open(path) as f:
        lines = [ln.strip() for ln in f if ln.strip()]
    out = {}
    i = lines.index("SPACE_POINTS")
    out["x"] = np.array([float(v) for v in lines[i + 1].split(",")])
    if "TIME_POINTS" in lines:
        j = lines.index("TIME_POINTS")
        out["t"] = np.array([float(v) for v in lines[j + 1].split(",")])
    k = lines.index("VALUES")
    vals = np.array([[float(v) for v in ln.split(",")] for ln in lines[k + 1:]])
    out["values"] = vals if "t" in out else vals[0]
    return out


def main():
    out = {}
    for name in GOLDEN_1D:
        for suffix, fp in (("double", "f64"), ("float", "f32")):
            path = os.path.join(REF, "outputs", f"{name}_approx_{suffix}.txt")
            if not os.path.exists(path):
                continue
            for key, arr in parse_curve(path).items():
                out[f"{name}|{fp}|{key}"] = arr
    np.savez_compressed(os.path.join(HERE, "reference_outputs_1d.npz"), **out)
    print(f"reference_outputs_1d.npz: {len(out)} arrays")

    small = {}
    for key, (kw, fp) in SMALL_1D.items():
        vals, _ = O.run_reference_1d(O.Heat1DProblem(**kw), fp, all_steps=True)
        small[key] = vals
    np.savez_compressed(os.path.join(HERE, "small_reference_1d.npz"), **small)
    print(f"small_reference_1d.npz: {len(small)} solutions")


if __name__ == "__main__":
    main()
