"""Regenerates the committed fixtures of tests/golden/ (run in a checkout that has the
reference at LSS_REFERENCE_DIR, default: a `reference` folder beside the repository's folder, and oracle/_ref built):

* reference_outputs.npz: the reference's own golden surfaces outputs/<name>_{double,float}.txt
  (6 significant digits) parsed into arrays x, y, values;
* small_reference.npz: full-precision surfaces of tests/golden/cases.py:SMALL computed by the
  compiled reference (oracle/_ref/ref_driver).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from cases import GOLDEN, SMALL  # noqa: E402
from oracle import oracle as O  # noqa: E402

REF = os.environ.get("LSS_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")


def parse_surface(path):
    with open(path) as f:
        lines = [ln.strip() for ln in f if ln.strip()]
    i = lines.index("SPACE_POINTS_X")
    x = np.array([float(v) for v in lines[i + 1].split(",")])
    j = lines.index("SPACE_POINTS_Y")
    y = np.array([float(v) for v in lines[j + 1].split(",")])
    k = lines.index("VALUES")
    vals = np.array([[float(v) for v in ln.split(",")] for ln in lines[k + 1:]])
    return x, y, vals


def main():
    out = {}
    for name in GOLDEN:
        for suffix, fp in (("double", "f64"), ("float", "f32")):
            path = os.path.join(REF, "outputs", f"{name}_{suffix}.txt")
            if not os.path.exists(path):
                continue
            x, y, v = parse_surface(path)
            out[f"{name}|{fp}|x"] = x
            out[f"{name}|{fp}|y"] = y
            out[f"{name}|{fp}|values"] = v
    np.savez_compressed(os.path.join(HERE, "reference_outputs.npz"), **out)
    print(f"reference_outputs.npz: {len(out) // 3} surfaces")

    small = {}
    for key, (kw, fp) in SMALL.items():
        p = O.Problem(**kw)
        surf, _ = O.run_reference(p, fp)
        small[key] = surf
    np.savez_compressed(os.path.join(HERE, "small_reference.npz"), **small)
    print(f"small_reference.npz: {len(small)} surfaces")


if __name__ == "__main__":
    main()
