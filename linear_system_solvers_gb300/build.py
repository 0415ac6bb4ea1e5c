"""In-tree build of the CUDA library ``_build/liblss_adi.so`` (sm_103a only).

Every translation unit is compiled by nvcc in parallel, then linked into one shared
library whose extern "C" symbols are the ones declared in ``include/lss_adi.h``.
Host code is compiled with ``-ffp-contract=off`` so the host-side table set-up keeps the
reference's two-rounding ``a*b+c``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "liblss_adi.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found (CUDA 13 toolkit required)")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "lss_adi.h"))
    files.append(os.path.join(INCLUDE, "lss_heat1d.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile (if needed) and return the path of liblss_adi.so."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    common = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-I", INCLUDE, "-I", CSRC,
                     "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-Xptxas", "-O3"]
    if os.environ.get("LSS_PTXAS_VERBOSE"):
        common += ["-Xptxas", "-v"]
    # extra nvcc flags, e.g. -DLSS_FWDADJ_MIN_CTAS=4 (register budget of the forward + adjoint kernel)
    common += os.environ.get("LSS_EXTRA_NVCC_FLAGS", "").split()

    def compile_one(src: str) -> str:
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, "-c", src, "-o", obj] + common
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr}")
        if verbose and res.stderr:
            sys.stderr.write(res.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", "-o", tmp] + ARCH + objs + ["-cudart", "shared"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
