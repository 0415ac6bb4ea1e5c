"""bench.py on the host: the reference arm's JSON line (the reference's own CPU path, no GPU), the
quiet exit of ranks other than 0, and the recomputed-fraction arithmetic behind `fp64_pipe`."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)


def _bench(args, env_extra=None, timeout=600):
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                          env=env, cwd=ROOT, timeout=timeout)


def test_reference_arm_prints_one_contract_line(lss):
    res = _bench(["--impl", "reference", "--steps", "1", "--warmup", "0"])
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in rec, key
    assert rec["impl"] == "reference" and rec["value"] > 0 and rec["higher_is_better"] is True
    assert rec["unit"] == "grid-point-steps/s" and rec["dtype"] == "f64" and rec["steps"] == 1
    assert "workload" in rec["config"]
    cb = rec["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == rec["value"]
    assert rec["e2e"] == {"value": rec["value"], "unit": rec["unit"], "h2d_bytes_per_step": 0,
                          "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_without_work():
    res = _bench(["--impl", "reference", "--steps", "1", "--warmup", "0"],
                 {"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, timeout=120)
    assert res.returncode == 0 and res.stdout.strip() == ""


def test_recompute_fraction():
    import bench
    from linear_system_solvers_gb300.batch import draw_batch

    probs = draw_batch(6, seed=3)
    steps = [p.nt - 1 for p in probs]
    # one segment per instance: nothing recomputed
    assert bench.recompute_fraction(probs, steps) == 0.0
    # interval 1: every step but the last segment's one
    w = [p.nx * p.ny for p in probs]
    want = sum(wi * (s - 1) for wi, s in zip(w, steps)) / sum(wi * s for wi, s in zip(w, steps))
    assert bench.recompute_fraction(probs, [1] * len(probs)) == pytest.approx(want)
    # default: ceil(sqrt(steps)) segments, the grid-point-step weighted share of all but the last
    import math

    num = den = 0
    for wi, s in zip(w, steps):
        c = math.ceil(math.sqrt(s))
        num += wi * ((s + c - 1) // c - 1) * c
        den += wi * s
    assert bench.recompute_fraction(probs) == pytest.approx(num / den)
    # the adjoint's count is what the forward + adjoint capture leaves after its forward passes
    assert 0.0 < bench.CAPTURE_RF < 1.0
    assert 0.0 < bench.FP64_INSTR_ADJ < bench.CAPTURE_FWDADJ
    assert 0.0 < bench.DRAM_BYTES_ADJ < bench.CAPTURE_DRAM_FWDADJ
    # forward only ignores the recomputed fraction; forward + adjoint grows with it by the forward's figure
    assert bench.per_gps(bench.DRAM_BYTES_FWD, bench.DRAM_BYTES_ADJ, 0, 0.7) == bench.DRAM_BYTES_FWD
    d = bench.per_gps(bench.DRAM_BYTES_FWD, bench.DRAM_BYTES_ADJ, 1, 0.7) - bench.per_gps(
        bench.DRAM_BYTES_FWD, bench.DRAM_BYTES_ADJ, 1, 0.2)
    assert d == pytest.approx(0.5 * bench.DRAM_BYTES_FWD)


def test_bench_functions_only_use_names_that_exist():
    """Every global name a function of bench.py reads is defined at module level or is a
    builtin (bench.py imports torch and the package inside functions, so a leg that forgets its
    own import would only fail on a GPU)."""
    import builtins
    import symtable

    import bench

    src = open(os.path.join(ROOT, "bench.py")).read()
    missing = []

    def walk(tab):
        for child in tab.get_children():
            if child.get_type() == "function":
                for sym in child.get_symbols():
                    if sym.is_global() and sym.is_referenced() and not sym.is_assigned():
                        name = sym.get_name()
                        if not hasattr(bench, name) and not hasattr(builtins, name):
                            missing.append((child.get_name(), name))
            walk(child)

    walk(symtable.symtable(src, "bench.py", "exec"))
    assert not missing, missing
