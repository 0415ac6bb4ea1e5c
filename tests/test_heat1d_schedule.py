"""Placement of the 1-D groups on the warps of the factorised sweep
(linear_system_solvers_gb300/csrc/heat1d_schedule.hpp), compiled on the host and checked without a
GPU: every group runs exactly once, in range, and the work of every SM sub-partition is balanced."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "heat1d_schedule_t.cpp")
SUBPARTITIONS = 4
SMS = 152
WARPS = 16


@pytest.fixture(scope="module")
def schedule_binary():
    out = os.path.join(tempfile.mkdtemp(), "heat1d_schedule_t")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "linear_system_solvers_gb300", "csrc"), SRC, "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def schedule(binary, work, sms=SMS, warps=WARPS):
    res = subprocess.run([binary, str(sms), str(warps)], input="\n".join(repr(float(w)) for w in work),
                         capture_output=True, text=True, check=True)
    lines = res.stdout.split("\n")
    head = lines[0].split()
    ctas, wpc = int(head[1]), int(head[3])
    lists = [[int(g) for g in ln.split()] for ln in lines[1:1 + ctas * wpc]]
    assert len(lists) == ctas * wpc
    return ctas, wpc, lists


def subpartition_loads(work, ctas, wpc, lists):
    loads = np.zeros((ctas, SUBPARTITIONS))
    for w, gl in enumerate(lists):
        loads[w // wpc, (w % wpc) % SUBPARTITIONS] += sum(work[g] for g in gl)
    return loads


def check(work, ctas, wpc, lists, sms=SMS, warps=WARPS):
    got = sorted(g for gl in lists for g in gl)
    assert got == list(range(len(work)))          # every group exactly once
    assert 0 <= ctas <= sms and wpc == warps
    if len(work):
        loads = subpartition_loads(work, ctas, wpc, lists)
        # greedy placement of the costliest first: no bin exceeds the mean over all bins by more
        # than the largest cost
        assert loads.max() <= sum(work) / (sms * SUBPARTITIONS) + max(work) + 1e-9


def groups_of(problems):
    """Group costs (points x steps) of a 1-D batch: instances sorted by size, then steps, both
    descending, cut into groups of 32 of equal size (batch_t::build)."""
    inst = sorted(((p.n, p.nt - 1) for p in problems), key=lambda t: (-t[0], -t[1]))
    work, q = [], 0
    while q < len(inst):
        n, l, steps = inst[q][0], 0, 0
        while q + l < len(inst) and l < 32 and inst[q + l][0] == n:
            steps = max(steps, inst[q + l][1])
            l += 1
        work.append(float(n * steps))
        q += l
    return work


def test_schedule_rejects_bad_arguments(schedule_binary):
    res = subprocess.run([schedule_binary], capture_output=True, text=True)
    assert res.returncode == 2
    assert schedule(schedule_binary, [])[0] == 0
    assert schedule(schedule_binary, [5.0, 3.0], warps=6)[0] == 0  # not a multiple of 4: nothing placed


@pytest.mark.parametrize("warps", [8, 16])  # CTA sizes of the FP64 and FP32 sweeps
@pytest.mark.parametrize("count", [1, 7, 152, 153, 608, 1216, 2432, 2433, 9000])
def test_schedule_places_every_group_once_and_balances(schedule_binary, count, warps):
    rng = np.random.default_rng(count)
    work = list(rng.integers(1, 1000, size=count) * rng.choice([128, 256, 384, 512], size=count))
    ctas, wpc, lists = schedule(schedule_binary, work, warps=warps)
    check(work, ctas, wpc, lists, warps=warps)
    if count <= SMS:  # few groups: one per SM
        assert ctas == count
        assert all(len([g for w in range(c * wpc, (c + 1) * wpc) for g in lists[w]]) == 1 for c in range(ctas))


def test_schedule_on_a_small_device(schedule_binary):
    work = [float(x) for x in range(1, 200)]
    ctas, wpc, lists = schedule(schedule_binary, work, sms=3)
    check(work, ctas, wpc, lists, sms=3)
    assert ctas == 3


@pytest.mark.parametrize("warps", [8, 16])
def test_schedule_balances_the_black_scholes_batch(schedule_binary, warps):
    """65536 uneven calls (n 128-512, 99-999 steps): placed one group per warp in creation order the
    busiest SM carries ~1.8x the mean; placed by cost every SM sub-partition is within a few per
    cent of the mean."""
    from linear_system_solvers_gb300.heat1d import draw_black_scholes

    work = groups_of(draw_black_scholes(65536))
    ctas, wpc, lists = schedule(schedule_binary, work, warps=warps)
    check(work, ctas, wpc, lists, warps=warps)
    assert ctas == SMS
    loads = subpartition_loads(work, ctas, wpc, lists)
    mean = sum(work) / (SMS * SUBPARTITIONS)
    assert loads.max() / mean < 1.05
    # group order of one warp per group, four warps per CTA, CTA b on SM b mod 152 (breadth-first)
    sm = np.zeros(SMS)
    for g, w in enumerate(work):
        sm[(g // 4) % SMS] += w
    assert sm.max() / sm.mean() > 1.5
