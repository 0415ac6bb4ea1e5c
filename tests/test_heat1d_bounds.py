"""Index arithmetic of the factorised 1-D sweep (k_h1_fast in linear_system_solvers_gb300/csrc/heat1d.cu)
checked on the host: the rows its register rings load, replayed for every size and boundary kind,
stay inside the point arrays (a group's 8 slots of n rows, plus H1_PAD rows after the last group).
The loops below mirror the kernel's: the first solved row, the forward ring (PF points ahead), the
last solved row, the back-substitution ring (PFB points behind)."""
import pytest

PF = 16   # H1_PF
PFB = 16  # H1_PFB
PAD_ROWS = PF + 2  # H1_PAD / 32 lanes
NSLOT = 8
S_B, S_D, S_M, S_G, S_U, S_Y = 1, 2, 3, 4, 6, 7


def loaded_rows(n, lo_dirichlet, hi_dirichlet):
    """(slot, row) of every load of one time step of k_h1_fast."""
    N = n - 1
    start = 1 if lo_dirichlet else 0
    end = n - 2 if hi_dirichlet else n - 1
    rows = []
    # first solved row
    if start:
        rows.append((S_U, 0))
    rows += [(S_U, start), (S_U, start + 1), (S_B, start), (S_D, start), (S_M, start)]
    # forward ring: prefetch, then PF points ahead while t + PF <= end
    t = start + 1
    for j in range(PF):
        rows += [(S_B, t + j), (S_D, t + j), (S_M, t + j), (S_U, t + j + 1)]
    while t + PF <= end:
        for j in range(PF):
            q = t + j + PF
            rows += [(S_B, q), (S_D, q), (S_M, q), (S_U, q + 1)]
        t += PF
    # last solved row
    if end > start:
        rows += [(S_B, end), (S_D, end), (S_M, end)]
        if end < N:
            rows.append((S_U, end + 1))
    # back substitution: prefetch, then PFB points behind while t - PFB >= start - 1
    t = end - 1
    for j in range(PFB):
        rows += [(S_Y, t - j), (S_G, t - j)]
    while t - PFB >= start - 1:
        for j in range(PFB):
            q = t - j - PFB
            rows += [(S_Y, q), (S_G, q)]
        t -= PFB
    return rows


@pytest.mark.parametrize("lo_dirichlet", [False, True])
@pytest.mark.parametrize("hi_dirichlet", [False, True])
def test_fast_sweep_loads_stay_in_the_point_arrays(lo_dirichlet, hi_dirichlet):
    for n in range(4, 700):  # lss_heat1d_batch_create rejects n < 4
        offs = [slot * n + row for slot, row in loaded_rows(n, lo_dirichlet, hi_dirichlet)]
        # first group of the arena: nothing below its slot 0; last group: nothing past H1_PAD
        assert min(offs) >= 0, n
        assert max(offs) < NSLOT * n + PAD_ROWS, n


def test_every_solved_row_is_loaded():
    """The rings cover every row the sweeps use (the loads past either end are the unused ones)."""
    for n in (4, 5, 17, 33, 128, 130):
        for lo in (False, True):
            for hi in (False, True):
                start = 1 if lo else 0
                end = n - 2 if hi else n - 1
                got = set(loaded_rows(n, lo, hi))
                for t in range(start, end + 1):
                    assert (S_B, t) in got and (S_M, t) in got
                for t in range(start, end):
                    assert (S_Y, t) in got and (S_G, t) in got
