"""Host replay of the index arithmetic of the partitioned line solves (k_wide_s_chunk,
k_wide_v_chunk and its shared-memory tiles, the adjoint chunk kernels): for every chunk count
and lines-per-CTA the autotuner or lss_adi_line_chunks can set, every row segment a warp's tile
copies stays inside its line, the chunks cover every row of a line exactly once, and the CTA
shapes fit the kernels' shared arrays.  No GPU: the kernels' formulas restated in Python
(linear_system_solvers_gb300/csrc/adi_batched.cu: chunk_range, set_wide_chunks, the own_*
lambdas of k_wide_v_chunk, carry2d)."""
import itertools

import pytest

VT = 4            # columns of a tile's recurrence window
MAX_CHUNKS = 128
CARRY = 1024      # values per carry array (carry2d)


def chunk_range(e, P, c):
    return 1 + (c * e) // P, ((c + 1) * e) // P


def chunk_ok(P, e):
    return 1 <= P <= MAX_CHUNKS and (P == 1 or e >= 4 * P)


def grid_for(n, b):
    return (n + b - 1) // b


def lines_per_cta(lines, sms=152):
    for l in (32, 16):
        if grid_for(lines, l) >= sms:
            return l
    return 8


def cta_shapes(nx, ny, ps, pv, ls=0, lv=0):
    """wide_ls / wide_lv as set_wide_chunks leaves them."""
    wls = ls if ls in (8, 16, 32) else lines_per_cta(ny - 2)
    wlv = lv if lv in (8, 16, 32) else lines_per_cta(nx - 2)
    if pv > 1 and (wlv * pv) % 32 != 0:
        wlv = 32
    while ps > 1 and wls * ps > 1024:
        wls >>= 1
    while pv > 1 and wlv * pv > 1024:
        wlv >>= 1
    return wls, wlv


SIZES = [(6, 6), (37, 41), (203, 131), (300, 100), (522, 300), (1030, 517), (4096, 2048)]


@pytest.mark.parametrize("nx,ny", SIZES)
def test_chunks_cover_every_row_once(nx, ny):
    for e in (nx - 2, ny - 2):
        for P in (1, 2, 4, 8, 16, 32, 64, 128):
            if not chunk_ok(P, e):
                continue
            rows = []
            for c in range(P):
                a, b = chunk_range(e, P, c)
                assert b >= a + (3 if P > 1 else -1)  # at least 4 rows per chunk when partitioned
                rows.extend(range(a, b + 1))
            assert rows == list(range(1, e + 1))


@pytest.mark.parametrize("nx,ny", SIZES)
def test_cta_shapes_fit_the_shared_arrays(nx, ny):
    for ps, pv in itertools.product((1, 2, 4, 8, 16, 32, 64, 128), repeat=2):
        if not (chunk_ok(ps, nx - 2) and chunk_ok(pv, ny - 2)):
            continue
        for ls, lv in itertools.product((0, 8, 16, 32), repeat=2):
            wls, wlv = cta_shapes(nx, ny, ps, pv, ls, lv)
            for L, P in ((wls, ps), (wlv, pv)):
                if P == 1:
                    continue
                assert L * P <= 1024 and L * P <= CARRY  # threads per CTA; carry arrays [c * L + lane]
                assert L in (8, 16, 32)
            if pv > 1:
                assert (wlv * pv) % 32 == 0  # whole warps: one vtile each


def tile_segments(nx, ny, L, P, block):
    """Every (offset, count) row segment the tiled partitioned v sweep copies, per warp and tile
    step, for CTA `block` (the own_in / own_h / own_b / own_f lambdas of k_wide_v_chunk)."""
    e = ny - 2
    warps = (L * P) // 32
    segs = []
    for w in range(warps):
        lanes = []
        for r in range(32):
            lr = (w << 5) + r
            cr, ir = lr // L, 1 + block * L + lr % L
            lanes.append((ir, cr))
        steps_max = max((chunk_range(e, P, cr)[1] - chunk_range(e, P, cr)[0] + VT) // VT for _, cr in lanes)
        for jt in range(steps_max):
            for ir, cr in lanes:
                a, b = chunk_range(e, P, cr)
                tb = a + jt * VT
                kk = min(VT, b - tb + 1)
                if ir <= nx - 2 and kk > 0:
                    segs.append((ir, tb - 1, kk + 2))   # own_in: columns t-1 .. t+VT of `in`
                    segs.append((ir, tb, kk))           # own_h / own_f: the chunk's columns
                te = b - jt * VT
                ts = max(a, te - VT + 1)
                if ir <= nx - 2 and te >= a:
                    segs.append((ir, ts, te - ts + 1))  # own_b: tiles from the chunk's end
    return segs


@pytest.mark.parametrize("nx,ny,P,L", [(37, 41, 8, 32), (203, 131, 32, 32), (300, 100, 16, 16),
                                       (522, 300, 64, 16), (1030, 517, 128, 8), (70, 516, 128, 8)])
def test_tile_copies_stay_inside_their_line(nx, ny, P, L):
    assert chunk_ok(P, ny - 2)
    blocks = grid_for(nx - 2, L)
    covered = set()
    for block in range(blocks):
        for ir, c0, cnt in tile_segments(nx, ny, L, P, block):
            assert 1 <= ir <= nx - 2
            assert 0 <= c0 and c0 + cnt - 1 <= ny - 1       # inside row ir of the state
            assert cnt <= VT + 2                             # the tile's width
            covered.update((ir, c) for c in range(max(c0, 1), min(c0 + cnt, ny - 1)))
    assert len(covered) == (nx - 2) * (ny - 2)               # every interior point is read
