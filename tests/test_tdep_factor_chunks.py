"""Host replay of the partitioned S-line refactorisation of time-dependent instances
(k_tdep_s_factor in linear_system_solvers_gb300/csrc/adi_batched.cu): the chunk products of the
Moebius matrices [[b_t, -a_t c_{t-1}], [1, 0]] (rescaled every 8 rows), the composition of the
chunks before a chunk giving its incoming beta, and the chunk's own recurrence reproduce the
serial Thomas factors beta_t = b_t - a_t c_{t-1} / beta_{t-1} to rounding, for every chunk count
the kernel uses (P <= 32 with at least 4 rows per chunk) on the scheme's line matrices
a = -theta M, b = 1 + theta Z, c = -theta P."""
import numpy as np
import pytest


def chunk_range(e, P, c):
    return 1 + (c * e) // P, ((c + 1) * e) // P


def serial(a, b, c):
    e = len(b) - 1  # rows 1..e (index 0 unused)
    beta = np.zeros(e + 1)
    for t in range(1, e + 1):
        beta[t] = b[t] if t == 1 else b[t] - a[t] * (c[t - 1] / beta[t - 1])
    return beta


def chunked(a, b, c, P):
    e = len(b) - 1
    maps = []
    for ch in range(P):
        t0, t1 = chunk_range(e, P, ch)
        m = np.array([[1.0, 0.0], [0.0, 1.0]])
        for t in range(t0, t1 + 1):
            ac = a[t] * c[t - 1] if t > 1 else 0.0
            m = np.array([[b[t], -ac], [1.0, 0.0]]) @ m
            if (t - t0) % 8 == 7:
                m = m / max(abs(m[0, 0]), abs(m[1, 0]))
        maps.append(m)
    beta = np.zeros(e + 1)
    for ch in range(P):
        t0, t1 = chunk_range(e, P, ch)
        x = 1.0
        for q in range(ch):
            m = maps[q]
            x = (m[0, 0] * x + m[0, 1]) / (m[1, 0] * x + m[1, 1])
        gam = c[t0 - 1] / x if t0 > 1 else 0.0
        for t in range(t0, t1 + 1):
            beta[t] = b[t] if t == 1 else b[t] - a[t] * gam
            gam = c[t] / beta[t]
    return beta


@pytest.mark.parametrize("e", [4, 37, 298, 598, 2046])
@pytest.mark.parametrize("seed", [0, 1])
def test_partitioned_recurrence_matches_serial(e, seed):
    r = np.random.default_rng(seed)
    theta = 0.5
    # M, P >= 0 and Z = M + P + (reaction): the implicit S-line matrices of the schemes are
    # diagonally dominant (1 + theta Z >= theta (M + P))
    M = r.uniform(0.0, 50.0, e + 1)
    Pc = r.uniform(0.0, 50.0, e + 1)
    Z = M + Pc + r.uniform(0.0, 1.0, e + 1)
    a, b, c = -theta * M, 1.0 + theta * Z, -theta * Pc
    want = serial(a, b, c)
    P = 1
    while P < 32 and e >= 8 * P:
        P *= 2
    for p in sorted({1, 2, P} & {q for q in (1, 2, 4, 8, 16, 32) if q == 1 or e >= 4 * q}):
        got = chunked(a, b, c, p)
        assert np.max(np.abs(got[1:] - want[1:]) / np.abs(want[1:])) < 1e-13, p
