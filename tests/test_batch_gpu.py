"""GPU parity of the batched persistent kernel (lss_adi_batch_*) against the CPU oracle."""
import dataclasses

import numpy as np
import pytest

from conftest import fp32_ok, fp64_tol, rel_err

pytestmark = pytest.mark.gpu

NU = dict(nonuniform=True, alpha_scale=10.0, beta_scale=24.0)


def mixed_batch(lss, schemes=("dr", "cs", "mcs", "hv"), seed=3, count=12):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        K = float(rng.uniform(80, 120))
        out.append(lss.HestonProblem(
            kappa=float(rng.uniform(0.5, 5)), theta_v=float(rng.uniform(0.01, 0.1)), sigma=float(rng.uniform(0.1, 1)),
            rho=float(rng.uniform(-0.95, 0)), rate=float(rng.uniform(0, 0.05)), maturity=float(rng.uniform(0.25, 2)),
            strike=K, acc_point=K, nx=int(rng.choice([4, 17, 64, 96, 130, 256])), ny=int(rng.choice([4, 9, 32, 48, 128])),
            nt=int(rng.integers(2, 40)), scheme=schemes[k % len(schemes)],
            zeta=0.8 if (schemes[k % len(schemes)] == "mcs" and k % 8 < 4) else 0.5, **NU))
    return out


def oracle_of(oracle, p):
    import dataclasses

    return oracle.Problem(**p.pde_fields())


@pytest.mark.parametrize("graph", [False, True])
def test_batch_fp64_matches_oracle(lss, oracle, graph):
    probs = mixed_batch(lss)
    b = lss.BatchSolver(probs, precision="f64")
    b.run(mode=0, graph=graph)
    values, _, status = b.results()
    assert np.all(status == 0)
    for k, p in enumerate(probs):
        want = oracle.solve(oracle_of(oracle, p), "f64")
        got = b.surface(k)
        assert rel_err(got, want) < fp64_tol(want, p.s_hi), (k, p.scheme, p.nx, p.ny, p.nt)
        s = lss.ImplicitHestonSolver(p, precision="f64", arith="fast")
        _, v = s.solve()
        assert abs(values[k] - v) <= fp64_tol(want, p.s_hi) * max(1.0, abs(v))


def test_batch_repeat_runs_are_identical(lss):
    probs = mixed_batch(lss, seed=11, count=9)
    b = lss.BatchSolver(probs, precision="f64")
    b.run(0)
    v1, _, _ = b.results()
    s1 = [b.surface(k) for k in range(len(probs))]
    b.run(0, graph=True)
    b.run(0, graph=True)
    v2, _, _ = b.results()
    assert np.array_equal(v1, v2)
    for k in range(len(probs)):
        assert np.array_equal(s1[k], b.surface(k))


def test_batch_fp32_matches_fp32_oracle(lss, oracle):
    probs = mixed_batch(lss, schemes=("dr", "mcs", "hv"), seed=5, count=6)
    b = lss.BatchSolver(probs, precision="f32")
    b.run(0)
    _, _, status = b.results()
    for k, p in enumerate(probs):
        op = oracle_of(oracle, p)
        ok, e_dev, e_ref = fp32_ok(b.surface(k), oracle.solve(op, "f32"), oracle.solve(op, "f64"))
        assert ok, (k, p.scheme, e_dev, e_ref)


def test_batch_config3_sample_within_1e10(lss, oracle):
    from linear_system_solvers_gb300.batch import draw_batch

    probs = draw_batch(24)
    for p in probs:  # keep the oracle side short: truncate the time loop
        p.nt = 21
    b = lss.BatchSolver(probs, precision="f64")
    b.run(0)
    for k, p in enumerate(probs):
        want = oracle.solve(oracle_of(oracle, p), "f64")
        assert rel_err(b.surface(k), want) < fp64_tol(want, p.s_hi)


def test_wide_single_instance_path_is_bitwise_the_batched_kernel(lss):
    """lss_adi_create(FAST) runs the same stage arithmetic as one kernel per stage over the
    whole GPU; for an instance that also fits the batched kernel the bits must agree."""
    probs = mixed_batch(lss, seed=21, count=8)
    b = lss.BatchSolver(probs, precision="f64")
    b.run(0)
    values, _, _ = b.results()
    for k, p in enumerate(probs):
        p.line_per_thread = True
        got, v = lss.ImplicitHestonSolver(p, precision="f64", arith="fast").solve()
        assert np.array_equal(got, b.surface(k), equal_nan=True)
        assert v == values[k] or (np.isnan(v) and np.isnan(values[k]))


@pytest.mark.parametrize("fp", ["f64", "f32"])
def test_wide_path_large_grid(lss, oracle, fp):
    kw = dict(model="heston", kappa=1.5, theta_v=0.04, sigma=0.3, rho=-0.5, rate=0.02, strike=100.0, maturity=1.0,
              s_lo=0.0, s_hi=200.0, v_lo=0.0, v_hi=1.2, nx=401, ny=201, nt=11, scheme="hv", acc_point=100.0, **NU)
    p = lss.HestonProblem(**kw)
    got, _ = lss.ImplicitHestonSolver(p, precision=fp, arith="fast").solve(graph=True)
    op = oracle_of(oracle, p)
    if fp == "f64":
        want = oracle.solve(op, "f64")
        assert rel_err(got, want) < fp64_tol(want, p.s_hi)
    else:
        ok, e_dev, e_ref = fp32_ok(got, oracle.solve(op, "f32"), oracle.solve(op, "f64"))
        assert ok, (e_dev, e_ref)


@pytest.mark.parametrize("scheme", ["dr", "cs", "mcs", "hv"])
@pytest.mark.parametrize("chunks", [(2, 3), (8, 4), (32, 16), (5, 32)])
def test_partitioned_line_solves_match_line_per_thread(lss, oracle, scheme, chunks):
    """Chunked S and v line solves (chunk products hf / hb and composed carries) against the
    thread-per-line solve of the same instance.  They differ by rounding only, which the
    reference's own scheme amplifies: the bound is 100x the spread that a 1e-15 relative
    perturbation of the terminal condition causes in the oracle (floor 1e-13)."""
    kw = dict(model="heston", kappa=2.0, theta_v=0.05, sigma=0.4, rho=-0.3, rate=0.02, strike=100.0, maturity=0.25,
              s_lo=0.0, s_hi=200.0, v_lo=0.0, v_hi=1.2, nx=203, ny=131, nt=17, scheme=scheme, zeta=1.0 / 3.0,
              acc_point=100.0, **NU)
    p = lss.HestonProblem(**kw)
    s = lss.ImplicitHestonSolver(p, precision="f64", arith="fast")
    assert s.line_chunks(*chunks) == chunks
    got, val = s.solve(graph=True)
    ref, rval = lss.ImplicitHestonSolver(dataclasses.replace(p, line_per_thread=True), precision="f64",
                                         arith="fast").solve()
    op = oracle_of(oracle, p)
    want = oracle.solve(op, "f64")
    x, _ = oracle.grid(op, "f64")
    pay = np.maximum(x[:, None] - p.strike, 0.0) * np.ones((1, p.ny))
    noisy = pay * (1.0 + 1e-15 * np.random.default_rng(1).standard_normal(pay.shape))
    amp = rel_err(oracle.solve(op, "f64", payoff=noisy), want)
    tol = max(1e-13, 100.0 * amp)
    assert rel_err(got, ref) < tol
    assert abs(val - rval) <= tol * max(1.0, abs(rval))
    assert rel_err(got, want) < fp64_tol(want, p.s_hi)


@pytest.mark.parametrize("scheme", ["cs", "hv"])
@pytest.mark.parametrize("chunks", [(64, 64), (128, 32)])
def test_many_chunks_match_line_per_thread(lss, oracle, scheme, chunks):
    """64 and 128 chunks per line (CTAs of 16 lines x 64 chunks, 8 x 128) on a grid with at least 4
    rows per chunk, against the thread-per-line solve: rounding-level differences, bounded as in
    the test above."""
    kw = dict(model="heston", kappa=2.0, theta_v=0.05, sigma=0.4, rho=-0.3, rate=0.02, strike=100.0, maturity=0.25,
              s_lo=0.0, s_hi=200.0, v_lo=0.0, v_hi=1.2, nx=522, ny=300, nt=9, scheme=scheme, acc_point=100.0, **NU)
    p = lss.HestonProblem(**kw)
    s = lss.ImplicitHestonSolver(p, precision="f64", arith="fast")
    assert s.line_chunks(*chunks) == chunks
    got, val = s.solve(graph=True)
    ref, rval = lss.ImplicitHestonSolver(dataclasses.replace(p, line_per_thread=True), precision="f64",
                                         arith="fast").solve()
    op = oracle_of(oracle, p)
    want = oracle.solve(op, "f64")
    x, _ = oracle.grid(op, "f64")
    pay = np.maximum(x[:, None] - p.strike, 0.0) * np.ones((1, p.ny))
    noisy = pay * (1.0 + 1e-15 * np.random.default_rng(1).standard_normal(pay.shape))
    amp = rel_err(oracle.solve(op, "f64", payoff=noisy), want)
    tol = max(1e-13, 100.0 * amp)
    assert rel_err(got, ref) < tol
    assert abs(val - rval) <= tol * max(1.0, abs(rval))
    assert rel_err(got, want) < fp64_tol(want, p.s_hi)


def test_partition_autotuner_and_limits(lss):
    p = lss.HestonProblem(scheme="hv", nx=300, ny=100, nt=5, nonuniform=True, acc_point=100.0, alpha_scale=10.0,
                          beta_scale=24.0)
    s = lss.ImplicitHestonSolver(p, precision="f64", arith="fast")
    ps, pv = s.line_chunks(0, 0)
    assert 1 <= ps <= 64 and 1 <= pv <= 64
    from linear_system_solvers_gb300 import _lib as L

    assert s.line_chunks(64, 1) == (64, 1)  # 298 rows: 64 chunks of at least 4
    with pytest.raises(L.LssError):
        s.line_chunks(128, 1)  # 298 rows: fewer than 4 per chunk
    with pytest.raises(L.LssError):
        s.line_chunks(256, 1)  # more than 128 chunks
    with pytest.raises(L.LssError):
        s.line_chunks(1, 32)  # 98 rows: fewer than 4 per chunk
    ref = lss.ImplicitHestonSolver(p, precision="f64", arith="reference")
    with pytest.raises(L.LssError):
        ref.line_chunks(2, 2)


@pytest.mark.parametrize("mode", [0, 1])
def test_cta_size_does_not_change_bits(lss, mode):
    """Each line is solved by one thread whatever the number of warps on an instance, so every cap
    the autotuner may pick gives the same surfaces and values bit for bit; the parameter
    sensitivities are sums over lines whose order follows the thread layout (rounding-level
    differences)."""
    from linear_system_solvers_gb300.batch import draw_batch

    probs = draw_batch(10, seed=77)
    for p in probs:
        p.nt = 15
    b = lss.BatchSolver(probs, precision="f64")
    ref = None
    for threads in (32, 64, 96, 128):
        assert b.autotune(mode=mode, threads=threads) == threads
        b.run(mode)
        v, g, _ = b.results()
        surf = [b.surface(k) for k in range(len(probs))]
        if ref is None:
            ref = (v, g, surf)
        else:
            assert np.array_equal(v, ref[0])
            np.testing.assert_allclose(g, ref[1], rtol=1e-11, atol=1e-14)
            assert all(np.array_equal(a, c) for a, c in zip(surf, ref[2]))
    assert b.autotune(mode=mode) in (32, 64, 128)


def test_batch_with_a_member_larger_than_256_rows(lss, oracle):
    """A batch may mix small instances with one of more than 256 S points (no fixed per-instance
    shared array): every member matches the single-instance fast path and the oracle."""
    from linear_system_solvers_gb300.batch import draw_batch

    probs = draw_batch(5, seed=21)
    for p in probs:
        p.nt = 13
    probs[2].nx, probs[2].ny = 300, 40
    b = lss.BatchSolver(probs, precision="f64")
    b.run(0)
    vals, _, status = b.results()
    for k, p in enumerate(probs):
        want = oracle.solve(oracle_of(oracle, p), "f64")
        got = b.surface(k)
        assert status[k] == 0
        assert rel_err(got, want) < fp64_tol(want, p.s_hi)
