"""GPU parity of the batched 1-D implicit heat / Black-Scholes path (include/lss_heat1d.h) against
the CPU oracle (oracle/lss_oracle_1d_impl.h, pinned bit for bit to the reference).

* reference arithmetic: bit-identical to the oracle, every time level, every boundary kind, both
  tridiagonal policies, heat source, both directions, FP64 and FP32;
* fast arithmetic: within 1e-10 relative (FP64) of the oracle; FP32 as close to the FP64 oracle
  as the reference's own FP32 run (3x, or 1e-4);
* uneven Black-Scholes batches (sizes, steps, calls and puts in one launch) and the values at
  the evaluation point; the end-to-end host call.
"""
import numpy as np
import pytest

from cases_1d import GOLDEN_1D, SMALL_1D
from conftest import fp32_ok, rel_err

pytestmark = pytest.mark.gpu

CASES = dict(SMALL_1D)
for _name, (_kw, _every) in GOLDEN_1D.items():
    CASES["golden_" + _name] = (_kw, "f64")

# decides what the FP32 bound compares against
ALL_FP = [(k, fp) for k in sorted(CASES) for fp in ("f64", "f32")]


def tables_problem(oracle, kw, fp):
    p = oracle.Heat1DProblem(**kw)
    t = oracle.tables_1d(p, fp)
    return p, dict(n=p.n, nt=p.nt, t_lo=p.t_lo, t_hi=p.t_hi, theta_scheme=p.theta_scheme, forward=p.forward,
                   lo_kind=oracle.BC_KINDS[p.lo_kind] if p.model == "const" else 0,
                   hi_kind=oracle.BC_KINDS[p.hi_kind] if p.model == "const" else 0,
                   coef=t["coef"], initial=t["init"], boundary=t["bnd"], source=t["src"])


def bs_oracle_problem(oracle, q):
    return oracle.Heat1DProblem(model="bs", sigma=q.sigma, rate=q.rate, strike=q.strike, put=q.put, x_lo=q.s_lo,
                                x_hi=q.s_hi, t_lo=0.0, t_hi=q.maturity, n=q.n, nt=q.nt, theta_scheme=q.theta_scheme,
                                nonuniform=q.nonuniform, acc_point=q.acc_point, alpha_scale=q.alpha_scale,
                                forward=False)


@pytest.mark.parametrize("key,fp", ALL_FP)
def test_heat1d_reference_arith_bitwise(lss, oracle, key, fp):
    kw, _ = CASES[key]
    p, tab = tables_problem(oracle, kw, fp)
    b = lss.tabulated_batch([tab], fp, "reference", all_steps=True, double_sweep=p.solver == "ds")
    b.run()
    got = b.solution(0)
    want = oracle.solve_1d(p, fp, all_steps=True)
    assert got.shape == want.shape
    assert np.array_equal(got, want), rel_err(got, want)


@pytest.mark.parametrize("key,fp", ALL_FP)
def test_heat1d_fast_arith_within_tolerance(lss, oracle, key, fp):
    kw, _ = CASES[key]
    p, tab = tables_problem(oracle, kw, fp)
    b = lss.tabulated_batch([tab], fp, "fast", all_steps=True)
    b.run()
    got = b.solution(0)
    want64 = oracle.solve_1d(p, "f64", all_steps=True)
    if fp == "f64":
        assert rel_err(got, want64) < 1e-10
    else:
        ok, e_dev, e_ref = fp32_ok(got, oracle.solve_1d(p, "f32", all_steps=True), want64)
        assert ok, (e_dev, e_ref)


def test_heat1d_mixed_batch_one_launch(lss, oracle):
    # every case of the table in one batch (equal sizes share a group of 32 lanes with different
    # boundary kinds, steps, directions and sources): each instance as if solved alone
    keys = sorted(SMALL_1D)
    probs, tabs = [], []
    for _ in range(3):
        for k in keys:
            kw, _ = SMALL_1D[k]
            p, t = tables_problem(oracle, kw, "f64")
            probs.append(p)
            tabs.append(t)
    for arith in ("reference", "fast"):
        # the double-sweep policy is a batch option: keep the Thomas-LU cases
        sel = [i for i, p in enumerate(probs) if p.solver != "ds"]
        b = lss.tabulated_batch([tabs[i] for i in sel], "f64", arith)
        b.run()
        for j, i in enumerate(sel):
            want = oracle.solve_1d(probs[i], "f64")
            got = b.solution(j)
            if arith == "reference":
                assert np.array_equal(got, want), (i, rel_err(got, want))
            else:
                assert rel_err(got, want) < 1e-10, i


def _bs_batch(lss, count, seed=7):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        K = float(rng.uniform(8.0, 12.0))
        out.append(lss.BlackScholesProblem(sigma=float(rng.uniform(0.15, 0.5)), rate=float(rng.uniform(0.0, 0.1)),
                                           strike=K, maturity=float(rng.uniform(0.25, 1.5)), put=bool(i % 3 == 0),
                                           s_lo=0.0, s_hi=4.0 * K, n=int(rng.choice([16, 24, 40, 64])),
                                           nt=int(rng.integers(2, 60)), theta_scheme="cn" if i % 4 else "euler",
                                           nonuniform=bool(i % 2), acc_point=K, alpha_scale=3.0, eval_s=K))
    return out


@pytest.mark.parametrize("fp", ["f64", "f32"])
def test_black_scholes_batch_reference_bitwise(lss, oracle, fp):
    qs = _bs_batch(lss, 77)
    b = lss.black_scholes_batch(qs, fp, "reference")
    vals, st = b.run_host()
    assert not st.any()
    for i, q in enumerate(qs):
        p = bs_oracle_problem(oracle, q)
        want = oracle.solve_1d(p, fp)
        assert np.array_equal(b.solution(i), want), i
        x = oracle.grid_1d(p, fp)
        assert np.array_equal(b.grid(i), x)
        j = max(0, min(int(np.searchsorted(x, q.eval_s, side="right")) - 1, q.n - 2))
        w = (q.eval_s - float(x[j])) / (float(x[j + 1]) - float(x[j]))
        w = min(1.0, max(0.0, w))
        assert vals[i] == pytest.approx((1 - w) * float(want[j]) + w * float(want[j + 1]), rel=1e-12, abs=1e-12)


def test_black_scholes_batch_fast_and_double_sweep(lss, oracle):
    qs = _bs_batch(lss, 70, seed=11)
    fast = lss.black_scholes_batch(qs, "f64", "fast")
    fast.run()
    ds = lss.black_scholes_batch(qs, "f64", "reference", double_sweep=True)
    ds.run()
    for i, q in enumerate(qs):
        p = bs_oracle_problem(oracle, q)
        assert rel_err(fast.solution(i), oracle.solve_1d(p, "f64")) < 1e-10, i
        p.solver = "ds"
        assert np.array_equal(ds.solution(i), oracle.solve_1d(p, "f64")), i


def test_black_scholes_batch_every_time_level(lss, oracle):
    qs = _bs_batch(lss, 9, seed=5)
    b = lss.black_scholes_batch(qs, "f64", "reference", all_steps=True)
    b.run()
    for i, q in enumerate(qs):
        want = oracle.solve_1d(bs_oracle_problem(oracle, q), "f64", all_steps=True)
        assert np.array_equal(b.solution(i), want), i


def test_run_host_new_initial_conditions(lss, oracle):
    # run_host uploads new initial conditions: equal to a batch created with them
    keys = ["heat_dirichlet_euler_f64", "heat_robin_robin_cn_f64", "bs_call_cn_bwd_f64"]
    tabs = [tables_problem(oracle, SMALL_1D[k][0], "f64")[1] for k in keys]
    b = lss.tabulated_batch(tabs, "f64", "reference")
    rng = np.random.default_rng(3)
    news = [rng.uniform(0.0, 1.0, t["n"]) for t in tabs]
    vals, st = b.run_host(np.concatenate(news))
    tabs2 = [dict(t, initial=nv) for t, nv in zip(tabs, news)]
    b2 = lss.tabulated_batch(tabs2, "f64", "reference")
    b2.run()
    for i in range(len(tabs)):
        assert np.array_equal(b.solution(i), b2.solution(i))
        assert vals[i] == b2.solution(i)[tabs[i]["n"] // 2]
    assert not st.any()


def test_general_heat_equation_front_end_matches_oracle(lss, oracle):
    # the Python front end samples callables as the reference does (double lambdas):
    # the reference's Black-Scholes test problem, bit for bit in reference arithmetic
    sig, r, K, T = 0.25, 0.2, 10.0, 1.0
    import math

    eq = lss.GeneralHeatEquation1D(
        a=lambda t, x: 0.5 * sig * sig * x * x, b=lambda t, x: r * x, c=lambda t, x: -r,
        initial=lambda x: max(0.0, x - K),
        boundary=(lss.Dirichlet(lambda t: 0.0), lss.Dirichlet(lambda t: 20.0 - K * math.exp(-r * (T - t)))),
        space=(0.0, 20.0), n=100, time=(0.0, T), nt=100, theta_scheme="cn", forward=False, arith="reference")
    want = oracle.solve_1d(oracle.Heat1DProblem(), "f64", all_steps=True)
    assert np.array_equal(eq.solve(), want[0])
    assert np.array_equal(eq.solve_all(), want)
    # Neumann / Robin data and a heat source through the same front end
    kw, _ = SMALL_1D["heat_source_neumann_robin_ds_f64"]
    p = oracle.Heat1DProblem(**kw)
    eq2 = lss.GeneralHeatEquation1D(
        a=lambda t, x: p.diff, b=lambda t, x: p.conv, c=lambda t, x: p.react,
        initial=lambda x: p.init0 + p.init1 * x, source=lambda t, x: p.src0 + p.src1 * x,
        boundary=(lss.Neumann(lambda t: p.lo_value), lss.Robin(lambda t: p.hi_linear, lambda t: p.hi_value)),
        space=(p.x_lo, p.x_hi), n=p.n, time=(p.t_lo, p.t_hi), nt=p.nt, theta_scheme=p.theta_scheme,
        forward=p.forward, double_sweep=True, arith="reference")
    assert np.array_equal(eq2.solve(), oracle.solve_1d(p, "f64"))


def test_minimal_sizes_and_single_step(lss, oracle):
    for kw in (dict(model="const", x_hi=1.0, t_hi=0.1, n=4, nt=2, forward=True, init0=0.0, init1=1.0),
               dict(model="const", x_hi=1.0, t_hi=0.1, n=4, nt=3, forward=True, lo_kind="neumann",
                    hi_kind="robin", hi_linear=0.5, hi_value=0.1, init0=0.2, init1=1.0),
               dict(model="bs", n=5, nt=2)):
        for arith in ("reference", "fast"):
            p, t = tables_problem(oracle, kw, "f64")
            b = lss.tabulated_batch([t], "f64", arith, all_steps=True)
            b.run()
            want = oracle.solve_1d(p, "f64", all_steps=True)
            got = b.solution(0)
            if arith == "reference":
                assert np.array_equal(got, want)
            else:
                assert rel_err(got, want) < 1e-10


def test_nonfinite_status(lss, oracle):
    # a NaN in one instance's initial condition reaches its whole line: its status flags it,
    # the other instances of the same group stay clean
    good = tables_problem(oracle, SMALL_1D["heat_dirichlet_euler_f64"][0], "f64")[1]
    init = good["initial"].copy()
    init[5] = np.nan
    bad = dict(good, initial=init)
    for arith in ("fast", "reference"):
        b = lss.tabulated_batch([good, bad, good], "f64", arith)
        vals, st = b.run_host()
        assert list(st) == [0, 1, 0]
        assert np.isfinite(vals[0]) and np.isfinite(vals[2])


@pytest.mark.parametrize("fp", ["f64", "f32"])
def test_heat1d_long_lines(lss, oracle, fp):
    # long lines: the prefetch rings run many full blocks and load past the last row of the last
    # group in the arena; sizes that are not multiples of the ring length
    qs = [lss.BlackScholesProblem(n=n, nt=6, s_hi=40.0, strike=10.0, nonuniform=True, acc_point=10.0, eval_s=10.0,
                                  theta_scheme=th) for n, th in ((997, "cn"), (2048, "euler"), (4099, "cn"))]
    fast = lss.black_scholes_batch(qs, fp, "fast")
    fast.run()
    ref = lss.black_scholes_batch(qs, fp, "reference")
    ref.run()
    for i, q in enumerate(qs):
        p = bs_oracle_problem(oracle, q)
        want = oracle.solve_1d(p, fp)
        assert np.array_equal(ref.solution(i), want), i
        want64 = oracle.solve_1d(p, "f64")
        if fp == "f64":
            assert rel_err(fast.solution(i), want64) < 1e-10, i
        else:
            ok, e_dev, e_ref = fp32_ok(fast.solution(i), want, want64)
            assert ok, (i, e_dev, e_ref)
