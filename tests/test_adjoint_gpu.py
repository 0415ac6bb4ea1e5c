"""Adjoint (lss_adi_adjoint / batch mode 1) against finite differences and linearity.

The reference has no sensitivities; its forward path is the check: dV/d(kappa, theta, sigma,
rho, r) against Richardson-extrapolated central finite differences of (a) the device forward
and (b) the CPU oracle (bit-exact with the reference's Thomas-LU path), and dV/d(payoff grid)
against the exact linearity of the scheme in the terminal condition.  Bumps: relative 1e-5
and 5e-6 (Heston), 1e-4 and 5e-5 (SABR); the extrapolation (error O(h^4)) is needed because
the reference's genuine modified Craig-Sneyd scheme (zeta != theta) grows by orders of
magnitude per step, so a plain central difference of it carries a relative truncation error
near 1e-5.
"""
import dataclasses

import numpy as np
import pytest

from conftest import oracle_unstable

pytestmark = pytest.mark.gpu

PARAMS = ("kappa", "theta_v", "sigma", "rho", "rate")
BASE = dict(model="heston", kappa=1.5, theta_v=0.04, sigma=0.3, rho=-0.6, rate=0.02, strike=100.0, maturity=1.0,
            s_lo=0.0, s_hi=200.0, v_lo=0.0, v_hi=1.2, nonuniform=True, acc_point=100.0, alpha_scale=10.0,
            beta_scale=24.0, eval_s=100.0, eval_v=0.04)


SABR = dict(model="sabr", sigma=0.4, rho=-0.3, sabr_beta=0.5, rate=0.0, strike=0.05, maturity=1.0, s_lo=0.0,
            s_hi=0.2, v_lo=0.0, v_hi=1.0, nonuniform=True, acc_point=0.05, alpha_scale=10.0, beta_scale=24.0,
            eval_s=0.05, eval_v=0.2)


def bilinear_value(surface, x, y, s0, v0):
    i = max(0, min(len(x) - 2, int(np.searchsorted(x, s0, side="right")) - 1))
    j = max(0, min(len(y) - 2, int(np.searchsorted(y, v0, side="right")) - 1))
    wx = min(1.0, max(0.0, (s0 - x[i]) / (x[i + 1] - x[i])))
    wy = min(1.0, max(0.0, (v0 - y[j]) / (y[j + 1] - y[j])))
    return ((1 - wx) * (1 - wy) * surface[i, j] + wx * (1 - wy) * surface[i + 1, j] + (1 - wx) * wy * surface[i, j + 1]
            + wx * wy * surface[i + 1, j + 1])


def device_value(lss, p):
    # thread-per-line solves: the autotuned chunk counts of a large instance may differ between
    # the bumped problems, which would put rounding noise into the differences
    return lss.ImplicitHestonSolver(dataclasses.replace(p, line_per_thread=True), precision="f64", arith="fast").solve()[1]


def oracle_value(oracle, lss, p):
    kw = p.pde_fields()
    op = oracle.Problem(**kw)
    surf = oracle.solve(op, "f64")
    x, y = oracle.grid(op, "f64")
    return bilinear_value(surf, x, y, p.eval_s, p.eval_v)


def fd_grad(fn, p, name, rel=None):
    base = getattr(p, name)

    def central(h):
        up = dataclasses.replace(p, **{name: base + h})
        dn = dataclasses.replace(p, **{name: base - h})
        return (fn(up) - fn(dn)) / (2 * h)

    if rel is None:
        # SABR sensitivities are ~1e-2 of the value: a larger bump keeps the rounding noise of the
        # differences (value x 1e-14 / h) well below 1e-6 of them
        rel = 1e-4 if p.model == "sabr" else 1e-5
    h = rel * (abs(base) if base != 0.0 else 1.0)  # r = 0: absolute bump rel
    return (4.0 * central(h / 2) - central(h)) / 3.0


CASES = {
    "mcs_64x32": dict(BASE, scheme="mcs", nx=64, ny=32, nt=51),
    "mcs_97x41": dict(BASE, scheme="mcs", nx=97, ny=41, nt=40, rho=-0.3, sigma=0.5, kappa=2.5),
    "cs_60x30": dict(BASE, scheme="cs", nx=60, ny=30, nt=31, rho=-0.2),
    "dr_70x35": dict(BASE, scheme="dr", nx=70, ny=35, nt=41),
    "mcs_z08_theta80": dict(BASE, scheme="mcs", zeta=0.8, theta_scheme="theta80", nx=48, ny=24, nt=31, rho=-0.4),
    "mcs_z08_cn": dict(BASE, scheme="mcs", zeta=0.8, nx=52, ny=26, nt=31, rho=-0.4),
    # SABR at r = 0 (sigma carries nu; kappa and theta do not enter): the r sensitivity comes
    # from d = rF, f = -r and the discount factors D(t) = exp(-r (T - t)) inside a and c
    "sabr_dr": dict(SABR, scheme="dr", nx=48, ny=26, nt=31),
    "sabr_cs": dict(SABR, scheme="cs", nx=44, ny=24, nt=25, rho=0.3),
    "sabr_mcs_z08": dict(SABR, scheme="mcs", zeta=0.8, theta_scheme="theta80", nx=40, ny=22, nt=21),
    # Hundsdorfer-Verwer: the second S stage acts on Y1 along the line, the last v stage on Y2
    "hv_60x30": dict(BASE, scheme="hv", nx=60, ny=30, nt=31),
    "hv_z07_theta80": dict(BASE, scheme="hv", zeta=0.7, theta_scheme="theta80", nx=50, ny=28, nt=21, rho=-0.2),
    "sabr_hv": dict(SABR, scheme="hv", nx=46, ny=24, nt=21),
    # large instances: the adjoint runs as one kernel per stage over the whole GPU
    "wide_heston_cs": dict(BASE, scheme="cs", nx=300, ny=64, nt=21, rho=-0.3),
    "wide_heston_mcs": dict(BASE, scheme="mcs", zeta=1.0 / 3.0, nx=264, ny=160, nt=9, rho=-0.2),
    "wide_sabr_dr": dict(SABR, scheme="dr", nx=280, ny=90, nt=17),
    "wide_heston_hv": dict(BASE, scheme="hv", nx=300, ny=70, nt=13),
    # SABR with r != 0 (the reference's SABR problem, unit_tests/common/lss_print_t.hpp:2039-2042):
    # a and c carry D(t)^(2(1-beta)) and D(t)^(1-beta) at every step's time, so the adjoint runs
    # on the wide kernels with the S-line tables rebuilt before every forward and adjoint step
    "sabr_dr_r03": dict(SABR, scheme="dr", rate=0.03, nx=48, ny=26, nt=31),
    "sabr_mcs_r03": dict(SABR, scheme="mcs", zeta=0.8, theta_scheme="theta80", rate=0.03, nx=40, ny=22, nt=21),
    "sabr_hv_r03": dict(SABR, scheme="hv", rate=0.05, nx=46, ny=24, nt=21),
    "wide_sabr_cs_r03": dict(SABR, scheme="cs", rate=0.03, nx=280, ny=90, nt=17, maturity=2.0),
    # forward time stepping: D(t) at t = k, 2k, ... (the tables and the adjoint's D(t) factors)
    "sabr_hv_fwd_r03": dict(SABR, scheme="hv", forward=True, rate=0.03, nx=44, ny=24, nt=21),
}


@pytest.mark.parametrize("key", sorted(CASES))
def test_parameter_gradients_match_device_finite_differences(lss, key):
    p = lss.HestonProblem(**CASES[key])
    s = lss.ImplicitHestonSolver(p, precision="f64", arith="fast")
    val, grads, _ = s.adjoint(want_payoff_grad=False)
    assert abs(val - device_value(lss, p)) <= 1e-12 * max(1.0, abs(val))
    for k, name in enumerate(PARAMS):
        fd = fd_grad(lambda q: device_value(lss, q), p, name)
        assert abs(grads[k] - fd) <= 1e-6 * max(abs(fd), 1e-3 * abs(val)), (name, grads[k], fd)


@pytest.mark.parametrize("key", ["mcs_64x32", "dr_70x35", "mcs_z08_cn", "sabr_dr", "sabr_mcs_z08", "wide_heston_cs",
                                 "wide_sabr_dr", "hv_60x30", "sabr_hv", "wide_heston_hv", "sabr_dr_r03", "sabr_hv_r03",
                                 "wide_sabr_cs_r03"])
def test_parameter_gradients_match_reference_bump_and_revalue(lss, oracle, key):
    p = lss.HestonProblem(**CASES[key])
    val, grads, _ = lss.ImplicitHestonSolver(p, precision="f64", arith="fast").adjoint(want_payoff_grad=False)
    for k, name in enumerate(PARAMS):
        fd = fd_grad(lambda q: oracle_value(oracle, lss, q), p, name)
        assert abs(grads[k] - fd) <= 1e-6 * max(abs(fd), 1e-3 * abs(val)), (name, grads[k], fd)


@pytest.mark.parametrize("key", ["mcs_64x32", "cs_60x30", "dr_70x35", "sabr_cs", "wide_heston_mcs", "hv_60x30",
                                 "wide_heston_hv", "sabr_mcs_r03", "wide_sabr_cs_r03"])
def test_payoff_gradient_is_the_linear_response(lss, key):
    p = lss.HestonProblem(**CASES[key])
    s = lss.ImplicitHestonSolver(p, precision="f64", arith="fast")
    rng = np.random.default_rng(1)
    payoff = rng.uniform(0.0, 100.0, size=(p.nx, p.ny))
    val, _, lam = s.adjoint(payoff=payoff)
    delta = rng.normal(size=(p.nx, p.ny))
    v1 = s.solve(payoff=payoff + delta)[1]
    v0 = s.solve(payoff=payoff)[1]
    assert abs(v0 - val) <= 1e-12 * max(1.0, abs(val))
    pred = float(np.sum(lam * delta))
    assert abs((v1 - v0) - pred) <= 1e-9 * max(1.0, np.sum(np.abs(lam * delta)))


@pytest.mark.parametrize("key", ["mcs_64x32", "wide_heston_cs", "hv_60x30", "sabr_dr_r03"])
def test_checkpoint_interval_does_not_change_results(lss, key):
    p = lss.HestonProblem(**CASES[key])
    s = lss.ImplicitHestonSolver(p, precision="f64", arith="fast")
    ref = None
    for ck in (0, 1, 3, 7, 50, 1000):
        val, g, lam = s.adjoint(checkpoint_every=ck)
        if ref is None:
            ref = (val, g, lam)
        else:
            assert val == ref[0]
            assert np.array_equal(g, ref[1])
            assert np.array_equal(lam, ref[2])


def test_batch_mode1_matches_single_instance_and_mode0(lss):
    from linear_system_solvers_gb300.batch import draw_batch

    probs = draw_batch(12)
    for p in probs:
        p.nt = 31
    b = lss.BatchSolver(probs, precision="f64")
    b.run(0)
    v0, _, _ = b.results()
    b.run(1)
    v1, g1, st = b.results()
    assert np.array_equal(v0, v1)
    for k in (0, 5, 11):
        val, g, lam = lss.ImplicitHestonSolver(probs[k], precision="f64", arith="fast").adjoint()
        assert val == v1[k]
        np.testing.assert_allclose(g1[k], g, rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(b.payoff_gradient(k), lam, rtol=1e-13, atol=1e-15)


def test_batch_checkpoint_plan(lss):
    """The batch plans each instance's checkpoint interval from the workspace it can hold: at
    least ceil(sqrt(steps)); a small batch on a large device keeps every step (one segment,
    no recomputation).  Results do not depend on the plan."""
    import math

    from linear_system_solvers_gb300.batch import draw_batch

    probs = draw_batch(6, seed=5)
    for p in probs:
        p.nt = 41
    b = lss.BatchSolver(probs, precision="f64")
    b.run(1)
    ck = b.checkpoints()
    v1, g1, _ = b.results()
    for k, p in enumerate(probs):
        steps = p.nt - 1
        assert math.ceil(math.sqrt(steps)) <= ck[k] <= steps
    assert (ck == 40).any()
    for k in (0, 3):
        val, g, _ = lss.ImplicitHestonSolver(probs[k], precision="f64", arith="fast").adjoint(checkpoint_every=7)
        assert val == v1[k]
        np.testing.assert_allclose(g1[k], g, rtol=1e-13, atol=1e-15)


def test_batch_gradients_finite_difference_sample(lss):
    """Config-4 style instances (uneven batch, MCS): stable members checked against FD."""
    from linear_system_solvers_gb300.batch import draw_batch

    probs = draw_batch(16, seed=20261204)
    for p in probs:
        p.nt = 21
        p.nx = min(p.nx, 96)
        p.ny = min(p.ny, 48)
    b = lss.BatchSolver(probs, precision="f64")
    b.run(1)
    vals, grads, _ = b.results()
    checked = 0
    for k, p in enumerate(probs):
        surf = b.surface(k)
        if oracle_unstable(surf, p.s_hi):
            continue
        for q, name in enumerate(PARAMS):
            fd = fd_grad(lambda pp: device_value(lss, pp), p, name)
            assert abs(grads[k, q] - fd) <= 1e-6 * max(abs(fd), 1e-3 * abs(vals[k])), (k, name, grads[k, q], fd)
        checked += 1
    assert checked >= 4


@pytest.mark.parametrize("key", ["wide_heston_mcs", "wide_heston_hv", "wide_sabr_dr"])
def test_wide_adjoint_partitioned_solves_match_line_per_thread(lss, key):
    """The wide adjoint's partitioned transposed solves (chunk products, composed carries)
    against its thread-per-line solves, with the forward chunked alike: the same derivatives
    up to rounding."""
    p = lss.HestonProblem(**CASES[key])
    ref = lss.ImplicitHestonSolver(dataclasses.replace(p, line_per_thread=True), precision="f64", arith="fast")
    v0, g0, l0 = ref.adjoint()
    for chunks in ((4, 2), (16, 8), (32, 4), (64, 2)):  # 64 chunks: CTAs of 16 lines
        s = lss.ImplicitHestonSolver(p, precision="f64", arith="fast")
        assert s.line_chunks(*chunks) == chunks
        v, g, lam = s.adjoint()
        assert abs(v - v0) <= 1e-12 * max(1.0, abs(v0))
        scale = max(np.abs(g0).max(), 1e-3 * abs(v0))
        assert np.max(np.abs(g - g0)) <= 1e-9 * scale, (chunks, g, g0)
        assert np.max(np.abs(lam - l0)) <= 1e-9 * np.abs(l0).max()


def test_plain_central_difference_error_is_the_difference_own_noise(lss, oracle):
    """A stable instance drawn as config 4 (seed 20261204): the adjoint gradient agrees with
    Richardson-extrapolated central differences of the oracle (bumps 1e-3 / 5e-4) to 5e-7, while
    the plain central difference at the relative bump 1e-5 sits farther from both -- by about the
    spread between two plain differences at nearby bumps (1e-5 and 1.25e-5), i.e. its own
    rounding noise: the oracle's value carries ~1e-13 relative rounding, divided by a bump of
    1e-5 relative.  The 1e-6 criterion against a plain 1e-5 difference therefore measures the
    difference, not the adjoint."""
    from linear_system_solvers_gb300.batch import draw_batch

    cands = draw_batch(64, seed=20261204)
    p = None
    for q in cands:
        q.nt = 61
        if q.nx <= 96 and q.ny <= 48:
            surf = oracle.solve(oracle.Problem(**q.pde_fields()), "f64")
            if not oracle_unstable(surf, q.s_hi):
                p = q
                break
    assert p is not None
    val, grads, _ = lss.ImplicitHestonSolver(p, precision="f64", arith="fast").adjoint(want_payoff_grad=False)

    def central(name, rel):
        base = getattr(p, name)
        h = rel * abs(base)
        up = oracle_value(oracle, lss, dataclasses.replace(p, **{name: base + h}))
        dn = oracle_value(oracle, lss, dataclasses.replace(p, **{name: base - h}))
        return (up - dn) / (2 * h)

    worst_rich = 0.0
    for k, name in enumerate(PARAMS):
        rich = (4.0 * central(name, 5e-4) - central(name, 1e-3)) / 3.0
        plain, plain2 = central(name, 1e-5), central(name, 1.25e-5)
        den = max(abs(rich), 1e-3 * abs(val))
        worst_rich = max(worst_rich, abs(grads[k] - rich) / den)
        # the plain difference's distance from the adjoint is within a small multiple of its
        # distance from the noise-free Richardson difference plus its own bump-to-bump spread
        assert abs(grads[k] - plain) <= 2.0 * (abs(plain - rich) + abs(plain - plain2)) + 5e-7 * den, name
    assert worst_rich < 5e-7


def test_workspace_cap_is_honoured_and_results_do_not_depend_on_it(lss):
    """lss_adi_batch_set_workspace bounds the forward + adjoint workspace: a tight cap holds less
    memory and recomputes more (shorter checkpoint intervals), the results stay the same --
    values and dV/d(initial condition) bit for bit, the parameter sums at rounding level (their
    order follows the warp groups)."""
    from linear_system_solvers_gb300.batch import draw_batch

    probs = draw_batch(20, seed=11)
    for p in probs:
        p.nt = 41
    b = lss.BatchSolver(probs, precision="f64")
    b.set_workspace(0.0)  # default: a quarter of the device memory
    b.run(1)
    v_big, g_big, _ = b.results()
    ck_big = b.checkpoints()
    lam_big = [b.payoff_gradient(k) for k in (0, 7)]
    cap = 64e6
    b.set_workspace(cap)
    b.run(1)
    assert 0 < b.workspace_bytes() <= cap
    v_small, g_small, _ = b.results()
    ck_small = b.checkpoints()
    assert (ck_small <= ck_big).all() and (ck_small < ck_big).any()
    assert np.array_equal(v_small, v_big)
    np.testing.assert_allclose(g_small, g_big, rtol=1e-12, atol=1e-14)
    for k, lam in zip((0, 7), lam_big):
        assert np.array_equal(b.payoff_gradient(k), lam)
    from linear_system_solvers_gb300 import _lib as L

    b.set_workspace(1e3)  # cannot hold the checkpoints of one instance
    with pytest.raises(L.LssError):
        b.run(1)
