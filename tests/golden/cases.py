"""Problem definitions of the reference's golden surfaces and of the small fixtures.

GOLDEN: the reference's own print tests that wrote outputs/*.txt (6 significant digits):
  unit_tests/common/lss_print_t.hpp:1724-1848  (CUDA QR policy, DR)        -> ImplHestonEquationCUDAQRSolverCrankNicolson
  unit_tests/common/lss_print_t.hpp:1850-1974  (Thomas LU, DR)             -> ImplHestonEquationThomasLUSolverCrankNicolson
  unit_tests/common/lss_print_t.hpp:1976-2102  (SABR, double sweep, DR)    -> ImplSABREquationDoubleSweepSolverCrankNicolson
  unit_tests/common/lss_print_t.hpp:2104-2222  (Thomas LU, DR, uniform)    -> ImplHestonEquationThomasLUSolverDouglasRachfordCrankNicolson
  unit_tests/common/lss_print_t.hpp:2224-2345  (Thomas LU, CS zeta=0.8)    -> ImplHestonEquationThomasLUSolverCraigSneydCrankNicolson
  unit_tests/common/lss_print_t.hpp:2347-2468  (Thomas LU, MCS)            -> ImplHestonEquationThomasLUSolverModCraigSneydCrankNicolson
  unit_tests/common/lss_print_t.hpp:2470-2591  (Thomas LU, HV)             -> ImplHestonEquationThomasLUSolverHundsdorferVerwerCrankNicolson
  unit_tests/builders/lss_2d_general_heston_equation_builder_t.hpp:55-162 (double sweep, DR)
                                                                            -> ImplHestonEquationDSSolverCrankNicolsonFromBuilder
SMALL: problems run through the compiled reference at full precision (make_golden.py).
"""

HESTON_TEST = dict(model="heston", kappa=2.0, theta_v=0.2, sigma=0.3, rho=0.2, rate=0.03, maturity=1.0)

GOLDEN = {
    "ImplHestonEquationThomasLUSolverCrankNicolson": dict(
        HESTON_TEST, strike=100.0, nx=150, ny=50, nt=200, s_lo=30.0, s_hi=200.0, v_lo=0.0, v_hi=1.2, scheme="dr",
        nonuniform=True, acc_point=100.0, alpha_scale=3.0, beta_scale=50.0, solver="tlu"),
    "ImplHestonEquationThomasLUSolverDouglasRachfordCrankNicolson": dict(
        HESTON_TEST, strike=100.0, nx=150, ny=50, nt=200, s_lo=50.0, s_hi=150.0, v_lo=0.0, v_hi=1.2, scheme="dr",
        nonuniform=False, acc_point=0.0, alpha_scale=3.0, beta_scale=50.0, solver="tlu"),
    "ImplHestonEquationThomasLUSolverCraigSneydCrankNicolson": dict(
        HESTON_TEST, strike=100.0, nx=150, ny=50, nt=200, s_lo=50.0, s_hi=200.0, v_lo=0.0, v_hi=1.2, scheme="cs",
        zeta=0.8, theta_scheme="theta80", nonuniform=True, acc_point=100.0, alpha_scale=3.0, beta_scale=50.0,
        solver="tlu"),
    "ImplHestonEquationThomasLUSolverModCraigSneydCrankNicolson": dict(
        HESTON_TEST, strike=100.0, nx=150, ny=50, nt=200, s_lo=50.0, s_hi=180.0, v_lo=0.0, v_hi=1.2, scheme="mcs",
        zeta=0.5, nonuniform=True, acc_point=100.0, alpha_scale=3.0, beta_scale=50.0, solver="tlu"),
    "ImplHestonEquationThomasLUSolverHundsdorferVerwerCrankNicolson": dict(
        HESTON_TEST, strike=100.0, nx=150, ny=50, nt=200, s_lo=50.0, s_hi=200.0, v_lo=0.0, v_hi=1.2, scheme="hv",
        nonuniform=True, acc_point=100.0, alpha_scale=3.0, beta_scale=50.0, solver="tlu"),
    "ImplHestonEquationCUDAQRSolverCrankNicolson": dict(
        HESTON_TEST, strike=10.0, nx=100, ny=50, nt=150, s_lo=0.0, s_hi=20.0, v_lo=0.0, v_hi=1.0, scheme="dr",
        nonuniform=True, acc_point=10.0, alpha_scale=10.0 / 3.0, beta_scale=1.0, solver="tlu"),
    "ImplHestonEquationDSSolverCrankNicolsonFromBuilder": dict(
        HESTON_TEST, strike=10.0, nx=100, ny=50, nt=150, s_lo=0.0, s_hi=20.0, v_lo=0.0, v_hi=1.5, scheme="dr",
        nonuniform=True, acc_point=10.0, alpha_scale=3.0, beta_scale=60.0, solver="ds"),
    "ImplSABREquationDoubleSweepSolverCrankNicolson": dict(
        model="sabr", sigma=0.081, rho=0.6, sabr_beta=0.7, rate=0.03, maturity=1.0, strike=100.0, nx=100, ny=50,
        nt=200, s_lo=50.0, s_hi=200.0, v_lo=0.0, v_hi=1.2, scheme="dr", nonuniform=True, acc_point=100.0,
        alpha_scale=3.0, beta_scale=50.0, solver="ds"),
}

# Benchmark configuration 1 (DR, FP64, 100 x 50, 200 steps, reference "Uniform" hints)
CONFIG1 = dict(model="heston", kappa=1.5, theta_v=0.04, sigma=0.3, rho=-0.9, rate=0.02, strike=100.0, maturity=1.0,
               s_lo=0.0, s_hi=200.0, v_lo=0.0, v_hi=1.2, nx=100, ny=50, nt=201, scheme="dr")

_NU = dict(nonuniform=True, acc_point=100.0, alpha_scale=10.0, beta_scale=24.0)
SMALL = {
    "dr_uniform_f64": (dict(CONFIG1, nx=37, ny=23, nt=41), "f64"),
    "dr_uniform_f32": (dict(CONFIG1, nx=37, ny=23, nt=41), "f32"),
    "cs_nu_f64": (dict(CONFIG1, scheme="cs", nx=48, ny=25, nt=31, **_NU), "f64"),
    "mcs_z08_f64": (dict(CONFIG1, scheme="mcs", zeta=0.8, theta_scheme="theta80", nx=41, ny=19, nt=31, **_NU), "f64"),
    "mcs_nu_f32": (dict(CONFIG1, scheme="mcs", nx=41, ny=19, nt=31, **_NU), "f32"),
    "hv_nu_f64": (dict(CONFIG1, scheme="hv", nx=50, ny=26, nt=33, **_NU), "f64"),
    "hv_euler_f64": (dict(CONFIG1, scheme="hv", theta_scheme="euler", nx=31, ny=17, nt=21, **_NU), "f64"),
    "dr_theta30_fwd_f64": (dict(CONFIG1, theta_scheme="theta30", forward=True, nx=30, ny=20, nt=25), "f64"),
    "dr_ds_f64": (dict(CONFIG1, solver="ds", nx=33, ny=21, nt=26), "f64"),
    "sabr_ds_f64": (dict(GOLDEN["ImplSABREquationDoubleSweepSolverCrankNicolson"], nx=40, ny=24, nt=30), "f64"),
    "cs_tiny4_f64": (dict(CONFIG1, scheme="cs", nx=4, ny=4, nt=5), "f64"),
    # explicit_solvers::general_heston_equation, host explicit Euler (stable: small time steps)
    "euler_f64": (dict(CONFIG1, scheme="euler", rho=-0.5, nx=30, ny=20, nt=401, maturity=0.25), "f64"),
    "euler_nu_f32": (dict(CONFIG1, scheme="euler", rho=-0.5, nx=24, ny=16, nt=301, maturity=0.2, nonuniform=True,
                          acc_point=100.0, alpha_scale=3.0, beta_scale=50.0), "f32"),
    "euler_fwd_f64": (dict(CONFIG1, scheme="euler", rho=-0.5, nx=20, ny=14, nt=201, maturity=0.1, forward=True), "f64"),
    "euler_sabr_f64": (dict(GOLDEN["ImplSABREquationDoubleSweepSolverCrankNicolson"], scheme="euler", nx=22, ny=16,
                            nt=301, maturity=0.2), "f64"),
}
