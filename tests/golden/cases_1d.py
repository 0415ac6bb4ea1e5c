"""1-D implicit heat / Black-Scholes cases of the reference's tests (keyword arguments of
oracle.Heat1DProblem).

GOLDEN_1D: the reference's own printed outputs outputs/<name>_{double,float}.txt, with the
problems of unit_tests/common/lss_print_t.hpp:105-566 (Black-Scholes, Thomas LU, Euler and
Crank-Nicolson, final values and every time level) and :949-1076 (advection-diffusion, forward
Crank-Nicolson, every time level).  Value: (kwargs, every time level printed).

SMALL_1D: small problems run through the compiled reference (oracle/_ref/ref_driver_1d) at full
precision (tests/golden/small_reference_1d.npz): every boundary kind on both ends, both
tridiagonal policies, the heat source, both directions, both theta schemes.
"""

BS = dict(model="bs", sigma=0.25, rate=0.2, strike=10.0, x_lo=0.0, x_hi=20.0, t_lo=0.0, t_hi=1.0, n=100, nt=100,
          forward=False)
UNIT = dict(model="const", x_lo=0.0, x_hi=1.0, t_lo=0.0, t_hi=0.1, forward=True)

GOLDEN_1D = {
    "ImplBlackScholesEquationDirichletBCThomasLUSolverEuler": (dict(BS, theta_scheme="euler"), False),
    "ImplBlackScholesEquationDirichletBCThomasLUSolverCrankNicolson": (dict(BS, theta_scheme="cn"), False),
    "ImplBlackScholesEquationDirichletBCThomasLUSolverEulerSurf": (dict(BS, theta_scheme="euler", acc_point=10.0), True),
    "ImplBlackScholesEquationDirichletBCThomasLUSolverSurf": (
        dict(BS, theta_scheme="cn", acc_point=10.0, alpha_scale=3.0, nonuniform=True), True),
    "ImplAdvDiffEquationDirichletBCThomasLUSolverCN": (
        dict(UNIT, diff=1.0, conv=-1.0, react=0.0, init0=1.0, init1=0.0, theta_scheme="cn", nonuniform=True,
             acc_point=0.5, alpha_scale=3.0, n=100, nt=100), True),
}

_S = dict(UNIT, n=24, nt=21)
SMALL_1D = {
    "bs_call_cn_bwd_f64": (dict(BS, n=40, nt=31), "f64"),
    "bs_put_euler_nonuniform_f32": (dict(BS, n=40, nt=31, put=True, theta_scheme="euler", nonuniform=True,
                                         acc_point=10.0), "f32"),
    "bs_call_ds_f64": (dict(BS, n=40, nt=31, solver="ds"), "f64"),
    "heat_dirichlet_euler_f64": (dict(_S, init0=0.0, init1=1.0, theta_scheme="euler"), "f64"),
    "heat_neumann_cn_f64": (dict(_S, init0=0.0, init1=1.0, lo_kind="neumann", hi_kind="neumann", lo_value=0.3,
                                 hi_value=-0.2), "f64"),
    "heat_robin_robin_cn_f64": (dict(_S, init0=0.3, init1=1.0, lo_kind="robin", lo_value=0.2, lo_linear=1.5,
                                     hi_kind="robin", hi_value=-0.1, hi_linear=-0.7), "f64"),
    "heat_robin_neumann_ds_f32": (dict(_S, init0=0.3, init1=1.0, lo_kind="robin", lo_value=0.2, lo_linear=1.5,
                                       hi_kind="neumann", hi_value=-0.1, solver="ds"), "f32"),
    "heat_source_neumann_robin_ds_f64": (dict(_S, init0=0.3, init1=1.0, lo_kind="neumann", lo_value=0.2,
                                              hi_kind="robin", hi_value=-0.1, hi_linear=0.4, solver="ds",
                                              has_source=True, src0=0.5, src1=1.0), "f64"),
    "advdiff_source_nonuniform_bwd_f64": (dict(_S, diff=0.7, conv=-1.0, react=-0.3, init0=1.0, init1=0.0,
                                               has_source=True, src1=1.0, nonuniform=True, acc_point=0.5,
                                               forward=False), "f64"),
}
