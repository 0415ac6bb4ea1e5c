/*
 * lss_oracle.h -- CPU oracle for the 2-D Heston/SABR ADI hot path and the 1-D implicit heat
 * path (the latter at the end of this header, lss_oracle_1d_impl.h).
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library, its
 * C-ABI, the Python package) may include, link or call this code.  Only the
 * tests, the smoke check and the CPU-baseline leg of bench.py use it, and only
 * as the checker.
 *
 * It is a plain-C restatement of the reference's host Thomas-LU / double-sweep
 * ADI path (MichalSara99/linear_system_solvers):
 *   - grid / sinh transform:   discretization/lss_grid_config.hpp:33-129,
 *                              discretization/lss_grid_transform_config.hpp:103-188
 *   - coefficient transform:   pde_solvers/transformation/lss_heat_data_transform.hpp:148-221
 *   - scheme coefficients:     pde_solvers/two_dimensional/heat_type/implicit_coefficients/
 *                              lss_2d_general_heston_equation_coefficients.hpp:43-99
 *   - time loop + boundaries:  .../lss_2d_general_heston_equation_implicit_kernel.hpp:63-207
 *   - explicit boundary:       .../lss_2d_general_heston_equation_explicit_boundary.hpp:39-238
 *   - splitting schemes:       .../splitting_method/lss_heat_{douglas_rachford,craig_sneyd,
 *                              modified_craig_sneyd,hundsdorfer_verwer}_method.hpp
 *   - line solvers:            sparse_solvers/tridiagonal/thomas_lu_solver/,
 *                              sparse_solvers/tridiagonal/double_sweep_solver/
 * with the model lambdas of the reference's own tests
 * (unit_tests/common/lss_print_t.hpp:1913-1918 Heston, :2039-2049 SABR).
 *
 * Every floating-point operation is evaluated in the reference's order and
 * precision (the user lambdas in double, everything else in the solver type),
 * so that compiled with -ffp-contract=off it reproduces the compiled reference
 * bit for bit.  Pinned against the reference by tests/test_oracle_pin.py
 * (reference golden files outputs/Impl*Heston*.txt, outputs/ImplSABR*.txt, and
 * the reference itself compiled under oracle/_ref when available).
 */
#ifndef LSS_ORACLE_H
#define LSS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { LSSO_HESTON = 0, LSSO_SABR = 1 };
enum { LSSO_DR = 0, LSSO_CS = 1, LSSO_MCS = 2, LSSO_HV = 3, LSSO_EXPLICIT_EULER = 4 };
enum { LSSO_EULER = 0, LSSO_THETA30 = 1, LSSO_CN = 2, LSSO_THETA80 = 3 };
enum { LSSO_THOMAS_LU = 0, LSSO_DOUBLE_SWEEP = 1 };

typedef struct lsso_problem {
    int model;            /* LSSO_HESTON | LSSO_SABR */
    /* Heston: kappa, theta, sigma, rho, r.  SABR: beta, nu, rho, r (alpha is the v axis). */
    double kappa, theta_v, sigma, rho, rate, sabr_beta;
    double strike, maturity;
    double s_lo, s_hi, v_lo, v_hi;
    int nx, ny;           /* space points */
    int nt;               /* time points: steps = nt - 1 */
    int scheme;           /* LSSO_DR .. LSSO_HV, or LSSO_EXPLICIT_EULER (explicit_solvers) */
    double zeta;          /* splitting weighting value */
    int theta_scheme;     /* LSSO_EULER .. LSSO_THETA80 */
    int nonuniform;       /* grid_enum::Nonuniform */
    double acc_point, alpha_scale, beta_scale;
    double neumann_value; /* value of the S_max Neumann boundary (reference sign convention: -1) */
    int solver;           /* LSSO_THOMAS_LU | LSSO_DOUBLE_SWEEP */
    int forward;          /* 0 = backward time stepping (the reference's *_bwd_* configs) */
} lsso_problem;

/* Solve; payoff NULL = the test's terminal condition max(0, S-K).  out is Nx*Ny row-major.
 * Returns 0 on success, >0 on invalid argument. */
int lsso_solve_f64(const lsso_problem *p, const double *payoff, double *out);
int lsso_solve_f32(const lsso_problem *p, const float *payoff, float *out);

/* Physical grid values X(zeta_i), Y(eta_j) in the solver type. */
int lsso_grid_f64(const lsso_problem *p, double *x, double *y);
int lsso_grid_f32(const lsso_problem *p, float *x, float *y);

/* Reference index_of remaps: imap[i] = (size_t)(zeta_i / h1), jmap[j] likewise. */
int lsso_index_maps_f64(const lsso_problem *p, int *imap, int *jmap);
int lsso_index_maps_f32(const lsso_problem *p, int *imap, int *jmap);

/* Scheme coefficient tables at time t (row-major Nx*Ny each):
 * order M, P, Z, Mt, Pt, W, C, D, E, F  -> out has 10*Nx*Ny entries. */
int lsso_coefficients_f64(const lsso_problem *p, double t, double *out);

/* ---- 1-D implicit heat equation u_t = a u_xx + b u_x + c u + F (lss_oracle_1d_impl.h) ----
 * The reference's implicit_solvers::general_heat_equation
 * (pde_solvers/one_dimensional/heat_type/lss_1d_general_heat_equation.hpp:140-250) with its
 * host Thomas-LU / double-sweep policies; theta = 1 (Euler) or 0.5 (Crank-Nicolson), the two
 * schemes its implicit kernel accepts (lss_1d_general_heat_equation_implicit_kernel.hpp:930-945). */
enum { LSSO_H1_BLACK_SCHOLES = 0, LSSO_H1_CONSTANT = 1 };
enum { LSSO_BC_DIRICHLET = 0, LSSO_BC_NEUMANN = 1, LSSO_BC_ROBIN = 2 };

typedef struct lsso_heat1d_problem {
    int model;                  /* LSSO_H1_BLACK_SCHOLES | LSSO_H1_CONSTANT */
    /* Black-Scholes (unit_tests/pde_solvers/one_dimensional/lss_black_scholes_equation_t.hpp:854-880):
     * a = 0.5 sigma^2 x^2, b = rate x, c = -rate; terminal max(0, x - K) (put: max(0, K - x));
     * Dirichlet data call V(x_lo) = 0, V(x_hi) = x_hi - K e^{-rate (t_hi - t)}
     * (put: V(x_lo) = K e^{-rate (t_hi - t)}, V(x_hi) = 0). */
    double sigma, rate, strike;
    int put;
    /* constant coefficients (pure heat / advection tests): a = diff, b = conv, c = react;
     * initial condition init0 + init1 x; boundary kinds LSSO_BC_* with constant data
     * (Robin: linear_value * u + value); heat source F = src0 + src1 x when has_source. */
    double diff, conv, react;
    double init0, init1;
    int lo_kind, hi_kind;
    double lo_value, lo_linear, hi_value, hi_linear;
    int has_source;
    double src0, src1;
    double x_lo, x_hi, t_lo, t_hi;
    int n, nt;                  /* space points >= 4, time points >= 2 */
    int theta_scheme;           /* LSSO_EULER | LSSO_CN */
    int nonuniform;             /* grid_config_hints_1d: Nonuniform */
    double acc_point, alpha_scale;
    int solver;                 /* LSSO_THOMAS_LU | LSSO_DOUBLE_SWEEP */
    int forward;                /* 1 = forward from t_lo (host_fwd_* configs), 0 = backward from t_hi */
} lsso_heat1d_problem;

/* Solve; out = final n values; all (may be NULL) = nt rows of n by time index (the
 * reference's solve(container_2d&) with run_with_stepping). */
int lsso_heat1d_solve_f64(const lsso_heat1d_problem *p, double *out, double *all);
int lsso_heat1d_solve_f32(const lsso_heat1d_problem *p, float *out, float *all);
int lsso_heat1d_grid_f64(const lsso_heat1d_problem *p, double *x);
int lsso_heat1d_grid_f32(const lsso_heat1d_problem *p, float *x);
/* coef[3n] = A_, B_, D_; init[n]; bnd[4*(nt-1)] = per step lo value, lo linear, hi value,
 * hi linear (transformed, at the step's time); src[nt*n] or NULL (row s: F at step s's time;
 * row nt-1: F at the last step's next time). */
int lsso_heat1d_tables_f64(const lsso_heat1d_problem *p, double *coef, double *init, double *bnd, double *src);
int lsso_heat1d_tables_f32(const lsso_heat1d_problem *p, float *coef, float *init, float *bnd, float *src);

#ifdef __cplusplus
}
#endif
#endif
