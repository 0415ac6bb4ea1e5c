/*
 * lss_oracle.h -- CPU oracle for the 2-D Heston/SABR ADI hot path.
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

#ifdef __cplusplus
}
#endif
#endif
