/*
 * lss_heat1d.h -- C-ABI of the GB300 (sm_103a) batched 1-D implicit heat / Black-Scholes solver.
 *
 * Device drop-in for the 1-D implicit time stepping of MichalSara99/linear_system_solvers:
 *
 *   implicit_solvers::general_heat_equation::solve(container&) and solve(container_2d&)
 *       (pde_solvers/one_dimensional/heat_type/lss_1d_general_heat_equation.hpp:140-355)
 *   -> general_heat_equation_implicit_kernel<Host, ThomasLUSolver | DoubleSweepSolver>
 *       (.../lss_1d_general_heat_equation_implicit_kernel.hpp:768-1015)
 *   -> heat_time_loop::run / run_with_stepping (.../implicit_kernel.hpp:83-251)
 *   -> heat_implicit_solver_method::solve: rhs / rhs_source, split, tridiagonal solve
 *       (.../solver_method/lss_heat_implicit_solver_method.hpp:34-262)
 *   -> thomas_lu_solver / double_sweep_solver with Dirichlet, Neumann or Robin ends
 *       (sparse_solvers/tridiagonal/thomas_lu_solver/lss_thomas_lu_solver.hpp:125-191,
 *        lss_thomas_lu_boundary.hpp:114-236; double_sweep_solver/lss_double_sweep_solver.hpp:112-155,
 *        lss_double_sweep_boundary.hpp:88-190)
 *
 * It plugs in where the reference picks the 1-D implicit kernel by tridiagonal_method_enum x
 * memory_space_enum (lss_1d_general_heat_equation.hpp:164-245): one more policy that owns the
 * whole time loop of many instances at once, one GPU thread per instance, instances of equal
 * size interleaved in groups of 32 so that every load of a warp is one coalesced line.
 *
 * Conventions, return codes, precision and arithmetic enums and lss_adi_last_error() are those
 * of lss_adi.h.  Solutions are the reference's std::vector of n values (x_i ascending), or with
 * LSS_HEAT1D_OPT_ALL_STEPS its container_2d<Row> of nt rows (row = time index) by n.
 */
#ifndef LSS_HEAT1D_H
#define LSS_HEAT1D_H

#include "lss_adi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* boundary_1d kinds (boundaries/lss_dirichlet_boundary.hpp, lss_neumann_boundary.hpp,
 * lss_robin_boundary.hpp): Robin data is u' = linear * u + value on the transformed grid */
enum lss_heat1d_bc { LSS_HEAT1D_DIRICHLET = 0, LSS_HEAT1D_NEUMANN = 1, LSS_HEAT1D_ROBIN = 2 };

/* options bits */
#define LSS_HEAT1D_OPT_ALL_STEPS 1    /* keep every time level (solve(container_2d&)) */
#define LSS_HEAT1D_OPT_DOUBLE_SWEEP 2 /* tridiagonal_method_enum::DoubleSweepSolver; with
                                       * LSS_ADI_ARITH_REFERENCE bit-identical to the reference's
                                       * double-sweep policy, FAST ignores it (same systems) */

/*
 * Tabulated problem: what general_heat_equation hands its implicit kernel, sampled on the
 * computational grid zeta_i = i/(n-1) by the caller, in the precision's type:
 *   coef:     3*n  A_, B_, D_ of general_heat_equation_coefficients
 *             (implicit_coefficients/lss_1d_general_heat_equation_coefficients.hpp:53-64) at
 *             (t, zeta_i); time-invariant (the device path checks nothing: the caller does);
 *   initial:  n    the transformed initial / terminal condition at zeta_i;
 *   boundary: 4*(nt-1)  for time step s (the s-th call of the time loop, at its time t_s =
 *             t_lo + (s+1)k forward or t_hi - (s+1)k backward, accumulated as the loop does):
 *             lower value, lower linear value, upper value, upper linear value of the
 *             transformed boundary pair (transformation/lss_boundary_transform.hpp:29-89);
 *             values may change from step to step, the Robin linear values may not
 *             (LSS_ADI_EUNSUPPORTED: the device path keeps them per instance);
 *   source:   NULL or nt*n: row s < nt-1 the transformed heat source at (t_s, zeta_i), row nt-1
 *             at the next time of the last step (rhs_source uses rows s and s+1).
 */
typedef struct lss_heat1d_tables {
    int n;              /* space points, >= 4 */
    int nt;             /* time points, >= 2 (steps = nt - 1) */
    double t_lo, t_hi;  /* time range; k = (t_hi - t_lo)/(nt - 1) in the solver type */
    int theta_scheme;   /* LSS_ADI_EULER (theta 1) or LSS_ADI_CRANK_NICOLSON (theta 0.5) */
    int forward;        /* 1 = forward from t_lo, 0 = backward from t_hi */
    int lo_kind, hi_kind; /* lss_heat1d_bc */
    const void *coef;
    const void *initial;
    const void *boundary;
    const void *source;
} lss_heat1d_tables;

/*
 * Parametric Black-Scholes problem, the model of the reference's 1-D tests
 * (unit_tests/pde_solvers/one_dimensional/lss_black_scholes_equation_t.hpp:823-910):
 * U_t = 0.5 sigma^2 S^2 U_SS + r S U_S - r U on [s_lo, s_hi] x [0, maturity], backward from the
 * terminal condition max(0, S - K) (put: max(0, K - S)), Dirichlet data
 * call U(s_lo) = 0, U(s_hi) = s_hi - K e^{-r (maturity - t)}; put U(s_lo) = K e^{-r (maturity - t)},
 * U(s_hi) = 0; grid_config_hints_1d(acc_point, alpha_scale, nonuniform).
 * The tables are built on the host in the reference's arithmetic (double user lambdas).
 */
typedef struct lss_heat1d_bs {
    double sigma, rate, strike, maturity;
    int put;
    double s_lo, s_hi;
    int n, nt;
    int theta_scheme;   /* LSS_ADI_EULER | LSS_ADI_CRANK_NICOLSON */
    int nonuniform;
    double acc_point, alpha_scale;
    double eval_s;      /* point of the scalar output V(eval_s): linear in S between grid points */
} lss_heat1d_bs;

typedef struct lss_heat1d_batch lss_heat1d_batch;

/* Builds a batch of independent problems (any sizes, steps, boundary kinds) and uploads it.
 * arith: LSS_ADI_ARITH_REFERENCE (the reference's operation order, IEEE divisions, no
 * contraction: bit-identical to its host policy) or LSS_ADI_ARITH_FAST (one factorisation per
 * instance, reciprocal pivots, FMA: within rounding of the reference).  options: LSS_HEAT1D_OPT_*. */
int lss_heat1d_batch_create(const lss_heat1d_tables *problems, int count, int precision, int arith, int options,
                            lss_heat1d_batch **b);
int lss_heat1d_batch_create_bs(const lss_heat1d_bs *problems, int count, int precision, int arith, int options,
                               lss_heat1d_batch **b);

/* Runs every instance's whole time loop: one kernel launch (device-resident, asynchronous on
 * `stream`).  The initial conditions are those uploaded by create or the last run_host. */
int lss_heat1d_batch_run(lss_heat1d_batch *b, void *stream);

/* End-to-end step: uploads `initials` (concatenated n values per instance in creation order,
 * host, precision type; NULL = keep), runs, downloads values[count] (host doubles; V(eval_s)
 * for Black-Scholes batches, the solution's middle point i = n/2 for tabulated ones) and, if
 * `status` is not NULL, status[count] (0 ok, 1 non-finite).  Copies happen on `stream`. */
int lss_heat1d_batch_run_host(lss_heat1d_batch *b, const void *initials, double *values, int *status, void *stream);

/* Results of the last run: values / status as lss_heat1d_batch_run_host (either may be NULL).
 * Synchronises the batch's stream. */
int lss_heat1d_batch_results(lss_heat1d_batch *b, double *values, int *status);

/* Final solution of instance `index` (n values, precision type, host), or with
 * LSS_HEAT1D_OPT_ALL_STEPS every time level (nt*n, row = time index). */
int lss_heat1d_batch_solution(lss_heat1d_batch *b, int index, void *out);

/* Physical grid of instance `index` of a Black-Scholes batch (n values, precision type). */
int lss_heat1d_batch_grid(const lss_heat1d_batch *b, int index, void *x);

/* Kernel launches of one run (own kernels only), and grid-point-steps of one run. */
int lss_heat1d_batch_launch_count(const lss_heat1d_batch *b);
double lss_heat1d_batch_point_steps(const lss_heat1d_batch *b);

void lss_heat1d_batch_destroy(lss_heat1d_batch *b);

#ifdef __cplusplus
}
#endif
#endif /* LSS_HEAT1D_H */
