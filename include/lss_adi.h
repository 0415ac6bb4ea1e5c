/*
 * lss_adi.h -- C-ABI of the GB300 (sm_103a) 2-D Heston/SABR ADI solver.
 *
 * This is the device drop-in for the implicit time-stepping path of
 * MichalSara99/linear_system_solvers:
 *
 *   implicit_solvers::general_heston_equation::solve
 *       (pde_solvers/two_dimensional/heat_type/lss_2d_general_heston_equation.hpp:183-307)
 *   -> general_heston_equation_implicit_kernel<Host, ThomasLUSolver>::operator()
 *       (.../lss_2d_general_heston_equation_implicit_kernel.hpp:958-1050)
 *   -> implicit_heston_time_loop::run  (.../implicit_kernel.hpp:150-207)
 *   -> heat_{douglas_rachford,craig_sneyd,modified_craig_sneyd,hundsdorfer_verwer}_method::solve
 *   -> thomas_lu_solver::solve per S-line and per v-line
 *       (sparse_solvers/tridiagonal/thomas_lu_solver/lss_thomas_lu_solver.hpp:52-83,125-191)
 *
 * The reference selects its solver policy by tridiagonal_method_enum x memory_space_enum
 * (common/lss_enumerations.hpp:46-52,84-88) at lss_2d_general_heston_equation.hpp:221-306.
 * The device path plugs in there as one more policy that owns the whole time loop,
 * because a per-line solve() call cannot be batched into coalesced sweeps.
 *
 * Conventions
 *   - Every function returns int: 0 = OK, > 0 = invalid argument, < 0 = device or
 *     runtime failure (see LSS_ADI_E*).  Nothing throws across this boundary.
 *     lss_adi_last_error() gives a message for the last failure of the calling thread.
 *   - Surfaces are Nx*Ny, row-major, V[i*Ny + j] with i the S index and j the v index
 *     (the reference's container_2d<by_enum::Row>).
 *   - Host buffers belong to the caller; device memory belongs to the handle.
 *   - A handle is used by one host thread at a time.  `stream` is a cudaStream_t
 *     (NULL = legacy default stream).
 *   - Precision: LSS_ADI_FP64 buffers are double, LSS_ADI_FP32 buffers are float.
 */
#ifndef LSS_ADI_H
#define LSS_ADI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LSS_ADI_ABI_VERSION 1

/* return codes */
#define LSS_ADI_OK 0
#define LSS_ADI_EINVAL 1        /* invalid argument */
#define LSS_ADI_EUNSUPPORTED 2  /* valid for the reference, not supported by this device path */
#define LSS_ADI_ECUDA (-1)      /* CUDA runtime error */
#define LSS_ADI_ENOMEM (-2)     /* device allocation failed */
#define LSS_ADI_ENONFINITE (-3) /* an instance produced NaN/Inf (status array says which) */

/* splitting_method_enum (common/lss_enumerations.hpp:35-41); EXPLICIT_EULER is the reference's
 * explicit_solvers::general_heston_equation with explicit_pde_schemes_enum::Euler
 * (pde_solvers/two_dimensional/heat_type/lss_2d_general_heston_equation.hpp:317-510,
 * explicit_schemes/lss_heston_euler_*_scheme.hpp): one explicit 9-point step per time step,
 * same boundaries; kernel-per-step path only, no adjoint, stability is the caller's (small k). */
enum lss_adi_scheme {
    LSS_ADI_DOUGLAS_RACHFORD = 0,
    LSS_ADI_CRAIG_SNEYD = 1,
    LSS_ADI_MODIFIED_CRAIG_SNEYD = 2,
    LSS_ADI_HUNDSDORFER_VERWER = 3,
    LSS_ADI_EXPLICIT_EULER = 4
};
/* implicit_pde_schemes_enum (common/lss_enumerations.hpp:102-108) */
enum lss_adi_theta { LSS_ADI_EULER = 0, LSS_ADI_THETA_30 = 1, LSS_ADI_CRANK_NICOLSON = 2, LSS_ADI_THETA_80 = 3 };
enum lss_adi_model { LSS_ADI_HESTON = 0, LSS_ADI_SABR = 1 };
enum lss_adi_precision { LSS_ADI_FP64 = 0, LSS_ADI_FP32 = 1 };
/* Arithmetic of the line solves:
 *   REFERENCE: the reference's operation order, no FMA contraction, IEEE divisions
 *              -> bit-identical to the reference's host Thomas-LU path;
 *   FAST:      time-invariant line factorisations precomputed once, FMA contraction
 *              (differs from the reference by rounding only, ~1e-14 relative). */
enum lss_adi_arith { LSS_ADI_ARITH_FAST = 0, LSS_ADI_ARITH_REFERENCE = 1 };
/* flags */
#define LSS_ADI_DEVICE_POINTERS 1 /* buffers passed to a call are device pointers */

/*
 * One pricing problem in the reference's terms.  Field meaning follows the reference
 * configs:
 *   space ranges / sizes / time points: pde_discretization_config_2d
 *       (pde_solvers/lss_pde_discretization_config.hpp:76-144; k = maturity/(nt-1));
 *   scheme + zeta: splitting_method_config (pde_solvers/lss_splitting_method_config.hpp:18-44);
 *   theta_scheme + forward: heat_implicit_solver_config (pde_solvers/lss_heat_solver_config.hpp:26-51);
 *   nonuniform / acc_point / alpha_scale / beta_scale: grid_config_hints_2d
 *       (discretization/lss_grid_config_hints.hpp:54-88);
 *   model coefficients: the Heston / SABR lambdas of the reference tests
 *       (unit_tests/common/lss_print_t.hpp:1913-1918, :2039-2049);
 *   boundaries: V(S_lo, v) = 0 (Dirichlet), dV/dS(S_hi, v) = neumann_value (Neumann, reference
 *       sign convention: -1 for a call), V(S, v_hi) = S (Dirichlet), degenerate PDE at v_lo;
 *   terminal condition max(0, S - strike) unless a payoff grid is supplied.
 */
typedef struct lss_adi_problem {
    int model;          /* lss_adi_model */
    double kappa, theta_v, sigma, rho, rate; /* Heston; SABR uses sigma = nu, rho, rate */
    double sabr_beta;   /* SABR only */
    double strike, maturity;
    double s_lo, s_hi, v_lo, v_hi;
    int nx, ny;         /* space points, each >= 4 */
    int nt;             /* time points, >= 2 (steps = nt - 1) */
    int scheme;         /* lss_adi_scheme */
    double zeta;        /* splitting weighting value (reference default 0.5) */
    int theta_scheme;   /* lss_adi_theta */
    int nonuniform;     /* 0 = grid_enum::Uniform (still sinh-mapped), 1 = Nonuniform */
    double acc_point, alpha_scale, beta_scale;
    double neumann_value;
    int forward;        /* 0 = backward stepping (reference *_bwd_* configs), 1 = forward */
    int precision;      /* lss_adi_precision */
    int arith;          /* lss_adi_arith */
    double eval_s, eval_v; /* point of the scalar output V(eval_s, eval_v): bilinear in (S, v) */
    int options;        /* LSS_ADI_OPT_* bits */
} lss_adi_problem;

/* options bits of lss_adi_problem
 * FP64_TABLES: for LSS_ADI_FP32, build grid, index_of remaps and coefficient tables in
 *   double and round them to float once.  The reference's own FP32 path computes the
 *   index_of remaps in float, which picks different neighbour lines than its FP64 path
 *   (e.g. 7 of 150 S indices differ), so its FP32 surfaces differ from its FP64 ones by
 *   up to ~10% at those boundary points; this option follows the FP64 problem instead. */
#define LSS_ADI_OPT_FP64_TABLES 1
/* DOUBLE_SWEEP: tridiagonal_method_enum::DoubleSweepSolver (common/lss_enumerations.hpp:46-52).
 *   The line solves run the double-sweep L/K recurrences of double_sweep_solver
 *   (sparse_solvers/tridiagonal/double_sweep_solver/lss_double_sweep_solver.hpp:114-155,
 *   lss_double_sweep_boundary.hpp:90-190) instead of Thomas LU; with LSS_ADI_ARITH_REFERENCE
 *   the surface is bit-identical to the reference's host double-sweep policy.  Both policies
 *   solve the same systems, so LSS_ADI_ARITH_FAST (one precomputed factorisation) serves
 *   both and ignores this bit. */
#define LSS_ADI_OPT_DOUBLE_SWEEP 2
/* LINE_PER_THREAD: LSS_ADI_ARITH_FAST single instance: solve every line with one thread (the
 *   batched kernel's arithmetic, bit for bit) instead of the autotuned partitioned line
 *   solves, which cut each line into chunks to occupy the whole GPU on one instance and
 *   differ from it by rounding only. */
#define LSS_ADI_OPT_LINE_PER_THREAD 4
/* WIDE_ADJOINT: lss_adi_adjoint runs the forward + adjoint of this instance as one kernel per
 *   stage over the whole GPU (partitioned line solves unless LINE_PER_THREAD) whatever its
 *   size, instead of one warp group of the batched kernel for instances of up to 256 x 160 points. */
#define LSS_ADI_OPT_WIDE_ADJOINT 8

/*
 * Tabulated drop-in: time-invariant scheme coefficients already sampled on the grid by
 * the caller (the reference's general_heston_equation_coefficients M_, P_, Z_, M_tilde_,
 * P_tilde_, W_, C_, D_, E_, F_ evaluated at (zeta_i, eta_j), implicit_coefficients/
 * lss_2d_general_heston_equation_coefficients.hpp:89-98).  Arrays are in the precision's
 * type.  Used by the C++ general_heston_equation front end for arbitrary user lambdas.
 */
typedef struct lss_adi_tables {
    int nx, ny, nt;
    double t_lo, t_hi;  /* time range; k = (t_hi - t_lo)/(nt - 1) in the solver type */
    int scheme, theta_scheme, forward, precision, arith;
    double zeta;
    const void *coef;     /* 7*nx*ny: M, P, Z, M~, P~, W, C */
    const void *coef_v0;  /* 3*nx: D, E, F at eta = 0 (degenerate v = v_lo line) */
    const void *s_lo_dirichlet; /* ny: V(S_lo, v_j) */
    const void *s_hi_neumann;   /* ny: transformed Neumann data dV/dzeta at S_hi (value * A(1)) */
    const void *v_hi_dirichlet; /* nx: V(S_i, v_hi) */
    const void *payoff;         /* nx*ny terminal/initial condition */
    int options;                /* LSS_ADI_OPT_DOUBLE_SWEEP, LSS_ADI_OPT_STEP_TABLES or 0 */
} lss_adi_tables;

/* STEP_TABLES (options of lss_adi_tables): time-dependent coefficients and boundaries.  coef,
 *   coef_v0, s_lo_dirichlet, s_hi_neumann and v_hi_dirichlet each hold nt - 1 consecutive blocks
 *   of the sizes above, block s sampled at the time of step s -- the running time of
 *   implicit_heston_time_loop::run (lss_2d_general_heston_equation_implicit_kernel.hpp:150-207):
 *   t_hi - k, t_hi - 2k, ... backward, t_lo + k, t_lo + 2k, ... forward, each obtained from the
 *   previous by one subtraction / addition of k in the solver type -- where the reference
 *   evaluates its coefficient functions M(t, zeta, eta), ..., F(t, zeta, eta) and boundary values
 *   (lss_2d_general_heston_equation_coefficients.hpp:31-40,89-98).  Runs the kernel-per-sweep
 *   path (line systems factorised every step, as the reference does) in either arithmetic; not
 *   for the explicit Euler scheme. */
#define LSS_ADI_OPT_STEP_TABLES 16

typedef struct lss_adi_handle lss_adi_handle;
typedef struct lss_adi_batch lss_adi_batch;

/* --- single instance ------------------------------------------------------------------ */

/* Builds the grid, index_of remaps and coefficient tables on the host in the reference's
 * arithmetic and uploads them.  Replaces general_heston_equation's constructor + the
 * solver setup of general_heston_equation_implicit_kernel<...>::operator()
 * (lss_2d_general_heston_equation.hpp:99-157; implicit_kernel.hpp:958-1030). */
int lss_adi_create(const lss_adi_problem *p, lss_adi_handle **h);
int lss_adi_create_tabulated(const lss_adi_tables *t, lss_adi_handle **h);

/* Runs the whole time loop (implicit_heston_time_loop::run, implicit_kernel.hpp:150-207).
 * payoff: NULL = the problem's terminal condition.  out_surface (may be NULL): final V.
 * out_value (may be NULL, host double): V(eval_s, eval_v).  Replaces
 * general_heston_equation::solve(container_2d&) (lss_2d_general_heston_equation.hpp:183-307). */
int lss_adi_forward(lss_adi_handle *h, const void *payoff, void *out_surface, double *out_value,
                    int flags, void *stream);

/* Same time loop with one kernel per sweep and CUDA-graph replay of the captured loop. */
int lss_adi_forward_graph(lss_adi_handle *h, const void *payoff, void *out_surface, double *out_value,
                          int flags, void *stream);

/* Adjoint of the whole forward solve (no counterpart in the reference, which has no
 * sensitivities): returns out_value = V(eval_s, eval_v), dV/d(kappa, theta, sigma, rho, r)
 * in dv_dparams[5] (host doubles; for SABR sigma is nu and kappa, theta give 0) and
 * dV/d(payoff grid) in dv_dpayoff (Nx*Ny, may be NULL).  FP64, all four splittings, Heston
 * and SABR (the r sensitivity includes the discount factors D(t) inside a and c).  Instances
 * larger than 256 x 160 points, and SABR with r != 0 (whose S-line tables are rebuilt at every
 * step's time), run the adjoint as one kernel per stage over the whole GPU.
 * Checkpoints every `checkpoint_every` steps; 0 = planned: instances of up to 256 x 160 points
 * take the longest interval the workspace allows (at least ceil(sqrt(steps))), larger ones
 * ceil(sqrt(steps)).  Results do not depend on the interval. */
int lss_adi_adjoint(lss_adi_handle *h, const void *payoff, double *out_value, double *dv_dparams,
                    void *dv_dpayoff, int checkpoint_every, int flags, void *stream);

/* Grid of the handle: x (nx) = S_i, y (ny) = v_j, in the precision's type (host). */
int lss_adi_grid(const lss_adi_handle *h, void *x, void *y);

/* Partitioned line solves of a LSS_ADI_ARITH_FAST single instance: every S line is cut into
 * s_chunks and every v line into v_chunks pieces solved concurrently (1 = thread per line;
 * at most 128; at least 4 rows per chunk).  0 for either picks it, with the number of lines
 * per CTA, by timing the sweeps (the autotuner lss_adi_create runs by default); a count set
 * here gets the lines per CTA that give every SM a CTA.  Neither changes the arithmetic of a
 * chunk: results depend on the chunk counts at rounding level only.  out_s / out_v (may be NULL) receive the
 * counts in use.  LSS_ADI_EUNSUPPORTED for handles on the kernel-per-sweep path.  No
 * counterpart in the reference, whose line solves are serial. */
int lss_adi_line_chunks(lss_adi_handle *h, int s_chunks, int v_chunks, int *out_s, int *out_v, void *stream);

void lss_adi_destroy(lss_adi_handle *h);

/* --- batched uneven instances ---------------------------------------------------------- */

/* Many independent problems with their own sizes, steps and parameters, advanced by one
 * persistent kernel per splitting scheme present (warp groups of 1-4 warps, about one thread
 * per S line, each on one instance at a time, longest first, pulled from device work
 * counters).  All problems share precision (FP64 or FP32); arith must be FAST. */
int lss_adi_batch_create(const lss_adi_problem *problems, int count, lss_adi_batch **b);

/* mode 0 = forward values only, 1 = forward + adjoint (values, the 5 parameter
 * sensitivities and dV/d(initial condition) per instance; FP64, every splitting, Heston and
 * SABR with r = 0; SABR with r != 0 has time-dependent coefficients and runs through
 * lss_adi_adjoint, one instance at a time).
 * The adjoint keeps a checkpoint every ceil(sqrt(steps)) steps or more (lss_adi_batch_checkpoints)
 * and recomputes each segment but the last once.  Device-resident: inputs were uploaded by
 * batch_create. */
int lss_adi_batch_run(lss_adi_batch *b, int mode, void *stream);

/* Captures lss_adi_batch_run(b, mode) once into a CUDA graph and launches the graph. */
int lss_adi_batch_graph_launch(lss_adi_batch *b, int mode, void *stream);

/* End-to-end step: uploads `payoffs` (concatenated Nx*Ny grids of all instances in order,
 * host, precision type; NULL = keep the terminal conditions) and `params` (count*5 host
 * doubles kappa,theta,sigma,rho,r; NULL = unchanged), runs, and downloads values[count]
 * and, for mode 1, grads[count*5] (host doubles).  Copies happen on `stream`. */
int lss_adi_batch_run_host(lss_adi_batch *b, int mode, const void *payoffs, double *values,
                           double *grads, void *stream);

/* Results of the last run (host doubles): values[count], grads[count*5] (NULL to skip),
 * status[count] (0 ok, 1 non-finite) (NULL to skip).  Synchronises the batch stream. */
int lss_adi_batch_results(lss_adi_batch *b, double *values, double *grads, int *status);

/* Final surface of instance `index` (host buffer of its Nx*Ny, precision type). */
int lss_adi_batch_surface(lss_adi_batch *b, int index, void *out_surface);

/* dV/d(initial condition grid) of instance `index` after a mode-1 run (host, FP64, Nx*Ny). */
int lss_adi_batch_payoff_gradient(lss_adi_batch *b, int index, void *out);

/* Lines-per-CTA autotuner: runs `mode` once per CTA size (32, 64, 128, 256 threads per
 * instance; each thread owns one S-line or v-line at a time) and keeps the fastest for later runs of
 * that mode.  With *threads_per_instance > 0 on entry it sets that size without timing; on
 * return it holds the size in use.  The runs overwrite the batch's results. */
int lss_adi_batch_autotune(lss_adi_batch *b, int mode, int *threads_per_instance, void *stream);

/* Kernel launches made by the last lss_adi_batch_run / graph launch (own kernels only). */
int lss_adi_batch_launch_count(const lss_adi_batch *b);

/* Checkpoint interval of every instance (creation order) that the last mode-1 run or autotune
 * planned: at least ceil(sqrt(steps)); longer where the adjoint workspace (one slice per
 * resident CTA, within the cap of lss_adi_batch_set_workspace) holds more stage
 * values, down to no recomputation at all when one segment covers the whole time loop. */
int lss_adi_batch_checkpoints(const lss_adi_batch *b, int *intervals);

/* Bounds the forward + adjoint workspace (checkpoints and the stored stage values of one
 * checkpoint segment, one slice per resident CTA): max_bytes = 0 restores the default, a
 * quarter of the device memory (never more than half of what is free when it is planned); a
 * max_bytes > 0 is honoured up to 90 % of the free memory.
 * checkpoint_every > 0 fixes every instance's checkpoint interval (capped at its step count);
 * 0 plans it from the cap.  A cap too small for one slice per resident CTA runs fewer CTAs; one
 * too small for a single slice makes the next mode-1 run return LSS_ADI_ENOMEM.  Takes effect
 * at the next mode-1 run or autotune.  Results do not depend on either setting.  No counterpart
 * in the reference, which has no adjoint. */
int lss_adi_batch_set_workspace(lss_adi_batch *b, double max_bytes, int checkpoint_every);

/* Bytes of device memory the batch's adjoint workspace holds now (0 before a mode-1 run). */
double lss_adi_batch_workspace_bytes(const lss_adi_batch *b);

void lss_adi_batch_destroy(lss_adi_batch *b);

/* --- line solver building block ------------------------------------------------------- */

/* Batched Thomas-LU solve of `lines` independent tridiagonal systems of size n >= 4 with
 * Dirichlet values at both ends, the reference's thomas_lu_solver with a Dirichlet
 * boundary_pair (lss_thomas_lu_solver.hpp:125-191, lss_thomas_lu_boundary.hpp:114-205).
 * lo/diag/up/rhs/x: n*lines, line-index fastest (element t of line l at t*lines + l);
 * bnd_lo/bnd_hi: lines.  Rows 1..n-2 are solved, x[0] = bnd_lo, x[n-1] = bnd_hi.
 * Always in the reference's operation order.  Device pointers.  Allocates n*lines
 * elements of stream-ordered device scratch (cudaMallocAsync) per call. */
int lss_tridiag_thomas_lu(int precision, int n, int lines, const void *lo, const void *diag,
                          const void *up, const void *rhs, const void *bnd_lo, const void *bnd_hi,
                          void *x, void *stream);

/* Same solve as lss_tridiag_thomas_lu for callers that must not allocate device memory
 * during the call (code inside a memory pool or allocator it does not control, real-time
 * paths, hosts that reserve all device memory up front).  No counterpart in the reference.
 * It allocates nothing: its scratch is a fixed 8 MiB array inside the library, held by every
 * GPU that loads the library until the process exits, so n*lines*element size must not exceed
 * 8 MiB (larger requests return LSS_ADI_EINVAL).  The first call on a device looks up the
 * array's device address and, under CUDA's lazy module loading (the default), that lookup
 * loads the array and the solver's code onto the device: the first call is the one time it
 * allocates.  Make a warm-up call with lines = 0 (it only does this set-up; other pointers may
 * be NULL) on every device before the code that must not allocate, and before any stream
 * capture -- or run with CUDA_MODULE_LOADING=EAGER.  A cudaDeviceReset between calls is not
 * supported (the looked-up address belongs to the reset context).  All calls on a device
 * share the array: calls whose kernels overlap on the GPU race. */
int lss_tridiag_thomas_lu_noalloc(int precision, int n, int lines, const void *lo, const void *diag,
                                  const void *up, const void *rhs, const void *bnd_lo, const void *bnd_hi,
                                  void *x, void *stream);

/* --- diagnostics ---------------------------------------------------------------------- */

/* Measured FP64 pipe rate of the current device (thread-level DFMA instructions per second):
 * eight independent DFMA chains per thread on four 256-thread CTAs per SM, best of three timed
 * launches after a warm-up.  The roofline denominator of the FP64-bound batched kernels.  No
 * counterpart in the reference. */
int lss_diag_fp64_rate(double *dfma_per_second, void *stream);

const char *lss_adi_last_error(void);
int lss_adi_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* LSS_ADI_H */
