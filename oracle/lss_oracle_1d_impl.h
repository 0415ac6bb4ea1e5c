/*
 * lss_oracle_1d_impl.h -- body of the 1-D implicit heat oracle, included once per solver type.
 * TEST INFRASTRUCTURE ONLY (see lss_oracle.h).
 *
 * Before inclusion define:  REAL (double|float), SFX(name) (name##_f64|_f32), ASINH, SINH, COSH.
 * It restates, in the reference's evaluation order:
 *   grid:                 discretization/lss_grid_config.hpp:21-52 (step 1/(n-1), zeta_i = step*i)
 *   sinh map:             discretization/lss_grid_transform_config.hpp:32-87
 *   coefficient transform: pde_solvers/transformation/lss_heat_data_transform.hpp:34-131
 *   boundary transform:   transformation/lss_boundary_transform.hpp:29-89
 *   scheme coefficients:  pde_solvers/one_dimensional/heat_type/implicit_coefficients/
 *                         lss_1d_general_heat_equation_coefficients.hpp:34-64
 *   right-hand sides:     .../solver_method/lss_heat_implicit_solver_method.hpp:34-181
 *   split + solve:        .../solver_method/lss_heat_implicit_solver_method.hpp:200-262
 *   time loops:           .../lss_1d_general_heat_equation_implicit_kernel.hpp:83-251
 *   Thomas LU:            sparse_solvers/tridiagonal/thomas_lu_solver/lss_thomas_lu_solver.hpp:125-191,
 *                         lss_thomas_lu_boundary.hpp:114-236
 *   double sweep:         sparse_solvers/tridiagonal/double_sweep_solver/lss_double_sweep_solver.hpp:112-155,
 *                         lss_double_sweep_boundary.hpp:88-190
 * with the model lambdas of the reference's 1-D tests (unit_tests/pde_solvers/one_dimensional/
 * lss_black_scholes_equation_t.hpp:854-880, lss_pure_heat_equation_t.hpp:1050-1070,2090-2105,
 * lss_advection_equation_t.hpp:1232-1250): user lambdas in double, returned as REAL.
 */

typedef struct SFX(h1) {
    const lsso_heat1d_problem *p;
    int n, steps;
    REAL step, k, theta, lambda, gamma, delta;
    REAL init, alpha, c0, c1, cdiff; /* sinh map */
    REAL *A, *B, *D;                 /* scheme coefficients A_, B_, D_ at zeta_i (time-invariant) */
} SFX(h1);

static REAL SFX(h1_arg)(const SFX(h1) *c, REAL z) { return c->c0 * z + c->c1 * ((REAL)1 - z); }
static REAL SFX(h1_x)(const SFX(h1) *c, REAL z) { return c->init + c->alpha * SINH(SFX(h1_arg)(c, z)); }
static REAL SFX(h1_ader)(const SFX(h1) *c, REAL z) { return c->alpha * c->cdiff * COSH(SFX(h1_arg)(c, z)); }
static REAL SFX(h1_bder)(const SFX(h1) *c, REAL z)
{
    return c->alpha * c->cdiff * c->cdiff * SINH(SFX(h1_arg)(c, z));
}

/* user lambdas a(t,x), b(t,x), c(t,x) */
static REAL SFX(h1_ua)(const lsso_heat1d_problem *p, REAL x)
{
    if (p->model == LSSO_H1_BLACK_SCHOLES) return (REAL)(0.5 * p->sigma * p->sigma * (double)x * (double)x);
    return (REAL)p->diff;
}
static REAL SFX(h1_ub)(const lsso_heat1d_problem *p, REAL x)
{
    if (p->model == LSSO_H1_BLACK_SCHOLES) return (REAL)(p->rate * (double)x);
    return (REAL)p->conv;
}
static REAL SFX(h1_uc)(const lsso_heat1d_problem *p, REAL x)
{
    (void)x;
    if (p->model == LSSO_H1_BLACK_SCHOLES) return (REAL)(-p->rate);
    return (REAL)p->react;
}
/* initial / terminal condition: Black-Scholes max<T>(0, x - K) (call) or max<T>(0, K - x) (put) */
static REAL SFX(h1_uinit)(const lsso_heat1d_problem *p, REAL x)
{
    if (p->model == LSSO_H1_BLACK_SCHOLES) {
        const REAL v = p->put ? (REAL)(p->strike - (double)x) : (REAL)((double)x - p->strike);
        return ((REAL)0.0 < v) ? v : (REAL)0.0;
    }
    return (REAL)(p->init0 + p->init1 * (double)x);
}
/* heat source F(t, x) = src0 + src1 x */
static REAL SFX(h1_usrc)(const lsso_heat1d_problem *p, REAL x) { return (REAL)(p->src0 + p->src1 * (double)x); }

/* untransformed boundary data at time t: Black-Scholes Dirichlet data
 * call: V(x_lo) = 0, V(x_hi) = x_hi - K e^{-r (T - t)}; put: V(x_lo) = K e^{-r (T - t)}, V(x_hi) = 0 */
static REAL SFX(h1_bvalue)(const lsso_heat1d_problem *p, int upper, REAL t)
{
    if (p->model == LSSO_H1_BLACK_SCHOLES) {
        const double disc = p->strike * exp(-p->rate * (p->t_hi - (double)t));
        if (p->put) return upper ? (REAL)0.0 : (REAL)disc;
        return upper ? (REAL)(p->x_hi - disc) : (REAL)0.0;
    }
    return upper ? (REAL)p->hi_value : (REAL)p->lo_value;
}
static REAL SFX(h1_blinear)(const lsso_heat1d_problem *p, int upper) { return upper ? (REAL)p->hi_linear : (REAL)p->lo_linear; }
static int SFX(h1_kind)(const lsso_heat1d_problem *p, int upper)
{
    if (p->model == LSSO_H1_BLACK_SCHOLES) return LSSO_BC_DIRICHLET;
    return upper ? p->hi_kind : p->lo_kind;
}

static int SFX(h1_init)(SFX(h1) *c, const lsso_heat1d_problem *p)
{
    memset(c, 0, sizeof(*c));
    c->p = p;
    c->n = p->n;
    c->steps = p->nt - 1;
    const REAL one = (REAL)1.0, two = (REAL)2.0, half = (REAL)0.5;
    /* grid_config_1d: step_ = one / (n - 1) */
    c->step = one / (REAL)(size_t)(p->n - 1);
    /* pde_discretization_config::time_step */
    c->k = ((REAL)p->t_hi - (REAL)p->t_lo) / (REAL)(size_t)(p->nt - 1);
    c->theta = (p->theta_scheme == LSSO_EULER) ? (REAL)1.0 : (REAL)0.5;
    /* general_heat_equation_coefficients::initialize (h = one / (space_size_ - 1)) */
    const REAL h = one / (REAL)(size_t)(p->n - 1);
    c->lambda = c->k / (h * h);
    c->gamma = c->k / (two * h);
    c->delta = half * c->k;
    /* grid_transform_config<One>::initialize */
    const REAL low = (REAL)p->x_lo, high = (REAL)p->x_hi, point = (REAL)p->acc_point;
    c->alpha = high - low;
    if (p->nonuniform) c->alpha = (point - low) / (REAL)p->alpha_scale;
    c->init = point;
    c->c0 = ASINH((high - point) / c->alpha);
    c->c1 = ASINH((low - point) / c->alpha);
    c->cdiff = c->c0 - c->c1;
    c->A = (REAL *)malloc(sizeof(REAL) * 3 * (size_t)p->n);
    if (!c->A) return -1;
    c->B = c->A + p->n;
    c->D = c->B + p->n;
    for (int i = 0; i < p->n; ++i) {
        const REAL zeta = c->step * (REAL)(size_t)i;
        const REAL x = SFX(h1_x)(c, zeta);
        /* heat_data_transform<One>: a_coeff_, b_coeff_, c_coeff_ */
        const REAL av = SFX(h1_ader)(c, zeta);
        const REAL ta = SFX(h1_ua)(p, x) / (SFX(h1_ader)(c, zeta) * SFX(h1_ader)(c, zeta));
        const REAL first = SFX(h1_ub)(p, x) / av;
        const REAL second = (SFX(h1_ua)(p, x) * SFX(h1_bder)(c, zeta)) / (av * av * av);
        const REAL tb = first - second;
        const REAL tc = SFX(h1_uc)(p, x);
        /* A_, B_, D_ lambdas */
        c->A[i] = c->lambda * ta - c->gamma * tb;
        c->B[i] = c->lambda * ta - c->delta * tc;
        c->D[i] = c->lambda * ta + c->gamma * tb;
    }
    return 0;
}
static void SFX(h1_free)(SFX(h1) *c) { free(c->A); }

/* transformed boundary value / linear value at time t (boundary_transform<One>) */
static REAL SFX(h1_tvalue)(const SFX(h1) *c, int upper, REAL t)
{
    const REAL v = SFX(h1_bvalue)(c->p, upper, t);
    if (SFX(h1_kind)(c->p, upper) == LSSO_BC_DIRICHLET) return v;
    return v * SFX(h1_ader)(c, upper ? (REAL)1.0 : (REAL)0.0);
}
static REAL SFX(h1_tlinear)(const SFX(h1) *c, int upper)
{
    if (SFX(h1_kind)(c->p, upper) != LSSO_BC_ROBIN) return (REAL)0.0;
    return SFX(h1_blinear)(c->p, upper) * SFX(h1_ader)(c, upper ? (REAL)1.0 : (REAL)0.0);
}

/* implicit_heat_scheme::rhs / rhs_source (lss_heat_implicit_solver_method.hpp:37-176) */
static void SFX(h1_rhs)(const SFX(h1) *c, const REAL *in, const REAL *src, const REAL *src_next, REAL t,
                        REAL *f)
{
    const REAL one = (REAL)1.0, two = (REAL)2.0;
    const REAL th = c->theta, h = c->step, k = c->k;
    const REAL *A = c->A, *B = c->B, *D = c->D;
    const int N = c->n - 1;
    const int lk = SFX(h1_kind)(c->p, 0), hk = SFX(h1_kind)(c->p, 1);
    if (lk == LSSO_BC_NEUMANN) {
        const REAL beta = two * h * SFX(h1_tvalue)(c, 0, t);
        f[0] = (one - th) * beta * A[0] + (one - two * (one - th) * B[0]) * in[0] + (one - th) * (A[0] + D[0]) * in[1];
        if (src) f[0] = f[0] + th * k * src_next[0] + (one - th) * k * src[0];
    } else if (lk == LSSO_BC_ROBIN) {
        const REAL beta = two * h * SFX(h1_tvalue)(c, 0, t);
        const REAL alpha = two * h * SFX(h1_tlinear)(c, 0);
        f[0] = (one - th) * beta * A[0] + (one - (one - th) * (two * B[0] - alpha * A[0])) * in[0] +
               (one - th) * (A[0] + D[0]) * in[1];
        if (src) f[0] = f[0] + th * k * src_next[0] + (one - th) * k * src[0];
    }
    if (hk == LSSO_BC_NEUMANN) {
        const REAL delta = two * h * SFX(h1_tvalue)(c, 1, t);
        f[N] = (one - th) * (A[N] + D[N]) * in[N - 1] + (one - two * (one - th) * B[N]) * in[N] -
               (one - th) * delta * D[N];
        if (src) f[N] = f[N] + th * k * src_next[N] + (one - th) * k * src[N];
    } else if (hk == LSSO_BC_ROBIN) {
        const REAL delta = two * h * SFX(h1_tvalue)(c, 1, t);
        const REAL gamma = two * h * SFX(h1_tlinear)(c, 1);
        f[N] = (one - th) * (A[N] + D[N]) * in[N - 1] + (one - (one - th) * (two * B[N] + gamma * D[N])) * in[N] -
               (one - th) * delta * D[N];
        if (src) f[N] = f[N] + th * k * src_next[N] + (one - th) * k * src[N];
    }
    for (int i = 1; i < N; ++i) {
        f[i] = (D[i] * (one - th) * in[i + 1]) + ((one - two * B[i] * (one - th)) * in[i]) + (A[i] * (one - th) * in[i - 1]);
        if (src) f[i] = f[i] + k * (th * src_next[i] + (one - th) * src[i]);
    }
}

/* thomas_lu_solver::kernel with thomas_lu_solver_boundary (Dirichlet / Neumann / Robin ends) */
static void SFX(h1_tlu)(const SFX(h1) *c, const REAL *a, const REAL *b, const REAL *cc, REAL *f, REAL t,
                        REAL *betav, REAL *gammav, REAL *sol, REAL *out)
{
    const REAL two = (REAL)2.0;
    const int n = c->n, N = n - 1;
    const REAL step = c->step; /* one / (n - 1), the solver's space_step */
    int start, end;
    REAL beta, gamma, z, an, bn, rn;
    const int lk = SFX(h1_kind)(c->p, 0), hk = SFX(h1_kind)(c->p, 1);
    const REAL lv = SFX(h1_tvalue)(c, 0, t), hv = SFX(h1_tvalue)(c, 1, t);
    if (lk == LSSO_BC_DIRICHLET) {
        start = 1;
        beta = b[1];
        gamma = cc[1] / beta;
        const REAL r = f[1] - a[1] * lv;
        z = r / beta;
    } else if (lk == LSSO_BC_NEUMANN) {
        const REAL cst = two * step * lv;
        start = 0;
        beta = b[0];
        gamma = (a[0] + cc[0]) / beta;
        const REAL r = f[0] - a[0] * cst;
        z = r / beta;
    } else {
        const REAL lin = two * step * SFX(h1_tlinear)(c, 0);
        const REAL cst = two * step * lv;
        start = 0;
        beta = b[0] + a[0] * lin;
        gamma = (a[0] + cc[0]) / beta;
        const REAL r = f[0] - a[0] * cst;
        z = r / beta;
    }
    if (hk == LSSO_BC_DIRICHLET) {
        end = n - 2;
        an = a[N - 1];
        bn = b[N - 1];
        rn = f[N - 1] - cc[N - 1] * hv;
    } else if (hk == LSSO_BC_NEUMANN) {
        const REAL cst = two * step * hv;
        end = n - 1;
        an = a[N] + cc[N];
        bn = b[N];
        rn = f[N] + cc[N] * cst;
    } else {
        const REAL lin = two * step * SFX(h1_tlinear)(c, 1);
        const REAL cst = two * step * hv;
        end = n - 1;
        an = a[N] + cc[N];
        bn = b[N] - cc[N] * lin;
        rn = f[N] + cc[N] * cst;
    }
    betav[start] = beta;
    gammav[start] = gamma;
    for (int i = start + 1; i < end; ++i) {
        betav[i] = b[i] - (a[i] * gammav[i - 1]);
        gammav[i] = cc[i] / betav[i];
    }
    betav[end] = bn - (an * gammav[end - 1]);
    sol[start] = z;
    for (int i = start + 1; i < end; ++i) sol[i] = (f[i] - (a[i] * sol[i - 1])) / betav[i];
    sol[end] = (rn - (an * sol[end - 1])) / betav[end];
    f[end] = sol[end];
    for (int i = end; i-- > start;) f[i] = sol[i] - (gammav[i] * f[i + 1]);
    memcpy(out, f, sizeof(REAL) * (size_t)n);
    if (start == 1) out[0] = lv;
    if (end == N - 1) out[N] = hv;
}

/* double_sweep_solver::kernel with double_sweep_boundary */
static void SFX(h1_ds)(const SFX(h1) *c, const REAL *a, const REAL *b, const REAL *cc, REAL *f, REAL t,
                       REAL *K, REAL *L, REAL *out)
{
    const REAL two = (REAL)2.0, one = (REAL)1.0, mone = (REAL)-1.0;
    const int n = c->n, N = n - 1;
    const REAL step = c->step;
    const int lk = SFX(h1_kind)(c->p, 0), hk = SFX(h1_kind)(c->p, 1);
    const REAL lv = SFX(h1_tvalue)(c, 0, t), hv = SFX(h1_tvalue)(c, 1, t);
    memset(K, 0, sizeof(REAL) * (size_t)n);
    memset(L, 0, sizeof(REAL) * (size_t)n);
    int start;
    if (lk == LSSO_BC_DIRICHLET) {
        start = 1;
        K[0] = lv;
        L[0] = (REAL)0.0;
    } else if (lk == LSSO_BC_NEUMANN) {
        start = 0;
        K[0] = (f[0] - a[0] * step * two * lv) / b[0];
        L[0] = mone * (a[0] + cc[0]) / b[0];
    } else {
        const REAL lin = SFX(h1_tlinear)(c, 0);
        start = 0;
        const REAL tmp = b[0] + a[0] * step * two * lin;
        K[0] = (f[0] - a[0] * step * two * lv) / tmp;
        L[0] = mone * (a[0] + cc[0]) / tmp;
    }
    const int end = (hk == LSSO_BC_DIRICHLET) ? n - 2 : n - 1;
    for (int i = 1; i <= end; ++i) {
        const REAL tmp = b[i] + (a[i] * L[i - 1]);
        L[i] = mone * cc[i] / tmp;
        K[i] = (f[i] - (a[i] * K[i - 1])) / tmp;
    }
    if (hk == LSSO_BC_DIRICHLET) {
        f[N] = hv;
    } else if (hk == LSSO_BC_NEUMANN) {
        const REAL cst = two * step * hv;
        f[N] = (L[N] * (K[N - 1] - cst) + K[N]) / (one - L[N] * L[N - 1]);
    } else {
        const REAL lin = two * step * SFX(h1_tlinear)(c, 1);
        const REAL cst = two * step * hv;
        f[N] = (L[N] * (K[N - 1] - cst) + K[N]) / (one - L[N] * (L[N - 1] - lin));
    }
    for (int i = N; i-- > start;) f[i] = (L[i] * f[i + 1]) + K[i];
    if (start == 1) f[0] = lv;
    memcpy(out, f, sizeof(REAL) * (size_t)n);
}

static int SFX(h1_validate)(const lsso_heat1d_problem *p)
{
    if (!p) return 1;
    if (p->n < 4 || p->nt < 2) return 1;
    if (p->theta_scheme != LSSO_EULER && p->theta_scheme != LSSO_CN) return 1;
    if (p->model != LSSO_H1_BLACK_SCHOLES && p->model != LSSO_H1_CONSTANT) return 1;
    if (p->model == LSSO_H1_CONSTANT &&
        (p->lo_kind < 0 || p->lo_kind > 2 || p->hi_kind < 0 || p->hi_kind > 2)) return 1;
    return 0;
}

/* heat_time_loop::run / run_with_stepping (implicit_kernel.hpp:83-251): `all` (may be NULL)
 * receives nt rows of n, row = time index. */
int SFX(lsso_heat1d_solve)(const lsso_heat1d_problem *p, REAL *out, REAL *all)
{
    int rc = SFX(h1_validate)(p);
    if (rc) return rc;
    SFX(h1) c;
    if (SFX(h1_init)(&c, p)) return -1;
    const int n = p->n, N = n - 1;
    const size_t nn = (size_t)n;
    REAL *buf = (REAL *)calloc(nn * 11, sizeof(REAL));
    if (!buf) { SFX(h1_free)(&c); return -1; }
    REAL *prev = buf, *next = buf + nn, *f = buf + 2 * nn, *a = buf + 3 * nn, *b = buf + 4 * nn, *cc = buf + 5 * nn;
    REAL *w1 = buf + 6 * nn, *w2 = buf + 7 * nn, *w3 = buf + 8 * nn, *src = buf + 9 * nn, *srcn = buf + 10 * nn;
    const REAL one = (REAL)1.0, two = (REAL)2.0;
    /* discretization<One>::of_function of the transformed initial condition */
    for (int i = 0; i < n; ++i) prev[i] = SFX(h1_uinit)(p, SFX(h1_x)(&c, c.step * (REAL)(size_t)i));
    /* split (heat_implicit_solver_method::split): time-invariant */
    for (int i = 0; i < n; ++i) {
        a[i] = (-c.theta * c.A[i]);
        b[i] = (one + two * c.theta * c.B[i]);
        cc[i] = (-c.theta * c.D[i]);
    }
    (void)N;
    const REAL k = c.k;
    const int steps = c.steps;
    const int fwd = p->forward;
    REAL time = fwd ? ((REAL)p->t_lo + k) : ((REAL)p->t_hi - k);
    REAL next_time = fwd ? (time + k) : (time - k);
    int idx = fwd ? 0 : steps;
    if (all) memcpy(all + (size_t)idx * nn, prev, sizeof(REAL) * nn);
    for (int s = 0; s < steps; ++s) {
        if (p->has_source) {
            for (int i = 0; i < n; ++i) {
                const REAL x = SFX(h1_x)(&c, c.step * (REAL)(size_t)i);
                src[i] = SFX(h1_usrc)(p, x);
                srcn[i] = SFX(h1_usrc)(p, x);
            }
            (void)next_time;
            SFX(h1_rhs)(&c, prev, src, srcn, time, f);
        } else {
            SFX(h1_rhs)(&c, prev, NULL, NULL, time, f);
        }
        if (p->solver == LSSO_DOUBLE_SWEEP)
            SFX(h1_ds)(&c, a, b, cc, f, time, w1, w2, next);
        else
            SFX(h1_tlu)(&c, a, b, cc, f, time, w1, w2, w3, next);
        memcpy(prev, next, sizeof(REAL) * nn);
        idx += fwd ? 1 : -1;
        if (all) memcpy(all + (size_t)idx * nn, prev, sizeof(REAL) * nn);
        if (fwd) { time += k; next_time += k; } else { time -= k; next_time -= k; }
    }
    memcpy(out, prev, sizeof(REAL) * nn);
    free(buf);
    SFX(h1_free)(&c);
    return 0;
}

/* Physical grid x(zeta_i). */
int SFX(lsso_heat1d_grid)(const lsso_heat1d_problem *p, REAL *x)
{
    int rc = SFX(h1_validate)(p);
    if (rc) return rc;
    SFX(h1) c;
    if (SFX(h1_init)(&c, p)) return -1;
    for (int i = 0; i < p->n; ++i) x[i] = SFX(h1_x)(&c, c.step * (REAL)(size_t)i);
    SFX(h1_free)(&c);
    return 0;
}

/* The tables a tabulated device problem takes (in the solver type):
 *   coef[3n]    A_, B_, D_ at zeta_i;   init[n] initial condition;
 *   bnd[4*(nt-1)] per step s: lo value, lo linear, hi value, hi linear (transformed) at the
 *                 step's time;
 *   src[nt*n] (may be NULL) row s < nt-1: F(time_s, x_i), row nt-1: F(next time of the last step). */
int SFX(lsso_heat1d_tables)(const lsso_heat1d_problem *p, REAL *coef, REAL *init, REAL *bnd, REAL *src)
{
    int rc = SFX(h1_validate)(p);
    if (rc) return rc;
    SFX(h1) c;
    if (SFX(h1_init)(&c, p)) return -1;
    const int n = p->n;
    memcpy(coef, c.A, sizeof(REAL) * 3 * (size_t)n);
    for (int i = 0; i < n; ++i) init[i] = SFX(h1_uinit)(p, SFX(h1_x)(&c, c.step * (REAL)(size_t)i));
    const REAL k = c.k;
    REAL time = p->forward ? ((REAL)p->t_lo + k) : ((REAL)p->t_hi - k);
    REAL last = time;
    for (int s = 0; s < c.steps; ++s) {
        bnd[4 * s + 0] = SFX(h1_tvalue)(&c, 0, time);
        bnd[4 * s + 1] = SFX(h1_tlinear)(&c, 0);
        bnd[4 * s + 2] = SFX(h1_tvalue)(&c, 1, time);
        bnd[4 * s + 3] = SFX(h1_tlinear)(&c, 1);
        if (src)
            for (int i = 0; i < n; ++i) src[(size_t)s * n + i] = SFX(h1_usrc)(p, SFX(h1_x)(&c, c.step * (REAL)(size_t)i));
        last = time;
        time = p->forward ? time + k : time - k;
    }
    (void)last;
    if (src)
        for (int i = 0; i < n; ++i) src[(size_t)c.steps * n + i] = SFX(h1_usrc)(p, SFX(h1_x)(&c, c.step * (REAL)(size_t)i));
    SFX(h1_free)(&c);
    return 0;
}
