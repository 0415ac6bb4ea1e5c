/*
 * lss_oracle_impl.h -- body of the CPU oracle, included once per solver type.
 * TEST INFRASTRUCTURE ONLY (see lss_oracle.h).
 *
 * Before inclusion define:  REAL (double|float) and SFX(name) (name##_f64|_f32).
 * Each operation keeps the reference's evaluation order; comments give the
 * reference file:line each block restates.
 */

/* ---------------------------------------------------------------------------
 * Sinh grid transform: discretization/lss_grid_transform_config.hpp:118-149,178-187
 * ------------------------------------------------------------------------ */
typedef struct SFX(gt) {
    REAL init1, init2, alpha, beta, c0, c1, d, cdiff;
} SFX(gt);

static void SFX(gt_init)(const lsso_problem *p, SFX(gt) *g)
{
    const REAL low1 = (REAL)p->s_lo, high1 = (REAL)p->s_hi;
    const REAL low2 = (REAL)p->v_lo, high2 = (REAL)p->v_hi;
    const REAL point = (REAL)p->acc_point;
    g->alpha = high1 - low1;
    g->beta = high2 - low2;
    if (p->nonuniform) {
        g->alpha = (point - low1) / (REAL)p->alpha_scale;
        g->beta = (high2 - low2) / (REAL)p->beta_scale;
    }
    g->init1 = point;
    g->init2 = low2;
    g->c0 = ASINH((high1 - point) / g->alpha);
    g->c1 = ASINH((low1 - point) / g->alpha);
    g->d = ASINH((high2 - low2) / g->beta);
    g->cdiff = g->c0 - g->c1;
}

static REAL SFX(gt_arg)(const SFX(gt) *g, REAL z) { return g->c0 * z + g->c1 * ((REAL)1 - z); }
static REAL SFX(gt_x)(const SFX(gt) *g, REAL z) { return g->init1 + g->alpha * SINH(SFX(gt_arg)(g, z)); }
static REAL SFX(gt_y)(const SFX(gt) *g, REAL e) { return g->init2 + g->beta * SINH(g->d * e); }
/* first / second derivatives of the map (a_der_, b_der_, c_der_, d_der_) */
static REAL SFX(gt_a)(const SFX(gt) *g, REAL z) { return g->alpha * g->cdiff * COSH(SFX(gt_arg)(g, z)); }
static REAL SFX(gt_b)(const SFX(gt) *g, REAL e) { return g->beta * g->d * COSH(g->d * e); }
static REAL SFX(gt_c)(const SFX(gt) *g, REAL z) { return g->alpha * g->cdiff * g->cdiff * SINH(SFX(gt_arg)(g, z)); }
static REAL SFX(gt_dd)(const SFX(gt) *g, REAL e) { return g->beta * g->d * g->d * SINH(g->d * e); }

/* ---------------------------------------------------------------------------
 * Model lambdas of the reference tests (computed in double, returned as REAL):
 * Heston unit_tests/common/lss_print_t.hpp:1913-1918; SABR :2039-2049.
 * ------------------------------------------------------------------------ */
static REAL SFX(user_a)(const lsso_problem *p, REAL t, REAL s, REAL v)
{
    if (p->model == LSSO_SABR) {
        const double D = exp(-p->rate * (p->maturity - (double)t));
        return (REAL)(0.5 * (double)v * (double)v * pow((double)s, 2.0 * p->sabr_beta) *
                      pow(D, 2.0 * (1.0 - p->sabr_beta)));
    }
    return (REAL)(0.5 * (double)v * (double)s * (double)s);
}
static REAL SFX(user_b)(const lsso_problem *p, REAL t, REAL s, REAL v)
{
    (void)t; (void)s;
    if (p->model == LSSO_SABR)
        return (REAL)(0.5 * p->sigma * p->sigma * (double)v * (double)v);
    return (REAL)(0.5 * p->sigma * p->sigma * (double)v);
}
static REAL SFX(user_c)(const lsso_problem *p, REAL t, REAL s, REAL v)
{
    if (p->model == LSSO_SABR) {
        const double D = exp(-p->rate * (p->maturity - (double)t));
        return (REAL)(p->rho * p->sigma * (double)v * (double)v * pow((double)s, p->sabr_beta) *
                      pow(D, (1.0 - p->sabr_beta)));
    }
    return (REAL)(p->rho * p->sigma * (double)v * (double)s);
}
static REAL SFX(user_d)(const lsso_problem *p, REAL t, REAL s, REAL v)
{
    (void)t; (void)v;
    return (REAL)(p->rate * (double)s);
}
static REAL SFX(user_e)(const lsso_problem *p, REAL t, REAL s, REAL v)
{
    (void)t; (void)s;
    if (p->model == LSSO_SABR)
        return (REAL)0.0;
    return (REAL)(p->kappa * (p->theta_v - (double)v));
}
static REAL SFX(user_f)(const lsso_problem *p, REAL t, REAL s, REAL v)
{
    (void)t; (void)s; (void)v;
    return (REAL)(-p->rate);
}
/* terminal condition max<T>(0, s - K) and the three boundary lambdas of the tests */
static REAL SFX(user_payoff)(const lsso_problem *p, REAL s)
{
    const REAL val = (REAL)((double)s - p->strike);
    return ((REAL)0.0 < val) ? val : (REAL)0.0;
}

/* ---------------------------------------------------------------------------
 * Everything fixed for a solve: sizes, steps, scalars (coefficients.hpp:43-74).
 * ------------------------------------------------------------------------ */
typedef struct SFX(ctx) {
    const lsso_problem *p;
    SFX(gt) g;
    int nx, ny;
    REAL h1, h2, k;
    REAL alpha, beta, gamma, delta, ni, rho, zeta, theta;
    REAL neu_trans; /* Neumann value * A(1): lss_heston_boundary_transform.hpp:59-62 */
    int *imap, *jmap;
    /* coefficient tables at the current time, row-major nx*ny */
    REAL *M, *P, *Z, *Mt, *Pt, *W, *C, *D, *E, *F;
} SFX(ctx);

/* Transformed coefficients a^..f^ at (t, zeta, eta): lss_heat_data_transform.hpp:174-214 */
static void SFX(coef_point)(const SFX(ctx) *c, REAL t, REAL zeta, REAL eta, REAL *out)
{
    const lsso_problem *p = c->p;
    const SFX(gt) *g = &c->g;
    const REAL x = SFX(gt_x)(g, zeta), y = SFX(gt_y)(g, eta);
    const REAL aval = SFX(gt_a)(g, zeta), bval = SFX(gt_b)(g, eta);
    const REAL A = SFX(user_a)(p, t, x, y), B = SFX(user_b)(p, t, x, y);
    const REAL ah = A / (aval * aval);
    const REAL bh = B / (bval * bval);
    const REAL ch = SFX(user_c)(p, t, x, y) / (aval * bval);
    const REAL dh = SFX(user_d)(p, t, x, y) / aval - (A * SFX(gt_c)(g, zeta)) / (aval * aval * aval);
    const REAL eh = SFX(user_e)(p, t, x, y) / bval - (B * SFX(gt_dd)(g, eta)) / (bval * bval * bval);
    const REAL fh = SFX(user_f)(p, t, x, y);
    const REAL two = (REAL)2.0, half = (REAL)0.5;
    /* lss_2d_general_heston_equation_coefficients.hpp:89-98 */
    out[0] = c->alpha * ah - c->delta * dh;                 /* M  */
    out[1] = c->alpha * ah + c->delta * dh;                 /* P  */
    out[2] = two * c->alpha * ah - half * c->rho * fh;      /* Z  */
    out[3] = c->beta * bh - c->ni * eh;                     /* M~ */
    out[4] = c->beta * bh + c->ni * eh;                     /* P~ */
    out[5] = two * c->beta * bh - half * c->rho * fh;       /* W  */
    out[6] = ch;                                            /* C  */
    out[7] = dh;                                            /* D  */
    out[8] = eh;                                            /* E  */
    out[9] = fh;                                            /* F  */
}

static void SFX(fill_tables)(SFX(ctx) *c, REAL t)
{
    REAL v[10];
    for (int i = 0; i < c->nx; ++i) {
        const REAL zeta = c->h1 * (REAL)i; /* grid_config::value_for_1 */
        for (int j = 0; j < c->ny; ++j) {
            const REAL eta = c->h2 * (REAL)j;
            const size_t o = (size_t)i * c->ny + j;
            SFX(coef_point)(c, t, zeta, eta, v);
            c->M[o] = v[0]; c->P[o] = v[1]; c->Z[o] = v[2];
            c->Mt[o] = v[3]; c->Pt[o] = v[4]; c->W[o] = v[5];
            c->C[o] = v[6]; c->D[o] = v[7]; c->E[o] = v[8]; c->F[o] = v[9];
        }
    }
}

static int SFX(validate)(const lsso_problem *p)
{
    if (!p) return 1;
    if (p->nx < 4 || p->ny < 4) return 2;
    if (p->nt < 2) return 3;
    if (p->scheme < LSSO_DR || p->scheme > LSSO_EXPLICIT_EULER) return 4;
    if (p->theta_scheme < 0 || p->theta_scheme > 3) return 5;
    if (p->solver != LSSO_THOMAS_LU && p->solver != LSSO_DOUBLE_SWEEP) return 6;
    if (!(p->s_hi > p->s_lo) || !(p->v_hi > p->v_lo) || !(p->maturity > 0.0)) return 7;
    if (p->model != LSSO_HESTON && p->model != LSSO_SABR) return 8;
    return 0;
}

static int SFX(ctx_init)(SFX(ctx) *c, const lsso_problem *p)
{
    memset(c, 0, sizeof(*c));
    c->p = p;
    c->nx = p->nx;
    c->ny = p->ny;
    SFX(gt_init)(p, &c->g);
    const REAL one = (REAL)1.0, half = (REAL)0.5, quarter = (REAL)0.25;
    /* lss_pde_discretization_config.hpp:140-143: k = (T_hi - T_lo) / (Nt - 1) */
    const REAL spread = (REAL)p->maturity - (REAL)0.0;
    c->k = spread / (REAL)(size_t)(p->nt - 1);
    c->h1 = one / (REAL)(size_t)(p->nx - 1);
    c->h2 = one / (REAL)(size_t)(p->ny - 1);
    c->alpha = c->k / (c->h1 * c->h1);
    c->beta = c->k / (c->h2 * c->h2);
    c->gamma = quarter * c->k / (c->h1 * c->h2);
    c->delta = half * c->k / c->h1;
    c->ni = half * c->k / c->h2;
    c->rho = c->k;
    c->zeta = (REAL)p->zeta;
    /* theta by scheme: lss_2d_general_heston_equation_implicit_kernel.hpp:978-995 */
    switch (p->theta_scheme) {
    case LSSO_EULER: c->theta = one; break;
    case LSSO_THETA30: c->theta = (REAL)0.3; break;
    case LSSO_THETA80: c->theta = (REAL)0.8; break;
    default: c->theta = half; break;
    }
    c->neu_trans = (REAL)p->neumann_value * SFX(gt_a)(&c->g, one);
    const size_t n = (size_t)p->nx * p->ny;
    c->imap = (int *)malloc(sizeof(int) * p->nx);
    c->jmap = (int *)malloc(sizeof(int) * p->ny);
    REAL *blk = (REAL *)malloc(sizeof(REAL) * n * 10);
    if (!c->imap || !c->jmap || !blk) return -1;
    c->M = blk; c->P = blk + n; c->Z = blk + 2 * n; c->Mt = blk + 3 * n; c->Pt = blk + 4 * n;
    c->W = blk + 5 * n; c->C = blk + 6 * n; c->D = blk + 7 * n; c->E = blk + 8 * n; c->F = blk + 9 * n;
    /* grid_config::index_of: (size_t)(zeta / step), lss_grid_config.hpp:56-59 */
    for (int i = 0; i < p->nx; ++i) c->imap[i] = (int)(size_t)((c->h1 * (REAL)i) / c->h1);
    for (int j = 0; j < p->ny; ++j) c->jmap[j] = (int)(size_t)((c->h2 * (REAL)j) / c->h2);
    return 0;
}

static void SFX(ctx_free)(SFX(ctx) *c)
{
    free(c->imap);
    free(c->jmap);
    free(c->M);
}

/* ---------------------------------------------------------------------------
 * Line solvers with Dirichlet values at both ends (the only case on this path).
 * a, b, c: sub-, main-, super-diagonal; f: right-hand side (rows 1..n-2 used).
 * ------------------------------------------------------------------------ */
/* thomas_lu_solver::kernel + thomas_lu_solver_boundary (Dirichlet/Dirichlet):
 * lss_thomas_lu_solver.hpp:127-191, lss_thomas_lu_boundary.hpp:114-183 */
static void SFX(thomas_lu)(int n, const REAL *a, const REAL *b, const REAL *c, REAL *f,
                           REAL lo, REAL hi, REAL *beta, REAL *gam, REAL *x)
{
    const int N = n - 1, s = 1, e = n - 2;
    beta[s] = b[1];
    gam[s] = c[1] / beta[s];
    const REAL r0 = f[1] - a[1] * lo;
    const REAL z0 = r0 / beta[s];
    const REAL an = a[N - 1], bn = b[N - 1];
    const REAL rn = f[N - 1] - c[N - 1] * hi;
    for (int t = s + 1; t < e; ++t) {
        beta[t] = b[t] - (a[t] * gam[t - 1]);
        gam[t] = c[t] / beta[t];
    }
    beta[e] = bn - (an * gam[e - 1]);
    x[s] = z0;
    for (int t = s + 1; t < e; ++t)
        x[t] = (f[t] - (a[t] * x[t - 1])) / beta[t];
    x[e] = (rn - (an * x[e - 1])) / beta[e];
    f[e] = x[e];
    for (int t = e; t-- > s;)
        f[t] = x[t] - (gam[t] * f[t + 1]);
    for (int t = 1; t <= e; ++t) x[t] = f[t];
    x[0] = lo;
    x[N] = hi;
}

/* double_sweep_solver::kernel + double_sweep_boundary (Dirichlet/Dirichlet):
 * lss_double_sweep_solver.hpp:114-155, lss_double_sweep_boundary.hpp:90-190 */
static void SFX(double_sweep)(int n, const REAL *a, const REAL *b, const REAL *c, REAL *f,
                              REAL lo, REAL hi, REAL *K, REAL *L, REAL *x)
{
    const int N = n - 1, e = n - 2;
    const REAL mone = (REAL)-1.0;
    K[0] = lo;
    L[0] = (REAL)0.0;
    for (int t = 1; t <= e; ++t) {
        const REAL tmp = b[t] + (a[t] * L[t - 1]);
        L[t] = mone * c[t] / tmp;
        K[t] = (f[t] - (a[t] * K[t - 1])) / tmp;
    }
    f[N] = hi;
    for (int t = N; t-- > 1;)
        f[t] = (L[t] * f[t + 1]) + K[t];
    f[0] = lo;
    for (int t = 0; t <= N; ++t) x[t] = f[t];
}

typedef struct SFX(work) {
    REAL *lo, *dg, *up, *rhs, *w1, *w2, *sol; /* line buffers, length max(nx, ny) */
} SFX(work);

static void SFX(line_solve)(const SFX(ctx) *c, SFX(work) *w, int n, REAL lo, REAL hi)
{
    if (c->p->solver == LSSO_DOUBLE_SWEEP)
        SFX(double_sweep)(n, w->lo, w->dg, w->up, w->rhs, lo, hi, w->w1, w->w2, w->sol);
    else
        SFX(thomas_lu)(n, w->lo, w->dg, w->up, w->rhs, lo, hi, w->w1, w->w2, w->sol);
}

#define IX(i, j) ((size_t)(i) * ny + (j))

/* split_0: S-line matrix for line j (lss_heat_douglas_rachford_method.hpp:159-169) */
static void SFX(split0)(const SFX(ctx) *c, SFX(work) *w, int j)
{
    const int ny = c->ny;
    for (int t = 0; t < c->nx; ++t) {
        w->lo[t] = (-c->theta * c->M[IX(t, j)]);
        w->dg[t] = ((REAL)1.0 + c->theta * c->Z[IX(t, j)]);
        w->up[t] = (-c->theta * c->P[IX(t, j)]);
    }
}
/* split_1: v-line matrix for line i (lss_heat_douglas_rachford_method.hpp:171-181) */
static void SFX(split1)(const SFX(ctx) *c, SFX(work) *w, int i)
{
    const int ny = c->ny;
    for (int t = 0; t < ny; ++t) {
        w->lo[t] = (-c->theta * c->Mt[IX(i, t)]);
        w->dg[t] = ((REAL)1.0 + c->theta * c->W[IX(i, t)]);
        w->up[t] = (-c->theta * c->Pt[IX(i, t)]);
    }
}

/* rhs_intermed_1: explicit 9-point operator (lss_heat_douglas_rachford_method.hpp:37-68;
 * identical in CS/MCS/HV) */
static void SFX(rhs1)(const SFX(ctx) *c, SFX(work) *w, int j, const REAL *U)
{
    const int ny = c->ny, N = c->nx - 1;
    const REAL one = (REAL)1.0, g = c->gamma, th = c->theta;
    for (int t = 1; t < N; ++t) {
        const size_t o = IX(t, j);
        const REAL C = c->C[o], M = c->M[o], P = c->P[o], Z = c->Z[o];
        const REAL Mt = c->Mt[o], Pt = c->Pt[o], W = c->W[o];
        w->rhs[t] = (g * C * U[IX(t - 1, j - 1)]) + ((one - th) * M * U[IX(t - 1, j)]) -
                    (g * C * U[IX(t - 1, j + 1)]) + (Mt * U[IX(t, j - 1)]) +
                    ((one - W - (one - th) * Z) * U[IX(t, j)]) + (Pt * U[IX(t, j + 1)]) -
                    (g * C * U[IX(t + 1, j - 1)]) + ((one - th) * P * U[IX(t + 1, j)]) +
                    (g * C * U[IX(t + 1, j + 1)]);
    }
}

/* v-line right-hand side: DR rhs (:106-126), CS rhs_intermed_2/rhs_final, MCS rhs, HV rhs */
static void SFX(rhs_v)(const SFX(ctx) *c, SFX(work) *w, int i, const REAL *in, const REAL *inh)
{
    const int ny = c->ny, N = ny - 1;
    const REAL th = c->theta;
    for (int t = 1; t < N; ++t) {
        const size_t o = IX(i, t);
        w->rhs[t] = (-th * c->Mt[o] * in[IX(i, t - 1)]) + (th * c->W[o] * in[IX(i, t)]) -
                    (th * c->Pt[o] * in[IX(i, t + 1)]) + inh[IX(i, t)];
    }
}

/* CS/MCS rhs_intermed_3 (lss_heat_craig_sneyd_method.hpp:128-156,
 * lss_heat_modified_craig_sneyd_method.hpp:128-165).  U = input, Y1 = inhom_input,
 * Y2 = inhom_input_next. */
static void SFX(rhs3_cs)(const SFX(ctx) *c, SFX(work) *w, int j, const REAL *U, const REAL *Y1,
                         const REAL *Y2, int modified)
{
    const int ny = c->ny, N = c->nx - 1;
    const REAL th = c->theta, g = c->gamma, ze = c->zeta;
    for (int t = 1; t < N; ++t) {
        const size_t o = IX(t, j);
        const REAL M = c->M[o], Z = c->Z[o], P = c->P[o], C = c->C[o];
        REAL val = (-th * M * U[IX(t - 1, j)]) + (th * Z * U[IX(t, j)]) - (th * P * U[IX(t + 1, j)]) +
                   (Y1[o]) +
                   (ze * g * C *
                    ((Y2[IX(t + 1, j + 1)] - U[IX(t + 1, j + 1)]) - (Y2[IX(t + 1, j - 1)] - U[IX(t + 1, j - 1)]) -
                     (Y2[IX(t - 1, j + 1)] - U[IX(t - 1, j + 1)]) + (Y2[IX(t - 1, j - 1)] - U[IX(t - 1, j - 1)])));
        if (modified) {
            val = val + ((ze - th) * (M * (Y2[IX(t - 1, j)] - U[IX(t - 1, j)]) -
                                      (Z + c->W[o]) * (Y2[o] - U[o]) - P * (Y2[IX(t + 1, j)] - U[IX(t + 1, j)]) +
                                      c->Mt[o] * (Y2[IX(t, j - 1)] - U[IX(t, j - 1)]) +
                                      c->Pt[o] * (Y2[IX(t, j + 1)] - U[IX(t, j + 1)])));
        }
        w->rhs[t] = val;
    }
}

/* HV rhs_intermed_3, full-grid stage (lss_heat_hundsdorfer_verwer_method.hpp:128-172).
 * input = U, inhom_input = Y1, inhom_input_next = Y2; writes interior of Y3. */
static void SFX(hv_stage3)(const SFX(ctx) *c, const REAL *U, const REAL *Y1, const REAL *Y2, REAL *Y3)
{
    const int ny = c->ny, rows = c->nx - 1, cols = ny - 1;
    const REAL one = (REAL)1.0, th = c->theta, g = c->gamma, ze = c->zeta;
    for (int r = 1; r < rows; ++r) {
        for (int q = 1; q < cols; ++q) {
            const size_t o = IX(r, q);
            const REAL M = c->M[o], Z = c->Z[o], P = c->P[o], C = c->C[o], W = c->W[o];
            const REAL val =
                (-th * M * Y1[IX(r - 1, q)]) + ((one + th * Z) * Y1[o]) - (th * P * Y1[IX(r + 1, q)]) +
                (th * M * U[IX(r - 1, q)]) - (th * Z * U[o]) + (th * P * U[IX(r + 1, q)]) +
                (ze * g * C *
                 ((Y2[IX(r + 1, q + 1)] - U[IX(r + 1, q + 1)]) - (Y2[IX(r + 1, q - 1)] - U[IX(r + 1, q - 1)]) -
                  (Y2[IX(r - 1, q + 1)] - U[IX(r - 1, q + 1)]) + (Y2[IX(r - 1, q - 1)] - U[IX(r - 1, q - 1)]))) +
                (ze * (M * (Y2[IX(r - 1, q)] - U[IX(r - 1, q)]) - (W + Z) * (Y2[o] - U[o]) +
                       P * (Y2[IX(r + 1, q)] - U[IX(r + 1, q)]) + c->Mt[o] * (Y2[IX(r, q - 1)] - U[IX(r, q - 1)]) +
                       c->Pt[o] * (Y2[IX(r, q + 1)] - U[IX(r, q + 1)])));
            Y3[o] = val;
        }
    }
}

/* HV rhs_intermed_4 (lss_heat_hundsdorfer_verwer_method.hpp:174-194): input = Y2, inhom = Y3 */
static void SFX(rhs4_hv)(const SFX(ctx) *c, SFX(work) *w, int j, const REAL *Y2, const REAL *Y3)
{
    const int ny = c->ny, N = c->nx - 1;
    const REAL th = c->theta;
    for (int t = 1; t < N; ++t) {
        const size_t o = IX(t, j);
        w->rhs[t] = (-th * c->M[o] * Y2[IX(t - 1, j)]) + (th * c->Z[o] * Y2[o]) -
                    (th * c->P[o] * Y2[IX(t + 1, j)]) + Y3[o];
    }
}

/* S-line sweep: for j = 1..ny-2, solve line j and store the full column (incl. both
 * Dirichlet ends) in Y.  Boundary values prev(0, jmap[j]) and prev(nx-1, jmap[j])
 * (implicit_heston_solver_boundaries::get_intermed_horizontal, implicit_kernel.hpp:86-101). */
typedef void (*SFX(rhs_s_fn))(const SFX(ctx) *, SFX(work) *, int, const REAL *, const REAL *, const REAL *, int);

static void SFX(s_sweep)(const SFX(ctx) *c, SFX(work) *w, const REAL *prev, int stage, const REAL *A1,
                         const REAL *A2, const REAL *A3, REAL *Y)
{
    const int ny = c->ny, nx = c->nx;
    for (int j = 1; j < ny - 1; ++j) {
        SFX(split0)(c, w, j);
        if (stage == 1)
            SFX(rhs1)(c, w, j, A1);
        else if (stage == 3)
            SFX(rhs3_cs)(c, w, j, A1, A2, A3, c->p->scheme == LSSO_MCS);
        else
            SFX(rhs4_hv)(c, w, j, A1, A2);
        const int jj = c->jmap[j];
        SFX(line_solve)(c, w, nx, prev[IX(0, jj)], prev[IX(nx - 1, jj)]);
        for (int t = 0; t < nx; ++t) Y[IX(t, j)] = w->sol[t];
    }
}

/* v-line sweep: for i = 1..nx-2 into rows of Y.  Boundary values next(imap[i], 0) and
 * next(imap[i], ny-1) of the post-boundary-update copy (get_vertical, implicit_kernel.hpp:69-84). */
static void SFX(v_sweep)(const SFX(ctx) *c, SFX(work) *w, const REAL *bcol0, const REAL *bcolN,
                         const REAL *in, const REAL *inh, REAL *Y)
{
    const int ny = c->ny, nx = c->nx;
    for (int i = 1; i < nx - 1; ++i) {
        SFX(split1)(c, w, i);
        SFX(rhs_v)(c, w, i, in, inh);
        const int ii = c->imap[i];
        SFX(line_solve)(c, w, ny, bcol0[ii], bcolN[ii]);
        for (int t = 0; t < ny; ++t) Y[IX(i, t)] = w->sol[t];
    }
}

/* explicit_boundary::solve #1: v = 0 column (explicit_heston_boundary_scheme::rhs) and
 * the v_max column (explicit_boundary.hpp:39-84,181-200). */
static void SFX(boundary1)(const SFX(ctx) *c, const REAL *prev, REAL *bcol0, REAL *bcolN)
{
    const int ny = c->ny, N = c->nx - 1;
    const REAL four = (REAL)4.0, three = (REAL)3.0, two = (REAL)2.0, one = (REAL)1.0;
    const REAL delta = c->delta, ni = c->ni, rho = c->rho;
    bcol0[0] = (REAL)0.0; /* Dirichlet V(0, v) = 0 of the tests */
    {
        const REAL D = c->D[IX(N, 0)], E = c->E[IX(N, 0)], F = c->F[IX(N, 0)];
        const REAL dlt = two * c->h1 * c->neu_trans;
        bcol0[N] = ((one - three * ni * E + rho * F) * prev[IX(N, 0)]) + (four * ni * E * prev[IX(N, 1)]) -
                   (ni * E * prev[IX(N, 2)]) - (delta * dlt * D);
    }
    for (int t = 1; t < N; ++t) {
        const REAL D = c->D[IX(t, 0)], E = c->E[IX(t, 0)], F = c->F[IX(t, 0)];
        bcol0[t] = (-delta * D * prev[IX(t - 1, 0)]) + ((one - three * ni * E + rho * F) * prev[IX(t, 0)]) +
                   (delta * D * prev[IX(t + 1, 0)]) - (ni * E * prev[IX(t, 2)]) + (four * ni * E * prev[IX(t, 1)]);
    }
    /* V(S, v_max) = S: dirichlet_high of the tests on the transformed grid */
    for (int t = 0; t <= N; ++t) bcolN[t] = SFX(gt_x)(&c->g, c->h1 * (REAL)t);
}

/* Explicit Euler interior (explicit_heston_scheme::rhs, solver_method/lss_heston_euler_solver_method.hpp:24-52):
 * the heston_euler_coefficients C is gamma * C (explicit_coefficients/lss_heston_euler_coefficients.hpp:53) */
static void SFX(euler_interior)(const SFX(ctx) *c, const REAL *in, REAL *out)
{
    const int nx = c->nx, ny = c->ny;
    const REAL one = (REAL)1.0;
    for (int r = 1; r < nx - 1; ++r)
        for (int q = 1; q < ny - 1; ++q) {
            const size_t o = IX(r, q);
            const REAL C = c->gamma * c->C[o];
            out[o] = C * in[IX(r - 1, q - 1)] + c->M[o] * in[IX(r - 1, q)] - C * in[IX(r - 1, q + 1)] +
                     c->Mt[o] * in[IX(r, q - 1)] + (one - c->Z[o] - c->W[o]) * in[o] + c->Pt[o] * in[IX(r, q + 1)] -
                     C * in[IX(r + 1, q - 1)] + c->P[o] * in[IX(r + 1, q)] + C * in[IX(r + 1, q + 1)];
        }
}

/* explicit_boundary::solve #2: row S = 0 and the S_max extrapolation row (:202-238) */
static void SFX(boundary2)(const SFX(ctx) *c, REAL *next)
{
    const int ny = c->ny, lri = c->nx - 1;
    const REAL two = (REAL)2.0, three = (REAL)3.0, four = (REAL)4.0;
    for (int j = 0; j < ny; ++j) next[IX(0, j)] = (REAL)0.0;
    for (int j = 0; j < ny; ++j) {
        const int jj = c->jmap[j];
        next[IX(lri, j)] = (((four * next[IX(lri - 1, jj)]) - next[IX(lri - 2, jj)] - (two * c->h1 * c->neu_trans)) / three);
    }
}

static int SFX(solve_impl)(const lsso_problem *p, const REAL *payoff, REAL *out)
{
    int rc = SFX(validate)(p);
    if (rc) return rc;
    SFX(ctx) c;
    if (SFX(ctx_init)(&c, p)) return -1;
    const int nx = p->nx, ny = p->ny;
    const size_t n = (size_t)nx * ny;
    const int L = nx > ny ? nx : ny;
    REAL *buf = (REAL *)calloc(n * 6 + (size_t)L * 9, sizeof(REAL));
    if (!buf) { SFX(ctx_free)(&c); return -1; }
    REAL *prev = buf, *next = buf + n, *Y1 = buf + 2 * n, *Y2 = buf + 3 * n, *Y3 = buf + 4 * n, *Y4 = buf + 5 * n;
    REAL *lb = buf + 6 * n;
    SFX(work) w = {lb, lb + L, lb + 2 * L, lb + 3 * L, lb + 4 * L, lb + 5 * L, lb + 6 * L};
    REAL *bcol0 = lb + 7 * L, *bcolN = lb + 8 * L;

    /* terminal condition on the grid (lss_2d_general_heston_equation.hpp:215) */
    for (int i = 0; i < nx; ++i) {
        const REAL x = SFX(gt_x)(&c.g, c.h1 * (REAL)i);
        for (int j = 0; j < ny; ++j)
            prev[IX(i, j)] = payoff ? payoff[IX(i, j)] : SFX(user_payoff)(p, x);
    }
    const int tdep = (p->model == LSSO_SABR) && p->rate != 0.0;
    const REAL k = c.k;
    /* implicit_heston_time_loop::run (implicit_kernel.hpp:150-207) */
    REAL time = p->forward ? ((REAL)0.0 + k) : ((REAL)p->maturity - k);
    const int steps = p->nt - 1;
    SFX(fill_tables)(&c, time);
    for (int s = 0; s < steps; ++s) {
        if (tdep && s > 0) SFX(fill_tables)(&c, time);
        SFX(boundary1)(&c, prev, bcol0, bcolN);
        if (p->scheme == LSSO_EXPLICIT_EULER) {
            /* heston_euler_time_loop::run (explicit_schemes/lss_heston_euler_solver_scheme.hpp:44-89): interior,
             * then boundary #1 writes the v = v_lo and v = v_hi columns of next
             * (explicit_boundary.hpp:181-199), then boundary #2 its first and last rows */
            SFX(euler_interior)(&c, prev, next);
            for (int i = 0; i < nx; ++i) {
                next[IX(i, 0)] = bcol0[i];
                next[IX(i, ny - 1)] = bcolN[i];
            }
            SFX(boundary2)(&c, next);
            memcpy(prev, next, sizeof(REAL) * n);
            time = p->forward ? (time + k) : (time - k);
            continue;
        }
        memset(Y1, 0, sizeof(REAL) * n);
        memset(Y2, 0, sizeof(REAL) * n);
        memset(Y3, 0, sizeof(REAL) * n);
        memset(Y4, 0, sizeof(REAL) * n);
        SFX(s_sweep)(&c, &w, prev, 1, prev, NULL, NULL, Y1);
        switch (p->scheme) {
        case LSSO_DR:
            SFX(v_sweep)(&c, &w, bcol0, bcolN, prev, Y1, next);
            break;
        case LSSO_CS:
        case LSSO_MCS:
            SFX(v_sweep)(&c, &w, bcol0, bcolN, prev, Y1, Y2);
            SFX(s_sweep)(&c, &w, prev, 3, prev, Y1, Y2, Y3);
            SFX(v_sweep)(&c, &w, bcol0, bcolN, prev, Y3, next);
            break;
        default: /* HV */
            SFX(v_sweep)(&c, &w, bcol0, bcolN, prev, Y1, Y2);
            SFX(hv_stage3)(&c, prev, Y1, Y2, Y3);
            SFX(s_sweep)(&c, &w, prev, 4, Y2, Y3, NULL, Y4);
            SFX(v_sweep)(&c, &w, bcol0, bcolN, Y2, Y4, next);
            break;
        }
        SFX(boundary2)(&c, next);
        memcpy(prev, next, sizeof(REAL) * n);
        time = p->forward ? (time + k) : (time - k);
    }
    memcpy(out, prev, sizeof(REAL) * n);
    free(buf);
    SFX(ctx_free)(&c);
    return 0;
}

int SFX(lsso_solve)(const lsso_problem *p, const REAL *payoff, REAL *out)
{
    return SFX(solve_impl)(p, payoff, out);
}

int SFX(lsso_grid)(const lsso_problem *p, REAL *x, REAL *y)
{
    int rc = SFX(validate)(p);
    if (rc) return rc;
    SFX(gt) g;
    SFX(gt_init)(p, &g);
    const REAL h1 = (REAL)1.0 / (REAL)(size_t)(p->nx - 1), h2 = (REAL)1.0 / (REAL)(size_t)(p->ny - 1);
    for (int i = 0; i < p->nx; ++i) x[i] = SFX(gt_x)(&g, h1 * (REAL)i);
    for (int j = 0; j < p->ny; ++j) y[j] = SFX(gt_y)(&g, h2 * (REAL)j);
    return 0;
}

int SFX(lsso_index_maps)(const lsso_problem *p, int *imap, int *jmap)
{
    int rc = SFX(validate)(p);
    if (rc) return rc;
    SFX(ctx) c;
    if (SFX(ctx_init)(&c, p)) return -1;
    memcpy(imap, c.imap, sizeof(int) * p->nx);
    memcpy(jmap, c.jmap, sizeof(int) * p->ny);
    SFX(ctx_free)(&c);
    return 0;
}

#undef IX
