// adi_tables.hpp -- host-side set-up of one 2-D Heston/SABR ADI instance.
//
// Builds, in the solver type T and in the reference's evaluation order, everything the
// device time loop needs and that does not change with time:
//   * sinh grid map            discretization/lss_grid_transform_config.hpp:118-149,178-187
//   * index_of remaps          discretization/lss_grid_config.hpp:56-59,110-118
//   * transformed coefficients pde_solvers/transformation/lss_heat_data_transform.hpp:174-214
//   * scheme coefficients      .../implicit_coefficients/lss_2d_general_heston_equation_coefficients.hpp:59-98
//   * boundary data            .../transformation/lss_heston_boundary_transform.hpp:47-65
//   * terminal condition       lss_2d_general_heston_equation.hpp:215
// with the Heston / SABR model lambdas of the reference tests
// (unit_tests/common/lss_print_t.hpp:1913-1918, :2039-2049), which compute in double and
// return the solver type.  This file is compiled with -ffp-contract=off so each a*b+c is
// rounded twice, like the reference build.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <string>
#include <type_traits>
#include <vector>

#include "lss_adi.h"

namespace lss_gb300 {

template <typename T> struct fpmath;
template <> struct fpmath<double> {
    static double asinh_(double v) { return std::asinh(v); }
    static double sinh_(double v) { return std::sinh(v); }
    static double cosh_(double v) { return std::cosh(v); }
};
template <> struct fpmath<float> {
    static float asinh_(float v) { return std::asinh(v); }
    static float sinh_(float v) { return std::sinh(v); }
    static float cosh_(float v) { return std::cosh(v); }
};

// grid_transform_config_2d: x(zeta) = p + alpha*sinh(c0*zeta + c1*(1-zeta)), y(eta) = v_lo + beta*sinh(d*eta)
template <typename T> struct sinh_map {
    T init1{}, init2{}, alpha{}, beta{}, c0{}, c1{}, d{}, cdiff{};

    void init(const lss_adi_problem &p)
    {
        const T low1 = static_cast<T>(p.s_lo), high1 = static_cast<T>(p.s_hi);
        const T low2 = static_cast<T>(p.v_lo), high2 = static_cast<T>(p.v_hi);
        const T point = static_cast<T>(p.acc_point);
        alpha = high1 - low1;
        beta = high2 - low2;
        if (p.nonuniform) {
            alpha = (point - low1) / static_cast<T>(p.alpha_scale);
            beta = (high2 - low2) / static_cast<T>(p.beta_scale);
        }
        init1 = point;
        init2 = low2;
        c0 = fpmath<T>::asinh_((high1 - point) / alpha);
        c1 = fpmath<T>::asinh_((low1 - point) / alpha);
        d = fpmath<T>::asinh_((high2 - low2) / beta);
        cdiff = c0 - c1;
    }
    T arg(T z) const { return c0 * z + c1 * (T(1) - z); }
    T x(T z) const { return init1 + alpha * fpmath<T>::sinh_(arg(z)); }
    T y(T e) const { return init2 + beta * fpmath<T>::sinh_(d * e); }
    T a_der(T z) const { return alpha * cdiff * fpmath<T>::cosh_(arg(z)); }
    T b_der(T e) const { return beta * d * fpmath<T>::cosh_(d * e); }
    T c_der(T z) const { return alpha * cdiff * cdiff * fpmath<T>::sinh_(arg(z)); }
    T d_der(T e) const { return beta * d * d * fpmath<T>::sinh_(d * e); }
};

// Scalars of one solve (coefficients.hpp:59-73 and implicit_kernel.hpp:978-995).
template <typename T> struct scheme_scalars {
    T k{}, h1{}, h2{}, alpha{}, beta{}, gamma{}, delta{}, ni{}, rho{}, zeta{}, theta{};
};

template <typename T>
inline scheme_scalars<T> make_scalars(int nx, int ny, int nt, T t_lo, T t_hi, double zeta, int theta_scheme)
{
    scheme_scalars<T> s;
    const T one = T(1.0), half = T(0.5), quarter = T(0.25);
    s.k = (t_hi - t_lo) / static_cast<T>(static_cast<std::size_t>(nt - 1));
    s.h1 = one / static_cast<T>(static_cast<std::size_t>(nx - 1));
    s.h2 = one / static_cast<T>(static_cast<std::size_t>(ny - 1));
    s.alpha = s.k / (s.h1 * s.h1);
    s.beta = s.k / (s.h2 * s.h2);
    s.gamma = quarter * s.k / (s.h1 * s.h2);
    s.delta = half * s.k / s.h1;
    s.ni = half * s.k / s.h2;
    s.rho = s.k;
    s.zeta = static_cast<T>(zeta);
    switch (theta_scheme) {
    case LSS_ADI_EULER: s.theta = one; break;
    case LSS_ADI_THETA_30: s.theta = T(0.3); break;
    case LSS_ADI_THETA_80: s.theta = T(0.8); break;
    default: s.theta = half; break;
    }
    return s;
}

// Host copy of everything the device time loop reads.
template <typename T> struct instance_tables {
    int nx = 0, ny = 0, steps = 0, scheme = 0, forward = 0;
    int double_sweep = 0;          // tridiagonal_method_enum::DoubleSweepSolver
    scheme_scalars<T> sc;
    T neu{};                       // Neumann data * A(1) (constant along S_hi on this path)
    std::vector<T> coef;           // 7*nx*ny: M, P, Z, Mt, Pt, W, C
    std::vector<T> coef_v0;        // 3*nx: D, E, F at eta = 0
    std::vector<T> s_lo;           // ny Dirichlet values at S_lo
    std::vector<T> s_hi_neu;       // ny transformed Neumann values at S_hi
    std::vector<T> v_hi;           // nx Dirichlet values at v_hi
    std::vector<int> imap, jmap;   // index_of remaps
    std::vector<T> payoff;         // nx*ny
    std::vector<T> x, y;           // physical grid
    T t_first{};                   // time of the first step
    // Caller-sampled time-dependent tables (LSS_ADI_OPT_STEP_TABLES): coef, coef_v0, s_lo,
    // s_hi_neu and v_hi hold one block per step, in step order.
    int step_tables = 0;
    // Time-dependent coefficients (SABR with r != 0: a and c carry D(t)^(2(1-beta)) and
    // D(t)^(1-beta), D(t) = exp(-r (T - t))).  Each step re-evaluates M, P, Z, C and the
    // D line from the time-independent factors below, in the reference's operation order.
    int tdep = 0;
    std::vector<double> a_static;  // nx*ny: (0.5 v) v S^(2 beta)            (double, as the lambda)
    std::vector<double> c_static;  // nx*ny: ((rho nu) v) v S^beta            (double)
    std::vector<T> ab;             // nx*ny: A(zeta_i) B(eta_j)
    std::vector<T> per_i;          // 5*nx: A, A*A, A*A*A, A'(zeta_i), user d(S_i)
    T two_alpha{}, half_rho_f{};   // 2*alpha, (0.5*rho)*f^
    std::vector<double> step_da, step_dc; // per step: D^(2(1-beta)), D^(1-beta)
};

// SABR with r != 0 is the one parametric problem whose coefficients depend on time.
inline bool time_dependent(const lss_adi_problem &p) { return p.model == LSS_ADI_SABR && p.rate != 0.0; }

int validate_problem(const lss_adi_problem &p, std::string &why);

template <typename T> inline void fill_index_maps(instance_tables<T> &it)
{
    it.imap.resize(it.nx);
    it.jmap.resize(it.ny);
    const T h1 = it.sc.h1, h2 = it.sc.h2;
    for (int i = 0; i < it.nx; ++i) it.imap[i] = static_cast<int>(static_cast<std::size_t>((h1 * static_cast<T>(i)) / h1));
    for (int j = 0; j < it.ny; ++j) it.jmap[j] = static_cast<int>(static_cast<std::size_t>((h2 * static_cast<T>(j)) / h2));
}

// Model lambdas of the reference tests, double arithmetic, solver-type result.
template <typename T> struct model_lambdas {
    const lss_adi_problem *p;
    T a(T t, T s, T v) const
    {
        if (p->model == LSS_ADI_SABR) {
            const double D = std::exp(-p->rate * (p->maturity - static_cast<double>(t)));
            return static_cast<T>(0.5 * static_cast<double>(v) * static_cast<double>(v) *
                                  std::pow(static_cast<double>(s), 2.0 * p->sabr_beta) *
                                  std::pow(D, 2.0 * (1.0 - p->sabr_beta)));
        }
        return static_cast<T>(0.5 * static_cast<double>(v) * static_cast<double>(s) * static_cast<double>(s));
    }
    T b(T, T, T v) const
    {
        if (p->model == LSS_ADI_SABR)
            return static_cast<T>(0.5 * p->sigma * p->sigma * static_cast<double>(v) * static_cast<double>(v));
        return static_cast<T>(0.5 * p->sigma * p->sigma * static_cast<double>(v));
    }
    T c(T t, T s, T v) const
    {
        if (p->model == LSS_ADI_SABR) {
            const double D = std::exp(-p->rate * (p->maturity - static_cast<double>(t)));
            return static_cast<T>(p->rho * p->sigma * static_cast<double>(v) * static_cast<double>(v) *
                                  std::pow(static_cast<double>(s), p->sabr_beta) * std::pow(D, (1.0 - p->sabr_beta)));
        }
        return static_cast<T>(p->rho * p->sigma * static_cast<double>(v) * static_cast<double>(s));
    }
    T d(T, T s, T) const { return static_cast<T>(p->rate * static_cast<double>(s)); }
    T e(T, T, T v) const
    {
        if (p->model == LSS_ADI_SABR) return static_cast<T>(0.0);
        return static_cast<T>(p->kappa * (p->theta_v - static_cast<double>(v)));
    }
    T f(T, T, T) const { return static_cast<T>(-p->rate); }
    T payoff(T s) const
    {
        const T val = static_cast<T>(static_cast<double>(s) - p->strike); // std::max<T>(0.0, s - K)
        return (T(0.0) < val) ? val : T(0.0);
    }
};

// Time-independent factors of the SABR coefficients and the per-step D(t) powers.  The
// lambdas evaluate ((((0.5 v) v) S^(2b)) D^(2(1-b))) and (((((rho nu) v) v) S^b) D^(1-b))
// left to right in double, so splitting off the last factor keeps every rounding.
template <typename T> inline void build_time_tables(const lss_adi_problem &p, const sinh_map<T> &g, instance_tables<T> &it)
{
    const auto &sc = it.sc;
    const int nx = p.nx, ny = p.ny;
    const std::size_t n = static_cast<std::size_t>(nx) * ny;
    it.tdep = 1;
    it.a_static.resize(n);
    it.c_static.resize(n);
    it.ab.resize(n);
    it.per_i.resize(5 * static_cast<std::size_t>(nx));
    for (int i = 0; i < nx; ++i) {
        const T zeta = sc.h1 * static_cast<T>(i);
        const T x = g.x(zeta), aval = g.a_der(zeta);
        it.per_i[0 * nx + i] = aval;
        it.per_i[1 * nx + i] = aval * aval;
        it.per_i[2 * nx + i] = aval * aval * aval;
        it.per_i[3 * nx + i] = g.c_der(zeta);
        it.per_i[4 * nx + i] = static_cast<T>(p.rate * static_cast<double>(x));
        for (int j = 0; j < ny; ++j) {
            const T eta = sc.h2 * static_cast<T>(j);
            const T y = g.y(eta), bval = g.b_der(eta);
            const double s = static_cast<double>(x), v = static_cast<double>(y);
            const std::size_t o = static_cast<std::size_t>(i) * ny + j;
            it.a_static[o] = 0.5 * v * v * std::pow(s, 2.0 * p.sabr_beta);
            it.c_static[o] = p.rho * p.sigma * v * v * std::pow(s, p.sabr_beta);
            it.ab[o] = aval * bval;
        }
    }
    const T two = T(2.0), half = T(0.5);
    it.two_alpha = two * sc.alpha;
    it.half_rho_f = half * sc.rho * static_cast<T>(-p.rate);
    it.step_da.resize(it.steps);
    it.step_dc.resize(it.steps);
    T t = it.t_first;
    for (int s = 0; s < it.steps; ++s) {
        const double D = std::exp(-p.rate * (p.maturity - static_cast<double>(t)));
        it.step_da[s] = std::pow(D, 2.0 * (1.0 - p.sabr_beta));
        it.step_dc[s] = std::pow(D, (1.0 - p.sabr_beta));
        t = p.forward ? (t + sc.k) : (t - sc.k);
    }
}

// Builds the tables of a parametric problem at time t (coefficients) -- Heston
// coefficients do not depend on t; SABR ones only through D(t) = exp(-r (T - t)).
template <typename T> inline void build_tables(const lss_adi_problem &p, instance_tables<T> &it)
{
    it.nx = p.nx;
    it.ny = p.ny;
    it.steps = p.nt - 1;
    it.scheme = p.scheme;
    it.forward = p.forward;
    it.double_sweep = (p.options & LSS_ADI_OPT_DOUBLE_SWEEP) ? 1 : 0;
    it.sc = make_scalars<T>(p.nx, p.ny, p.nt, T(0.0), static_cast<T>(p.maturity), p.zeta, p.theta_scheme);
    sinh_map<T> g;
    g.init(p);
    model_lambdas<T> m{&p};
    const T one = T(1.0), two = T(2.0), half = T(0.5);
    const auto &sc = it.sc;
    it.t_first = p.forward ? (T(0.0) + sc.k) : (static_cast<T>(p.maturity) - sc.k);
    const T t = it.t_first;
    const std::size_t n = static_cast<std::size_t>(p.nx) * p.ny;
    it.coef.assign(7 * n, T(0));
    it.coef_v0.assign(3 * static_cast<std::size_t>(p.nx), T(0));
    for (int i = 0; i < p.nx; ++i) {
        const T zeta = sc.h1 * static_cast<T>(i);
        for (int j = 0; j < p.ny; ++j) {
            const T eta = sc.h2 * static_cast<T>(j);
            const T x = g.x(zeta), y = g.y(eta);
            const T aval = g.a_der(zeta), bval = g.b_der(eta);
            const T A = m.a(t, x, y), B = m.b(t, x, y);
            const T ah = A / (aval * aval);
            const T bh = B / (bval * bval);
            const T ch = m.c(t, x, y) / (aval * bval);
            const T dh = m.d(t, x, y) / aval - (A * g.c_der(zeta)) / (aval * aval * aval);
            const T eh = m.e(t, x, y) / bval - (B * g.d_der(eta)) / (bval * bval * bval);
            const T fh = m.f(t, x, y);
            const std::size_t o = static_cast<std::size_t>(i) * p.ny + j;
            it.coef[0 * n + o] = sc.alpha * ah - sc.delta * dh;          // M
            it.coef[1 * n + o] = sc.alpha * ah + sc.delta * dh;          // P
            it.coef[2 * n + o] = two * sc.alpha * ah - half * sc.rho * fh; // Z
            it.coef[3 * n + o] = sc.beta * bh - sc.ni * eh;              // M~
            it.coef[4 * n + o] = sc.beta * bh + sc.ni * eh;              // P~
            it.coef[5 * n + o] = two * sc.beta * bh - half * sc.rho * fh;  // W
            it.coef[6 * n + o] = ch;                                     // C
            if (j == 0) {
                it.coef_v0[0 * p.nx + i] = dh;
                it.coef_v0[1 * p.nx + i] = eh;
                it.coef_v0[2 * p.nx + i] = fh;
            }
        }
    }
    // boundaries of the tests, transformed (lss_heston_boundary_transform.hpp:47-65)
    it.neu = static_cast<T>(p.neumann_value) * g.a_der(one);
    it.s_lo.assign(p.ny, static_cast<T>(0.0));
    it.s_hi_neu.assign(p.ny, it.neu);
    it.x.resize(p.nx);
    it.y.resize(p.ny);
    it.v_hi.resize(p.nx);
    for (int i = 0; i < p.nx; ++i) {
        it.x[i] = g.x(sc.h1 * static_cast<T>(i));
        it.v_hi[i] = it.x[i];
    }
    for (int j = 0; j < p.ny; ++j) it.y[j] = g.y(sc.h2 * static_cast<T>(j));
    it.payoff.resize(n);
    for (int i = 0; i < p.nx; ++i)
        for (int j = 0; j < p.ny; ++j) it.payoff[static_cast<std::size_t>(i) * p.ny + j] = m.payoff(it.x[i]);
    fill_index_maps(it);
    if (time_dependent(p)) build_time_tables(p, g, it);
}

// Tables from caller-sampled coefficients (lss_adi_tables).
template <typename T> inline void build_tables(const lss_adi_tables &t, instance_tables<T> &it)
{
    it.nx = t.nx;
    it.ny = t.ny;
    it.steps = t.nt - 1;
    it.scheme = t.scheme;
    it.forward = t.forward;
    it.double_sweep = (t.options & LSS_ADI_OPT_DOUBLE_SWEEP) ? 1 : 0;
    it.sc = make_scalars<T>(t.nx, t.ny, t.nt, static_cast<T>(t.t_lo), static_cast<T>(t.t_hi), t.zeta, t.theta_scheme);
    const std::size_t n = static_cast<std::size_t>(t.nx) * t.ny;
    it.step_tables = (t.options & LSS_ADI_OPT_STEP_TABLES) ? 1 : 0;
    const std::size_t blocks = it.step_tables ? static_cast<std::size_t>(it.steps) : 1;
    const T *c = static_cast<const T *>(t.coef);
    it.coef.assign(c, c + 7 * n * blocks);
    const T *v0 = static_cast<const T *>(t.coef_v0);
    it.coef_v0.assign(v0, v0 + 3 * static_cast<std::size_t>(t.nx) * blocks);
    const T *slo = static_cast<const T *>(t.s_lo_dirichlet);
    it.s_lo.assign(slo, slo + static_cast<std::size_t>(t.ny) * blocks);
    const T *shi = static_cast<const T *>(t.s_hi_neumann);
    it.s_hi_neu.assign(shi, shi + static_cast<std::size_t>(t.ny) * blocks);
    it.neu = it.s_hi_neu[0];
    const T *vhi = static_cast<const T *>(t.v_hi_dirichlet);
    it.v_hi.assign(vhi, vhi + static_cast<std::size_t>(t.nx) * blocks);
    const T *pay = static_cast<const T *>(t.payoff);
    it.payoff.assign(pay, pay + n);
    it.x.assign(t.nx, T(0));
    it.y.assign(t.ny, T(0));
    it.t_first = t.forward ? (static_cast<T>(t.t_lo) + it.sc.k) : (static_cast<T>(t.t_hi) - it.sc.k);
    fill_index_maps(it);
}

// Converts tables built in double to the solver type (LSS_ADI_OPT_FP64_TABLES).
template <typename T> inline void convert_tables(const instance_tables<double> &d, instance_tables<T> &t)
{
    auto cv = [](const std::vector<double> &v) { return std::vector<T>(v.begin(), v.end()); };
    t.nx = d.nx;
    t.ny = d.ny;
    t.steps = d.steps;
    t.scheme = d.scheme;
    t.forward = d.forward;
    t.double_sweep = d.double_sweep;
    t.sc.k = static_cast<T>(d.sc.k);
    t.sc.h1 = static_cast<T>(d.sc.h1);
    t.sc.h2 = static_cast<T>(d.sc.h2);
    t.sc.alpha = static_cast<T>(d.sc.alpha);
    t.sc.beta = static_cast<T>(d.sc.beta);
    t.sc.gamma = static_cast<T>(d.sc.gamma);
    t.sc.delta = static_cast<T>(d.sc.delta);
    t.sc.ni = static_cast<T>(d.sc.ni);
    t.sc.rho = static_cast<T>(d.sc.rho);
    t.sc.zeta = static_cast<T>(d.sc.zeta);
    t.sc.theta = static_cast<T>(d.sc.theta);
    t.neu = static_cast<T>(d.neu);
    t.coef = cv(d.coef);
    t.coef_v0 = cv(d.coef_v0);
    t.s_lo = cv(d.s_lo);
    t.s_hi_neu = cv(d.s_hi_neu);
    t.v_hi = cv(d.v_hi);
    t.imap = d.imap;
    t.jmap = d.jmap;
    t.payoff = cv(d.payoff);
    t.x = cv(d.x);
    t.y = cv(d.y);
    t.t_first = static_cast<T>(d.t_first);
    t.tdep = d.tdep;
    t.a_static = d.a_static;
    t.c_static = d.c_static;
    t.ab = cv(d.ab);
    t.per_i = cv(d.per_i);
    t.two_alpha = static_cast<T>(d.two_alpha);
    t.half_rho_f = static_cast<T>(d.half_rho_f);
    t.step_da = d.step_da;
    t.step_dc = d.step_dc;
}

// Parametric problem -> tables in T, honouring LSS_ADI_OPT_FP64_TABLES.
template <typename T> inline void build_tables_for(const lss_adi_problem &p, instance_tables<T> &it)
{
    if (!std::is_same<T, double>::value && (p.options & LSS_ADI_OPT_FP64_TABLES)) {
        instance_tables<double> d;
        build_tables<double>(p, d);
        convert_tables(d, it);
    } else {
        build_tables<T>(p, it);
    }
}

} // namespace lss_gb300
