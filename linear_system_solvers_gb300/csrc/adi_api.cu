// adi_api.cu -- the extern "C" entry points declared in include/lss_adi.h.
#include <cmath>
#include <memory>
#include <new>
#include <string>

#include "adi_batched.hpp"
#include "adi_common.hpp"
#include "adi_plain.hpp"
#include "adi_tables.hpp"

namespace lss_gb300 {

static thread_local std::string g_last_error;

int set_error(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}
void clear_error()
{
    g_last_error.clear();
    (void)cudaGetLastError(); // drop a stale non-sticky error of an earlier, unrelated call
}

// Mirrors the checks of general_heston_equation::initialize (lss_2d_general_heston_equation.hpp:104-131)
// plus the size limits of the Dirichlet/Dirichlet Thomas LU path (n >= 4).
int validate_problem(const lss_adi_problem &p, std::string &why)
{
    if (p.model != LSS_ADI_HESTON && p.model != LSS_ADI_SABR) return why = "model must be LSS_ADI_HESTON or LSS_ADI_SABR", LSS_ADI_EINVAL;
    if (p.nx < 4 || p.ny < 4) return why = "nx and ny must be >= 4", LSS_ADI_EINVAL;
    if (p.nt < 2) return why = "nt (number of time points) must be >= 2", LSS_ADI_EINVAL;
    if (static_cast<long long>(p.nx) * p.ny > (1LL << 30)) return why = "grid larger than 2^30 points", LSS_ADI_EINVAL;
    if (p.scheme < LSS_ADI_DOUGLAS_RACHFORD || p.scheme > LSS_ADI_EXPLICIT_EULER) return why = "unknown splitting scheme", LSS_ADI_EINVAL;
    if (p.theta_scheme < LSS_ADI_EULER || p.theta_scheme > LSS_ADI_THETA_80) return why = "unknown theta scheme", LSS_ADI_EINVAL;
    if (p.precision != LSS_ADI_FP64 && p.precision != LSS_ADI_FP32) return why = "precision must be LSS_ADI_FP64 or LSS_ADI_FP32", LSS_ADI_EINVAL;
    if (p.arith != LSS_ADI_ARITH_FAST && p.arith != LSS_ADI_ARITH_REFERENCE) return why = "unknown arithmetic mode", LSS_ADI_EINVAL;
    if (!(p.s_hi > p.s_lo) || !(p.v_hi > p.v_lo)) return why = "space ranges must be increasing", LSS_ADI_EINVAL;
    if (!(p.maturity > 0.0) || !std::isfinite(p.maturity)) return why = "maturity must be positive", LSS_ADI_EINVAL;
    if (p.nonuniform && (!(p.alpha_scale > 0.0) || !(p.beta_scale > 0.0))) return why = "grid scales must be positive", LSS_ADI_EINVAL;
    if (p.nonuniform && !(p.acc_point > p.s_lo)) return why = "accumulation point must lie above s_lo for a nonuniform grid", LSS_ADI_EINVAL;
    const double vals[] = {p.kappa, p.theta_v, p.sigma, p.rho, p.rate, p.sabr_beta, p.strike, p.zeta, p.neumann_value, p.acc_point};
    for (double v : vals)
        if (!std::isfinite(v)) return why = "non-finite model parameter", LSS_ADI_EINVAL;
    if (p.options & ~(LSS_ADI_OPT_FP64_TABLES | LSS_ADI_OPT_DOUBLE_SWEEP | LSS_ADI_OPT_LINE_PER_THREAD |
                      LSS_ADI_OPT_WIDE_ADJOINT))
        return why = "unknown option bits", LSS_ADI_EINVAL;
    return LSS_ADI_OK;
}

} // namespace lss_gb300

using namespace lss_gb300;

struct lss_adi_handle {
    int precision = LSS_ADI_FP64;
    bool parametric = false;
    lss_adi_problem prob{};
    std::unique_ptr<plain_solver<double>> s64;
    std::unique_ptr<plain_solver<float>> s32;
    std::unique_ptr<wide_solver_base> wide;
    std::unique_ptr<adjoint_solver> adj;
};

template <typename T> static void tables_from(const lss_adi_problem &p, instance_tables<T> &tab) { build_tables_for<T>(p, tab); }
template <typename T> static void tables_from(const lss_adi_tables &t, instance_tables<T> &tab) { build_tables<T>(t, tab); }

template <typename T, typename Src>
static int make_plain(const Src &src, int arith, double es, double ev, std::unique_ptr<plain_solver<T>> &out)
{
    instance_tables<T> tab;
    tables_from<T>(src, tab);
    std::unique_ptr<plain_solver<T>> s(new (std::nothrow) plain_solver<T>());
    if (!s) return set_error(LSS_ADI_ENOMEM, "host allocation failed");
    int rc = s->init(std::move(tab), arith, es, ev);
    if (rc) return rc;
    out = std::move(s);
    return LSS_ADI_OK;
}

extern "C" {

int lss_adi_abi_version(void) { return LSS_ADI_ABI_VERSION; }

const char *lss_adi_last_error(void) { return g_last_error.c_str(); }

int lss_adi_create(const lss_adi_problem *p, lss_adi_handle **h)
{
    clear_error();
    if (!p || !h) return set_error(LSS_ADI_EINVAL, "lss_adi_create: null argument");
    *h = nullptr;
    std::string why;
    int rc = validate_problem(*p, why);
    if (rc) return set_error(rc, "lss_adi_create: " + why);
    std::unique_ptr<lss_adi_handle> hh(new (std::nothrow) lss_adi_handle());
    if (!hh) return set_error(LSS_ADI_ENOMEM, "host allocation failed");
    hh->precision = p->precision;
    hh->parametric = true;
    hh->prob = *p;
    try {
        // time-dependent coefficients (SABR, r != 0) rebuild their S-line factorisation before
        // every step: on the factorised wide path in FP64, on the kernel-per-sweep path (which
        // refactorises every sweep anyway) in FP32.  The explicit Euler scheme has no line
        // solves: kernel-per-step path.
        if (p->arith == LSS_ADI_ARITH_FAST && (!time_dependent(*p) || p->precision == LSS_ADI_FP64) &&
            p->scheme != LSS_ADI_EXPLICIT_EULER)
            rc = make_wide_solver(*p, hh->wide);
        else
            rc = p->precision == LSS_ADI_FP64 ? make_plain<double>(*p, p->arith, p->eval_s, p->eval_v, hh->s64)
                                              : make_plain<float>(*p, p->arith, p->eval_s, p->eval_v, hh->s32);
    } catch (const std::bad_alloc &) {
        return set_error(LSS_ADI_ENOMEM, "lss_adi_create: host allocation failed");
    }
    if (rc) return rc;
    *h = hh.release();
    return LSS_ADI_OK;
}

int lss_adi_create_tabulated(const lss_adi_tables *t, lss_adi_handle **h)
{
    clear_error();
    if (!t || !h) return set_error(LSS_ADI_EINVAL, "lss_adi_create_tabulated: null argument");
    *h = nullptr;
    if (t->nx < 4 || t->ny < 4 || t->nt < 2) return set_error(LSS_ADI_EINVAL, "lss_adi_create_tabulated: nx, ny >= 4 and nt >= 2 required");
    if (!t->coef || !t->coef_v0 || !t->s_lo_dirichlet || !t->s_hi_neumann || !t->v_hi_dirichlet || !t->payoff)
        return set_error(LSS_ADI_EINVAL, "lss_adi_create_tabulated: null table");
    if (t->scheme < 0 || t->scheme > LSS_ADI_EXPLICIT_EULER || t->theta_scheme < 0 || t->theta_scheme > 3)
        return set_error(LSS_ADI_EINVAL, "lss_adi_create_tabulated: unknown scheme");
    if (t->precision != LSS_ADI_FP64 && t->precision != LSS_ADI_FP32)
        return set_error(LSS_ADI_EINVAL, "lss_adi_create_tabulated: unknown precision");
    if (t->arith != LSS_ADI_ARITH_FAST && t->arith != LSS_ADI_ARITH_REFERENCE)
        return set_error(LSS_ADI_EINVAL, "lss_adi_create_tabulated: unknown arithmetic mode");
    if (!(t->t_hi > t->t_lo)) return set_error(LSS_ADI_EINVAL, "lss_adi_create_tabulated: empty time range");
    if (t->options & ~(LSS_ADI_OPT_DOUBLE_SWEEP | LSS_ADI_OPT_STEP_TABLES))
        return set_error(LSS_ADI_EINVAL, "lss_adi_create_tabulated: unknown option bits");
    if ((t->options & LSS_ADI_OPT_STEP_TABLES) && t->scheme == LSS_ADI_EXPLICIT_EULER)
        return set_error(LSS_ADI_EUNSUPPORTED, "lss_adi_create_tabulated: per-step tables are for the splitting schemes");
    std::unique_ptr<lss_adi_handle> hh(new (std::nothrow) lss_adi_handle());
    if (!hh) return set_error(LSS_ADI_ENOMEM, "host allocation failed");
    hh->precision = t->precision;
    int rc;
    try {
        rc = t->precision == LSS_ADI_FP64 ? make_plain<double>(*t, t->arith, 0.0, 0.0, hh->s64)
                                          : make_plain<float>(*t, t->arith, 0.0, 0.0, hh->s32);
    } catch (const std::bad_alloc &) {
        return set_error(LSS_ADI_ENOMEM, "lss_adi_create_tabulated: host allocation failed");
    }
    if (rc) return rc;
    *h = hh.release();
    return LSS_ADI_OK;
}

static int forward_impl(lss_adi_handle *h, const void *payoff, void *out_surface, double *out_value, int flags,
                        void *stream, bool graph)
{
    clear_error();
    if (!h) return set_error(LSS_ADI_EINVAL, "lss_adi_forward: null handle");
    if (h->wide) return h->wide->forward(payoff, out_surface, out_value, flags, stream, graph);
    if (h->s64) return h->s64->forward(payoff, out_surface, out_value, flags, stream, graph);
    if (h->s32) return h->s32->forward(payoff, out_surface, out_value, flags, stream, graph);
    return set_error(LSS_ADI_EINVAL, "lss_adi_forward: empty handle");
}

int lss_adi_forward(lss_adi_handle *h, const void *payoff, void *out_surface, double *out_value, int flags, void *stream)
{
    return forward_impl(h, payoff, out_surface, out_value, flags, stream, false);
}

int lss_adi_forward_graph(lss_adi_handle *h, const void *payoff, void *out_surface, double *out_value, int flags,
                          void *stream)
{
    return forward_impl(h, payoff, out_surface, out_value, flags, stream, true);
}

int lss_adi_adjoint(lss_adi_handle *h, const void *payoff, double *out_value, double *dv_dparams, void *dv_dpayoff,
                    int checkpoint_every, int flags, void *stream)
{
    clear_error();
    if (!h) return set_error(LSS_ADI_EINVAL, "lss_adi_adjoint: null handle");
    if (!h->parametric || h->precision != LSS_ADI_FP64)
        return set_error(LSS_ADI_EUNSUPPORTED, "lss_adi_adjoint: parametric FP64 problems only");
    if (checkpoint_every < 0) return set_error(LSS_ADI_EINVAL, "lss_adi_adjoint: checkpoint_every must be >= 0");
    if (!h->adj) {
        std::unique_ptr<adjoint_solver> a(new (std::nothrow) adjoint_solver());
        if (!a) return set_error(LSS_ADI_ENOMEM, "host allocation failed");
        int rc = a->init(h->prob);
        if (rc) return rc;
        if (h->wide) { // the forward's chunk counts, so both passes solve alike
            int ps = 1, pv = 1, ls = 0, lv = 0;
            h->wide->current_chunks(ps, pv, ls, lv);
            rc = a->set_chunks(ps, pv, ls, lv, stream);
            if (rc) return rc;
        }
        h->adj = std::move(a);
    }
    return h->adj->run(payoff, out_value, dv_dparams, dv_dpayoff, checkpoint_every, flags, stream);
}

int lss_adi_grid(const lss_adi_handle *h, void *x, void *y)
{
    clear_error();
    if (!h || !x || !y) return set_error(LSS_ADI_EINVAL, "lss_adi_grid: null argument");
    if (h->wide) return h->wide->grid(x, y);
    if (h->s64) {
        std::copy(h->s64->tab_.x.begin(), h->s64->tab_.x.end(), static_cast<double *>(x));
        std::copy(h->s64->tab_.y.begin(), h->s64->tab_.y.end(), static_cast<double *>(y));
    } else if (h->s32) {
        std::copy(h->s32->tab_.x.begin(), h->s32->tab_.x.end(), static_cast<float *>(x));
        std::copy(h->s32->tab_.y.begin(), h->s32->tab_.y.end(), static_cast<float *>(y));
    }
    return LSS_ADI_OK;
}

int lss_adi_line_chunks(lss_adi_handle *h, int s_chunks, int v_chunks, int *out_s, int *out_v, void *stream)
{
    clear_error();
    if (!h) return set_error(LSS_ADI_EINVAL, "lss_adi_line_chunks: null handle");
    if (!h->wide) return set_error(LSS_ADI_EUNSUPPORTED, "lss_adi_line_chunks: not a partitioned (fast single-instance) handle");
    int ps = 1, pv = 1, ls = 0, lv = 0;
    int rc = h->wide->chunks(s_chunks, v_chunks, &ps, &pv, stream);
    if (rc) return rc;
    if (h->adj) {
        h->wide->current_chunks(ps, pv, ls, lv);
        rc = h->adj->set_chunks(ps, pv, ls, lv, stream);
        if (rc) return rc;
    }
    if (out_s) *out_s = ps;
    if (out_v) *out_v = pv;
    return LSS_ADI_OK;
}

void lss_adi_destroy(lss_adi_handle *h) { delete h; }

} // extern "C"
