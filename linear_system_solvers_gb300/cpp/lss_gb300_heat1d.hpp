// lss_gb300_heat1d.hpp -- C++17 front end of the GB300 1-D implicit heat path with the
// reference's names.
//
// Mirrors the user-facing pieces of MichalSara99/linear_system_solvers that the 1-D implicit
// path takes (same class names, constructor arguments and meaning):
//   lss_boundary::dirichlet/neumann/robin_boundary_1d   boundaries/lss_dirichlet_boundary.hpp,
//                                                       lss_neumann_boundary.hpp, lss_robin_boundary.hpp
//   lss_grids::grid_config_hints_1d                     discretization/lss_grid_config_hints.hpp:21-49
//   lss_pde_solvers::pde_discretization_config_1d,      pde_solvers/lss_pde_discretization_config.hpp:18-71
//   heat_{coefficient,initial,source}_data_config_1d,   pde_solvers/lss_heat_data_config.hpp
//   heat_data_config_1d
//   lss_pde_solvers::one_dimensional::implicit_solvers::general_heat_equation
//                                                       .../lss_1d_general_heat_equation.hpp:60-355
// plus the shared types of lss_gb300_heston.hpp (range, enumerations, container_2d,
// heat_implicit_solver_config).  solve() runs the device policies
// (tridiagonal_method_enum::GB300ThomasLUSolver / GB300DoubleSweepSolver on
// memory_space_enum::Device) through include/lss_heat1d.h: the user's functions are transformed
// to the computational grid and sampled exactly as the reference does (grid transform
// lss_grid_transform_config.hpp:32-87, lss_heat_data_transform.hpp:34-131,
// lss_boundary_transform.hpp:29-89, lss_1d_general_heat_equation_coefficients.hpp:34-64, the time
// sequence of heat_time_loop::run, implicit_kernel.hpp:83-163) and handed to
// lss_heat1d_batch_create as one tabulated instance.  Errors throw, as in the reference.
#pragma once

#include "lss_gb300_heston.hpp"
#include "lss_heat1d.h"

namespace lss_gb300 {

namespace lss_boundary {
template <typename T> class boundary_1d {
  public:
    virtual ~boundary_1d() = default;
    virtual T value(T t) const = 0;
};
template <typename T> class dirichlet_boundary_1d : public boundary_1d<T> {
    std::function<T(T)> v_;

  public:
    explicit dirichlet_boundary_1d(std::function<T(T)> const &v) : v_{v} {}
    T value(T t) const override { return v_(t); }
};
template <typename T> class neumann_boundary_1d : public boundary_1d<T> {
    std::function<T(T)> v_;

  public:
    explicit neumann_boundary_1d(std::function<T(T)> const &v) : v_{v} {}
    T value(T t) const override { return v_(t); }
};
template <typename T> class robin_boundary_1d : public boundary_1d<T> {
    std::function<T(T)> l_, v_;

  public:
    robin_boundary_1d(std::function<T(T)> const &linear_value, std::function<T(T)> const &value)
        : l_{linear_value}, v_{value}
    {
    }
    T linear_value(T t) const { return l_(t); }
    T value(T t) const override { return v_(t); }
};
template <typename T> using boundary_1d_ptr = std::shared_ptr<boundary_1d<T>>;
template <typename T> using boundary_1d_pair = std::pair<boundary_1d_ptr<T>, boundary_1d_ptr<T>>;
} // namespace lss_boundary

namespace lss_grids {
template <typename T> class grid_config_hints_1d {
    T point_, alpha_scale_;
    lss_enumerations::grid_enum grid_;

  public:
    explicit grid_config_hints_1d(T accumulation_point = T(0.0), T alpha_scale = T(3.0),
                                  lss_enumerations::grid_enum grid = lss_enumerations::grid_enum::Uniform)
        : point_{accumulation_point}, alpha_scale_{alpha_scale}, grid_{grid}
    {
    }
    T accumulation_point() const { return point_; }
    T alpha_scale() const { return alpha_scale_; }
    lss_enumerations::grid_enum grid() const { return grid_; }
};
template <typename T> using grid_config_hints_1d_ptr = std::shared_ptr<grid_config_hints_1d<T>>;
} // namespace lss_grids

namespace lss_pde_solvers {

template <typename T> class pde_discretization_config_1d {
    range<T> r_, rt_;
    std::size_t n_, nt_;

  public:
    pde_discretization_config_1d(range<T> const &space_range, std::size_t number_of_space_points,
                                 range<T> const &time_range, std::size_t number_of_time_points)
        : r_{space_range}, rt_{time_range}, n_{number_of_space_points}, nt_{number_of_time_points}
    {
    }
    range<T> const &space_range() const { return r_; }
    range<T> const &time_range() const { return rt_; }
    std::size_t number_of_space_points() const { return n_; }
    std::size_t number_of_time_points() const { return nt_; }
    T time_step() const { return (rt_.spread()) / static_cast<T>(nt_ - 1); }
};
template <typename T> using pde_discretization_config_1d_ptr = std::shared_ptr<pde_discretization_config_1d<T>>;

template <typename T> using fn2 = std::function<T(T, T)>;
template <typename T> class heat_coefficient_data_config_1d {
  public:
    fn2<T> a, b, c;
    heat_coefficient_data_config_1d(fn2<T> const &a_coefficient, fn2<T> const &b_coefficient,
                                    fn2<T> const &c_coefficient)
        : a{a_coefficient}, b{b_coefficient}, c{c_coefficient}
    {
    }
};
template <typename T> class heat_initial_data_config_1d {
  public:
    std::function<T(T)> initial_condition;
    explicit heat_initial_data_config_1d(std::function<T(T)> const &ic) : initial_condition{ic} {}
};
template <typename T> class heat_source_data_config_1d {
  public:
    fn2<T> heat_source;
    explicit heat_source_data_config_1d(fn2<T> const &src) : heat_source{src} {}
};
template <typename T> class heat_data_config_1d {
  public:
    std::shared_ptr<heat_coefficient_data_config_1d<T>> coefficients;
    std::shared_ptr<heat_initial_data_config_1d<T>> initial;
    std::shared_ptr<heat_source_data_config_1d<T>> source;
    heat_data_config_1d(std::shared_ptr<heat_coefficient_data_config_1d<T>> const &coefficient_data_config,
                        std::shared_ptr<heat_initial_data_config_1d<T>> const &initial_data_config,
                        std::shared_ptr<heat_source_data_config_1d<T>> const &source_data_config = nullptr)
        : coefficients{coefficient_data_config}, initial{initial_data_config}, source{source_data_config}
    {
    }
};
template <typename T> using heat_data_config_1d_ptr = std::shared_ptr<heat_data_config_1d<T>>;

namespace default_heat_solver_configs {
// the device counterparts of the reference's host_{fwd,bwd}_tlusolver_{euler,cn}_solver_config_ptr
// (pde_solvers/lss_heat_solver_config.hpp:155-240)
inline heat_implicit_solver_config_ptr make_dev_gb300(lss_enumerations::traverse_direction_enum d,
                                                      lss_enumerations::implicit_pde_schemes_enum s)
{
    return std::make_shared<heat_implicit_solver_config>(lss_enumerations::memory_space_enum::Device, d,
                                                         lss_enumerations::tridiagonal_method_enum::GB300ThomasLUSolver,
                                                         lss_enumerations::factorization_enum::None, s);
}
inline heat_implicit_solver_config_ptr const dev_fwd_gb300_euler_solver_config_ptr =
    make_dev_gb300(lss_enumerations::traverse_direction_enum::Forward, lss_enumerations::implicit_pde_schemes_enum::Euler);
inline heat_implicit_solver_config_ptr const dev_fwd_gb300_cn_solver_config_ptr = make_dev_gb300(
    lss_enumerations::traverse_direction_enum::Forward, lss_enumerations::implicit_pde_schemes_enum::CrankNicolson);
inline heat_implicit_solver_config_ptr const dev_bwd_gb300_euler_solver_config_ptr =
    make_dev_gb300(lss_enumerations::traverse_direction_enum::Backward, lss_enumerations::implicit_pde_schemes_enum::Euler);
} // namespace default_heat_solver_configs

namespace one_dimensional {
namespace implicit_solvers {

/*
 * general_heat_equation with the GB300 device policy.  arith: LSS_ADI_ARITH_REFERENCE
 * (bit-identical to the reference's host Thomas-LU / double-sweep policy) or LSS_ADI_ARITH_FAST.
 * The coefficients must not depend on t (checked at the first and last time of the loop).
 */
template <typename T> class general_heat_equation {
    heat_data_config_1d_ptr<T> data_;
    pde_discretization_config_1d_ptr<T> disc_;
    lss_boundary::boundary_1d_pair<T> bnd_;
    lss_grids::grid_config_hints_1d_ptr<T> hints_;
    heat_implicit_solver_config_ptr cfg_;
    int arith_;

    static void verify(bool ok, const char *msg)
    {
        if (!ok) throw std::invalid_argument(msg);
    }
    static int kind(lss_boundary::boundary_1d_ptr<T> const &b)
    {
        if (std::dynamic_pointer_cast<lss_boundary::dirichlet_boundary_1d<T>>(b)) return LSS_HEAT1D_DIRICHLET;
        if (std::dynamic_pointer_cast<lss_boundary::neumann_boundary_1d<T>>(b)) return LSS_HEAT1D_NEUMANN;
        return LSS_HEAT1D_ROBIN;
    }

    void run(bool all, std::vector<T> &out)
    {
        const std::size_t n = disc_->number_of_space_points(), nt = disc_->number_of_time_points();
        verify(n >= 4 && nt >= 2, "the discretisation needs at least 4 space and 2 time points");
        const T one = T(1.0), two = T(2.0), half = T(0.5);
        // grid_config_1d and grid_transform_config<One>
        const T step = one / (n - 1);
        const T low = disc_->space_range().lower(), high = disc_->space_range().upper();
        const T point = hints_->accumulation_point();
        T alpha = high - low;
        if (hints_->grid() == lss_enumerations::grid_enum::Nonuniform) alpha = (point - low) / hints_->alpha_scale();
        const T c0 = std::asinh((high - point) / alpha), c1 = std::asinh((low - point) / alpha);
        const T cdiff = c0 - c1;
        auto X = [&](T z) { return point + alpha * std::sinh(c0 * z + c1 * (one - z)); };
        auto Ad = [&](T z) { return alpha * cdiff * std::cosh(c0 * z + c1 * (one - z)); };
        auto Bd = [&](T z) { return alpha * cdiff * cdiff * std::sinh(c0 * z + c1 * (one - z)); };
        // general_heat_equation_coefficients
        const T k = disc_->time_step();
        const T h = one / (n - 1);
        const T lambda = k / (h * h), gamma = k / (two * h), delta = half * k;
        const auto &cf = *data_->coefficients;
        auto fill = [&](T t, std::vector<T> &coef) {
            coef.assign(3 * n, T(0));
            for (std::size_t i = 0; i < n; ++i) {
                const T zeta = step * i;
                const T x = X(zeta);
                const T av = Ad(zeta);
                const T ta = cf.a(t, x) / (Ad(zeta) * Ad(zeta));
                const T first = cf.b(t, x) / av;
                const T second = (cf.a(t, x) * Bd(zeta)) / (av * av * av);
                const T tb = first - second;
                const T tc = cf.c(t, x);
                coef[i] = lambda * ta - gamma * tb;
                coef[n + i] = lambda * ta - delta * tc;
                coef[2 * n + i] = lambda * ta + gamma * tb;
            }
        };
        const bool fwd = cfg_->traverse_direction() == lss_enumerations::traverse_direction_enum::Forward;
        const range<T> tr = disc_->time_range();
        std::vector<T> times(nt - 1);
        T time = fwd ? (tr.lower() + k) : (tr.upper() - k);
        for (std::size_t s = 0; s + 1 < nt; ++s) {
            times[s] = time;
            time = fwd ? time + k : time - k;
        }
        const T after = time;
        std::vector<T> coef, coef_last;
        fill(times.front(), coef);
        fill(times.back(), coef_last);
        if (coef != coef_last) throw std::invalid_argument("the device policy needs time-invariant coefficients");
        std::vector<T> init(n), bnd(4 * (nt - 1), T(0)), src;
        for (std::size_t i = 0; i < n; ++i) init[i] = data_->initial->initial_condition(X(step * i));
        // boundary_transform<One>: Neumann / Robin data times A(0) / A(1)
        const T a0 = Ad(T(0.0)), a1 = Ad(T(1.0));
        auto side = [&](lss_boundary::boundary_1d_ptr<T> const &b, T aval, T t, T *v, T *l) {
            if (kind(b) == LSS_HEAT1D_DIRICHLET) {
                *v = b->value(t);
            } else {
                *v = b->value(t) * aval;
                if (auto r = std::dynamic_pointer_cast<lss_boundary::robin_boundary_1d<T>>(b)) *l = r->linear_value(t) * aval;
            }
        };
        for (std::size_t s = 0; s + 1 < nt; ++s) {
            side(bnd_.first, a0, times[s], &bnd[4 * s], &bnd[4 * s + 1]);
            side(bnd_.second, a1, times[s], &bnd[4 * s + 2], &bnd[4 * s + 3]);
        }
        if (data_->source) {
            src.resize(nt * n);
            for (std::size_t s = 0; s < nt; ++s) {
                const T t = s + 1 < nt ? times[s] : after;
                for (std::size_t i = 0; i < n; ++i) src[s * n + i] = data_->source->heat_source(t, X(step * i));
            }
        }
        lss_heat1d_tables tb{};
        tb.n = static_cast<int>(n);
        tb.nt = static_cast<int>(nt);
        tb.t_lo = static_cast<double>(tr.lower());
        tb.t_hi = static_cast<double>(tr.upper());
        tb.theta_scheme = static_cast<int>(cfg_->implicit_pde_scheme());
        tb.forward = fwd ? 1 : 0;
        tb.lo_kind = kind(bnd_.first);
        tb.hi_kind = kind(bnd_.second);
        tb.coef = coef.data();
        tb.initial = init.data();
        tb.boundary = bnd.data();
        tb.source = src.empty() ? nullptr : src.data();
        int options = all ? LSS_HEAT1D_OPT_ALL_STEPS : 0;
        if (cfg_->tridiagonal_method() == lss_enumerations::tridiagonal_method_enum::GB300DoubleSweepSolver)
            options |= LSS_HEAT1D_OPT_DOUBLE_SWEEP;
        const int prec = std::is_same<T, double>::value ? LSS_ADI_FP64 : LSS_ADI_FP32;
        lss_heat1d_batch *b = nullptr;
        if (lss_heat1d_batch_create(&tb, 1, prec, arith_, options, &b) != LSS_ADI_OK)
            throw std::runtime_error(lss_adi_last_error());
        int rc = lss_heat1d_batch_run(b, nullptr);
        if (rc == LSS_ADI_OK) {
            out.resize(all ? nt * n : n);
            rc = lss_heat1d_batch_solution(b, 0, out.data());
        }
        lss_heat1d_batch_destroy(b);
        if (rc != LSS_ADI_OK) throw std::runtime_error(lss_adi_last_error());
    }

  public:
    general_heat_equation(heat_data_config_1d_ptr<T> const &heat_data_config,
                          pde_discretization_config_1d_ptr<T> const &discretization_config,
                          lss_boundary::boundary_1d_pair<T> const &boundary_pair,
                          lss_grids::grid_config_hints_1d_ptr<T> const &grid_config_hints,
                          heat_implicit_solver_config_ptr const &solver_config =
                              default_heat_solver_configs::dev_fwd_gb300_euler_solver_config_ptr,
                          std::map<std::string, T> const & = std::map<std::string, T>(),
                          int arith = LSS_ADI_ARITH_REFERENCE)
        : data_{heat_data_config}, disc_{discretization_config}, bnd_{boundary_pair}, hints_{grid_config_hints},
          cfg_{solver_config}, arith_{arith}
    {
        verify(data_ != nullptr && data_->coefficients && data_->initial, "heat_data_config must not be null");
        verify(disc_ != nullptr, "discretization_config must not be null");
        verify(bnd_.first != nullptr && bnd_.second != nullptr, "boundary_pair must not be null");
        verify(hints_ != nullptr, "grid_config_hints must not be null");
        verify(cfg_ != nullptr, "solver_config must not be null");
        if (cfg_->memory_space() != lss_enumerations::memory_space_enum::Device ||
            (cfg_->tridiagonal_method() != lss_enumerations::tridiagonal_method_enum::GB300ThomasLUSolver &&
             cfg_->tridiagonal_method() != lss_enumerations::tridiagonal_method_enum::GB300DoubleSweepSolver))
            throw std::invalid_argument("this front end runs the Device/GB300ThomasLUSolver and "
                                        "Device/GB300DoubleSweepSolver policies only; host policies stay in the "
                                        "reference library");
        if (cfg_->implicit_pde_scheme() != lss_enumerations::implicit_pde_schemes_enum::Euler &&
            cfg_->implicit_pde_scheme() != lss_enumerations::implicit_pde_schemes_enum::CrankNicolson)
            throw std::invalid_argument("Unreachable"); // the reference's 1-D kernel accepts Euler and CN only
    }

    // solve(container&): the final values (n)
    void solve(std::vector<T> &solution)
    {
        verify(solution.size() == disc_->number_of_space_points(),
               "The input solution container must have the correct size");
        std::vector<T> out;
        run(false, out);
        solution = out;
    }

    // solve(container_2d&): every time level, row = time index
    void solve(lss_containers::container_2d<lss_enumerations::by_enum::Row, T> &solutions)
    {
        const std::size_t n = disc_->number_of_space_points(), nt = disc_->number_of_time_points();
        verify(solutions.rows() == nt && solutions.columns() == n,
               "The input solution 2D container must have the correct size");
        std::vector<T> out;
        run(true, out);
        std::copy(out.begin(), out.end(), solutions.data());
    }
};

} // namespace implicit_solvers
} // namespace one_dimensional
} // namespace lss_pde_solvers
} // namespace lss_gb300
