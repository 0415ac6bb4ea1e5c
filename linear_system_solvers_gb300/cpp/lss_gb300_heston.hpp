// lss_gb300_heston.hpp -- C++17 front end of the GB300 ADI path with the reference's names.
//
// Mirrors the user-facing pieces of MichalSara99/linear_system_solvers that the implicit 2-D
// Heston path takes (same class names, constructor arguments and meaning):
//   lss_utility::range                        common/lss_utility.hpp:130-186
//   lss_enumerations::*                       common/lss_enumerations.hpp:15-129
//   lss_containers::container_2d<Row>         containers/lss_container_2d.hpp:22-205
//   lss_boundary::dirichlet/neumann_boundary_2d  boundaries/lss_dirichlet_boundary.hpp, lss_neumann_boundary.hpp
//   lss_grids::grid_config_hints_2d           discretization/lss_grid_config_hints.hpp:54-88
//   lss_pde_solvers::pde_discretization_config_2d, heat_*_config_2d, splitting_method_config,
//                    heat_implicit_solver_config          pde_solvers/lss_*config*.hpp
//   lss_pde_solvers::two_dimensional::implicit_solvers::general_heston_equation
//                                             .../lss_2d_general_heston_equation.hpp:83-307
//   lss_pde_solvers::two_dimensional::explicit_solvers::general_heston_equation
//                                             .../lss_2d_general_heston_equation.hpp:317-510
//   lss_pde_solvers::general_heston_equation_builder   builders/lss_2d_general_heston_equation_builder.hpp:57-128
// solve() runs the device policies (tridiagonal_method_enum::GB300ThomasLUSolver or
// GB300DoubleSweepSolver on memory_space_enum::Device; the explicit Euler scheme) through the
// C-ABI of include/lss_adi.h: the user's coefficient
// functions are transformed to the computational grid and sampled exactly as the reference
// does (lss_heat_data_transform.hpp:174-214, lss_2d_general_heston_equation_coefficients.hpp:89-98),
// then handed to lss_adi_create_tabulated.  Host policies are not provided here (they stay in
// the reference).  Errors throw, as in the reference.
#pragma once

#include <cmath>
#include <cstddef>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "lss_adi.h"

namespace lss_gb300 {

namespace lss_utility {
template <typename T> using sptr_t = std::shared_ptr<T>;
template <typename T> class range {
    T l_{}, u_{};

  public:
    range() = default;
    range(T lower, T upper) : l_{lower}, u_{upper} {}
    T lower() const { return l_; }
    T upper() const { return u_; }
    T spread() const { return (u_ - l_); }
};
} // namespace lss_utility

namespace lss_enumerations {
enum class by_enum { Row, Column };
enum class factorization_enum { QRMethod, LUMethod, CholeskyMethod, None };
enum class splitting_method_enum { DouglasRachford, CraigSneyd, ModifiedCraigSneyd, HundsdorferVerwer };
enum class tridiagonal_method_enum {
    CUDASolver,
    DoubleSweepSolver,
    SORSolver,
    ThomasLUSolver,
    GB300ThomasLUSolver,     // device policies of this library: Thomas LU ...
    GB300DoubleSweepSolver   // ... and the double sweep (bit-identical to the host policies)
};
enum class grid_enum { Uniform, Nonuniform };
enum class traverse_direction_enum { Forward, Backward };
enum class memory_space_enum { Host, Device };
enum class implicit_pde_schemes_enum { Euler, Theta_30, CrankNicolson, Theta_80 };
enum class explicit_pde_schemes_enum { Euler, ADEBarakatClark, ADESaulyev };
} // namespace lss_enumerations

namespace lss_containers {
template <lss_enumerations::by_enum by, typename T> class container_2d;
template <typename T> class container_2d<lss_enumerations::by_enum::Row, T> {
    std::size_t rows_, cols_;
    std::vector<T> data_;

  public:
    container_2d(std::size_t rows, std::size_t columns, T value = T{})
        : rows_{rows}, cols_{columns}, data_(rows * columns, value)
    {
    }
    std::size_t rows() const { return rows_; }
    std::size_t columns() const { return cols_; }
    T operator()(std::size_t r, std::size_t c) const
    {
        if (r >= rows_ || c >= cols_) throw std::out_of_range("container_2d: index out of range");
        return data_[r * cols_ + c];
    }
    void operator()(std::size_t r, std::size_t c, T value)
    {
        if (r >= rows_ || c >= cols_) throw std::out_of_range("container_2d: index out of range");
        data_[r * cols_ + c] = value;
    }
    T *data() { return data_.data(); }
    const T *data() const { return data_.data(); }
};
} // namespace lss_containers

namespace lss_boundary {
template <typename T> class boundary_2d {
  public:
    virtual ~boundary_2d() = default;
    virtual T value(T t, T s) const = 0;
};
template <typename T> class dirichlet_boundary_2d : public boundary_2d<T> {
    std::function<T(T, T)> v_;

  public:
    explicit dirichlet_boundary_2d(std::function<T(T, T)> const &v) : v_{v} {}
    T value(T t, T s) const override { return v_(t, s); }
};
template <typename T> class neumann_boundary_2d : public boundary_2d<T> {
    std::function<T(T, T)> v_;

  public:
    explicit neumann_boundary_2d(std::function<T(T, T)> const &v) : v_{v} {}
    T value(T t, T s) const override { return v_(t, s); }
};
template <typename T> using boundary_2d_ptr = std::shared_ptr<boundary_2d<T>>;
template <typename T> using boundary_2d_pair = std::pair<boundary_2d_ptr<T>, boundary_2d_ptr<T>>;
} // namespace lss_boundary

namespace lss_grids {
template <typename T> class grid_config_hints_2d {
    T point_, alpha_scale_, beta_scale_;
    lss_enumerations::grid_enum grid_;

  public:
    explicit grid_config_hints_2d(T accumulation_point = T(0.0), T alpha_scale = T(3.0), T beta_scale = T(50.0),
                                  lss_enumerations::grid_enum grid = lss_enumerations::grid_enum::Uniform)
        : point_{accumulation_point}, alpha_scale_{alpha_scale}, beta_scale_{beta_scale}, grid_{grid}
    {
    }
    T accumulation_point() const { return point_; }
    T alpha_scale() const { return alpha_scale_; }
    T beta_scale() const { return beta_scale_; }
    lss_enumerations::grid_enum grid() const { return grid_; }
};
template <typename T> using grid_config_hints_2d_ptr = std::shared_ptr<grid_config_hints_2d<T>>;
} // namespace lss_grids

namespace lss_pde_solvers {
using lss_utility::range;

template <typename T> class pde_discretization_config_2d {
    range<T> r1_, r2_, rt_;
    std::size_t n1_, n2_, nt_;

  public:
    pde_discretization_config_2d(range<T> const &space_range_1, range<T> const &space_range_2,
                                 std::size_t number_of_space_points_1, std::size_t number_of_space_points_2,
                                 range<T> const &time_range, std::size_t number_of_time_points)
        : r1_{space_range_1}, r2_{space_range_2}, rt_{time_range}, n1_{number_of_space_points_1},
          n2_{number_of_space_points_2}, nt_{number_of_time_points}
    {
    }
    std::pair<range<T>, range<T>> space_range() const { return {r1_, r2_}; }
    range<T> const &time_range() const { return rt_; }
    std::pair<std::size_t, std::size_t> number_of_space_points() const { return {n1_, n2_}; }
    std::size_t number_of_time_points() const { return nt_; }
    T time_step() const { return (rt_.spread()) / static_cast<T>(nt_ - 1); }
};
template <typename T> using pde_discretization_config_2d_ptr = std::shared_ptr<pde_discretization_config_2d<T>>;

template <typename T> using fn3 = std::function<T(T, T, T)>;
template <typename T> class heat_coefficient_data_config_2d {
  public:
    fn3<T> a, b, c, d, e, f;
    heat_coefficient_data_config_2d(fn3<T> const &a_coefficient, fn3<T> const &b_coefficient,
                                    fn3<T> const &c_coefficient, fn3<T> const &d_coefficient,
                                    fn3<T> const &e_coefficient, fn3<T> const &f_coefficient)
        : a{a_coefficient}, b{b_coefficient}, c{c_coefficient}, d{d_coefficient}, e{e_coefficient}, f{f_coefficient}
    {
    }
};
template <typename T> class heat_initial_data_config_2d {
  public:
    std::function<T(T, T)> initial_condition;
    explicit heat_initial_data_config_2d(std::function<T(T, T)> const &ic) : initial_condition{ic} {}
};
template <typename T> class heat_data_config_2d {
  public:
    std::shared_ptr<heat_coefficient_data_config_2d<T>> coefficients;
    std::shared_ptr<heat_initial_data_config_2d<T>> initial;
    heat_data_config_2d(std::shared_ptr<heat_coefficient_data_config_2d<T>> const &coefficient_data_config,
                        std::shared_ptr<heat_initial_data_config_2d<T>> const &initial_data_config)
        : coefficients{coefficient_data_config}, initial{initial_data_config}
    {
    }
};
template <typename T> using heat_data_config_2d_ptr = std::shared_ptr<heat_data_config_2d<T>>;

template <typename T> class splitting_method_config {
    lss_enumerations::splitting_method_enum m_;
    T w_;

  public:
    explicit splitting_method_config(lss_enumerations::splitting_method_enum m, T weighting_value = T(0.5))
        : m_{m}, w_{weighting_value}
    {
    }
    lss_enumerations::splitting_method_enum splitting_method() const { return m_; }
    T weighting_value() const { return w_; }
};
template <typename T> using splitting_method_config_ptr = std::shared_ptr<splitting_method_config<T>>;

class heat_implicit_solver_config {
    lss_enumerations::memory_space_enum mem_;
    lss_enumerations::traverse_direction_enum dir_;
    lss_enumerations::tridiagonal_method_enum tri_;
    lss_enumerations::factorization_enum fac_;
    lss_enumerations::implicit_pde_schemes_enum sch_;

  public:
    heat_implicit_solver_config(lss_enumerations::memory_space_enum memory_space,
                                lss_enumerations::traverse_direction_enum traverse_direction,
                                lss_enumerations::tridiagonal_method_enum tridiagonal_method,
                                lss_enumerations::factorization_enum tridiagonal_factorization,
                                lss_enumerations::implicit_pde_schemes_enum implicit_pde_scheme)
        : mem_{memory_space}, dir_{traverse_direction}, tri_{tridiagonal_method}, fac_{tridiagonal_factorization},
          sch_{implicit_pde_scheme}
    {
    }
    lss_enumerations::memory_space_enum memory_space() const { return mem_; }
    lss_enumerations::traverse_direction_enum traverse_direction() const { return dir_; }
    lss_enumerations::tridiagonal_method_enum tridiagonal_method() const { return tri_; }
    lss_enumerations::implicit_pde_schemes_enum implicit_pde_scheme() const { return sch_; }
};
using heat_implicit_solver_config_ptr = std::shared_ptr<heat_implicit_solver_config>;

// heat_explicit_solver_config (pde_solvers/lss_heat_solver_config.hpp:56-78)
class heat_explicit_solver_config {
    lss_enumerations::memory_space_enum mem_;
    lss_enumerations::traverse_direction_enum dir_;
    lss_enumerations::explicit_pde_schemes_enum sch_;

  public:
    heat_explicit_solver_config(lss_enumerations::memory_space_enum memory_space,
                                lss_enumerations::traverse_direction_enum traverse_direction,
                                lss_enumerations::explicit_pde_schemes_enum explicit_pde_scheme)
        : mem_{memory_space}, dir_{traverse_direction}, sch_{explicit_pde_scheme}
    {
    }
    lss_enumerations::memory_space_enum memory_space() const { return mem_; }
    lss_enumerations::traverse_direction_enum traverse_direction() const { return dir_; }
    lss_enumerations::explicit_pde_schemes_enum explicit_pde_scheme() const { return sch_; }
};
using heat_explicit_solver_config_ptr = std::shared_ptr<heat_explicit_solver_config>;

namespace default_heat_solver_configs {
// the device counterparts of the reference's host_bwd_tlusolver_*_solver_config_ptr
inline heat_implicit_solver_config_ptr const dev_bwd_gb300_cn_solver_config_ptr =
    std::make_shared<heat_implicit_solver_config>(
        lss_enumerations::memory_space_enum::Device, lss_enumerations::traverse_direction_enum::Backward,
        lss_enumerations::tridiagonal_method_enum::GB300ThomasLUSolver, lss_enumerations::factorization_enum::None,
        lss_enumerations::implicit_pde_schemes_enum::CrankNicolson);
inline heat_implicit_solver_config_ptr const dev_bwd_gb300_o8_solver_config_ptr =
    std::make_shared<heat_implicit_solver_config>(
        lss_enumerations::memory_space_enum::Device, lss_enumerations::traverse_direction_enum::Backward,
        lss_enumerations::tridiagonal_method_enum::GB300ThomasLUSolver, lss_enumerations::factorization_enum::None,
        lss_enumerations::implicit_pde_schemes_enum::Theta_80);
// the reference's dev_expl_{fwd,bwd}_euler_solver_config_ptr (lss_heat_solver_config.hpp:244-252)
inline heat_explicit_solver_config_ptr const dev_expl_fwd_euler_solver_config_ptr =
    std::make_shared<heat_explicit_solver_config>(lss_enumerations::memory_space_enum::Device,
                                                  lss_enumerations::traverse_direction_enum::Forward,
                                                  lss_enumerations::explicit_pde_schemes_enum::Euler);
inline heat_explicit_solver_config_ptr const dev_expl_bwd_euler_solver_config_ptr =
    std::make_shared<heat_explicit_solver_config>(lss_enumerations::memory_space_enum::Device,
                                                  lss_enumerations::traverse_direction_enum::Backward,
                                                  lss_enumerations::explicit_pde_schemes_enum::Euler);
} // namespace default_heat_solver_configs

namespace two_dimensional {
namespace detail {
// The user's coefficient functions transformed to the computational grid and sampled exactly as
// the reference does (lss_heat_data_transform.hpp:174-214, coefficients.hpp:89-98), the
// boundaries and the terminal condition on the grid, then the device time loop through
// lss_adi_create_tabulated / lss_adi_forward.  Coefficients and boundaries are sampled at every
// step's time (the running time of implicit_heston_time_loop::run, implicit_kernel.hpp:150-207);
// when any of them changes with t the device gets one block of tables per step
// (LSS_ADI_OPT_STEP_TABLES), otherwise one.
template <typename T>
void tabulated_solve(heat_data_config_2d_ptr<T> const &data, pde_discretization_config_2d_ptr<T> const &disc,
                     lss_boundary::boundary_2d_ptr<T> const &ver, lss_boundary::boundary_2d_pair<T> const &hor,
                     lss_grids::grid_config_hints_2d_ptr<T> const &hints, bool fwd, int scheme, int theta_scheme,
                     double zeta, int arith, int options,
                     lss_containers::container_2d<lss_enumerations::by_enum::Row, T> &solution)
{
    const auto sizes = disc->number_of_space_points();
    const std::size_t nx = sizes.first, ny = sizes.second;
    if (!(solution.rows() == nx && solution.columns() == ny))
        throw std::invalid_argument("The input solution container must have the correct size");
    const auto sp = disc->space_range();
    const T one = T(1.0), two = T(2.0), half = T(0.5), quarter = T(0.25);
    // sinh grid map (discretization/lss_grid_transform_config.hpp:118-149)
    const T low1 = sp.first.lower(), high1 = sp.first.upper(), low2 = sp.second.lower(), high2 = sp.second.upper();
    const T point = hints->accumulation_point();
    T alpha = high1 - low1, beta = high2 - low2;
    if (hints->grid() == lss_enumerations::grid_enum::Nonuniform) {
        alpha = (point - low1) / hints->alpha_scale();
        beta = (high2 - low2) / hints->beta_scale();
    }
    const T c0 = std::asinh((high1 - point) / alpha), c1 = std::asinh((low1 - point) / alpha);
    const T dd = std::asinh((high2 - low2) / beta), cdiff = c0 - c1;
    auto X = [&](T z) { return point + alpha * std::sinh(c0 * z + c1 * (one - z)); };
    auto Y = [&](T e) { return low2 + beta * std::sinh(dd * e); };
    auto Ad = [&](T z) { return alpha * cdiff * std::cosh(c0 * z + c1 * (one - z)); };
    auto Bd = [&](T e) { return beta * dd * std::cosh(dd * e); };
    auto Cd = [&](T z) { return alpha * cdiff * cdiff * std::sinh(c0 * z + c1 * (one - z)); };
    auto Dd = [&](T e) { return beta * dd * dd * std::sinh(dd * e); };
    // scheme scalars (implicit_coefficients/...coefficients.hpp:59-73)
    const T k = disc->time_step();
    const T h1 = one / static_cast<T>(nx - 1), h2 = one / static_cast<T>(ny - 1);
    const T al = k / (h1 * h1), be = k / (h2 * h2), de = half * k / h1, ni = half * k / h2, rho = k;
    (void)quarter;
    const auto &cf = *data->coefficients;
    const T t_first = fwd ? (disc->time_range().lower() + k) : (disc->time_range().upper() - k);
    const T t_last = fwd ? disc->time_range().upper() : disc->time_range().lower() + k;
    const std::size_t n = nx * ny;
    auto fill = [&](T t, std::vector<T> &coef, std::vector<T> &v0) {
        coef.assign(7 * n, T(0));
        v0.assign(3 * nx, T(0));
        for (std::size_t i = 0; i < nx; ++i) {
            const T z = h1 * static_cast<T>(i);
            for (std::size_t j = 0; j < ny; ++j) {
                const T e = h2 * static_cast<T>(j);
                const T x = X(z), y = Y(e);
                const T av = Ad(z), bv = Bd(e);
                const T A = cf.a(t, x, y), B = cf.b(t, x, y);
                const T ah = A / (av * av), bh = B / (bv * bv), ch = cf.c(t, x, y) / (av * bv);
                const T dh = cf.d(t, x, y) / av - (A * Cd(z)) / (av * av * av);
                const T eh = cf.e(t, x, y) / bv - (B * Dd(e)) / (bv * bv * bv);
                const T fh = cf.f(t, x, y);
                const std::size_t o = i * ny + j;
                coef[o] = al * ah - de * dh;
                coef[n + o] = al * ah + de * dh;
                coef[2 * n + o] = two * al * ah - half * rho * fh;
                coef[3 * n + o] = be * bh - ni * eh;
                coef[4 * n + o] = be * bh + ni * eh;
                coef[5 * n + o] = two * be * bh - half * rho * fh;
                coef[6 * n + o] = ch;
                if (j == 0) {
                    v0[i] = dh;
                    v0[nx + i] = eh;
                    v0[2 * nx + i] = fh;
                }
            }
        }
    };
    (void)t_last;
    // boundaries on the computational grid (lss_heston_boundary_transform.hpp:47-65)
    const T A1 = Ad(one);
    auto fill_bnd = [&](T t, std::vector<T> &slo, std::vector<T> &neu, std::vector<T> &vhi) {
        slo.resize(ny);
        neu.resize(ny);
        vhi.resize(nx);
        for (std::size_t j = 0; j < ny; ++j) {
            const T y = Y(h2 * static_cast<T>(j));
            slo[j] = hor.first->value(t, y);
            neu[j] = hor.second->value(t, y) * A1;
        }
        for (std::size_t i = 0; i < nx; ++i) vhi[i] = ver->value(t, X(h1 * static_cast<T>(i)));
    };
    // every step's tables; kept as one block while they all equal the first step's
    const std::size_t steps = disc->number_of_time_points() - 1;
    std::vector<T> coef, v0, slo, neu, vhi;
    fill(t_first, coef, v0);
    fill_bnd(t_first, slo, neu, vhi);
    const std::vector<T> coef1 = coef, v01 = v0, slo1 = slo, neu1 = neu, vhi1 = vhi;
    bool varies = false;
    T ts = t_first;
    std::vector<T> c2, w2, s2, n2, h2v;
    for (std::size_t st = 1; st < steps; ++st) {
        ts = fwd ? ts + k : ts - k;
        fill(ts, c2, w2);
        fill_bnd(ts, s2, n2, h2v);
        if (!varies && (c2 != coef1 || w2 != v01 || s2 != slo1 || n2 != neu1 || h2v != vhi1)) {
            varies = true;
            for (std::size_t b = 1; b < st; ++b) { // the steps before were equal to the first
                coef.insert(coef.end(), coef1.begin(), coef1.end());
                v0.insert(v0.end(), v01.begin(), v01.end());
                slo.insert(slo.end(), slo1.begin(), slo1.end());
                neu.insert(neu.end(), neu1.begin(), neu1.end());
                vhi.insert(vhi.end(), vhi1.begin(), vhi1.end());
            }
        }
        if (varies) {
            coef.insert(coef.end(), c2.begin(), c2.end());
            v0.insert(v0.end(), w2.begin(), w2.end());
            slo.insert(slo.end(), s2.begin(), s2.end());
            neu.insert(neu.end(), n2.begin(), n2.end());
            vhi.insert(vhi.end(), h2v.begin(), h2v.end());
        }
    }
    if (varies && scheme == LSS_ADI_EXPLICIT_EULER)
        throw std::invalid_argument("the device explicit Euler scheme needs time-invariant coefficients and boundaries");
    if (varies) options |= LSS_ADI_OPT_STEP_TABLES;
    std::vector<T> pay(n);
    for (std::size_t i = 0; i < nx; ++i) {
        const T x = X(h1 * static_cast<T>(i));
        for (std::size_t j = 0; j < ny; ++j) pay[i * ny + j] = data->initial->initial_condition(x, Y(h2 * static_cast<T>(j)));
    }
    lss_adi_tables t{};
    t.nx = static_cast<int>(nx);
    t.ny = static_cast<int>(ny);
    t.nt = static_cast<int>(disc->number_of_time_points());
    t.t_lo = static_cast<double>(disc->time_range().lower());
    t.t_hi = static_cast<double>(disc->time_range().upper());
    t.scheme = scheme;
    t.theta_scheme = theta_scheme;
    t.forward = fwd ? 1 : 0;
    t.precision = std::is_same<T, double>::value ? LSS_ADI_FP64 : LSS_ADI_FP32;
    t.arith = arith;
    t.zeta = zeta;
    t.coef = coef.data();
    t.coef_v0 = v0.data();
    t.s_lo_dirichlet = slo.data();
    t.s_hi_neumann = neu.data();
    t.v_hi_dirichlet = vhi.data();
    t.payoff = pay.data();
    t.options = options;
    lss_adi_handle *h = nullptr;
    if (lss_adi_create_tabulated(&t, &h) != LSS_ADI_OK) throw std::runtime_error(lss_adi_last_error());
    const int rc = lss_adi_forward(h, nullptr, solution.data(), nullptr, 0, nullptr);
    lss_adi_destroy(h);
    if (rc != LSS_ADI_OK) throw std::runtime_error(lss_adi_last_error());
}
} // namespace detail

namespace implicit_solvers {

/*
 * general_heston_equation with the GB300 device policy.  arith selects the line-solve
 * arithmetic: LSS_ADI_ARITH_REFERENCE (bit-identical to the reference's host Thomas-LU
 * policy) or LSS_ADI_ARITH_FAST.
 */
template <typename T> class general_heston_equation {
    heat_data_config_2d_ptr<T> data_;
    pde_discretization_config_2d_ptr<T> disc_;
    lss_boundary::boundary_2d_ptr<T> ver_;
    lss_boundary::boundary_2d_pair<T> hor_;
    splitting_method_config_ptr<T> split_;
    lss_grids::grid_config_hints_2d_ptr<T> hints_;
    heat_implicit_solver_config_ptr cfg_;
    int arith_;

    static void verify(bool ok, const char *msg)
    {
        if (!ok) throw std::invalid_argument(msg);
    }

  public:
    general_heston_equation(heat_data_config_2d_ptr<T> const &heat_data_config,
                            pde_discretization_config_2d_ptr<T> const &discretization_config,
                            lss_boundary::boundary_2d_ptr<T> const &vertical_upper_boundary_ptr,
                            lss_boundary::boundary_2d_pair<T> const &horizontal_boundary_pair,
                            splitting_method_config_ptr<T> const &splitting_method_config,
                            lss_grids::grid_config_hints_2d_ptr<T> const &grid_config_hints,
                            heat_implicit_solver_config_ptr const &solver_config =
                                default_heat_solver_configs::dev_bwd_gb300_cn_solver_config_ptr,
                            std::map<std::string, T> const & = std::map<std::string, T>(),
                            int arith = LSS_ADI_ARITH_REFERENCE)
        : data_{heat_data_config}, disc_{discretization_config}, ver_{vertical_upper_boundary_ptr},
          hor_{horizontal_boundary_pair}, split_{splitting_method_config}, hints_{grid_config_hints},
          cfg_{solver_config}, arith_{arith}
    {
        // the checks of general_heston_equation::initialize (lss_2d_general_heston_equation.hpp:104-126)
        verify(data_ != nullptr, "heat_data_config must not be null");
        verify(disc_ != nullptr, "discretization_config must not be null");
        verify(std::dynamic_pointer_cast<lss_boundary::dirichlet_boundary_2d<T>>(ver_) != nullptr,
               "vertical_upper_boundary_ptr must be of dirichlet type only");
        verify(std::dynamic_pointer_cast<lss_boundary::dirichlet_boundary_2d<T>>(hor_.first) != nullptr,
               "horizontal_boundary_pair.first must be of dirichlet type only");
        verify(std::dynamic_pointer_cast<lss_boundary::neumann_boundary_2d<T>>(hor_.second) != nullptr,
               "horizontal_boundary_pair.second must be of neumann type only");
        verify(split_ != nullptr, "splitting_method_config must not be null");
        verify(cfg_ != nullptr, "solver_config must not be null");
        verify(hints_ != nullptr, "grid_config_hints must not be null");
        if (cfg_->memory_space() != lss_enumerations::memory_space_enum::Device ||
            (cfg_->tridiagonal_method() != lss_enumerations::tridiagonal_method_enum::GB300ThomasLUSolver &&
             cfg_->tridiagonal_method() != lss_enumerations::tridiagonal_method_enum::GB300DoubleSweepSolver))
            throw std::invalid_argument("this front end runs the Device/GB300ThomasLUSolver and "
                                        "Device/GB300DoubleSweepSolver policies only; host policies stay in the "
                                        "reference library");
    }

    void solve(lss_containers::container_2d<lss_enumerations::by_enum::Row, T> &solution)
    {
        int scheme = 0;
        switch (split_->splitting_method()) {
        case lss_enumerations::splitting_method_enum::DouglasRachford: scheme = LSS_ADI_DOUGLAS_RACHFORD; break;
        case lss_enumerations::splitting_method_enum::CraigSneyd: scheme = LSS_ADI_CRAIG_SNEYD; break;
        case lss_enumerations::splitting_method_enum::ModifiedCraigSneyd: scheme = LSS_ADI_MODIFIED_CRAIG_SNEYD; break;
        default: scheme = LSS_ADI_HUNDSDORFER_VERWER; break;
        }
        const bool fwd = cfg_->traverse_direction() == lss_enumerations::traverse_direction_enum::Forward;
        const int options =
            cfg_->tridiagonal_method() == lss_enumerations::tridiagonal_method_enum::GB300DoubleSweepSolver
                ? LSS_ADI_OPT_DOUBLE_SWEEP
                : 0;
        detail::tabulated_solve<T>(data_, disc_, ver_, hor_, hints_, fwd, scheme, static_cast<int>(cfg_->implicit_pde_scheme()),
                                   static_cast<double>(split_->weighting_value()), arith_, options, solution);
    }
};
} // namespace implicit_solvers

namespace explicit_solvers {

/*
 * explicit_solvers::general_heston_equation (lss_2d_general_heston_equation.hpp:317-510) with
 * the device explicit Euler scheme: the whole time loop runs on the GPU with the coefficients
 * resident there.  arith: LSS_ADI_ARITH_REFERENCE (bit-identical to the reference's host
 * Euler scheme) or LSS_ADI_ARITH_FAST.  Stability is the caller's, as in the reference.
 */
template <typename T> class general_heston_equation {
    heat_data_config_2d_ptr<T> data_;
    pde_discretization_config_2d_ptr<T> disc_;
    lss_boundary::boundary_2d_ptr<T> ver_;
    lss_boundary::boundary_2d_pair<T> hor_;
    lss_grids::grid_config_hints_2d_ptr<T> hints_;
    heat_explicit_solver_config_ptr cfg_;
    int arith_;

  public:
    general_heston_equation(heat_data_config_2d_ptr<T> const &heat_data_config,
                            pde_discretization_config_2d_ptr<T> const &discretization_config,
                            lss_boundary::boundary_2d_ptr<T> const &vertical_upper_boundary_ptr,
                            lss_boundary::boundary_2d_pair<T> const &horizontal_boundary_pair,
                            lss_grids::grid_config_hints_2d_ptr<T> const &grid_config_hints,
                            heat_explicit_solver_config_ptr const &solver_config =
                                default_heat_solver_configs::dev_expl_fwd_euler_solver_config_ptr,
                            int arith = LSS_ADI_ARITH_REFERENCE)
        : data_{heat_data_config}, disc_{discretization_config}, ver_{vertical_upper_boundary_ptr},
          hor_{horizontal_boundary_pair}, hints_{grid_config_hints}, cfg_{solver_config}, arith_{arith}
    {
        // the checks of the reference's initialize (lss_2d_general_heston_equation.hpp:375-402)
        if (!data_) throw std::invalid_argument("heat_data_config must not be null");
        if (!disc_) throw std::invalid_argument("discretization_config must not be null");
        if (!std::dynamic_pointer_cast<lss_boundary::dirichlet_boundary_2d<T>>(ver_))
            throw std::invalid_argument("vertical_upper_boundary_ptr must be of dirichlet type only");
        if (!std::dynamic_pointer_cast<lss_boundary::dirichlet_boundary_2d<T>>(hor_.first))
            throw std::invalid_argument("horizontal_boundary_pair.first must be of dirichlet type only");
        if (!std::dynamic_pointer_cast<lss_boundary::neumann_boundary_2d<T>>(hor_.second))
            throw std::invalid_argument("horizontal_boundary_pair.second must be of neumann type only");
        if (!cfg_) throw std::invalid_argument("solver_config must not be null");
        if (!hints_) throw std::invalid_argument("grid_config_hints must not be null");
        if (cfg_->memory_space() != lss_enumerations::memory_space_enum::Device ||
            cfg_->explicit_pde_scheme() != lss_enumerations::explicit_pde_schemes_enum::Euler)
            throw std::invalid_argument("this front end runs the Device explicit Euler scheme only "
                                        "(the reference supports no other on the device either)");
    }

    void solve(lss_containers::container_2d<lss_enumerations::by_enum::Row, T> &solution)
    {
        const bool fwd = cfg_->traverse_direction() == lss_enumerations::traverse_direction_enum::Forward;
        detail::tabulated_solve<T>(data_, disc_, ver_, hor_, hints_, fwd, LSS_ADI_EXPLICIT_EULER, LSS_ADI_CRANK_NICOLSON,
                                   0.5, arith_, 0, solution);
    }
};

} // namespace explicit_solvers
} // namespace two_dimensional

template <typename T> class general_heston_equation_builder {
    heat_data_config_2d_ptr<T> data_;
    pde_discretization_config_2d_ptr<T> disc_;
    lss_boundary::boundary_2d_ptr<T> ver_;
    lss_boundary::boundary_2d_pair<T> hor_;
    splitting_method_config_ptr<T> split_;
    lss_grids::grid_config_hints_2d_ptr<T> hints_;
    heat_implicit_solver_config_ptr cfg_ = default_heat_solver_configs::dev_bwd_gb300_cn_solver_config_ptr;
    std::map<std::string, T> details_;

  public:
    general_heston_equation_builder &heat_data_config(heat_data_config_2d_ptr<T> const &v) { data_ = v; return *this; }
    general_heston_equation_builder &discretization_config(pde_discretization_config_2d_ptr<T> const &v) { disc_ = v; return *this; }
    general_heston_equation_builder &vertical_upper_boundary(lss_boundary::boundary_2d_ptr<T> const &v) { ver_ = v; return *this; }
    general_heston_equation_builder &horizontal_boundary(lss_boundary::boundary_2d_pair<T> const &v) { hor_ = v; return *this; }
    general_heston_equation_builder &splitting_method_config(splitting_method_config_ptr<T> const &v) { split_ = v; return *this; }
    general_heston_equation_builder &grid_hints(lss_grids::grid_config_hints_2d_ptr<T> const &v) { hints_ = v; return *this; }
    general_heston_equation_builder &solver_config(heat_implicit_solver_config_ptr const &v) { cfg_ = v; return *this; }
    general_heston_equation_builder &solver_config_details(std::map<std::string, T> const &v) { details_ = v; return *this; }
    std::shared_ptr<two_dimensional::implicit_solvers::general_heston_equation<T>> build()
    {
        return std::make_shared<two_dimensional::implicit_solvers::general_heston_equation<T>>(
            data_, disc_, ver_, hor_, split_, hints_, cfg_, details_);
    }
};

} // namespace lss_pde_solvers
} // namespace lss_gb300
