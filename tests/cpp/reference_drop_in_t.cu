// reference_drop_in_t.cu -- the GB300 device policy inside the reference's own solver (TEST
// INFRASTRUCTURE ONLY; built by tests/cpp/build_reference_drop_in.sh against a build-time copy of
// the reference with the enumerator and dispatch branch added).
//
// Every case sets a problem up as the reference's tests do (unit_tests/common/lss_print_t.hpp:
// 1850-1974 Heston, 1976-2102 SABR) and solves it twice with the reference's
// implicit_solvers::general_heston_equation: once with its Host ThomasLUSolver policy, once with
// memory_space_enum::Device and tridiagonal_method_enum::GB300ThomasLUSolver (the kernel
// specialisation of linear_system_solvers_gb300/cpp/lss_gb300_reference_kernel.hpp, running the
// time loop on the GPU).  One case goes through the reference's general_heston_equation_builder.
// Prints one line per case: name, 1 if the two surfaces are identical bit for bit, the largest
// absolute difference; exit 0 when every case is identical.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "builders/lss_2d_general_heston_equation_builder.hpp"
#include "pde_solvers/two_dimensional/heat_type/lss_2d_general_heston_equation.hpp"

#include "lss_gb300_reference_kernel.hpp"

using namespace lss_pde_solvers;
using lss_boundary::dirichlet_boundary_2d;
using lss_boundary::neumann_boundary_2d;
using lss_containers::container_2d;
using lss_enumerations::by_enum;
using lss_enumerations::factorization_enum;
using lss_enumerations::grid_enum;
using lss_enumerations::implicit_pde_schemes_enum;
using lss_enumerations::memory_space_enum;
using lss_enumerations::splitting_method_enum;
using lss_enumerations::traverse_direction_enum;
using lss_enumerations::tridiagonal_method_enum;
using lss_grids::grid_config_hints_2d;
using lss_utility::range;

struct drop_case {
    const char *name;
    bool sabr;
    splitting_method_enum scheme;
    double zeta;
    implicit_pde_schemes_enum theta;
    std::size_t nx, ny, nt;
    double rate;
    bool forward, builder;
};

template <typename T> static int run_case(const drop_case &c)
{
    typedef container_2d<by_enum::Row, T, std::vector, std::allocator<T>> rcontainer_2d_t;
    typedef two_dimensional::implicit_solvers::general_heston_equation<T, std::vector, std::allocator<T>> pde_solver;
    const double maturity = 1.0, rate = c.rate;
    const double strike = c.sabr ? 0.05 : 100.0;
    range<T> sx(static_cast<T>(0.0), static_cast<T>(c.sabr ? 0.2 : 200.0));
    range<T> sy(static_cast<T>(0.0), static_cast<T>(c.sabr ? 1.0 : 1.2));
    range<T> tr(static_cast<T>(0.0), static_cast<T>(maturity));
    auto const disc = std::make_shared<pde_discretization_config_2d<T>>(sx, sy, c.nx, c.ny, tr, c.nt);
    std::shared_ptr<heat_coefficient_data_config_2d<T>> coeffs;
    if (c.sabr) {
        const double beta = 0.5, nu = 0.4, rho = -0.3;
        auto D = [=](T t) { return std::exp(-rate * (maturity - t)); };
        auto ca = [=](T t, T s, T a) {
            return (0.5 * a * a * std::pow(s, 2.0 * beta) * std::pow(D(t), 2.0 * (1.0 - beta)));
        };
        auto cb = [=](T t, T s, T a) { return (0.5 * nu * nu * a * a); };
        auto cc = [=](T t, T s, T a) { return (rho * nu * a * a * std::pow(s, beta) * std::pow(D(t), (1.0 - beta))); };
        auto cd = [=](T t, T s, T a) { return (rate * s); };
        auto ce = [=](T t, T s, T a) { return 0.0; };
        auto cf = [=](T t, T s, T a) { return (-rate); };
        coeffs = std::make_shared<heat_coefficient_data_config_2d<T>>(ca, cb, cc, cd, ce, cf);
    } else {
        const double kappa = 1.5, theta_v = 0.04, sigma = 0.3, rho = -0.6;
        auto ca = [=](T t, T s, T v) { return (0.5 * v * s * s); };
        auto cb = [=](T t, T s, T v) { return (0.5 * sigma * sigma * v); };
        auto cc = [=](T t, T s, T v) { return (rho * sigma * v * s); };
        auto cd = [=](T t, T s, T v) { return (rate * s); };
        auto ce = [=](T t, T s, T v) { return (kappa * (theta_v - v)); };
        auto cf = [=](T t, T s, T v) { return (-rate); };
        coeffs = std::make_shared<heat_coefficient_data_config_2d<T>>(ca, cb, cc, cd, ce, cf);
    }
    auto terminal = [=](T s, T v) { return std::max<T>(0.0, s - strike); };
    auto const init = std::make_shared<heat_initial_data_config_2d<T>>(terminal);
    auto const data = std::make_shared<heat_data_config_2d<T>>(coeffs, init);
    auto const &lo = [=](T t, T v) { return 0.0; };
    auto const &hi = [=](T t, T s) { return -1.0; };
    auto const &lo_ptr = std::make_shared<dirichlet_boundary_2d<T>>(lo);
    auto const &hi_ptr = std::make_shared<neumann_boundary_2d<T>>(hi);
    auto const &hpair = std::make_pair(lss_boundary::boundary_2d_ptr<T>(lo_ptr), lss_boundary::boundary_2d_ptr<T>(hi_ptr));
    auto const &vtop = [=](T t, T s) { return s; };
    auto const &vtop_ptr = std::make_shared<dirichlet_boundary_2d<T>>(vtop);
    auto const &split = std::make_shared<splitting_method_config<T>>(c.scheme, static_cast<T>(c.zeta));
    auto const &hints = std::make_shared<grid_config_hints_2d<T>>(static_cast<T>(strike), static_cast<T>(10.0),
                                                                  static_cast<T>(24.0), grid_enum::Nonuniform);
    const traverse_direction_enum dir = c.forward ? traverse_direction_enum::Forward : traverse_direction_enum::Backward;
    auto const host_cfg = std::make_shared<heat_implicit_solver_config>(
        memory_space_enum::Host, dir, tridiagonal_method_enum::ThomasLUSolver, factorization_enum::None, c.theta);
    auto const dev_cfg = std::make_shared<heat_implicit_solver_config>(
        memory_space_enum::Device, dir, tridiagonal_method_enum::GB300ThomasLUSolver, factorization_enum::None, c.theta);

    rcontainer_2d_t host(c.nx, c.ny, T{}), dev(c.nx, c.ny, T{});
    {
        pde_solver s(data, disc, vtop_ptr, hpair, split, hints, host_cfg);
        s.solve(host);
    }
    if (c.builder) {
        auto s = two_dimensional::implicit_solvers::general_heston_equation_builder<T>()
                     .heat_data_config(data)
                     .discretization_config(disc)
                     .vertical_upper_boundary(vtop_ptr)
                     .horizontal_boundary(hpair)
                     .splitting_method_config(split)
                     .grid_hints(hints)
                     .solver_config(dev_cfg)
                     .build();
        s->solve(dev);
    } else {
        pde_solver s(data, disc, vtop_ptr, hpair, split, hints, dev_cfg);
        s.solve(dev);
    }
    // identical bits, except that a NaN equals any NaN (the host's and the GPU's arithmetic give
    // NaNs of different sign and payload where the scheme overflows); one NaN against a number
    // is a mismatch
    bool same = true;
    double worst = 0.0;
    int nans = 0;
    for (std::size_t i = 0; i < c.nx; ++i)
        for (std::size_t j = 0; j < c.ny; ++j) {
            const T a = host(i, j), b = dev(i, j);
            if (std::isnan(a) || std::isnan(b)) {
                if (!(std::isnan(a) && std::isnan(b))) {
                    same = false;
                    worst = INFINITY;
                }
                ++nans;
                continue;
            }
            if (std::memcmp(&a, &b, sizeof(T)) != 0) same = false;
            worst = std::max(worst, std::fabs(static_cast<double>(a) - static_cast<double>(b)));
        }
    std::printf("%s%s %d %.3e %d\n", c.name, sizeof(T) == 4 ? "_f32" : "_f64", same ? 1 : 0, worst, nans);
    return same ? 0 : 1;
}

int main()
{
    const drop_case cases[] = {
        {"heston_dr", false, splitting_method_enum::DouglasRachford, 0.5, implicit_pde_schemes_enum::CrankNicolson, 60,
         30, 41, 0.02, false, false},
        {"heston_cs", false, splitting_method_enum::CraigSneyd, 0.5, implicit_pde_schemes_enum::CrankNicolson, 48, 26, 31,
         0.02, false, true},
        {"heston_mcs_zeta_third", false, splitting_method_enum::ModifiedCraigSneyd, 1.0 / 3.0,
         implicit_pde_schemes_enum::Theta_80, 50, 25, 31, 0.02, false, false},
        {"heston_hv_forward", false, splitting_method_enum::HundsdorferVerwer, 0.5, implicit_pde_schemes_enum::CrankNicolson,
         45, 33, 27, 0.02, true, false},
        {"sabr_dr_time_dependent", true, splitting_method_enum::DouglasRachford, 0.5,
         implicit_pde_schemes_enum::CrankNicolson, 40, 22, 26, 0.03, false, false},
        {"sabr_hv_time_dependent", true, splitting_method_enum::HundsdorferVerwer, 0.5, implicit_pde_schemes_enum::Euler,
         36, 20, 21, 0.03, false, false},
    };
    int bad = 0;
    try {
        for (const drop_case &c : cases) {
            bad += run_case<double>(c);
            bad += run_case<float>(c);
        }
    } catch (std::exception const &e) {
        std::fprintf(stderr, "reference_drop_in_t: %s\n", e.what());
        return 2;
    }
    return bad ? 1 : 0;
}
