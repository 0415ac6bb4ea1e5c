// heston_front_end_t.cpp -- the reference's Heston print tests, written against the C++ front
// end (linear_system_solvers_gb300/cpp/lss_gb300_heston.hpp) with the device policy.  Same
// set-up as unit_tests/common/lss_print_t.hpp:1850-1974 / :2104-2591 of the reference, with
// the parameters taken from the command line; writes the final surface (raw, row-major).
//
// usage: heston_front_end_t <f32|f64> <dr|cs|mcs|hv> nx ny nt kappa theta sigma rho rate
//        strike maturity s_lo s_hi v_lo v_hi zeta theta_scheme nonuniform acc alpha_s beta_s
//        arith(0 fast|1 reference) builder(0|1) method(tlu|ds|euler) out.bin [sabr:<beta>]
// method: tridiagonal_method_enum::GB300ThomasLUSolver / GB300DoubleSweepSolver, or the
// explicit_solvers::general_heston_equation with the device explicit Euler scheme.
// sabr:<beta>: the SABR model of unit_tests/common/lss_print_t.hpp:2039-2050 instead (sigma is nu,
// F in place of S, alpha in place of v), whose coefficients change with t through the discount
// factor D(t) = exp(-r (T - t)) when r != 0: the front end then hands the device one block of
// tables per step.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <string>

#include "lss_gb300_heston.hpp"

using namespace lss_gb300;
using lss_boundary::dirichlet_boundary_2d;
using lss_boundary::neumann_boundary_2d;
using lss_containers::container_2d;
using lss_enumerations::by_enum;
using lss_enumerations::grid_enum;
using lss_enumerations::splitting_method_enum;
using lss_grids::grid_config_hints_2d;
using lss_pde_solvers::heat_coefficient_data_config_2d;
using lss_pde_solvers::heat_data_config_2d;
using lss_pde_solvers::heat_implicit_solver_config;
using lss_pde_solvers::heat_initial_data_config_2d;
using lss_pde_solvers::pde_discretization_config_2d;
using lss_pde_solvers::splitting_method_config;
using lss_pde_solvers::two_dimensional::implicit_solvers::general_heston_equation;
using lss_utility::range;

template <typename T> static int run(int argc, char **argv)
{
    int k = 2;
    const std::string scheme = argv[k++];
    const std::size_t Sd = std::strtoul(argv[k++], nullptr, 10), Vd = std::strtoul(argv[k++], nullptr, 10),
                      Td = std::strtoul(argv[k++], nullptr, 10);
    const double sig_kappa = std::atof(argv[k++]), sig_theta = std::atof(argv[k++]), sig_sig = std::atof(argv[k++]);
    const double rho = std::atof(argv[k++]), rate = std::atof(argv[k++]), strike = std::atof(argv[k++]);
    const double maturity = std::atof(argv[k++]);
    const double s_lo = std::atof(argv[k++]), s_hi = std::atof(argv[k++]), v_lo = std::atof(argv[k++]),
                 v_hi = std::atof(argv[k++]), zeta = std::atof(argv[k++]);
    const int theta_scheme = std::atoi(argv[k++]), nonuniform = std::atoi(argv[k++]);
    const double acc = std::atof(argv[k++]), alpha_s = std::atof(argv[k++]), beta_s = std::atof(argv[k++]);
    const int arith = std::atoi(argv[k++]), use_builder = std::atoi(argv[k++]);
    const std::string method = argv[k++];
    const std::string out = argv[k++];
    (void)argc;

    range<T> spacex_range(static_cast<T>(s_lo), static_cast<T>(s_hi));
    range<T> spacey_range(static_cast<T>(v_lo), static_cast<T>(v_hi));
    range<T> time_range(static_cast<T>(0.0), static_cast<T>(maturity));
    auto const discretization_ptr =
        std::make_shared<pde_discretization_config_2d<T>>(spacex_range, spacey_range, Sd, Vd, time_range, Td);
    const std::string model = argc > 27 ? argv[27] : "heston";
    const bool sabr = model.rfind("sabr:", 0) == 0;
    const double beta = sabr ? std::atof(model.c_str() + 5) : 0.0;
    std::function<T(T, T, T)> a = [=](T t, T s, T v) { return (0.5 * v * s * s); };
    std::function<T(T, T, T)> b = [=](T t, T s, T v) { return (0.5 * sig_sig * sig_sig * v); };
    std::function<T(T, T, T)> c = [=](T t, T s, T v) { return (rho * sig_sig * v * s); };
    std::function<T(T, T, T)> d = [=](T t, T s, T v) { return (rate * s); };
    std::function<T(T, T, T)> e = [=](T t, T s, T v) { return (sig_kappa * (sig_theta - v)); };
    std::function<T(T, T, T)> f = [=](T t, T s, T v) { return (-rate); };
    if (sabr) {
        // double arithmetic, evaluated left to right as the reference's lambdas
        a = [=](T t, T s, T v) {
            const double D = std::exp(-rate * (maturity - static_cast<double>(t)));
            return static_cast<T>(0.5 * static_cast<double>(v) * static_cast<double>(v) *
                                  std::pow(static_cast<double>(s), 2.0 * beta) * std::pow(D, 2.0 * (1.0 - beta)));
        };
        b = [=](T t, T s, T v) {
            return static_cast<T>(0.5 * sig_sig * sig_sig * static_cast<double>(v) * static_cast<double>(v));
        };
        c = [=](T t, T s, T v) {
            const double D = std::exp(-rate * (maturity - static_cast<double>(t)));
            return static_cast<T>(rho * sig_sig * static_cast<double>(v) * static_cast<double>(v) *
                                  std::pow(static_cast<double>(s), beta) * std::pow(D, (1.0 - beta)));
        };
        d = [=](T t, T s, T v) { return static_cast<T>(rate * static_cast<double>(s)); };
        e = [=](T t, T s, T v) { return static_cast<T>(0.0); };
        f = [=](T t, T s, T v) { return static_cast<T>(-rate); };
    }
    auto const heat_coeffs_data_ptr = std::make_shared<heat_coefficient_data_config_2d<T>>(a, b, c, d, e, f);
    auto terminal_condition = [=](T s, T v) { return std::max<T>(0.0, s - strike); };
    auto const heat_init_data_ptr = std::make_shared<heat_initial_data_config_2d<T>>(terminal_condition);
    auto const heat_data_ptr = std::make_shared<heat_data_config_2d<T>>(heat_coeffs_data_ptr, heat_init_data_ptr);
    auto const &dirichlet_low = [=](T t, T v) { return 0.0; };
    auto const &neumann_high = [=](T t, T s) { return -1.0; };
    auto const &boundary_low_ptr = std::make_shared<dirichlet_boundary_2d<T>>(dirichlet_low);
    auto const &boundary_high_ptr = std::make_shared<neumann_boundary_2d<T>>(neumann_high);
    auto const &horizontal_boundary_pair =
        std::make_pair(lss_boundary::boundary_2d_ptr<T>(boundary_low_ptr), lss_boundary::boundary_2d_ptr<T>(boundary_high_ptr));
    auto const &dirichlet_high = [=](T t, T s) { return s; };
    auto const &vertical_upper_boundary_ptr = std::make_shared<dirichlet_boundary_2d<T>>(dirichlet_high);
    splitting_method_enum sm = splitting_method_enum::DouglasRachford;
    if (scheme == "cs") sm = splitting_method_enum::CraigSneyd;
    else if (scheme == "mcs") sm = splitting_method_enum::ModifiedCraigSneyd;
    else if (scheme == "hv") sm = splitting_method_enum::HundsdorferVerwer;
    auto const &splitting_config_ptr = std::make_shared<splitting_method_config<T>>(sm, static_cast<T>(zeta));
    auto const &grid_config_hints_ptr = std::make_shared<grid_config_hints_2d<T>>(
        static_cast<T>(acc), static_cast<T>(alpha_s), static_cast<T>(beta_s),
        nonuniform ? grid_enum::Nonuniform : grid_enum::Uniform);
    auto const solver_cfg = std::make_shared<heat_implicit_solver_config>(
        lss_enumerations::memory_space_enum::Device, lss_enumerations::traverse_direction_enum::Backward,
        method == "ds" ? lss_enumerations::tridiagonal_method_enum::GB300DoubleSweepSolver
                       : lss_enumerations::tridiagonal_method_enum::GB300ThomasLUSolver,
        lss_enumerations::factorization_enum::None, static_cast<lss_enumerations::implicit_pde_schemes_enum>(theta_scheme));

    container_2d<by_enum::Row, T> solution(Sd, Vd, T{});
    try {
        if (method == "euler") {
            lss_pde_solvers::two_dimensional::explicit_solvers::general_heston_equation<T> pdesolver(
                heat_data_ptr, discretization_ptr, vertical_upper_boundary_ptr, horizontal_boundary_pair,
                grid_config_hints_ptr, lss_pde_solvers::default_heat_solver_configs::dev_expl_bwd_euler_solver_config_ptr,
                arith);
            pdesolver.solve(solution);
        } else if (use_builder) {
            auto pdesolver = lss_pde_solvers::general_heston_equation_builder<T>()
                                 .heat_data_config(heat_data_ptr)
                                 .discretization_config(discretization_ptr)
                                 .vertical_upper_boundary(vertical_upper_boundary_ptr)
                                 .horizontal_boundary(horizontal_boundary_pair)
                                 .splitting_method_config(splitting_config_ptr)
                                 .grid_hints(grid_config_hints_ptr)
                                 .solver_config(solver_cfg)
                                 .build();
            pdesolver->solve(solution);
        } else {
            general_heston_equation<T> pdesolver(heat_data_ptr, discretization_ptr, vertical_upper_boundary_ptr,
                                                 horizontal_boundary_pair, splitting_config_ptr, grid_config_hints_ptr,
                                                 solver_cfg, {}, arith);
            pdesolver.solve(solution);
        }
    } catch (std::exception const &ex) {
        std::fprintf(stderr, "heston_front_end_t: %s\n", ex.what());
        return 3;
    }
    FILE *fo = std::fopen(out.c_str(), "wb");
    if (!fo) return 4;
    std::fwrite(solution.data(), sizeof(T), Sd * Vd, fo);
    std::fclose(fo);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc != 27 && argc != 28) {
        std::fprintf(stderr, "heston_front_end_t: expected 26 arguments, got %d\n", argc - 1);
        return 2;
    }
    return std::string(argv[1]) == "f32" ? run<float>(argc, argv) : run<double>(argc, argv);
}
