// ref_driver.cu -- runs the UNMODIFIED reference 2-D Heston/SABR implicit solver
// (MichalSara99/linear_system_solvers, host Thomas-LU / double-sweep policies) on one
// problem given on the command line and writes the final surface as raw binary.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.sh into oracle/_ref/ from a
// build-time copy of the reference sources (4 mechanical portability patches, see the
// script).  It pins the C restatement in oracle/lss_oracle.c and serves as the
// reference CPU baseline.  The problem is set up exactly like the reference's tests
// (unit_tests/common/lss_print_t.hpp:1850-1974 Heston, :1976-2102 SABR).
//
// usage: ref_driver <f32|f64> <heston|sabr> <dr|cs|mcs|hv|euler> <tlu|ds> nx ny nt
//        kappa theta_v sigma rho rate sabr_beta strike maturity s_lo s_hi v_lo v_hi
//        zeta theta_scheme(0..3) nonuniform acc_point alpha_scale beta_scale neumann
//        forward(0|1) repeat out.bin
#include <cmath>
#include <stdexcept>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pde_solvers/two_dimensional/heat_type/lss_2d_general_heston_equation.hpp"

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

struct args_t {
    std::string fp, model, scheme, solver;
    std::size_t nx, ny, nt;
    double kappa, theta_v, sigma, rho, rate, sabr_beta, strike, maturity;
    double s_lo, s_hi, v_lo, v_hi, zeta;
    int theta_scheme, nonuniform;
    double acc, alpha_scale, beta_scale, neumann;
    int forward, repeat;
    std::string out;
};

template <typename T> static int run(const args_t &a)
{
    typedef container_2d<by_enum::Row, T, std::vector, std::allocator<T>> rcontainer_2d_t;
    typedef two_dimensional::implicit_solvers::general_heston_equation<T, std::vector, std::allocator<T>> pde_solver;

    const double strike = a.strike, maturity = a.maturity, rate = a.rate, sig_sig = a.sigma;
    const double sig_kappa = a.kappa, sig_theta = a.theta_v, rho = a.rho, beta = a.sabr_beta;
    const double neu = a.neumann;

    range<T> spacex_range(static_cast<T>(a.s_lo), static_cast<T>(a.s_hi));
    range<T> spacey_range(static_cast<T>(a.v_lo), static_cast<T>(a.v_hi));
    range<T> time_range(static_cast<T>(0.0), static_cast<T>(maturity));
    auto const discretization_ptr =
        std::make_shared<pde_discretization_config_2d<T>>(spacex_range, spacey_range, a.nx, a.ny, time_range, a.nt);

    std::shared_ptr<heat_coefficient_data_config_2d<T>> coeffs;
    if (a.model == "sabr") {
        auto D = [=](T t, T s, T alpha) { return std::exp(-rate * (maturity - t)); };
        auto ca = [=](T t, T s, T alpha) {
            return (0.5 * alpha * alpha * std::pow(s, 2.0 * beta) * std::pow(D(t, s, alpha), 2.0 * (1.0 - beta)));
        };
        auto cb = [=](T t, T s, T alpha) { return (0.5 * sig_sig * sig_sig * alpha * alpha); };
        auto cc = [=](T t, T s, T alpha) {
            return (rho * sig_sig * alpha * alpha * std::pow(s, beta) * std::pow(D(t, s, alpha), (1.0 - beta)));
        };
        auto cd = [=](T t, T s, T alpha) { return (rate * s); };
        auto ce = [=](T t, T s, T alpha) { return 0.0; };
        auto cf = [=](T t, T s, T alpha) { return (-rate); };
        coeffs = std::make_shared<heat_coefficient_data_config_2d<T>>(ca, cb, cc, cd, ce, cf);
    } else {
        auto ca = [=](T t, T s, T v) { return (0.5 * v * s * s); };
        auto cb = [=](T t, T s, T v) { return (0.5 * sig_sig * sig_sig * v); };
        auto cc = [=](T t, T s, T v) { return (rho * sig_sig * v * s); };
        auto cd = [=](T t, T s, T v) { return (rate * s); };
        auto ce = [=](T t, T s, T v) { return (sig_kappa * (sig_theta - v)); };
        auto cf = [=](T t, T s, T v) { return (-rate); };
        coeffs = std::make_shared<heat_coefficient_data_config_2d<T>>(ca, cb, cc, cd, ce, cf);
    }
    auto terminal_condition = [=](T s, T v) { return std::max<T>(0.0, s - strike); };
    auto const heat_init_data_ptr = std::make_shared<heat_initial_data_config_2d<T>>(terminal_condition);
    auto const heat_data_ptr = std::make_shared<heat_data_config_2d<T>>(coeffs, heat_init_data_ptr);
    auto const &dirichlet_low = [=](T t, T v) { return 0.0; };
    auto const &neumann_high = [=](T t, T s) { return neu; };
    auto const &boundary_low_ptr = std::make_shared<dirichlet_boundary_2d<T>>(dirichlet_low);
    auto const &boundary_high_ptr = std::make_shared<neumann_boundary_2d<T>>(neumann_high);
    auto const &horizontal_boundary_pair = std::make_pair(boundary_low_ptr, boundary_high_ptr);
    auto const &dirichlet_high = [=](T t, T s) { return s; };
    auto const &vertical_upper_boundary_ptr = std::make_shared<dirichlet_boundary_2d<T>>(dirichlet_high);

    splitting_method_enum sm = splitting_method_enum::DouglasRachford;
    if (a.scheme == "cs") sm = splitting_method_enum::CraigSneyd;
    else if (a.scheme == "mcs") sm = splitting_method_enum::ModifiedCraigSneyd;
    else if (a.scheme == "hv") sm = splitting_method_enum::HundsdorferVerwer;
    auto const &splitting_config_ptr = std::make_shared<splitting_method_config<T>>(sm, static_cast<T>(a.zeta));

    auto const &grid_config_hints_ptr = std::make_shared<grid_config_hints_2d<T>>(
        static_cast<T>(a.acc), static_cast<T>(a.alpha_scale), static_cast<T>(a.beta_scale),
        a.nonuniform ? grid_enum::Nonuniform : grid_enum::Uniform);

    const implicit_pde_schemes_enum schemes[4] = {implicit_pde_schemes_enum::Euler, implicit_pde_schemes_enum::Theta_30,
                                                  implicit_pde_schemes_enum::CrankNicolson,
                                                  implicit_pde_schemes_enum::Theta_80};
    auto const solver_cfg = std::make_shared<heat_implicit_solver_config>(
        memory_space_enum::Host, a.forward ? traverse_direction_enum::Forward : traverse_direction_enum::Backward,
        a.solver == "ds" ? tridiagonal_method_enum::DoubleSweepSolver : tridiagonal_method_enum::ThomasLUSolver,
        factorization_enum::None, schemes[a.theta_scheme]);

    rcontainer_2d_t solution(a.nx, a.ny, T{});
    double secs = 0.0;
    for (int r = 0; r < a.repeat; ++r) {
        auto t0 = std::chrono::steady_clock::now();
        if (a.scheme == "euler") {
            // explicit_solvers::general_heston_equation with the host explicit Euler scheme
            typedef two_dimensional::explicit_solvers::general_heston_equation<T, std::vector, std::allocator<T>> expl_solver;
            auto const expl_cfg = std::make_shared<heat_explicit_solver_config>(
                memory_space_enum::Host, a.forward ? traverse_direction_enum::Forward : traverse_direction_enum::Backward,
                lss_enumerations::explicit_pde_schemes_enum::Euler);
            expl_solver pdesolver(heat_data_ptr, discretization_ptr, vertical_upper_boundary_ptr, horizontal_boundary_pair,
                                  grid_config_hints_ptr, expl_cfg);
            pdesolver.solve(solution);
        } else {
            pde_solver pdesolver(heat_data_ptr, discretization_ptr, vertical_upper_boundary_ptr, horizontal_boundary_pair,
                                 splitting_config_ptr, grid_config_hints_ptr, solver_cfg);
            pdesolver.solve(solution);
        }
        secs += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    std::vector<T> flat(a.nx * a.ny);
    for (std::size_t i = 0; i < a.nx; ++i)
        for (std::size_t j = 0; j < a.ny; ++j) flat[i * a.ny + j] = solution(i, j);
    FILE *f = std::fopen(a.out.c_str(), "wb");
    if (!f) return 3;
    std::fwrite(flat.data(), sizeof(T), flat.size(), f);
    std::fclose(f);
    std::printf("{\"seconds\": %.9f, \"repeat\": %d}\n", secs, a.repeat);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc != 30) {
        std::fprintf(stderr, "ref_driver: expected 29 arguments, got %d\n", argc - 1);
        return 2;
    }
    args_t a;
    int k = 1;
    a.fp = argv[k++]; a.model = argv[k++]; a.scheme = argv[k++]; a.solver = argv[k++];
    a.nx = std::strtoul(argv[k++], nullptr, 10);
    a.ny = std::strtoul(argv[k++], nullptr, 10);
    a.nt = std::strtoul(argv[k++], nullptr, 10);
    a.kappa = std::atof(argv[k++]); a.theta_v = std::atof(argv[k++]); a.sigma = std::atof(argv[k++]);
    a.rho = std::atof(argv[k++]); a.rate = std::atof(argv[k++]); a.sabr_beta = std::atof(argv[k++]);
    a.strike = std::atof(argv[k++]); a.maturity = std::atof(argv[k++]);
    a.s_lo = std::atof(argv[k++]); a.s_hi = std::atof(argv[k++]);
    a.v_lo = std::atof(argv[k++]); a.v_hi = std::atof(argv[k++]);
    a.zeta = std::atof(argv[k++]);
    a.theta_scheme = std::atoi(argv[k++]); a.nonuniform = std::atoi(argv[k++]);
    a.acc = std::atof(argv[k++]); a.alpha_scale = std::atof(argv[k++]); a.beta_scale = std::atof(argv[k++]);
    a.neumann = std::atof(argv[k++]);
    a.forward = std::atoi(argv[k++]); a.repeat = std::atoi(argv[k++]);
    a.out = argv[k++];
    try {
        return a.fp == "f32" ? run<float>(a) : run<double>(a);
    } catch (std::exception const &e) {
        std::fprintf(stderr, "ref_driver: %s\n", e.what());
        return 4;
    }
}
