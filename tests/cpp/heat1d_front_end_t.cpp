// heat1d_front_end_t.cpp -- the reference's 1-D implicit tests written against the C++ front end
// (linear_system_solvers_gb300/cpp/lss_gb300_heat1d.hpp) with the device policy.  Same set-up as
// unit_tests/pde_solvers/one_dimensional/lss_black_scholes_equation_t.hpp:823-910 (Black-Scholes
// call, Dirichlet ends) and lss_pure_heat_equation_t.hpp:1422-1520, :2053-2160 (pure heat with
// Neumann / Robin ends and a heat source), with the parameters taken from the command line;
// writes the final values or every time level (raw).
//
// usage: heat1d_front_end_t <f32|f64> <bs|heat> n nt theta(euler|cn) fwd(0|1) nonuniform acc
//        alpha_s arith(0 fast|1 reference) method(tlu|ds) all(0|1) out.bin
// bs: sigma 0.25, r 0.2, K 10, T 1 on [0, 20]; heat: a = 1, b = -0.5, c = -0.25 on [0, 1] x
// [0, 0.1], initial 0.3 + x, Neumann 0.2 at x = 0, Robin u' = 0.4 u - 0.1 at x = 1, source x.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "lss_gb300_heat1d.hpp"

using namespace lss_gb300;
using lss_boundary::dirichlet_boundary_1d;
using lss_boundary::neumann_boundary_1d;
using lss_boundary::robin_boundary_1d;
using lss_containers::container_2d;
using lss_enumerations::by_enum;
using lss_enumerations::grid_enum;
using lss_grids::grid_config_hints_1d;
using lss_pde_solvers::heat_coefficient_data_config_1d;
using lss_pde_solvers::heat_data_config_1d;
using lss_pde_solvers::heat_implicit_solver_config;
using lss_pde_solvers::heat_initial_data_config_1d;
using lss_pde_solvers::heat_source_data_config_1d;
using lss_pde_solvers::pde_discretization_config_1d;
using lss_pde_solvers::one_dimensional::implicit_solvers::general_heat_equation;
using lss_utility::range;

template <typename T> static int run(char **argv)
{
    int k = 2;
    const std::string model = argv[k++];
    const std::size_t Sd = std::strtoul(argv[k++], nullptr, 10), Td = std::strtoul(argv[k++], nullptr, 10);
    const std::string theta = argv[k++];
    const int fwd = std::atoi(argv[k++]), nonuniform = std::atoi(argv[k++]);
    const double acc = std::atof(argv[k++]), alpha_s = std::atof(argv[k++]);
    const int arith = std::atoi(argv[k++]);
    const std::string method = argv[k++];
    const int all = std::atoi(argv[k++]);
    const std::string out = argv[k++];

    std::shared_ptr<pde_discretization_config_1d<T>> disc;
    std::shared_ptr<heat_data_config_1d<T>> data;
    lss_boundary::boundary_1d_pair<T> bnd;
    if (model == "bs") {
        auto const &strike = 10;
        auto const &maturity = 1.0;
        auto const &rate = 0.2;
        auto const &sig = 0.25;
        disc = std::make_shared<pde_discretization_config_1d<T>>(range<T>(T(0.0), T(20.0)), Sd,
                                                                 range<T>(T(0.0), T(maturity)), Td);
        auto a = [=](T t, T x) { return 0.5 * sig * sig * x * x; };
        auto b = [=](T t, T x) { return rate * x; };
        auto c = [=](T t, T x) { return -rate; };
        auto coeffs = std::make_shared<heat_coefficient_data_config_1d<T>>(a, b, c);
        auto terminal = [=](T x) { return std::max<T>(0.0, x - strike); };
        data = std::make_shared<heat_data_config_1d<T>>(coeffs, std::make_shared<heat_initial_data_config_1d<T>>(terminal));
        auto const &low = [=](T t) { return 0.0; };
        auto const &high = [=](T t) { return (20.0 - strike * std::exp(-rate * (maturity - t))); };
        bnd = std::make_pair(std::make_shared<dirichlet_boundary_1d<T>>(low), std::make_shared<dirichlet_boundary_1d<T>>(high));
    } else {
        disc = std::make_shared<pde_discretization_config_1d<T>>(range<T>(T(0.0), T(1.0)), Sd, range<T>(T(0.0), T(0.1)), Td);
        auto a = [](T t, T x) { return 1.0; };
        auto b = [](T t, T x) { return -0.5; };
        auto c = [](T t, T x) { return -0.25; };
        auto coeffs = std::make_shared<heat_coefficient_data_config_1d<T>>(a, b, c);
        auto initial = [](T x) { return 0.3 + 1.0 * x; };
        auto source = [](T t, T x) { return 0.0 + 1.0 * x; };
        data = std::make_shared<heat_data_config_1d<T>>(coeffs, std::make_shared<heat_initial_data_config_1d<T>>(initial),
                                                        std::make_shared<heat_source_data_config_1d<T>>(source));
        auto const &neu = [](T t) { return 0.2; };
        auto const &rlin = [](T t) { return 0.4; };
        auto const &rval = [](T t) { return -0.1; };
        bnd = std::make_pair(std::make_shared<neumann_boundary_1d<T>>(neu), std::make_shared<robin_boundary_1d<T>>(rlin, rval));
    }
    auto hints = std::make_shared<grid_config_hints_1d<T>>(T(acc), T(alpha_s), nonuniform ? grid_enum::Nonuniform : grid_enum::Uniform);
    auto cfg = std::make_shared<heat_implicit_solver_config>(
        lss_enumerations::memory_space_enum::Device,
        fwd ? lss_enumerations::traverse_direction_enum::Forward : lss_enumerations::traverse_direction_enum::Backward,
        method == "ds" ? lss_enumerations::tridiagonal_method_enum::GB300DoubleSweepSolver
                       : lss_enumerations::tridiagonal_method_enum::GB300ThomasLUSolver,
        lss_enumerations::factorization_enum::None,
        theta == "euler" ? lss_enumerations::implicit_pde_schemes_enum::Euler
                         : lss_enumerations::implicit_pde_schemes_enum::CrankNicolson);
    std::vector<T> flat;
    try {
        general_heat_equation<T> pdesolver(data, disc, bnd, hints, cfg, {}, arith);
        if (all) {
            container_2d<by_enum::Row, T> solutions(Td, Sd);
            pdesolver.solve(solutions);
            flat.assign(solutions.data(), solutions.data() + Td * Sd);
        } else {
            std::vector<T> solution(Sd, T{});
            pdesolver.solve(solution);
            flat = solution;
        }
    } catch (std::exception const &ex) {
        std::fprintf(stderr, "heat1d_front_end_t: %s\n", ex.what());
        return 3;
    }
    FILE *fo = std::fopen(out.c_str(), "wb");
    if (!fo) return 4;
    std::fwrite(flat.data(), sizeof(T), flat.size(), fo);
    std::fclose(fo);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc != 14) {
        std::fprintf(stderr, "heat1d_front_end_t: expected 13 arguments, got %d\n", argc - 1);
        return 2;
    }
    return std::string(argv[1]) == "f32" ? run<float>(argv) : run<double>(argv);
}
