// ref_driver_1d.cu -- runs the UNMODIFIED reference 1-D implicit heat solver
// (MichalSara99/linear_system_solvers, implicit_solvers::general_heat_equation with the host
// Thomas-LU / double-sweep policies) on one problem given on the command line and writes the
// final solution (or every time level) as raw binary.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.sh into oracle/_ref/ from the same
// build-time copy of the reference sources as ref_driver.  It pins the C restatement in
// oracle/lss_oracle_1d_impl.h and serves as the reference CPU baseline of the 1-D path.  The
// problems are set up like the reference's tests (unit_tests/pde_solvers/one_dimensional/
// lss_black_scholes_equation_t.hpp:823-910, lss_pure_heat_equation_t.hpp:1028-1120,2053-2160,
// lss_advection_equation_t.hpp:1211-1300).
//
// usage: ref_driver_1d <f32|f64> <bs|const> <tlu|ds> n nt sigma rate strike put diff conv react
//        init0 init1 lo_kind hi_kind lo_value lo_linear hi_value hi_linear has_source src0 src1
//        x_lo x_hi t_lo t_hi theta_scheme(0|2) nonuniform acc_point alpha_scale forward all
//        repeat out.bin
#include <cmath>
#include <stdexcept>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pde_solvers/one_dimensional/heat_type/lss_1d_general_heat_equation.hpp"

using namespace lss_pde_solvers;
using lss_boundary::boundary_1d_ptr;
using lss_boundary::dirichlet_boundary_1d;
using lss_boundary::neumann_boundary_1d;
using lss_boundary::robin_boundary_1d;
using lss_containers::container_2d;
using lss_enumerations::by_enum;
using lss_enumerations::factorization_enum;
using lss_enumerations::grid_enum;
using lss_enumerations::implicit_pde_schemes_enum;
using lss_enumerations::memory_space_enum;
using lss_enumerations::traverse_direction_enum;
using lss_enumerations::tridiagonal_method_enum;
using lss_grids::grid_config_hints_1d;
using lss_utility::range;

struct args_t {
    std::string fp, model, solver;
    std::size_t n, nt;
    double sigma, rate, strike;
    int put;
    double diff, conv, react, init0, init1;
    int lo_kind, hi_kind;
    double lo_value, lo_linear, hi_value, hi_linear;
    int has_source;
    double src0, src1, x_lo, x_hi, t_lo, t_hi;
    int theta_scheme, nonuniform;
    double acc, alpha_scale;
    int forward, all, repeat;
    std::string out;
};

template <typename T> static boundary_1d_ptr<T> make_boundary(int kind, double value, double linear)
{
    auto const v = [=](T t) { return value; };
    if (kind == 1) return std::make_shared<neumann_boundary_1d<T>>(v);
    if (kind == 2) {
        auto const l = [=](T t) { return linear; };
        return std::make_shared<robin_boundary_1d<T>>(l, v);
    }
    return std::make_shared<dirichlet_boundary_1d<T>>(v);
}

template <typename T> static int run(const args_t &a)
{
    typedef one_dimensional::implicit_solvers::general_heat_equation<T, std::vector, std::allocator<T>> pde_solver;
    typedef container_2d<by_enum::Row, T, std::vector, std::allocator<T>> rcontainer_2d_t;

    const double sig = a.sigma, rate = a.rate, strike = a.strike, maturity = a.t_hi, x_hi = a.x_hi;
    const double diff = a.diff, conv = a.conv, react = a.react, init0 = a.init0, init1 = a.init1;
    const double src0 = a.src0, src1 = a.src1;
    const bool bs = a.model == "bs";
    const int put = a.put;

    range<T> space_range(static_cast<T>(a.x_lo), static_cast<T>(a.x_hi));
    range<T> time_range(static_cast<T>(a.t_lo), static_cast<T>(a.t_hi));
    auto const discretization_ptr = std::make_shared<pde_discretization_config_1d<T>>(space_range, a.n, time_range, a.nt);

    std::shared_ptr<heat_coefficient_data_config_1d<T>> coeffs;
    std::shared_ptr<heat_initial_data_config_1d<T>> init;
    boundary_1d_ptr<T> lo, hi;
    if (bs) {
        auto ca = [=](T t, T x) { return 0.5 * sig * sig * x * x; };
        auto cb = [=](T t, T x) { return rate * x; };
        auto cc = [=](T t, T x) { return -rate; };
        coeffs = std::make_shared<heat_coefficient_data_config_1d<T>>(ca, cb, cc);
        auto terminal = [=](T x) { return put ? std::max<T>(0.0, strike - x) : std::max<T>(0.0, x - strike); };
        init = std::make_shared<heat_initial_data_config_1d<T>>(terminal);
        auto const disc = [=](T t) { return strike * std::exp(-rate * (maturity - t)); };
        auto const low = [=](T t) { return put ? disc(t) : 0.0; };
        auto const high = [=](T t) { return put ? 0.0 : (x_hi - strike * std::exp(-rate * (maturity - t))); };
        lo = std::make_shared<dirichlet_boundary_1d<T>>(low);
        hi = std::make_shared<dirichlet_boundary_1d<T>>(high);
    } else {
        auto ca = [=](T t, T x) { return diff; };
        auto cb = [=](T t, T x) { return conv; };
        auto cc = [=](T t, T x) { return react; };
        coeffs = std::make_shared<heat_coefficient_data_config_1d<T>>(ca, cb, cc);
        auto initial = [=](T x) { return init0 + init1 * x; };
        init = std::make_shared<heat_initial_data_config_1d<T>>(initial);
        lo = make_boundary<T>(a.lo_kind, a.lo_value, a.lo_linear);
        hi = make_boundary<T>(a.hi_kind, a.hi_value, a.hi_linear);
    }
    std::shared_ptr<heat_data_config_1d<T>> heat_data_ptr;
    if (a.has_source) {
        auto source = [=](T t, T x) { return src0 + src1 * x; };
        auto const src_ptr = std::make_shared<heat_source_data_config_1d<T>>(source);
        heat_data_ptr = std::make_shared<heat_data_config_1d<T>>(coeffs, init, src_ptr);
    } else {
        heat_data_ptr = std::make_shared<heat_data_config_1d<T>>(coeffs, init);
    }
    auto const boundary_pair = std::make_pair(lo, hi);
    auto const grid_config_hints_ptr = std::make_shared<grid_config_hints_1d<T>>(
        static_cast<T>(a.acc), static_cast<T>(a.alpha_scale), a.nonuniform ? grid_enum::Nonuniform : grid_enum::Uniform);
    auto const solver_cfg = std::make_shared<heat_implicit_solver_config>(
        memory_space_enum::Host, a.forward ? traverse_direction_enum::Forward : traverse_direction_enum::Backward,
        a.solver == "ds" ? tridiagonal_method_enum::DoubleSweepSolver : tridiagonal_method_enum::ThomasLUSolver,
        factorization_enum::None,
        a.theta_scheme == 0 ? implicit_pde_schemes_enum::Euler : implicit_pde_schemes_enum::CrankNicolson);

    std::vector<T> flat;
    double secs = 0.0;
    for (int r = 0; r < a.repeat; ++r) {
        auto t0 = std::chrono::steady_clock::now();
        pde_solver pdesolver(heat_data_ptr, discretization_ptr, boundary_pair, grid_config_hints_ptr, solver_cfg);
        if (a.all) {
            rcontainer_2d_t solutions(a.nt, a.n);
            pdesolver.solve(solutions);
            flat.assign(a.nt * a.n, T{});
            for (std::size_t t = 0; t < a.nt; ++t)
                for (std::size_t i = 0; i < a.n; ++i) flat[t * a.n + i] = solutions(t, i);
        } else {
            std::vector<T> solution(a.n, T{});
            pdesolver.solve(solution);
            flat = solution;
        }
        secs += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    FILE *f = std::fopen(a.out.c_str(), "wb");
    if (!f) return 3;
    std::fwrite(flat.data(), sizeof(T), flat.size(), f);
    std::fclose(f);
    std::printf("{\"seconds\": %.9f, \"repeat\": %d}\n", secs, a.repeat);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc != 36) {
        std::fprintf(stderr, "ref_driver_1d: expected 35 arguments, got %d\n", argc - 1);
        return 2;
    }
    args_t a;
    int k = 1;
    a.fp = argv[k++]; a.model = argv[k++]; a.solver = argv[k++];
    a.n = std::strtoul(argv[k++], nullptr, 10);
    a.nt = std::strtoul(argv[k++], nullptr, 10);
    a.sigma = std::atof(argv[k++]); a.rate = std::atof(argv[k++]); a.strike = std::atof(argv[k++]);
    a.put = std::atoi(argv[k++]);
    a.diff = std::atof(argv[k++]); a.conv = std::atof(argv[k++]); a.react = std::atof(argv[k++]);
    a.init0 = std::atof(argv[k++]); a.init1 = std::atof(argv[k++]);
    a.lo_kind = std::atoi(argv[k++]); a.hi_kind = std::atoi(argv[k++]);
    a.lo_value = std::atof(argv[k++]); a.lo_linear = std::atof(argv[k++]);
    a.hi_value = std::atof(argv[k++]); a.hi_linear = std::atof(argv[k++]);
    a.has_source = std::atoi(argv[k++]);
    a.src0 = std::atof(argv[k++]); a.src1 = std::atof(argv[k++]);
    a.x_lo = std::atof(argv[k++]); a.x_hi = std::atof(argv[k++]);
    a.t_lo = std::atof(argv[k++]); a.t_hi = std::atof(argv[k++]);
    a.theta_scheme = std::atoi(argv[k++]); a.nonuniform = std::atoi(argv[k++]);
    a.acc = std::atof(argv[k++]); a.alpha_scale = std::atof(argv[k++]);
    a.forward = std::atoi(argv[k++]); a.all = std::atoi(argv[k++]); a.repeat = std::atoi(argv[k++]);
    a.out = argv[k++];
    try {
        return a.fp == "f32" ? run<float>(a) : run<double>(a);
    } catch (std::exception const &e) {
        std::fprintf(stderr, "ref_driver_1d: %s\n", e.what());
        return 4;
    }
}
