// lss_gb300_reference_kernel.hpp -- the GB300 device policy as one more kernel specialisation of
// the reference's own general_heston_equation_implicit_kernel
// (pde_solvers/two_dimensional/heat_type/lss_2d_general_heston_equation_implicit_kernel.hpp:209-1056),
// for the new value tridiagonal_method_enum::GB300ThomasLUSolver (common/lss_enumerations.hpp:46-52)
// with memory_space_enum::Device.
//
// This is the code a maintainer adds to the reference, together with the enumerator and one
// dispatch branch in general_heston_equation::solve
// (pde_solvers/two_dimensional/heat_type/lss_2d_general_heston_equation.hpp:221-252) that
// constructs this kernel like the Host ThomasLUSolver one and takes next_solution.  Include it
// after the reference's headers.  The builders, configs, boundaries, transforms and coefficient
// holder stay the reference's: the kernel samples the reference's transformed coefficient
// functions (general_heston_equation_coefficients, ...coefficients.hpp:89-98) and transformed
// boundaries at every step's time -- the running time of implicit_heston_time_loop::run
// (implicit_kernel.hpp:150-207) -- on the reference's computational grid, and hands the whole
// time loop to the device through the C-ABI (lss_adi_create_tabulated, include/lss_adi.h) in the
// reference's operation order, so the surface is the Host ThomasLUSolver's bit for bit.
#pragma once

#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>

#include "lss_adi.h"

namespace lss_pde_solvers
{
namespace two_dimensional
{

template <typename fp_type, template <typename, typename> typename container, typename allocator>
class general_heston_equation_implicit_kernel<memory_space_enum::Device, tridiagonal_method_enum::GB300ThomasLUSolver,
                                              fp_type, container, allocator>
{
    typedef container_2d<by_enum::Row, fp_type, container, allocator> rcontainer_2d_t;
    typedef container_3d<by_enum::Row, fp_type, container, allocator> rcontainer_3d_t;

  private:
    boundary_2d_ptr<fp_type> boundary_ver_;
    boundary_2d_pair<fp_type> boundary_pair_hor_;
    heat_data_transform_2d_ptr<fp_type> heat_data_cfg_;
    pde_discretization_config_2d_ptr<fp_type> discretization_cfg_;
    splitting_method_config_ptr<fp_type> splitting_cfg_;
    heat_implicit_solver_config_ptr solver_cfg_;
    grid_config_2d_ptr<fp_type> grid_cfg_;

    static int scheme_of(lss_enumerations::splitting_method_enum m)
    {
        switch (m) {
        case lss_enumerations::splitting_method_enum::DouglasRachford: return LSS_ADI_DOUGLAS_RACHFORD;
        case lss_enumerations::splitting_method_enum::CraigSneyd: return LSS_ADI_CRAIG_SNEYD;
        case lss_enumerations::splitting_method_enum::ModifiedCraigSneyd: return LSS_ADI_MODIFIED_CRAIG_SNEYD;
        case lss_enumerations::splitting_method_enum::HundsdorferVerwer: return LSS_ADI_HUNDSDORFER_VERWER;
        default: throw std::runtime_error("GB300ThomasLUSolver: unknown splitting method");
        }
    }

  public:
    general_heston_equation_implicit_kernel(boundary_2d_ptr<fp_type> const &vertical_upper_boundary_ptr,
                                            boundary_2d_pair<fp_type> const &horizontal_boundary_pair,
                                            heat_data_transform_2d_ptr<fp_type> const &heat_data_config,
                                            pde_discretization_config_2d_ptr<fp_type> const &discretization_config,
                                            splitting_method_config_ptr<fp_type> const &splitting_config,
                                            heat_implicit_solver_config_ptr const &solver_config,
                                            grid_config_2d_ptr<fp_type> const &grid_config)
        : boundary_ver_{vertical_upper_boundary_ptr}, boundary_pair_hor_{horizontal_boundary_pair},
          heat_data_cfg_{heat_data_config}, discretization_cfg_{discretization_config},
          splitting_cfg_{splitting_config}, solver_cfg_{solver_config}, grid_cfg_{grid_config}
    {
    }

    void operator()(rcontainer_2d_t &prev_solution, rcontainer_2d_t &next_solution, bool is_heat_sourse_set,
                    std::function<fp_type(fp_type, fp_type, fp_type)> const &heat_source)
    {
        (void)heat_source;
        // the reference's 2-D heat-source branch does nothing (implicit_kernel.hpp:1028-1039)
        if (is_heat_sourse_set) return;
        const range<fp_type> time = discretization_cfg_->time_range();
        const fp_type k = discretization_cfg_->time_step();
        const auto &sizes = discretization_cfg_->number_of_space_points();
        const std::size_t nx = std::get<0>(sizes), ny = std::get<1>(sizes), n = nx * ny;
        const std::size_t steps = discretization_cfg_->number_of_time_points() - 1;
        const bool fwd = solver_cfg_->traverse_direction() == traverse_direction_enum::Forward;
        int theta_scheme = LSS_ADI_CRANK_NICOLSON;
        fp_type theta = static_cast<fp_type>(0.5);
        switch (solver_cfg_->implicit_pde_scheme()) { // the theta of the Host kernels (implicit_kernel.hpp:978-995)
        case implicit_pde_schemes_enum::Euler:
            theta = static_cast<fp_type>(1.0);
            theta_scheme = LSS_ADI_EULER;
            break;
        case implicit_pde_schemes_enum::Theta_30:
            theta = static_cast<fp_type>(0.3);
            theta_scheme = LSS_ADI_THETA_30;
            break;
        case implicit_pde_schemes_enum::Theta_80:
            theta = static_cast<fp_type>(0.8);
            theta_scheme = LSS_ADI_THETA_80;
            break;
        default:
            break;
        }
        auto const cf =
            std::make_shared<general_heston_equation_coefficients<fp_type>>(heat_data_cfg_, discretization_cfg_,
                                                                            splitting_cfg_, theta);
        std::vector<fp_type> zeta(nx), eta(ny);
        for (std::size_t i = 0; i < nx; ++i) zeta[i] = grid_cfg_->value_for_1(i);
        for (std::size_t j = 0; j < ny; ++j) eta[j] = grid_cfg_->value_for_2(j);
        // one step's tables: M, P, Z, M~, P~, W, C on the grid; D, E, F on the v = v_lo line;
        // the transformed boundary values
        auto sample = [&](fp_type t, std::vector<fp_type> &c, std::vector<fp_type> &v0, std::vector<fp_type> &slo,
                          std::vector<fp_type> &shi, std::vector<fp_type> &vhi) {
            c.resize(7 * n);
            v0.resize(3 * nx);
            slo.resize(ny);
            shi.resize(ny);
            vhi.resize(nx);
            for (std::size_t i = 0; i < nx; ++i)
                for (std::size_t j = 0; j < ny; ++j) {
                    const std::size_t o = i * ny + j;
                    const fp_type x = zeta[i], y = eta[j];
                    c[o] = cf->M_(t, x, y);
                    c[n + o] = cf->P_(t, x, y);
                    c[2 * n + o] = cf->Z_(t, x, y);
                    c[3 * n + o] = cf->M_tilde_(t, x, y);
                    c[4 * n + o] = cf->P_tilde_(t, x, y);
                    c[5 * n + o] = cf->W_(t, x, y);
                    c[6 * n + o] = cf->C_(t, x, y);
                }
            for (std::size_t i = 0; i < nx; ++i) {
                v0[i] = cf->D_(t, zeta[i], eta[0]);
                v0[nx + i] = cf->E_(t, zeta[i], eta[0]);
                v0[2 * nx + i] = cf->F_(t, zeta[i], eta[0]);
                vhi[i] = boundary_ver_->value(t, zeta[i]);
            }
            for (std::size_t j = 0; j < ny; ++j) {
                slo[j] = boundary_pair_hor_.first->value(t, eta[j]);
                shi[j] = boundary_pair_hor_.second->value(t, eta[j]);
            }
        };
        // every step's tables, one block while they all equal the first step's
        fp_type ts = fwd ? time.lower() + k : time.upper() - k;
        std::vector<fp_type> coef, v0, slo, shi, vhi;
        sample(ts, coef, v0, slo, shi, vhi);
        const std::vector<fp_type> c1 = coef, w1 = v0, s1 = slo, h1 = shi, u1 = vhi;
        std::vector<fp_type> c2, w2, s2, h2, u2;
        bool varies = false;
        for (std::size_t st = 1; st < steps; ++st) {
            ts = fwd ? ts + k : ts - k;
            sample(ts, c2, w2, s2, h2, u2);
            if (!varies && (c2 != c1 || w2 != w1 || s2 != s1 || h2 != h1 || u2 != u1)) {
                varies = true;
                for (std::size_t b = 1; b < st; ++b) {
                    coef.insert(coef.end(), c1.begin(), c1.end());
                    v0.insert(v0.end(), w1.begin(), w1.end());
                    slo.insert(slo.end(), s1.begin(), s1.end());
                    shi.insert(shi.end(), h1.begin(), h1.end());
                    vhi.insert(vhi.end(), u1.begin(), u1.end());
                }
            }
            if (varies) {
                coef.insert(coef.end(), c2.begin(), c2.end());
                v0.insert(v0.end(), w2.begin(), w2.end());
                slo.insert(slo.end(), s2.begin(), s2.end());
                shi.insert(shi.end(), h2.begin(), h2.end());
                vhi.insert(vhi.end(), u2.begin(), u2.end());
            }
        }
        std::vector<fp_type> pay(n), out(n);
        for (std::size_t i = 0; i < nx; ++i)
            for (std::size_t j = 0; j < ny; ++j) pay[i * ny + j] = prev_solution(i, j);
        lss_adi_tables tb{};
        tb.nx = static_cast<int>(nx);
        tb.ny = static_cast<int>(ny);
        tb.nt = static_cast<int>(steps + 1);
        tb.t_lo = static_cast<double>(time.lower());
        tb.t_hi = static_cast<double>(time.upper());
        tb.scheme = scheme_of(splitting_cfg_->splitting_method());
        tb.theta_scheme = theta_scheme;
        tb.forward = fwd ? 1 : 0;
        tb.precision = std::is_same<fp_type, double>::value ? LSS_ADI_FP64 : LSS_ADI_FP32;
        tb.arith = LSS_ADI_ARITH_REFERENCE;
        tb.zeta = static_cast<double>(splitting_cfg_->weighting_value());
        tb.coef = coef.data();
        tb.coef_v0 = v0.data();
        tb.s_lo_dirichlet = slo.data();
        tb.s_hi_neumann = shi.data();
        tb.v_hi_dirichlet = vhi.data();
        tb.payoff = pay.data();
        tb.options = varies ? LSS_ADI_OPT_STEP_TABLES : 0;
        lss_adi_handle *h = nullptr;
        if (lss_adi_create_tabulated(&tb, &h) != LSS_ADI_OK) throw std::runtime_error(lss_adi_last_error());
        const int rc = lss_adi_forward(h, nullptr, out.data(), nullptr, 0, nullptr);
        lss_adi_destroy(h);
        if (rc != LSS_ADI_OK) throw std::runtime_error(lss_adi_last_error());
        for (std::size_t i = 0; i < nx; ++i)
            for (std::size_t j = 0; j < ny; ++j) {
                next_solution(i, j, out[i * ny + j]);
                prev_solution(i, j, out[i * ny + j]);
            }
    }

    void operator()(rcontainer_2d_t &prev_solution, rcontainer_2d_t &next_solution, bool is_heat_sourse_set,
                    std::function<fp_type(fp_type, fp_type, fp_type)> const &heat_source, rcontainer_3d_t &solutions)
    {
        (void)prev_solution;
        (void)next_solution;
        (void)is_heat_sourse_set;
        (void)heat_source;
        (void)solutions;
        throw std::runtime_error("GB300ThomasLUSolver: the per-step surfaces are not recorded");
    }
};

} // namespace two_dimensional
} // namespace lss_pde_solvers
