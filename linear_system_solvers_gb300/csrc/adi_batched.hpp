// adi_batched.hpp -- batched persistent-kernel solver and the adjoint solver.
#pragma once

#include <memory>
#include <vector>

#include "adi_common.hpp"
#include "adi_device.cuh"
#include "adi_tables.hpp"

namespace lss_gb300 {

struct batch_impl;   // defined in adi_batched.cu
struct adjoint_impl; // defined in adi_adjoint.cu

// Forward + adjoint of one parametric FP64 Heston problem (behind lss_adi_adjoint).
struct adjoint_solver {
    std::unique_ptr<adjoint_impl> impl;
    adjoint_solver();
    ~adjoint_solver();
    int init(const lss_adi_problem &p);
    int run(const void *payoff, double *out_value, double *dv_dparams, void *dv_dpayoff, int checkpoint_every, int flags,
            void *stream);
    // chunk counts and lines per CTA of the partitioned solves of a large instance (0 lines: by
    // SM count; no effect on one-CTA instances)
    int set_chunks(int s_chunks, int v_chunks, int s_lines, int v_lines, void *stream);
};

// Single instance on the factorised ("fast") arithmetic: one kernel per stage over the whole
// GPU, graph-replayed time loop (behind lss_adi_create with LSS_ADI_ARITH_FAST).
struct wide_solver_base {
    virtual ~wide_solver_base() = default;
    virtual int forward(const void *payoff, void *out_surface, double *out_value, int flags, void *stream,
                        bool use_graph) = 0;
    virtual int grid(void *x, void *y) const = 0;
    virtual int chunks(int s_chunks, int v_chunks, int *out_s, int *out_v, void *stream) = 0;
    virtual void current_chunks(int &s_chunks, int &v_chunks, int &s_lines, int &v_lines) const = 0;
};
int make_wide_solver(const lss_adi_problem &p, std::unique_ptr<wide_solver_base> &out);

} // namespace lss_gb300
