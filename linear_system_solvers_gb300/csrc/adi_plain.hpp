// adi_plain.hpp -- single-instance solver object behind lss_adi_handle.
#pragma once

#include "adi_common.hpp"
#include "adi_device.cuh"
#include "adi_tables.hpp"

namespace lss_gb300 {

template <typename T> struct plain_solver {
    instance_tables<T> tab_;
    int arith_ = LSS_ADI_ARITH_REFERENCE;
    dev_instance<T> d_{};
    dbuf<T> coef_, small_, state_, tdep_t_;
    dbuf<double> tdep_d_;
    dbuf<int> maps_;
    dbuf<double> value_;
    bilinear bil_{};
    cudaGraphExec_t graph_exec_ = nullptr;
    long long launches_ = 0, graph_launches_ = 0;

    plain_solver() = default;
    plain_solver(const plain_solver &) = delete;
    plain_solver &operator=(const plain_solver &) = delete;
    ~plain_solver();

    int init(instance_tables<T> &&tab, int arith, double eval_s, double eval_v);
    int forward(const void *payoff, void *out_surface, double *out_value, int flags, void *stream, bool use_graph);

    template <bool X> void enqueue_steps(cudaStream_t s, T *&U, T *&V);
};

} // namespace lss_gb300
