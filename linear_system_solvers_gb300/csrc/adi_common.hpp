// adi_common.hpp -- error reporting and CUDA helpers shared by the library's sources.
#pragma once

#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "lss_adi.h"

namespace lss_gb300 {

// Records the message for lss_adi_last_error() of the calling thread; returns `code`.
int set_error(int code, const std::string &msg);
void clear_error();

// Evaluates a CUDA runtime call; on failure records "<what>: <cuda message>" and returns
// LSS_ADI_ECUDA (LSS_ADI_ENOMEM for allocation failures) from the enclosing function.
#define LSS_CUDA_TRY(call, what)                                                                                     \
    do {                                                                                                             \
        cudaError_t lss_err_ = (call);                                                                               \
        if (lss_err_ != cudaSuccess) {                                                                               \
            return ::lss_gb300::set_error(lss_err_ == cudaErrorMemoryAllocation ? LSS_ADI_ENOMEM : LSS_ADI_ECUDA,   \
                                          std::string(what) + ": " + cudaGetErrorString(lss_err_));                  \
        }                                                                                                            \
    } while (0)

// Device buffer owned by a handle.
template <typename T> struct dbuf {
    T *p = nullptr;
    size_t n = 0;
    dbuf() = default;
    dbuf(const dbuf &) = delete;
    dbuf &operator=(const dbuf &) = delete;
    ~dbuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t alloc(size_t count)
    {
        release();
        n = count;
        if (count == 0) return cudaSuccess;
        return cudaMalloc(reinterpret_cast<void **>(&p), count * sizeof(T));
    }
    cudaError_t upload(const T *src, size_t count, cudaStream_t s = nullptr)
    {
        return cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, s);
    }
};

inline int grid_for(long long n, int block) { return static_cast<int>((n + block - 1) / block); }

// Bilinear weights of (s, v) on a tensor grid x[0..nx), y[0..ny) (host, double).
struct bilinear {
    int i0 = 0, j0 = 0;
    double w00 = 1, w10 = 0, w01 = 0, w11 = 0;
};
template <typename T> bilinear make_bilinear(const T *x, int nx, const T *y, int ny, double s, double v)
{
    auto locate = [](const T *g, int n, double q, int &k, double &w) {
        k = 0;
        while (k < n - 2 && static_cast<double>(g[k + 1]) <= q) ++k;
        const double g0 = static_cast<double>(g[k]), g1 = static_cast<double>(g[k + 1]);
        w = (q - g0) / (g1 - g0);
        if (w < 0.0) w = 0.0;
        if (w > 1.0) w = 1.0;
    };
    bilinear b;
    double wx, wy;
    locate(x, nx, s, b.i0, wx);
    locate(y, ny, v, b.j0, wy);
    b.w00 = (1.0 - wx) * (1.0 - wy);
    b.w10 = wx * (1.0 - wy);
    b.w01 = (1.0 - wx) * wy;
    b.w11 = wx * wy;
    return b;
}

} // namespace lss_gb300
