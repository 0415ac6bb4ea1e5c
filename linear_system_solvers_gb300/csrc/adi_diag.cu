// adi_diag.cu -- measured denominators of the FP64 roofline.
//
// The batched ADI kernels run out of FP64 issue slots before HBM bandwidth on GB300, so their
// roofline is the FP64 pipe.  lss_diag_fp64_rate measures that pipe's rate on the device in the
// calling process: every thread runs eight independent chains of dependent DFMA (no loads, no
// other FP64 work), on enough resident warps to keep every SM sub-partition issuing.
#include <algorithm>

#include "adi_common.hpp"

namespace lss_gb300 {

constexpr int FP64_RATE_CHAINS = 8;

__global__ void __launch_bounds__(256) k_fp64_rate(double *sink, int iters, double a, double b)
{
    double x[FP64_RATE_CHAINS];
#pragma unroll
    for (int q = 0; q < FP64_RATE_CHAINS; ++q) x[q] = 1e-3 * (threadIdx.x + q);
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int q = 0; q < FP64_RATE_CHAINS; ++q) x[q] = fma(x[q], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < FP64_RATE_CHAINS; ++q) s += x[q];
    if (s == -1.0) sink[blockIdx.x] = s; // never true for these inputs: keeps the chains live
}

} // namespace lss_gb300

using namespace lss_gb300;

extern "C" int lss_diag_fp64_rate(double *dfma_per_second, void *stream)
{
    clear_error();
    if (!dfma_per_second) return set_error(LSS_ADI_EINVAL, "lss_diag_fp64_rate: null output");
    int dev = 0, sms = 0;
    LSS_CUDA_TRY(cudaGetDevice(&dev), "lss_diag_fp64_rate: cudaGetDevice");
    LSS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "lss_diag_fp64_rate: SM count");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int blocks = 4 * sms, threads = 256, iters = 8192;
    double *sink = nullptr;
    LSS_CUDA_TRY(cudaMallocAsync(&sink, blocks * sizeof(double), s), "lss_diag_fp64_rate: scratch");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    cudaError_t err = cudaSuccess;
    for (int rep = 0; rep < 4 && err == cudaSuccess; ++rep) {
        cudaEventRecord(e0, s);
        k_fp64_rate<<<blocks, threads, 0, s>>>(sink, iters, 0.9999999, 1e-7);
        cudaEventRecord(e1, s);
        err = cudaEventSynchronize(e1);
        if (err == cudaSuccess) err = cudaGetLastError();
        float ms = 0.f;
        if (err == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms > 0.f) best = std::min(best, ms); // the first run warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(sink, s);
    LSS_CUDA_TRY(err, "lss_diag_fp64_rate: run");
    *dfma_per_second = static_cast<double>(blocks) * threads * iters * FP64_RATE_CHAINS / (best * 1e-3);
    return LSS_ADI_OK;
}
