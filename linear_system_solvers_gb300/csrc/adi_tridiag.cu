// adi_tridiag.cu -- batched Thomas LU line solver (lss_tridiag_thomas_lu).
//
// The reference's thomas_lu_solver with a Dirichlet boundary_pair
// (sparse_solvers/tridiagonal/thomas_lu_solver/lss_thomas_lu_solver.hpp:125-191,
// lss_thomas_lu_boundary.hpp:114-205), one thread per line, lines fastest in memory so
// every access of a warp is one coalesced row.  Reference operation order, no FMA
// contraction (bit-identical to the host policy).
#include <mutex>
#include <string>

#include "adi_common.hpp"
#include "adi_device.cuh"

namespace lss_gb300 {

template <typename T>
__global__ void k_thomas_lu_lines(int n, int lines, const T *__restrict__ lo, const T *__restrict__ dg,
                                  const T *__restrict__ up, const T *__restrict__ rhs, const T *__restrict__ blo,
                                  const T *__restrict__ bhi, T *__restrict__ x, T *__restrict__ gam_scratch)
{
    using R = ar<true>;
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= lines) return;
    const size_t L = static_cast<size_t>(lines);
    const int e = n - 2;
    const T bl = blo[l], bh = bhi[l];
    T gam = T(0), y = T(0);
    for (int t = 1; t <= e; ++t) {
        const size_t o = static_cast<size_t>(t) * L + l;
        const T a = lo[o], b = dg[o], c = up[o], f = rhs[o];
        if (t == 1) {
            gam = R::div(c, b);
            y = R::div(R::sub(f, R::mul(a, bl)), b);
        } else if (t < e) {
            const T beta = R::sub(b, R::mul(a, gam));
            y = R::div(R::sub(f, R::mul(a, y)), beta);
            gam = R::div(c, beta);
        } else {
            const T beta = R::sub(b, R::mul(a, gam));
            y = R::div(R::sub(R::sub(f, R::mul(c, bh)), R::mul(a, y)), beta);
        }
        gam_scratch[o] = gam;
        x[o] = y;
    }
    T xv = y;
    for (int t = e - 1; t >= 1; --t) {
        const size_t o = static_cast<size_t>(t) * L + l;
        xv = R::sub(x[o], R::mul(gam_scratch[o], xv));
        x[o] = xv;
    }
    x[l] = bl;
    x[static_cast<size_t>(n - 1) * L + l] = bh;
}

} // namespace lss_gb300

using namespace lss_gb300;

extern "C" int lss_tridiag_thomas_lu(int precision, int n, int lines, const void *lo, const void *diag, const void *up,
                                     const void *rhs, const void *bnd_lo, const void *bnd_hi, void *x, void *stream)
{
    clear_error();
    if (n < 4) return set_error(LSS_ADI_EINVAL, "lss_tridiag_thomas_lu: n must be >= 4");
    if (lines < 0) return set_error(LSS_ADI_EINVAL, "lss_tridiag_thomas_lu: lines must be >= 0");
    if (lines == 0) return LSS_ADI_OK;
    if (!lo || !diag || !up || !rhs || !bnd_lo || !bnd_hi || !x)
        return set_error(LSS_ADI_EINVAL, "lss_tridiag_thomas_lu: null pointer");
    if (precision != LSS_ADI_FP64 && precision != LSS_ADI_FP32)
        return set_error(LSS_ADI_EINVAL, "lss_tridiag_thomas_lu: unknown precision");
    const size_t elem = precision == LSS_ADI_FP64 ? sizeof(double) : sizeof(float);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // stream-ordered scratch for the gamma factors: concurrent calls on other streams
    // get their own buffer
    void *scratch = nullptr;
    LSS_CUDA_TRY(cudaMallocAsync(&scratch, static_cast<size_t>(n) * lines * elem, s), "allocating line-solver scratch");
    const int bs = 128;
    if (precision == LSS_ADI_FP64)
        k_thomas_lu_lines<double><<<grid_for(lines, bs), bs, 0, s>>>(
            n, lines, static_cast<const double *>(lo), static_cast<const double *>(diag), static_cast<const double *>(up),
            static_cast<const double *>(rhs), static_cast<const double *>(bnd_lo), static_cast<const double *>(bnd_hi),
            static_cast<double *>(x), static_cast<double *>(scratch));
    else
        k_thomas_lu_lines<float><<<grid_for(lines, bs), bs, 0, s>>>(
            n, lines, static_cast<const float *>(lo), static_cast<const float *>(diag), static_cast<const float *>(up),
            static_cast<const float *>(rhs), static_cast<const float *>(bnd_lo), static_cast<const float *>(bnd_hi),
            static_cast<float *>(x), static_cast<float *>(scratch));
    const cudaError_t launch = cudaGetLastError();
    cudaFreeAsync(scratch, s);
    LSS_CUDA_TRY(launch, "launching k_thomas_lu_lines");
    return LSS_ADI_OK;
}

// ------------------------------------------------------------------------------------------
// lss_tridiag_thomas_lu_noalloc: the same batched Thomas LU solve for callers that may not
// allocate device memory at call time -- code running under a memory pool or allocator it
// does not own, real-time paths that forbid allocator round trips, or hosts that reserve
// all device memory up front.  Its only scratch (the gamma factors) is the fixed array
// below, part of the library image: every GPU that loads the library holds these
// LSS_NOALLOC_SCRATCH_BYTES until the process exits.  The array is shared by all calls on a
// device and keeps the last call's contents; nothing in it needs to start at zero (every
// gamma factor is written before it is read).  Calls whose kernels overlap on the GPU
// (different streams, or different host threads) race on the array.
// ------------------------------------------------------------------------------------------
#define LSS_NOALLOC_SCRATCH_BYTES (8u << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[LSS_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {};
}

// Device address of the scratch array for the current device, looked up once per device
// with that device current (the host-side symbol is not a device address).  Under CUDA's lazy
// module loading (the default) this first lookup is what loads this file's module -- the 8 MiB
// array and the kernels' code -- onto the device, so it allocates device memory once; the
// kernels' code is loaded here too (cudaFuncGetAttributes) so that the first real solve loads
// nothing.  The cached address belongs to the device's primary context: a cudaDeviceReset
// between calls invalidates it and is not supported.
static int noalloc_scratch(void **out)
{
    int dev = 0;
    LSS_CUDA_TRY(cudaGetDevice(&dev), "lss_tridiag_thomas_lu_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= 64) return set_error(LSS_ADI_EINVAL, "lss_tridiag_thomas_lu_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        LSS_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch), "lss_tridiag_thomas_lu_noalloc: cudaGetSymbolAddress");
        cudaFuncAttributes fa;
        LSS_CUDA_TRY(cudaFuncGetAttributes(&fa, k_thomas_lu_lines<double>), "lss_tridiag_thomas_lu_noalloc: loading the kernel");
        LSS_CUDA_TRY(cudaFuncGetAttributes(&fa, k_thomas_lu_lines<float>), "lss_tridiag_thomas_lu_noalloc: loading the kernel");
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return LSS_ADI_OK;
}

extern "C" int lss_tridiag_thomas_lu_noalloc(int precision, int n, int lines, const void *lo, const void *diag,
                                             const void *up, const void *rhs, const void *bnd_lo, const void *bnd_hi,
                                             void *x, void *stream)
{
    clear_error();
    if (n < 4) return set_error(LSS_ADI_EINVAL, "lss_tridiag_thomas_lu_noalloc: n must be >= 4");
    if (lines < 0) return set_error(LSS_ADI_EINVAL, "lss_tridiag_thomas_lu_noalloc: lines must be >= 0");
    void *scratch = nullptr;
    int rc = noalloc_scratch(&scratch); // lines == 0: the per-device warm-up, nothing else
    if (rc) return rc;
    if (lines == 0) return LSS_ADI_OK;
    if (!lo || !diag || !up || !rhs || !bnd_lo || !bnd_hi || !x)
        return set_error(LSS_ADI_EINVAL, "lss_tridiag_thomas_lu_noalloc: null pointer");
    if (precision != LSS_ADI_FP64 && precision != LSS_ADI_FP32)
        return set_error(LSS_ADI_EINVAL, "lss_tridiag_thomas_lu_noalloc: unknown precision");
    const size_t elem = precision == LSS_ADI_FP64 ? sizeof(double) : sizeof(float);
    const size_t need = static_cast<size_t>(n) * static_cast<size_t>(lines) * elem;
    if (need > LSS_NOALLOC_SCRATCH_BYTES)
        return set_error(LSS_ADI_EINVAL, "lss_tridiag_thomas_lu_noalloc: n*lines*element size " + std::to_string(need) +
                                             " bytes exceeds the fixed scratch of " +
                                             std::to_string(LSS_NOALLOC_SCRATCH_BYTES) + " bytes");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int bs = 128;
    if (precision == LSS_ADI_FP64)
        k_thomas_lu_lines<double><<<grid_for(lines, bs), bs, 0, s>>>(
            n, lines, static_cast<const double *>(lo), static_cast<const double *>(diag), static_cast<const double *>(up),
            static_cast<const double *>(rhs), static_cast<const double *>(bnd_lo), static_cast<const double *>(bnd_hi),
            static_cast<double *>(x), static_cast<double *>(scratch));
    else
        k_thomas_lu_lines<float><<<grid_for(lines, bs), bs, 0, s>>>(
            n, lines, static_cast<const float *>(lo), static_cast<const float *>(diag), static_cast<const float *>(up),
            static_cast<const float *>(rhs), static_cast<const float *>(bnd_lo), static_cast<const float *>(bnd_hi),
            static_cast<float *>(x), static_cast<float *>(scratch));
    LSS_CUDA_TRY(cudaGetLastError(), "launching k_thomas_lu_lines (no-alloc)");
    return LSS_ADI_OK;
}
