// Allocation-free residual entry point.
//
// Some callers must not have a library call cudaMalloc or cudaFree: runtimes
// that own all device memory through their own pool (CUDA.jl's or PyTorch's
// caching allocator, a serving process with a fixed memory budget) and code
// that cannot afford the device-wide synchronisation cudaMalloc/cudaFree may
// imply.  fdfd_residual_noalloc computes the same FP64 residual and norms as
// the handle path (residual_kernel + reduce_partials_kernel) from caller-owned
// buffers only.  Its one piece of scratch — the per-block partial sums of
// |r|² and |b|² — lives in the file-scope device array below.  The array comes
// into being when this library's module is loaded on a device (with lazy module
// loading, the CUDA default, at its first use there) and every GPU that loads
// it holds it until the process exits.
#include "fdfd_cuda.h"
#include "kernels.cuh"

#include <mutex>

// (thread block, right-hand side) pairs whose partial sums fit the array:
// 65536 pairs x 2 doubles = 1 MiB per device.  The right-hand sides form the
// grid's y dimension, so nrhs is also bounded by 65535.
#define FDFD_NOALLOC_MAX_PARTIALS 65536
#define FDFD_NOALLOC_MAX_RHS 65535
#define FDFD_NOALLOC_BLOCK 256
#define FDFD_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_partials[2 * FDFD_NOALLOC_MAX_PARTIALS];

namespace {
std::mutex g_mu;
double* g_partials_ptr[FDFD_NOALLOC_MAX_DEVICES] = {nullptr};
}  // namespace

extern "C" int fdfd_residual_noalloc(int Nx, int Ny, int nrhs, const double* stencil, const double* x,
                                     const double* b, double* r, double* norms, void* stream) {
    if (Nx < 1 || Ny < 1 || nrhs < 1 || !stencil || !x || !r || !norms) return FDFD_EINVAL;
    const long long N = (long long)Nx * Ny;
    const long long nblocks = (N + FDFD_NOALLOC_BLOCK - 1) / FDFD_NOALLOC_BLOCK;
    if (nrhs > FDFD_NOALLOC_MAX_RHS) return FDFD_EINVAL;                  // grid y limit
    if (nblocks * nrhs > FDFD_NOALLOC_MAX_PARTIALS) return FDFD_EINVAL;   // scratch too small
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= FDFD_NOALLOC_MAX_DEVICES) {
        cudaGetLastError();
        return FDFD_ECUDA;
    }
    double* part = nullptr;
    {
        // set-up, once per device, with that device current: the host-side name
        // of the array is not a device address, so resolve it here.  The cached
        // address belongs to the device's primary context: it must not outlive a
        // cudaDeviceReset (or a release and re-creation of that context)
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_partials_ptr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess || !p) {
                cudaGetLastError();
                return FDFD_ECUDA;
            }
            g_partials_ptr[dev] = static_cast<double*>(p);
        }
        part = g_partials_ptr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // every (block, rhs) entry the reduction reads is written by residual_kernel
    // first, so nothing has to be cleared between calls
    residual_kernel<<<dim3((unsigned)nblocks, nrhs), FDFD_NOALLOC_BLOCK, 0, s>>>(
        Nx, Ny, nrhs, reinterpret_cast<const cplx<double>*>(stencil), reinterpret_cast<const cplx<double>*>(x),
        reinterpret_cast<const cplx<double>*>(b), reinterpret_cast<cplx<double>*>(r), part);
    reduce_partials_kernel<<<nrhs, 256, 0, s>>>(part, (int)nblocks, 2, norms);
    if (cudaGetLastError() != cudaSuccess) return FDFD_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return FDFD_ECUDA;
    }
    return FDFD_OK;
}
