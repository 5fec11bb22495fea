// noalloc.cu — a Coulomb (J) build that allocates no memory.
//
// Some callers cannot call cudaMalloc: code that runs inside another framework's memory
// pool or allocator hooks, real-time or embedded hosts that forbid allocation after
// start-up, and drivers that capture a fixed set of buffers once.  This entry point serves
// them: the caller passes every input and output buffer, and the one intermediate the
// J build needs, the fitted density d_Q (naux doubles), lives in a file-scope __device__
// array of fixed size that every GPU loading this library holds until the process exits.
//
// The computation is the same two passes as the regular J build (DFHelper::compute_J_symm),
// but over the Q-major packed-triangle layout the caller already holds:
//   pass 1  d_Q  = sum_{m>=n} B[Q][mn] * (D_mn + D_nm)   (D_mm once on the diagonal)
//   pass 2  J_mn = J_nm = sum_Q B[Q][mn] * d_Q
// Both passes use fixed-order reductions, so results are reproducible.
#include <cuda_runtime.h>

#include <string>

#include "common.cuh"
#include "gdfjk.h"

namespace gdfjk {

// Shared scratch for d_Q.  Every call overwrites entries [0, naux) before reading them, so
// nothing has to start at zero; two calls whose kernels overlap on the GPU race on it.
static __device__ __align__(256) double g_noalloc_dq[GDFJK_NOALLOC_MAX_NAUX];

namespace {

constexpr int NA_THREADS = 256;

__global__ void __launch_bounds__(NA_THREADS) noalloc_pass1_kernel(const double* __restrict__ B,
                                                                   const double* __restrict__ D, int nbf,
                                                                   double* __restrict__ dq) {
    __shared__ double sh[NA_THREADS / 32];
    int Q = blockIdx.x;
    size_t npair = (size_t)nbf * (nbf + 1) / 2;
    const double* row = B + (size_t)Q * npair;
    // One flat, coalesced walk over the packed triangle: thread t reads pairs t, t+256, ...
    // and keeps its own (m, n) decoding of the packed index, advanced without a square root.
    size_t p = threadIdx.x;
    size_t m = 0, n = p;
    while (m < (size_t)nbf && n > m) {
        n -= m + 1;
        ++m;
    }
    double acc = 0.0;
    for (; p < npair; p += NA_THREADS) {
        double w = (n == m) ? D[m * nbf + m] : D[m * nbf + n] + D[n * nbf + m];
        acc = fma(__ldg(row + p), w, acc);
        n += NA_THREADS;
        while (m < (size_t)nbf && n > m) {
            n -= m + 1;
            ++m;
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x % 32 == 0) sh[threadIdx.x / 32] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < NA_THREADS / 32; ++k) s += sh[k];
        dq[Q] = s;
    }
}

__global__ void __launch_bounds__(NA_THREADS) noalloc_pass2_kernel(const double* __restrict__ B,
                                                                   const double* __restrict__ dq, int nbf, int naux,
                                                                   double* __restrict__ J) {
    size_t npair = (size_t)nbf * (nbf + 1) / 2;
    for (size_t p = blockIdx.x * (size_t)NA_THREADS + threadIdx.x; p < npair; p += (size_t)gridDim.x * NA_THREADS) {
        double acc = 0.0;
        for (int Q = 0; Q < naux; ++Q) acc = fma(__ldg(B + (size_t)Q * npair + p), __ldg(dq + Q), acc);
        size_t m = (size_t)((sqrt(8.0 * (double)p + 1.0) - 1.0) * 0.5);
        while (m * (m + 1) / 2 > p) --m;
        while ((m + 1) * (m + 2) / 2 <= p) ++m;
        size_t n = p - m * (m + 1) / 2;
        J[m * nbf + n] = acc;
        J[n * nbf + m] = acc;
    }
}

}  // namespace
}  // namespace gdfjk

extern "C" int gdfjk_coulomb_noalloc(int nbf, int naux, const double* B, const double* D, double* J, void* stream) {
    using namespace gdfjk;
    if (nbf <= 0 || naux <= 0 || !B || !D || !J) return report_error(GDFJK_ERR_ARG, "coulomb_noalloc: bad sizes or null buffer");
    if (naux > GDFJK_NOALLOC_MAX_NAUX)
        return report_error(GDFJK_ERR_ARG, "coulomb_noalloc: naux " + std::to_string(naux) + " exceeds the fixed scratch of " +
                                               std::to_string(GDFJK_NOALLOC_MAX_NAUX) + " fitting functions");
    // The array's device address belongs to the CUDA context current on this thread, so it
    // is looked up on every call (no allocation; the first call in a context may load the
    // module, which is why that first call should come before any stream capture).  A cached
    // address would go stale after cudaDeviceReset or under a caller's own non-primary context.
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_dq);
    if (e != cudaSuccess)
        return report_error(GDFJK_ERR_CUDA, std::string("coulomb_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    double* dq = static_cast<double*>(p);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    noalloc_pass1_kernel<<<naux, NA_THREADS, 0, s>>>(B, D, nbf, dq);
    size_t npair = (size_t)nbf * (nbf + 1) / 2;
    int blocks = (int)((npair + NA_THREADS - 1) / NA_THREADS);
    if (blocks > 152 * 16) blocks = 152 * 16;
    noalloc_pass2_kernel<<<blocks, NA_THREADS, 0, s>>>(B, dq, nbf, naux, J);
    e = cudaGetLastError();
    if (e != cudaSuccess) return report_error(GDFJK_ERR_CUDA, std::string("coulomb_noalloc: launch: ") + cudaGetErrorString(e));
    return GDFJK_OK;
}
