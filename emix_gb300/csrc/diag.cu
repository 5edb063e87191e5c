// diag.cu -- device diagnostics used by the benchmark's roofline report.
#include "common.cuh"

namespace emix {
namespace {

// Eight independent FMA chains per thread; the loop count is fixed, so the
// kernel always ends.  Values stay finite (|a| < 1 contraction towards b/(1-a)).
__global__ void k_dfma_chain(double *out, double a, double b, int iters) {
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 0.1, x2 = x0 + 0.2, x3 = x0 + 0.3, x4 = x0 + 0.4,
           x5 = x0 + 0.5, x6 = x0 + 0.6, x7 = x0 + 0.7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// The library's reciprocal and square-root helpers beside CUDA's own
// operators, evaluated on the same arguments in the same kernel: out[k*n + q]
// for k = 0..5 is rcp_fast, 1.0/x, sqrt_fast, sqrt, rsqrt_fast, 1.0/sqrt.
__global__ void k_math_selftest(const double *__restrict__ x, double *__restrict__ out, long n) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const double v = x[q];
        out[q] = rcp_fast(v);
        out[n + q] = 1.0 / v;
        out[2 * n + q] = sqrt_fast(v);
        out[3 * n + q] = sqrt(v);
        out[4 * n + q] = rsqrt_fast(v);
        out[5 * n + q] = 1.0 / sqrt(v);
    }
}

} // namespace
} // namespace emix

using namespace emix;

extern "C" int emix_math_selftest_dev(const double *x, double *out, long n, void *stream) {
    if (!x || !out || n < 1) return EMIX_ERR_ARG;
    k_math_selftest<<<grid_cap(n, 8), 256, 0, (cudaStream_t)stream>>>(x, out, n);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

extern "C" int emix_fp64_peak(double *lane_ops_per_s) {
    if (!lane_ops_per_s) return EMIX_ERR_ARG;
    int dev = 0, sms = 0;
    EMIX_CUDA_TRY(cudaGetDevice(&dev));
    EMIX_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256, iters = 2000;
    double *d = nullptr;
    if (cudaMalloc(&d, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return EMIX_ERR_ALLOC;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0);
        k_dfma_chain<<<blocks, threads>>>(d, 0.999999, 1e-9, iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (e != cudaSuccess) {
        set_last_error(e, "k_dfma_chain", __FILE__, __LINE__);
        return EMIX_ERR_CUDA;
    }
    *lane_ops_per_s = (double)blocks * threads * iters * 8 / (best * 1e-3);
    return EMIX_OK;
}
