// FMA throughput probe used as the FP64 / FP32 compute roofline denominator
// (the measured peaks cover HBM bandwidth and bf16 tensor throughput
// only).  Eight independent in-register FMA chains per thread, one output
// value per thread, grid sized as a multiple of the SM count.
#include <cuda_runtime.h>

#include "../../include/ks.h"

namespace {

template <typename T>
__global__ void k_fma_chain(T* out, T a, T b, int iters) {
    T x0 = (T)threadIdx.x, x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
    T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
    for (int i = 0; i < iters; ++i) {
        x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
        x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
    out[blockIdx.x * (long long)blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int run(double* gflops, void* scratch, int sms) {
    const int threads = 256, blocks = sms * 8, iters = 4096;
    T* out = static_cast<T*>(scratch);
    k_fma_chain<T><<<blocks, threads>>>(out, T(0.999), T(0.001), 16);
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return KS_ERR_CUDA;
    cudaEventRecord(a);
    k_fma_chain<T><<<blocks, threads>>>(out, T(0.999), T(0.001), iters);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *gflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e9;
    return cudaGetLastError() == cudaSuccess ? KS_OK : KS_ERR_CUDA;
}

}  // namespace

extern "C" int ks_fma_peak(int fp64, double* gflops) {
    if (!gflops) return KS_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return KS_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return KS_ERR_CUDA;
    void* scratch = nullptr;
    const size_t bytes = (size_t)sms * 8 * 256 * sizeof(double);
    if (cudaMalloc(&scratch, bytes) != cudaSuccess) return KS_ERR_OOM;
    const int rc = fp64 ? run<double>(gflops, scratch, sms) : run<float>(gflops, scratch, sms);
    cudaFree(scratch);
    return rc;
}
