// peaks.cu -- live FP32 / FP64 FMA throughput of the current GPU.
//
// The pair sweeps are bound by the FP32 (and, for the FP64 path, FP64)
// pipes.  Measured HBM and bf16 tensor peaks say nothing about these, so
// this probe measures them on the device the library runs on:
// independent FMA chains per thread over a grid of 8 blocks per SM.
#include "hz_internal.cuh"

namespace hz {
namespace {

template <typename T>
__global__ void __launch_bounds__(256) fma_chains(T *out, int iters, T a, T b)
{
    T x0 = threadIdx.x * (T)1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
      x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
        x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
        x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int time_chains(int iters, double &tflops)
{
    int dev = 0, sms = 0;
    HZ_CHECK_CUDA(cudaGetDevice(&dev));
    HZ_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256;
    DevBuf out;
    HZ_TRY(out.ensure((size_t)blocks * threads * sizeof(T)));
    cudaEvent_t e0, e1;
    HZ_CHECK_CUDA(cudaEventCreate(&e0));
    HZ_CHECK_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(e0);
        fma_chains<T><<<blocks, threads>>>(out.as<T>(), iters, (T)0.999, (T)0.001);
        cudaEventRecord(e1);
        HZ_CHECK_LAUNCH();
        HZ_CHECK_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
    return HZ_OK;
}

}  // namespace
}  // namespace hz

extern "C" HZ_API int hz_measure_fma_peaks(double *fp32_tflops, double *fp64_tflops)
{
    double a = 0, b = 0;
    HZ_TRY(hz::time_chains<float>(100000, a));
    HZ_TRY(hz::time_chains<double>(1500, b));
    if (fp32_tflops) *fp32_tflops = a;
    if (fp64_tflops) *fp64_tflops = b;
    return HZ_OK;
}
