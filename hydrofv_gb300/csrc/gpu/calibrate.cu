/*
 * calibrate.cu -- arithmetic-throughput calibration for roofline reporting.
 *
 * The FP64 MUSCL-Hancock step is bound by the FP64 pipe, not by HBM, and the
 * GB300's FP64 rate is not a published per-SKU constant we can rely on, so
 * the benchmark measures it: independent fused multiply-add chains (8 per
 * thread, enough to cover the pipe latency), one wave of 8 CTAs of 256
 * threads per SM, timed with CUDA events.  1 FMA = 2 FLOP.
 */
#include <cuda_runtime.h>

#include "hydro_gpu.h"

namespace {

template <class T>
__global__ void fma_chains(T *out, int iters, T a, T b)
{
    T x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = (T) (threadIdx.x + k) * (T) 1e-3;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k];
    if (s == (T) 12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class T>
int measure(int sms, int iters, double *tflops)
{
    const int blocks = sms * 8, threads = 256;
    T *out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains<T><<<blocks, threads>>>(out, iters / 8, (T) 0.999, (T) 1e-3);  /* warm-up */
    cudaEventRecord(e0);
    fma_chains<T><<<blocks, threads>>>(out, iters, (T) 0.999, (T) 1e-3);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0) return -1;
    const double flop = 2.0 * 8.0 * (double) iters * blocks * threads;
    *tflops = flop / (ms * 1e-3) / 1e12;
    return 0;
}

}  // namespace

extern "C" int hydro_gpu_sm_count(int device)
{
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return sms;
}

extern "C" int hydro_gpu_calibrate(int device, double *fp64_tflops, double *fp32_tflops)
{
    if (cudaSetDevice(device) != cudaSuccess) return -1;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return -1;
    if (fp64_tflops && measure<double>(sms, 1 << 12, fp64_tflops)) return -1;
    if (fp32_tflops && measure<float>(sms, 1 << 16, fp32_tflops)) return -1;
    return 0;
}
