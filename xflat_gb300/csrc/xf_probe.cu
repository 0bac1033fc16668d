// FP64 FMA throughput probe: the denominator of the FP64-pipe roofline.
#include <cuda_runtime.h>

#include "xflat_gpu.h"

namespace {

__global__ void k_dfma_loop(double* out, int iters, double a, double b)
{
    double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace

extern "C" int xf_probe_fp64_peak(double ms, double* tflops)
{
    if (!tflops || !(ms > 0.)) return XF_EINVAL;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return XF_ECUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return XF_ECUDA;
    const int blocks = sms * 8, threads = 256;
    double* out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return XF_ENOMEM;
    cudaStream_t st;
    cudaEvent_t e0, e1;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int iters = 256;
    float t = 0.f;
    k_dfma_loop<<<blocks, threads, 0, st>>>(out, iters, 1.0000001, 1e-9);
    // grow the loop (at most 16x per round, at most 2^20 iterations, which is
    // a few seconds at GB300's FP64 rate) until one launch takes about `ms`
    for (int rep = 0; rep < 8; ++rep) {
        cudaEventRecord(e0, st);
        k_dfma_loop<<<blocks, threads, 0, st>>>(out, iters, 1.0000001, 1e-9);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&t, e0, e1);
        if (t <= 0.f || t >= 0.5 * ms || iters >= (1 << 20)) break;
        double f = ms / t;
        f = f > 16. ? 16. : f;
        const double next = iters * f + 1.;
        iters = next > (double)(1 << 20) ? (1 << 20) : (int)next;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    cudaFree(out);
    if (err != cudaSuccess || t <= 0.f) return XF_ECUDA;
    *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (t * 1e-3) / 1e12;
    return XF_OK;
}
