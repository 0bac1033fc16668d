// Probes: the FP64 FMA throughput (the denominator of the FP64-pipe
// roofline) and the double-float propagator coefficients on given inputs.
#include <cuda_runtime.h>

#include "xf_df.cuh"
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

// ------------------------------------------------------------------ double-float propagator

namespace {

__global__ void k_df_propagator(int n, const double* __restrict__ h, const double* __restrict__ dl, int half,
                                double* __restrict__ cm, double* __restrict__ S)
{
    using namespace xf::dfp;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = i < n ? i : n - 1;  // lanes past n repeat the last input: every lane takes part
    const DF h00 = dsplit(h[3 * j]), h01r = dsplit(h[3 * j + 1]), h01i = dsplit(h[3 * j + 2]);
    const DLen bm = dlen(dsplit(dl[j]));
    const DK k = half ? dcoeffs<1>(h00, h01r, dsq(h01i), bm) : dcoeffs<0>(h00, h01r, dsq(h01i), bm);
    if (i < n) {
        cm[i] = df_value(k.cm);
        S[i] = df_value(k.S);
    }
}

}  // namespace

extern "C" int xf_probe_df_propagator(int n, const double* h, const double* dl, int half, double* cm, double* S)
{
    if (n <= 0 || n > (1 << 26) || !h || !dl || !cm || !S) return XF_EINVAL;
    double* d = nullptr;
    const size_t nb = (size_t)n * sizeof(double);
    if (cudaMalloc(&d, 6 * nb) != cudaSuccess) return XF_ENOMEM;
    double *dh = d, *ddl = d + 3 * (size_t)n, *dcm = d + 4 * (size_t)n, *dS = d + 5 * (size_t)n;
    cudaError_t err = cudaMemcpy(dh, h, 3 * nb, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(ddl, dl, nb, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) {
        k_df_propagator<<<(n + 255) / 256, 256>>>(n, dh, ddl, half, dcm, dS);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaMemcpy(cm, dcm, nb, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemcpy(S, dS, nb, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return err == cudaSuccess ? XF_OK : XF_ECUDA;
}
