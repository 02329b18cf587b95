// peak_fma.cu -- sustained FMA throughput of the device (the roofline denominator
// of the path kernel, which is bound by the FP64 pipe in FP64 mode and by the
// FP32 pipe in mixed mode; neither is a tensor-core or HBM bound).
//
// Every thread runs kChains independent dependent FMA chains; the grid fills
// every SM many times over.  Flops = 2 * FMAs.
#include <cuda_runtime.h>

#include "hjm_kernels.h"

namespace hjm {

constexpr int kChains = 8;
constexpr int kPeakThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kPeakThreads) fma_chains(int iters, T b, T c, T* __restrict__ sink)
{
    T a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) a[i] = (T)(threadIdx.x + i) * (T)1e-3;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
#pragma unroll
            for (int i = 0; i < kChains; ++i) a[i] = fma(a[i], b, c);
        }
    }
    T s = 0;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += a[i];
    if (s == (T)-1) sink[threadIdx.x] = s;  // never true; keeps the chains alive
}

template <typename T>
static cudaError_t time_chains(int iters, int blocks, cudaStream_t s, T* sink, float* ms)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    fma_chains<T><<<blocks, kPeakThreads, 0, s>>>(iters, (T)0.999999, (T)1e-7, sink);
    cudaEventRecord(e1, s);
    cudaError_t err = cudaEventSynchronize(e1);
    if (err == cudaSuccess) err = cudaGetLastError();
    cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return err;
}

cudaError_t measure_fma_peak(bool fp64, cudaStream_t s, int n_sms, double* tflops)
{
    void* sink = nullptr;
    cudaError_t err = cudaMalloc(&sink, sizeof(double) * kPeakThreads);
    if (err != cudaSuccess) return err;
    const int blocks = n_sms * 8;
    int iters = fp64 ? 16 : 256;
    float ms = 0.f;
    // grow the work until one launch takes >= 20 ms, then take the best of 3
    for (int round = 0; round < 12; ++round) {
        err = fp64 ? time_chains<double>(iters, blocks, s, (double*)sink, &ms)
                   : time_chains<float>(iters, blocks, s, (float*)sink, &ms);
        if (err != cudaSuccess || ms >= 20.f) break;
        iters *= 2;
    }
    float best = ms;
    for (int r = 0; r < 3 && err == cudaSuccess; ++r) {
        err = fp64 ? time_chains<double>(iters, blocks, s, (double*)sink, &ms)
                   : time_chains<float>(iters, blocks, s, (float*)sink, &ms);
        if (ms < best) best = ms;
    }
    cudaFree(sink);
    if (err != cudaSuccess) return err;
    const double fmas = (double)blocks * kPeakThreads * (double)iters * 16.0 * kChains;
    *tflops = 2.0 * fmas / ((double)best * 1e-3) / 1e12;
    return cudaSuccess;
}

}  // namespace hjm
