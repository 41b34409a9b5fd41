// bs_probe.cu -- FP64 throughput of the current GPU, measured by a chain of
// dependent fused multiply-adds.
//
// The FP64-pipe-bound kernels of the step (the search and the assembly in
// both forms, the FGMRES column passes in the FP64 form) are judged against
// the GPU's FP64 rate.  This probe measures that rate on the part itself
// instead of quoting a data-sheet figure: every thread runs NCH independent
// chains a <- a * m + c (one DFMA each, 2 flops), enough chains per thread
// and threads per SM to cover the pipe's latency, on a grid of several
// blocks per SM; time by CUDA events on a private stream.
#include <cuda_runtime.h>

#include "bs_internal.cuh"

namespace {

constexpr int NCH = 8;   // independent chains per thread

__global__ void __launch_bounds__(256) k_dfma_chain(int iters, double m, double c, double* __restrict__ sink) {
    double a[NCH];
#pragma unroll
    for (int q = 0; q < NCH; ++q) a[q] = 1.0 + 1e-3 * (threadIdx.x + q);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int q = 0; q < NCH; ++q) a[q] = fma(a[q], m, c);
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < NCH; ++q) s += a[q];
    // a data-dependent store the compiler cannot drop (never taken for m < 1)
    if (s == -1.0) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int bs_measure_fp64_peak(double* tflops) {
    if (!tflops) return BS_E_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return BS_E_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return BS_E_CUDA;
    const int threads = 256, blocks = sms * 8, iters = 1 << 14;
    double* sink = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = BS_OK;
    if (cudaMalloc(&sink, sizeof(double) * (size_t)blocks * threads) != cudaSuccess) return BS_E_NOMEM;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        rc = BS_E_CUDA;
    } else {
        float best = 1e30f;
        for (int rep = 0; rep < 6 && rc == BS_OK; ++rep) {   // first launch warms up
            cudaEventRecord(e0, st);
            k_dfma_chain<<<blocks, threads, 0, st>>>(iters, 0.999999, 1e-7, sink);
            cudaEventRecord(e1, st);
            float ms = 0.0f;
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
                rc = BS_E_CUDA;
            else if (rep > 0 && ms < best)
                best = ms;
        }
        if (rc == BS_OK) {
            const double flops = 2.0 * NCH * (double)iters * threads * blocks;
            *tflops = flops / (best * 1e-3) / 1e12;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaFree(sink);
    return (rc == BS_OK && cudaGetLastError() == cudaSuccess) ? BS_OK : (rc ? rc : BS_E_CUDA);
}
