// peaks.cu -- the float64 FMA throughput of the device, measured: the
// FP64-ALU roofline of the float64 kernels (on GB300 far below the HBM one).
#include <cuda_runtime.h>

#include "f2d_common.cuh"
#include "../../include/fluid2d_gb300.h"

namespace f2d {

// eight independent FMA chains per thread; the sum keeps them live
__global__ void k_dfma_chains(double *out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4,
           x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int it = 0; it < iters; it++) {
        x0 = fma(x0, a, b);
        x1 = fma(x1, a, b);
        x2 = fma(x2, a, b);
        x3 = fma(x3, a, b);
        x4 = fma(x4, a, b);
        x5 = fma(x5, a, b);
        x6 = fma(x6, a, b);
        x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace f2d

extern "C" {

int f2d_fp64_peak(double *tflops) {
    if (!tflops) return f2d::ERR_ARG;
    int dev = 0, sms = 0;
    int st0 = f2d::cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (!st0)
        st0 = f2d::cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                               "SM count");
    if (st0) return st0;
    const int blocks = 8 * (sms > 0 ? sms : 1), threads = 256, iters = 4096;
    double *out = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int st = f2d::cuda_status(cudaMalloc((void **)&out, sizeof(double) * blocks * threads),
                              "peak buffer");
    if (!st) st = f2d::cuda_status(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
    if (!st) st = f2d::cuda_status(cudaEventCreate(&e0), "event");
    if (!st) st = f2d::cuda_status(cudaEventCreate(&e1), "event");
    double best = 0.;
    for (int rep = 0; rep < 4 && !st; rep++) {
        cudaEventRecord(e0, s);
        f2d::k_dfma_chains<<<blocks, threads, 0, s>>>(out, iters, 0.999, 1e-3);
        cudaEventRecord(e1, s);
        st = f2d::cuda_status(cudaEventSynchronize(e1), "peak kernel");
        float ms = 0.f;
        if (!st) st = f2d::cuda_status(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
        const double flops = 2.0 * 8 * iters * (double)blocks * threads;
        if (!st && rep > 0 && ms > 0.f && flops / (ms * 1e-3) / 1e12 > best)
            best = flops / (ms * 1e-3) / 1e12;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (out) cudaFree(out);
    if (!st) *tflops = best;
    return st;
}

}  // extern "C"
