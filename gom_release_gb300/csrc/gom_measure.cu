// gom_measure.cu -- the FP64 arithmetic peak of the GPU, measured, for the FP64 roofline of the
// plain FP64 path (whose kernels are bound by FP64 issue on GB300, not by HBM bandwidth).
#include "gom_launch.h"

namespace {

// eight independent FMA chains per thread, so that the FP64 pipe never waits on a result
__global__ void k_fp64_fma_peak(double *sink, int iters, double add) {
    double a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    const double m = 0.999999;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, m, add);
        a1 = fma(a1, m, add);
        a2 = fma(a2, m, add);
        a3 = fma(a3, m, add);
        a4 = fma(a4, m, add);
        a5 = fma(a5, m, add);
        a6 = fma(a6, m, add);
        a7 = fma(a7, m, add);
    }
    // never true for these inputs; keeps the chains alive
    if (a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7 == -1.0) sink[0] = a0;
}

// the same chains on the first `lanes` lanes of each warp only: the FP64 warp-instruction rate
// with that many lanes active
__global__ void k_fp64_fma_lanes(double *sink, int iters, double add, int lanes) {
    if ((int)(threadIdx.x & 31) >= lanes) return;
    double a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    const double m = 0.999999;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, m, add);
        a1 = fma(a1, m, add);
        a2 = fma(a2, m, add);
        a3 = fma(a3, m, add);
        a4 = fma(a4, m, add);
        a5 = fma(a5, m, add);
        a6 = fma(a6, m, add);
        a7 = fma(a7, m, add);
    }
    if (a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7 == -1.0) sink[0] = a0;
}

}  // namespace

extern "C" int gom_measure_fp64_issue(int32_t active_lanes, double *warp_instr_per_s) {
    if (!warp_instr_per_s || active_lanes < 1 || active_lanes > 32) return GOM_E_ARG;
    *warp_instr_per_s = 0.0;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GOM_E_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GOM_E_CUDA;
    double *sink = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = GOM_E_CUDA;
    const int blocks = 4 * sms, threads = 256, iters = 20000;
    float ms = 0.0f;
    if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess) return GOM_E_NOMEM;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
        cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
        k_fp64_fma_lanes<<<blocks, threads, 0, st>>>(sink, 200, 1e-9, active_lanes);   // warm-up
        cudaEventRecord(e0, st);
        k_fp64_fma_lanes<<<blocks, threads, 0, st>>>(sink, iters, 1e-9, active_lanes);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.0f) {
            const double warp_instr = 8.0 * (double)iters * blocks * (threads / 32);
            *warp_instr_per_s = warp_instr / (ms * 1e-3);
            rc = GOM_OK;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaFree(sink);
    return rc;
}

extern "C" int gom_measure_fp64_peak(double *gflops) {
    if (!gflops) return GOM_E_ARG;
    *gflops = 0.0;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GOM_E_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GOM_E_CUDA;
    double *sink = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = GOM_E_CUDA;
    const int blocks = 4 * sms, threads = 256, iters = 20000;
    float ms = 0.0f;
    if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess) return GOM_E_NOMEM;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
        cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
        k_fp64_fma_peak<<<blocks, threads, 0, st>>>(sink, 200, 1e-9);   // warm-up
        cudaEventRecord(e0, st);
        k_fp64_fma_peak<<<blocks, threads, 0, st>>>(sink, iters, 1e-9);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.0f) {
            const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;   // an FMA is 2 flops
            *gflops = flops / (ms * 1e-3) / 1e9;
            rc = GOM_OK;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaFree(sink);
    return rc;
}
