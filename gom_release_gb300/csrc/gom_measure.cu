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

// the comparisons on bit patterns against the FP comparisons they stand for, over every pair of a
// table of special and ordinary values (signed zeros, subnormals, normals, infinities, NaNs of
// both signs), each helper only where its precondition holds
template <typename R> __device__ long long compare_mismatches(const R *v, int n, long long *checked) {
    long long bad = 0, seen = 0;
    for (int a = 0; a < n; ++a) {
        const R x = v[a];
        bad += gom::is_zero(x) != (x == R(0));
        bad += gom::pos_finite_or_inf(x) != (x > R(0));
        bad += gom::nan_bits(x) != (x != x);
        seen += 3;
        for (int b = 0; b < n; ++b) {
            const R y = v[b];
            if (gom::fbits(y) >= 0 || gom::nan_bits(y)) {   // y >= +0 or NaN, never -0
                bad += gom::gt_nonneg(x, y) != (x > y);
                ++seen;
            }
            if (gom::fbits(x) >= 0) {   // x with its sign bit clear
                bad += gom::lt_of_nonneg(x, y) != (x < y);
                ++seen;
            }
        }
    }
    *checked += seen;
    return bad;
}

__global__ void k_selftest_compares(const double *vd, int nd, const float *vf, int nf, long long *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    long long checked = 0;
    long long bad = compare_mismatches(vd, nd, &checked);
    bad += compare_mismatches(vf, nf, &checked);
    out[0] = checked;
    out[1] = bad;
}

}  // namespace

extern "C" int gom_selftest_compares(int64_t *checked, int64_t *mismatches) {
    if (!checked || !mismatches) return GOM_E_ARG;
    *checked = *mismatches = 0;
    const double dinf = __builtin_huge_val(), dnan = __builtin_nan("");
    const float finf = __builtin_huge_valf(), fnan = __builtin_nanf("");
    const double dbase[] = {0.0, 4.9406564584124654e-324, 2.2250738585072009e-308, 2.2250738585072014e-308, 1e-300,
                            1e-9, 0.25, 0.5, 1.0, 1.0000000000000002, 2.0, 50.0, 1e300, 1.7976931348623157e308,
                            dinf, dnan, 3.14159, 0.1};
    const float fbase[] = {0.0f, 1.4e-45f, 1.1754942e-38f, 1.17549435e-38f, 1e-30f, 1e-5f, 0.5f, 1.0f, 1.0000001f,
                           2.0f, 50.0f, 3.4028235e38f, finf, fnan, 0.1f};
    const int nd0 = sizeof(dbase) / sizeof(double), nf0 = sizeof(fbase) / sizeof(float);
    double vd[2 * nd0];
    float vf[2 * nf0];
    for (int k = 0; k < nd0; ++k) {
        vd[2 * k] = dbase[k];
        vd[2 * k + 1] = -dbase[k];   // -0, negative values, -inf and a NaN with its sign bit set
    }
    for (int k = 0; k < nf0; ++k) {
        vf[2 * k] = fbase[k];
        vf[2 * k + 1] = -fbase[k];
    }
    double *dd = nullptr;
    float *df = nullptr;
    long long *dout = nullptr;
    int rc = GOM_E_CUDA;
    if (cudaMalloc(&dd, sizeof(vd)) == cudaSuccess && cudaMalloc(&df, sizeof(vf)) == cudaSuccess &&
        cudaMalloc(&dout, 2 * sizeof(long long)) == cudaSuccess &&
        cudaMemcpy(dd, vd, sizeof(vd), cudaMemcpyHostToDevice) == cudaSuccess &&
        cudaMemcpy(df, vf, sizeof(vf), cudaMemcpyHostToDevice) == cudaSuccess) {
        k_selftest_compares<<<1, 32>>>(dd, 2 * nd0, df, 2 * nf0, dout);
        long long out[2] = {0, 0};
        if (cudaMemcpy(out, dout, sizeof(out), cudaMemcpyDeviceToHost) == cudaSuccess) {
            *checked = out[0];
            *mismatches = out[1];
            rc = GOM_OK;
        }
    }
    cudaFree(dd);
    cudaFree(df);
    cudaFree(dout);
    return rc;
}

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
