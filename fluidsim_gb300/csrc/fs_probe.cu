// fs_probe.cu -- FP64 issue-rate microbenchmark of the current GPU.
//
// The plain path's particle and assembly kernels are limited by the FP64
// pipe, not by HBM: GB300 issues one warp-wide DFMA per SM every 16 cycles
// or so.  This measures that roof on the card the library runs on: a grid of
// 8 CTAs per SM, each thread running eight independent DFMA chains (enough
// independent work to hide the DFMA latency), timed with CUDA events on a
// private stream.  No clocks or device settings are touched.
#include <cuda_runtime.h>
#include <stdint.h>
#include "fluidsim_gpu.h"
#include "fs_fastmath.cuh"

namespace {

// Each thread runs CH independent DFMA chains (enough independent work to hide
// the DFMA latency); each chain contracts toward a fixed point, so its values
// stay normal.
template <int CH>
__global__ void __launch_bounds__(256) k_dfma_rate(double *sink, int iters, double seed) {
    double a[CH];
#pragma unroll
    for (int c = 0; c < CH; ++c) a[c] = seed + 1e-9 * (threadIdx.x + 37 * c);
    const double m = 0.9999999999, k = 1e-12;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < CH; ++c) a[c] = fma(a[c], m, k);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < CH; ++c) s += a[c];
    if (s == 1234.5678) sink[blockIdx.x] = s;   // never true; keeps the chains live
}

__global__ void k_math_eval(int fn, const double *x, double *y, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = x[i];
        y[i] = fn == 0 ? fs_log(v) : fn == 1 ? fs_exp(v) : fn == 2 ? log(v) : exp(v);
    }
}

}  // namespace

// Evaluates one of the kernels' FP64 elementary functions on n host values
// (accuracy tests): fn 0 fs_log, 1 fs_exp (the table-driven ones the FP64
// kernels use), 2 CUDA log, 3 CUDA exp, on the current device.
extern "C" int fs_math_eval(int32_t fn, const double *x, double *y, int64_t n) {
    if (fn < 0 || fn > 3 || n < 0 || (n > 0 && (!x || !y))) return FS_ERR_INVALID;
    if (n == 0) return FS_OK;
    double *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(double) * 2 * (size_t)n);
    if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? FS_ERR_NOMEM : FS_ERR_NO_DEVICE;
    e = cudaMemcpy(d, x, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
        k_math_eval<<<blocks, 256>>>(fn, d, d + n, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(y, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? FS_OK : FS_ERR_CUDA;
}

extern "C" int fs_fp64_rate(int32_t device, double *dfma_per_s) {
    if (!dfma_per_s) return FS_ERR_INVALID;
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess) return FS_ERR_NO_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return FS_ERR_NO_DEVICE;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int iters = 4096;
    double *sink = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = FS_OK;
    double best = 0.0;
    if (cudaMalloc(&sink, sizeof(double) * 16 * sms) != cudaSuccess ||
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        rc = FS_ERR_CUDA;
    } else {
        // 8 and 16 chains per thread, 4 to 16 CTAs of 256 threads per SM: the
        // best rate of all shapes (each timed 5 times after a warm-up launch)
        for (int shape = 0; shape < 6 && rc == FS_OK; ++shape) {
            const int chains = shape < 3 ? 8 : 16, per_sm = 4 << (shape % 3), blocks = per_sm * sms;
            for (int rep = 0; rep < 6 && rc == FS_OK; ++rep) {
                cudaEventRecord(e0, st);
                if (chains == 8) k_dfma_rate<8><<<blocks, 256, 0, st>>>(sink, iters, 1.0 + rep);
                else k_dfma_rate<16><<<blocks, 256, 0, st>>>(sink, iters / 2, 1.0 + rep);
                cudaEventRecord(e1, st);
                if (cudaEventSynchronize(e1) != cudaSuccess) { rc = FS_ERR_CUDA; break; }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                const double rate = (double)blocks * 256 * 8 * (double)iters / (ms * 1e-3);
                if (rep > 0 && rate > best) best = rate;   // the first launch is a warm-up
            }
        }
        if (rc == FS_OK && cudaGetLastError() != cudaSuccess) rc = FS_ERR_CUDA;
    }
    if (rc == FS_OK) *dfma_per_s = best;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (sink) cudaFree(sink);
    cudaSetDevice(prev);
    return rc;
}
