// fs_fastmath.cuh -- table-driven FP64 natural logarithm and exponential for
// the FP64-issue-bound kernels (RK stage, Poisson assembly, ion face data).
//
// GB300 issues FP64 arithmetic at 1/64 of its FP32 rate, so in those kernels
// the cost of a logarithm or an exponential is the number of FP64 pipe
// instructions it takes.  Both functions here follow P. T. P. Tang's
// table-driven methods (ACM TOMS 15(2), 1989, for exp; 16(4), 1990, for log):
// a small table removes most of the argument range, and a short Taylor
// polynomial covers the rest.  Each takes about a dozen FP64 instructions.
// Tables and coefficients: fs_mathtab.h (make_mathtab.py, 60-digit decimal
// arithmetic rounded once).  Arguments outside the ranges handled here
// (non-positive, subnormal or non-finite for the logarithm; |x| >= 700 or
// NaN for the exponential) go to the CUDA functions.  Accuracy: within 2 ulp
// of the CUDA functions (tests/test_gpu_fastmath.py).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fs_mathtab.h"

// ln x.  x = 2^e m with m in [1, 2); F = 1 + j/128 is m rounded to 7
// fraction bits (when m rounds up to 2, x is taken as 2^(e+1) (m/2) with
// F = 1), r = (m - F)/F with |r| <= 2^-8, ln x = e ln 2 + ln F + ln(1 + r),
// the last by its Taylor series to r^7 (truncation < 2^-64 |r|).  ln 2 and
// ln F are head + tail pairs whose heads lie on the 2^-32 grid, so
// e ln2_head + lnF_head is exact and the cancellation near x = 1 (e = -1,
// F near 2) loses nothing: the result keeps its relative accuracy there.
__device__ __forceinline__ double fs_log(double x) {
    const int64_t b = __double_as_longlong(x);
    // positive normal finite: the exponent field in [1, 2046], sign clear
    if ((uint64_t)(b - 0x0010000000000000LL) >= (uint64_t)(0x7FF0000000000000LL - 0x0010000000000000LL))
        return log(x);
    int64_t mb = (b & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL;
    int j = (int)(((mb >> 44) & 0xFF) + 1) >> 1;                        // 0..128
    const int up = j >> 7;                                              // m rounds to 2
    mb -= (int64_t)up << 52;                                            // m / 2
    j &= 127;
    const int e = (int)(b >> 52) - 1023 + up;
    const double m = __longlong_as_double(mb);
    const double F = __longlong_as_double(0x3FF0000000000000LL + ((int64_t)j << 45));
    const double invF = __ldg(fs_log_tab + 3 * j), lnF_hi = __ldg(fs_log_tab + 3 * j + 1),
                 lnF_lo = __ldg(fs_log_tab + 3 * j + 2);
    const double r = (m - F) * invF;
    double q = fma(FS_LOG_C7, r, FS_LOG_C6);
    q = fma(q, r, FS_LOG_C5);
    q = fma(q, r, FS_LOG_C4);
    q = fma(q, r, FS_LOG_C3);
    q = fma(q, r, FS_LOG_C2);
    const double p = fma(r * r, q, r);
    const double ed = (double)e;
    const double hi = fma(ed, FS_LN2_HI, lnF_hi);   // exact: both terms on the 2^-32 grid
    const double lo = p + fma(ed, FS_LN2_LO, lnF_lo);
    return hi + lo;
}

// e^x.  k = rint(64 x / ln 2) = 64 m + j, r = x - k ln2/64 (|r| <= ln2/128,
// k ln2/64 in two parts so the first product is exact),
// e^x = 2^m 2^(j/64) (1 + p(r)) with p the Taylor series of e^r - 1 to r^6
// (truncation < 2^-60 |r|) and 2^(j/64) as a head + tail pair.
__device__ __forceinline__ double fs_exp(double x) {
    const int64_t b = __double_as_longlong(x);
    if ((b & 0x7FFFFFFFFFFFFFFFLL) >= 0x4085E00000000000LL)   // |x| >= 700 or NaN / inf
        return exp(x);
    const double shifter = 0x1.8p52;
    const double t = fma(x, FS_EXP_INV_L, shifter);
    const int k = (int)(uint32_t)__double_as_longlong(t);     // rint(x * 64/ln2), two's complement
    const double kd = t - shifter;
    const double r = fma(-kd, FS_EXP_L2, fma(-kd, FS_EXP_L1, x));
    double q = fma(FS_EXP_C6, r, FS_EXP_C5);
    q = fma(q, r, FS_EXP_C4);
    q = fma(q, r, FS_EXP_C3);
    q = fma(q, r, FS_EXP_C2);
    const double p = fma(r * r, q, r);
    const int j = k & 63, m = k >> 6;
    const double shi = __ldg(fs_exp_tab + 2 * j), slo = __ldg(fs_exp_tab + 2 * j + 1);
    const double s = shi + fma(shi, p, slo);
    return s * __longlong_as_double((int64_t)(m + 1023) << 52);
}
