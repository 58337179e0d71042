// FP64 elementary functions for the plain path.
//
// On GB300 the FP64 pipe issues about 0.63 T FMA/s for the whole GPU (measured), 1/60 of the FP32 rate,
// and every kernel of the plain path is bound by it. CUDA's double exp, log and division cost about
// 20, 37 and 8 FP64-pipe slots each on this part (measured), so the hot loops use the routines below,
// which spend as few FP64 instructions as possible, do their bookkeeping with integer operations, and
// stay within about one ulp (checked against CUDA's functions by the GPU tests):
//
//  exp_fast (9 FP64 ops): Tang's table-driven method (P. T. P. Tang, "Table-driven implementation of the
//    exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989) with 256 table
//    points: x = (256 m + j) ln2/256 + r, |r| <= ln2/512, exp(x) = 2^m 2^(j/256) (1 + q(r)), q the
//    degree-4 Taylor polynomial of e^r - 1 (truncation below 4e-17). n = 256 m + j comes from the
//    round-to-nearest shifter 1.5 * 2^52, ln2/256 is split so n * hi is exact, and 2^m is added to the
//    exponent field with an integer add.
//  log_fast (15 FP64 ops): x = 2^e f, f in [1, 2), c = 1 + j/256 the table point nearest f,
//    log x = e ln2 + ln c + log1p(u), u = (f - c) / c formed with the tabulated reciprocal of c
//    (f - c is exact) plus one residual correction, log1p(u) by its alternating series to u^6
//    (|u| <= 2^-9, truncation below 2^-54 relative); ln2 and ln c are double-doubles (Tang,
//    "Table-driven implementation of the logarithm function in IEEE floating-point arithmetic",
//    ACM TOMS 16(4), 1990, with a reciprocal table). Within 2 ulps where ln c and log1p(u) cancel.
//  rcp_fast (3 FP64 ops): the hardware estimate rcp.approx.ftz.f64 refined by one third-order Newton
//    step r' = r + r (e + e^2), e = 1 - y r (Muller et al., Handbook of Floating-Point Arithmetic,
//    2nd ed., section 4.7), enough to take a 2^-20 estimate below one ulp.
// Arguments outside each fast path's range (zero, subnormal, infinite, NaN, |x| >= 708 for exp) take
// CUDA's own function instead, so special values behave exactly as IEEE / CUDA define them.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tables.h"

namespace cbg {

// Out-of-line slow paths: kept as real (almost never taken) branches. Inlined, the compiler turns them
// into predicated code that every call executes, and predicated-off FP64 instructions still occupy the
// FP64 pipe (measured: about 2k extra warp-level FP64 instructions per cell in the rates kernels).
static __device__ __noinline__ double exp_slow(double x) { return exp(x); }
static __device__ __noinline__ double log_slow(double x) { return log(x); }
static __device__ __noinline__ double rcp_slow(double y) { return 1.0 / y; }

__device__ __forceinline__ double exp_fast(double x, const double* __restrict__ exp2j) {
    const int hi = __double2hiint(x);
    if ((hi & 0x7fffffff) >= 0x40862000) return exp_slow(x);  // |x| >= 708, inf or NaN
    const double t = fma(x, 0x1.71547652b82fep+8, 0x1.8p52);  // 256/ln2, round-to-nearest shifter
    const int n = __double2loint(t);
    const double nd = t - 0x1.8p52;
    double r = fma(nd, -0x1.62e42ff000000p-9, x);   // ln2/256, high part (32 significant bits)
    r = fma(nd, 0x1.718432a1b0e26p-43, r);          // minus the low part
    double a = fma(r, 1.0 / 24.0, 1.0 / 6.0);
    a = fma(a, r, 0.5);
    const double q = fma(a, r * r, r);
    const double tj = exp2j[n & 255];
    const double y = fma(tj, q, tj);
    return __hiloint2double(__double2hiint(y) + ((n >> 8) << 20), __double2loint(y));
}

__device__ __forceinline__ double log_fast(double x, const MathTables& T) {
    const int hi = __double2hiint(x), lo = __double2loint(x);
    if (hi < 0x00100000 || hi >= 0x7ff00000) return log_slow(x);  // <= 0, subnormal, inf or NaN
    const int e = (hi >> 20) - 1023;
    const int mant = hi & 0x000fffff;
    const int j = ((mant >> 11) + 1) >> 1;  // nearest multiple of 1/256
    const double f = __hiloint2double(mant | 0x3ff00000, lo);
    const double c = __hiloint2double(0x3ff00000 + (j << 12), 0);
    const double d = f - c;                        // exact
    const double u0 = d * T.rcp[j];
    const double u = fma(fma(-c, u0, d), T.rcp[j], u0);  // one correction: d / c to half an ulp
    double p = fma(u, -1.0 / 6.0, 1.0 / 5.0);
    p = fma(p, u, -0.25);
    p = fma(p, u, 1.0 / 3.0);
    p = fma(p, u, -0.5);
    const double l = fma(p, u * u, u);
    // (double)e without an FP64 conversion instruction: 2^52 + 2^31 + e, minus the offset.
    const double ed = __hiloint2double(0x43300000, (int)(0x80000000u ^ (unsigned)e)) - 0x1.00000800p+52;
    const double s = fma(ed, 0x1.62e42fefa4000p-1, T.log_hi[j]);
    return s + (l + fma(ed, -0x1.8432a1b0e2634p-43, T.log_lo[j]));
}

__device__ __forceinline__ double rcp_fast(double y) {
    const int ahi = __double2hiint(y) & 0x7fffffff;
    if (ahi < 0x00200000 || ahi >= 0x7fd00000) return rcp_slow(y);  // 0, tiny, huge, inf or NaN
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(y));
    const double e = fma(-y, r, 1.0);
    return fma(r, fma(e, e, e), r);
}

__device__ __forceinline__ double div_fast(double a, double b) { return a * rcp_fast(b); }

}  // namespace cbg
