// FP64 elementary functions for the plain path.
//
// On GB300 the FP64 pipe issues about 0.6 T FMA/s for the whole GPU (measured), 1/62 of the FP32 rate,
// and every kernel of the plain path is bound by it. CUDA's double exp, log and division cost about
// 20, 37 and 8 FMA-pipe slots each on this part, so the hot loops use the routines below, built to
// spend as few FP64 instructions as possible while staying within about one ulp:
//
//  exp_fast: Tang's table-driven method (P. T. P. Tang, "Table-driven implementation of the exponential
//    function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989): x = (m*256 + j) ln2/256 + r
//    with |r| <= ln2/512, exp(x) = 2^m * 2^(j/256) * (1 + p(r)), p a degree-5 Taylor polynomial.
//    The 256-entry table of 2^(j/256) lives in shared memory; index and scaling use integer ops only.
//  log_fast: x = 2^e * f, f in [sqrt(1/2), sqrt(2)), table point c_j = 1 + j/128 nearest f,
//    log(x) = e ln2 + ln(c_j) + log1p((f - c_j) / c_j), the quotient formed with the exactly
//    representable reciprocal table 1/c_j rounded, log1p by its alternating Taylor series
//    (Tang, "Table-driven implementation of the logarithm function", ACM TOMS 16(4), 1990).
//  rcp_fast: a seed from the hardware approximation rcp.approx.ftz.f64 refined by one third-order
//    Newton step r' = r + r (e + e^2), e = 1 - y r (the standard iteration for 1/y; see Muller et al.,
//    Handbook of Floating-Point Arithmetic, ch. 5).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cbg {

struct MathTables {
    double exp2_j[256];   // 2^(j/256)
    double log_c[128];    // ln(c_j), c_j = 1 + j/128 (then folded for f >= sqrt(2)... see log_fast)
    double rcp_c[128];    // 1/c_j rounded
};

__device__ __forceinline__ double rcp_fast(double y) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(y));
    double e = fma(-y, r, 1.0);
    double t = fma(e, e, e);
    return fma(r, t, r);
}

// Plain-path switches: the first correct version uses CUDA's own functions everywhere.
__device__ __forceinline__ double exp64(double x) { return exp(x); }
__device__ __forceinline__ double log64(double x) { return log(x); }
__device__ __forceinline__ double div64(double a, double b) { return a / b; }
__device__ __forceinline__ double rcp64(double b) { return 1.0 / b; }

}  // namespace cbg
