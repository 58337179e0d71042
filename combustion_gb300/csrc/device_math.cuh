// Per-block shared copy of the elementary-function tables and the FP64 functions the kernels call,
// plus the integer-only conversions between FP32 and FP64 used by the mixed-precision form.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fp64_math.cuh"
#include "tables.h"

namespace cbg {

constexpr double kF32Max = 3.4028234663852886e+38;     // f32::MAX as f64
constexpr double kF32MinPos = 1.1754943508222875e-38;  // f32::MIN_POSITIVE as f64

// Dynamic shared memory of every kernel here. It starts with the MathTables (lane-divergent lookups),
// which every table blob carries first: either the whole blob is staged there, or only its first
// kMathBytes.
extern __shared__ __align__(16) uint8_t cb_dsmem[];

__device__ __forceinline__ const MathTables& smath() { return *reinterpret_cast<const MathTables*>(cb_dsmem); }
__device__ __forceinline__ double exp64(double x) { return exp_fast(x, smath().exp2j); }
__device__ __forceinline__ double log64(double x) { return log_fast(x, smath()); }
__device__ __forceinline__ double rcp64(double x) { return rcp_fast(x); }
__device__ __forceinline__ double div64(double a, double b) { return div_fast(a, b); }

// Copies the math tables at the start of a global blob into dynamic shared memory (whole block).
__device__ __forceinline__ void load_math(const uint8_t* gtab) {
    const double* src = reinterpret_cast<const double*>(gtab);
    double* dst = reinterpret_cast<double*>(cb_dsmem);
    for (int q = threadIdx.x; q < kMathBytes / (int)sizeof(double); q += blockDim.x) dst[q] = src[q];
    __syncthreads();
}

// FP64 -> FP32 by truncating the mantissa (error below one FP32 ulp); magnitudes below the FP32 normal
// range give signed zero, above it signed infinity. Integer instructions only: on this GPU the FP64 pipe
// is the scarce unit, and these conversions stay off it.
__device__ __forceinline__ float dbl_to_flt(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    if (e < -126) return __uint_as_float(sign);
    if (e > 127) return __uint_as_float(sign | (((b >> 52) & 0x7ff) == 0x7ff && (b & 0xfffffffffffffull) ? 0x7fc00000u : 0x7f800000u));
    return __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7fffff));
}

// FP32 -> FP64 exactly (subnormal FP32 inputs give zero), integer instructions only.
__device__ __forceinline__ double flt_to_dbl(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    const unsigned e = (u >> 23) & 0xff;
    if (e == 0) return __longlong_as_double((long long)sign);
    const unsigned long long de = e == 0xff ? 0x7ffull : (unsigned long long)(e - 127 + 1023);
    return __longlong_as_double((long long)(sign | (de << 52) | ((unsigned long long)(u & 0x7fffff) << 29)));
}

// exp(x) for an FP32 argument, accurate to a few FP32 ulps, returned as a double so that the result
// keeps the full double range (rate constants overflow FP32). x log2(e) = n + f with the product's
// rounding error recovered by an FMA; 2^f by exp2f, 2^n added to the double's exponent field.
__device__ __forceinline__ double exp_f32x(float x) {
    const float L = 0x1.715476p+0f, Llo = 0x1.4ae0c0p-26f;  // log2(e) = L + Llo
    const float t = x * L;
    const float n = rintf(t);
    const float f = (t - n) + fmaf(x, L, -t) + x * Llo;
    const float p = exp2f(f);
    if (!(fabsf(n) < 1000.0f)) return n > 0.0f ? __longlong_as_double(0x7ff0000000000000ll) : 0.0;
    const unsigned pb = __float_as_uint(p);
    const int e = (int)((pb >> 23) & 0xff) - 127 + (int)n + 1023;
    return __longlong_as_double((long long)(((unsigned long long)e << 52) | ((unsigned long long)(pb & 0x7fffff) << 29)));
}

// ln(d) in FP32 accuracy for a positive normal double of any magnitude.
__device__ __forceinline__ float log_dbl_f32(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    const float m = __uint_as_float(0x3f800000u | (unsigned)((b >> 29) & 0x7fffff));
    return fmaf((float)e, 0x1.62e430p-1f, logf(m));
}

__device__ __forceinline__ float rcp_f32(float y) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y));
    return r;
}

}  // namespace cbg
