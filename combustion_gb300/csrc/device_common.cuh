// Device helpers: bounded bulk-TMA staging of a table blob into shared memory, FP64 bit tricks.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cbg {

// Kernel status bits written to the mechanism's device status word.
enum DeviceStatus : int { kStatusStageTimeout = 1 };

// Spin limits for every wait in these kernels: a wait that runs out sets a status bit and returns.
constexpr long long kWaitLimit = 1ll << 24;

// Polls of stage_to_shared's first wait (one copy per translation unit). Only a test hook lowers it
// (cb_debug_stage_wait_polls, for the plain FP64 kernels): that wait then runs out while the second,
// full-length wait still lets the copy land before the block exits.
static __device__ long long g_stage_wait_polls = kWaitLimit;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    return done != 0;
}

// Copies `bytes` (a multiple of 16, both addresses 16-byte aligned) from global memory into this
// block's shared memory with 1-D bulk TMA (cp.async.bulk) completing on an mbarrier. Returns false,
// with a status bit set, if the copy does not complete within the spin limit.
__device__ inline bool stage_to_shared(void* dst, const void* src, uint32_t bytes, uint64_t* bar, int* status) {
    const uint32_t b = smem_u32(bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
        const uint32_t chunk = 32768;
        for (uint32_t off = 0; off < bytes; off += chunk) {
            uint32_t n = bytes - off < chunk ? bytes - off : chunk;
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(static_cast<char*>(dst) + off)),
                "l"(static_cast<const char*>(src) + off), "r"(n), "r"(b)
                : "memory");
        }
    }
    bool ok = false;
    const long long polls = g_stage_wait_polls;
    for (long long it = 0; it < polls; ++it)
        if (mbar_try_wait(b, 0)) { ok = true; break; }
    if (!ok) {
        atomicOr(status, kStatusStageTimeout);
        // Give copies still in flight a second bounded chance to land before the block exits.
        for (long long it = 0; it < kWaitLimit; ++it)
            if (mbar_try_wait(b, 0)) break;
    }
    __syncthreads();
    return __syncthreads_and(ok);
}

// For non-negative doubles the IEEE bit pattern orders like the value: compares on it cost no FP64
// pipe slot (the FP64 pipe is the bottleneck of every kernel here).
__device__ __forceinline__ long long bits(double x) { return __double_as_longlong(x); }

// min(c, x) for x >= 0 (or NaN: gives c, like f64::min), c a positive constant.
__device__ __forceinline__ double min_pos(double c, double x) { return bits(x) > bits(c) ? c : x; }

// max(0, x) as f64::max(0., x): negative values (and negative zero) give +0.
__device__ __forceinline__ double max0(double x) { return bits(x) < 0 ? 0.0 : x; }

}  // namespace cbg
