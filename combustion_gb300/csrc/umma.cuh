// Blackwell (sm_103a) tensor-core primitives in inline PTX: mbarriers, 2-D TMA tile loads and stores, TMEM
// allocation, tcgen05.mma (kind::f16, BF16 operands, FP32 accumulator in TMEM), tcgen05.commit and
// tcgen05.ld. Operand tiles are K-major or MN-major, with the 128-byte swizzle that TMA writes.
//
// Shared-memory operand tile (one "K block" of 64 BF16 = 128 bytes per row):
//   row r of the tile at byte r * 128; its eight 16-byte chunks j stored at chunk j ^ (r % 8)
//   (CU_TENSOR_MAP_SWIZZLE_128B); 8-row groups 1024 bytes apart; tile base 1024-byte aligned.
// Matrix descriptor (tcgen05 shared-memory descriptor): start address >> 4 in bits 0-13, leading byte
// offset >> 4 in bits 16-29 (unused by swizzled K-major layouts), stride byte offset >> 4 in bits 32-45
// (1024: the distance between 8-row groups), the fixed version value 1 in bits 46-47, base offset 0,
// layout type in bits 61-63 (2 = 128-byte swizzle). A K step of 16 elements inside the 128-byte row
// advances the start address by 32 bytes; the hardware applies the swizzle to the final address.
// MN-major operand tile (the weight-gradient GEMM reads row-major activations with the batch as K): TMA
// boxes of 64 MN elements (128 bytes, the same swizzle) by 64 K rows, box j of the tile holding MN
// elements [64 j, 64 j + 64) at byte 8192 j. Descriptor: leading byte offset = the distance between
// 64-element MN blocks (8192), stride byte offset = the distance between 8-row K groups (1024); a K step
// of 16 rows advances the start address by 2048 bytes (whole swizzle atoms).
// Instruction descriptor (kind::f16): D format in bits 4-5 (1 = F32), A and B formats in bits 7-9 and
// 10-12 (1 = BF16), A and B major in bits 15 and 16 (0 = K-major, 1 = MN-major), N >> 3 in bits 17-22,
// M >> 4 in bits 24-28.
// TMEM accumulator of an M = 128 MMA: row m in lane m, column n in column n (32-bit cells). A warp reads
// the 32 lanes [32 (w % 4), 32 (w % 4) + 32) only, w its index in the block.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"

namespace cbg {
namespace umma {

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Waits for the phase of the given parity to complete; false when the spin limit runs out (the waits of
// one GEMM tile last microseconds: 2^20 polls is far beyond any legitimate wait).
constexpr long long kMmaWaitLimit = 1ll << 20;
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (long long it = 0; it < kMmaWaitLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Generic-proxy writes to shared memory made visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 2-D tiled TMA load into shared memory, completing on an mbarrier (x: inner coordinate in elements,
// a multiple of 64 for the BF16 tiles here, so 16-byte aligned).
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
        : "memory");
}

// 2-D tiled TMA store of a shared-memory box to global memory (bulk async group of this thread); x,
// the inner coordinate in elements, a multiple of 64 BF16 here (16-byte aligned), y >= 0.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, uint32_t src, int x, int y) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(src), "r"(x), "r"(y)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// This thread's bulk stores have read their shared-memory sources (which may then be rewritten).
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// This thread's bulk stores have completed.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;            // leading byte offset (ignored for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset: 8 rows x 128 bytes
    d |= (uint64_t)1 << 46;            // descriptor version
    d |= (uint64_t)2 << 61;            // 128-byte swizzle
    return d;
}

constexpr uint32_t kMnBlockBytes = 64 * 64 * 2;  // one MN-major box: 64 K rows x 128 bytes

__device__ __forceinline__ uint64_t sdesc_sw128_mn(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(kMnBlockBytes >> 4) << 16;  // leading byte offset: next 64-element MN block
    d |= (uint64_t)(1024 >> 4) << 32;           // stride byte offset: next 8 K rows
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N, bool a_mn = false, bool b_mn = false) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, one elected thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// Arrives on the mbarrier once every MMA this thread issued before has completed.
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// One 32-bit column of this thread's TMEM lane, waited for before returning.
__device__ __forceinline__ float tmem_ld1(uint32_t taddr) {
    uint32_t r;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r)
        : "r"(taddr)
        : "memory");
    return __uint_as_float(r);
}

// 32 consecutive 32-bit columns of this thread's TMEM lane, waited for before returning.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int j = 0; j < 32; j++) v[j] = __uint_as_float(r[j]);
}

}  // namespace umma
}  // namespace cbg
