// Kernels of the learned transport surrogate (declarations and roles in surrogate_kernels.cuh).
//
// The GEMM is D[M][N] = A[M][K] B[N][K]^T over BF16 operands with an FP32 accumulator in tensor memory:
// 128 x BN output tiles taken in turn by a persistent block per SM (two accumulators in tensor memory,
// so that one tile's epilogue runs under the next tile's MMAs), operands streamed through a ring of
// shared-memory stages by TMA (128-byte swizzle, K-major or MN-major per GEMM: the weight gradients read
// both operands MN-major, the data gradients B), tcgen05.mma issued by one thread, the accumulator read
// back by eight
// epilogue warps (one TMEM lane, i.e. one output row, per thread; two warps per lane quarter, each on
// half of the columns) which apply the layer's element-wise work before anything is written to global
// memory. Every mbarrier wait is bounded: a wait that runs
// out sets a status bit, lets in-flight copies land and the block still frees its tensor memory.
#include <cuda_bf16.h>

#include <cstring>

#include "device_common.cuh"
#include "device_math.cuh"
#include "surrogate_kernels.cuh"
#include "umma.cuh"

namespace cbg {
namespace sur {

// sigmoid(z) = (1 + tanh(z / 2)) / 2 on the hardware tanh (one SFU operation; its ~2^-11 relative
// error stays below the BF16 rounding of the activations). Training and inference use the same form.
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// silu(z) and silu'(z) from one tanh: with h = z / 2 and t = tanh(h), sigmoid(z) = (1 + t) / 2, so
// silu(z) = h (1 + t) and silu'(z) = sigmoid(z) (1 + z (1 - sigmoid(z))) = (1 + t + h (1 - t^2)) / 2.
__device__ __forceinline__ void silu_and_derivative(float z, float& s, float& d) {
    const float h = 0.5f * z, t = tanh_approx(h);
    s = fmaf(h, t, h);
    d = fmaf(0.5f, fmaf(h, fmaf(-t, t, 1.f), t), 0.5f);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}

// 32 values of one row, columns [n, n + 32), as BF16 (64 contiguous bytes).
__device__ __forceinline__ void store_row_bf16(__nv_bfloat16* base, int ld, int row, int n, const float* a) {
    uint4* dst = reinterpret_cast<uint4*>(base + (size_t)row * ld + n);
#pragma unroll
    for (int j = 0; j < 4; j++)
        dst[j] = make_uint4(pack_bf16(a[8 * j], a[8 * j + 1]), pack_bf16(a[8 * j + 2], a[8 * j + 3]),
                            pack_bf16(a[8 * j + 4], a[8 * j + 5]), pack_bf16(a[8 * j + 6], a[8 * j + 7]));
}

// Row r (this lane) of a 32 x 64 BF16 box in the 128-byte swizzle of its TMA store map: columns
// [32 half, 32 half + 32) are the 16-byte chunks 4 half .. 4 half + 3, chunk c of row r stored at
// chunk position c ^ (r % 8) (eight consecutive rows hit eight different bank groups).
__device__ __forceinline__ void stage_row_half(uint8_t* box, int r, int half, const float* a) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int c = 4 * half + j;
        *reinterpret_cast<uint4*>(box + r * 128 + ((c ^ (r & 7)) << 4)) =
            make_uint4(pack_bf16(a[8 * j], a[8 * j + 1]), pack_bf16(a[8 * j + 2], a[8 * j + 3]),
                       pack_bf16(a[8 * j + 4], a[8 * j + 5]), pack_bf16(a[8 * j + 6], a[8 * j + 7]));
    }
}

// SiLU-derivative tiles of the data-gradient epilogue: one 32-row x 64-column box per warp, loaded by TMA
// into the warp's second box one 64-column pair ahead of its use (the first pair of an item while the
// item's MMAs run), completing on the warp's mbarrier.
struct DLoad {
    uint32_t bar, phase;
    bool pending;
};

__device__ __forceinline__ void d_issue(DLoad& dl, const RowMaps& rm, uint8_t* box, int lane, int x, int y) {
    if (lane == 0) {
        umma::mbar_expect_tx(dl.bar, 32 * 128);
        umma::tma_load_2d(smem_u32(box), &rm.dact, dl.bar, x, y);
    }
    dl.pending = true;
}

// The epilogue of one tile for one warp: its 32 rows (TMEM lane quarter q) and its half h of the columns,
// 32 columns per TMEM load. The hidden-layer and data-gradient epilogues (tiles at least 128 wide) put
// their row-major BF16 outputs into 32 x 64 boxes in shared memory and store each box with one TMA store
// (lane 0); the other outputs are written directly.
// (nm0, nn0): the origin of the warp's next item (nm0 < 0: none), where the data-gradient epilogue's
// SiLU-derivative prefetch goes after the item's last pair. False when a wait ran out.
template <int BN, int EPI>
__device__ __forceinline__ bool epilogue(const GemmParams& p, const RowMaps& rm, uint32_t tmem, int warp, int lane,
                                         int m0, int n0, int z, int mt, uint8_t* box0, uint8_t* box1, DLoad& dl,
                                         int nm0, int nn0) {
    constexpr bool kTmaRows = (EPI == kEpiHidden || EPI == kEpiDgrad) && BN >= 128;
    const int q = warp & 3;          // the TMEM lane quarter this warp may read
    const int h = (warp - 2) >> 2;   // and its half of the tile's columns
    const int row = m0 + q * 32 + lane;
    const int trow0 = (p.dyn & kDynTarget) ? *p.row0 : 0;
    float lsum = 0.f;
    uint4 dr[EPI == kEpiDgrad ? 8 : 1];  // the pair's SiLU derivatives (BF16), 16-byte chunks in column order
#pragma unroll 1
    for (int c = h * (BN / 2); c < (h + 1) * (BN / 2); c += 32) {
        const int half = (c >> 5) & 1;  // which half of its 64-column box (BN / 2 is a multiple of 64)
        if constexpr (kTmaRows) {
            if (half == 0) {  // the boxes' previous stores have read them
                if (lane == 0) umma::bulk_wait_read();
                __syncwarp();
            }
        }
        float v[32];
        umma::tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c, v);
        const int n = n0 + c;
        if constexpr (EPI == kEpiPartial) {
            float4* dst = reinterpret_cast<float4*>(p.outf + (size_t)z * p.split_stride + (size_t)row * p.ld_outf + n);
#pragma unroll
            for (int j = 0; j < 8; j++) dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        } else if constexpr (EPI == kEpiLinear) {
            float4* dst = reinterpret_cast<float4*>(p.outf + (size_t)row * p.ld_outf + n);
            const float4* b4 = reinterpret_cast<const float4*>(p.bias + n);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const float4 b = b4[j];
                dst[j] = make_float4(v[4 * j] + b.x, v[4 * j + 1] + b.y, v[4 * j + 2] + b.z, v[4 * j + 3] + b.w);
            }
        } else if constexpr (EPI == kEpiHidden) {  // a = silu(z); v = silu'(z) for the backward
            const float4* b4 = reinterpret_cast<const float4*>(p.bias + n);  // 16-byte aligned: n % 32 == 0
            float a[32];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const float4 b = b4[j];
                const float bb[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                for (int e = 0; e < 4; e++) silu_and_derivative(v[4 * j + e] + bb[e], a[4 * j + e], v[4 * j + e]);
            }
            if constexpr (kTmaRows) {
                if (p.out) stage_row_half(box0, lane, half, v);
                stage_row_half(box1, lane, half, a);
            } else {
                if (p.out) store_row_bf16(p.out, p.ld_out, row, n, v);
                store_row_bf16(p.out2, p.ld_out2, row, n, a);
            }
        } else if constexpr (EPI == kEpiLoss) {
            const float4* t4 = reinterpret_cast<const float4*>(p.target + (size_t)(trow0 + row) * p.ld_target + n);
            const float4* b4 = reinterpret_cast<const float4*>(p.bias + n);
            float a[32];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const float4 b = b4[j], t = t4[j];
                const float bb[4] = {b.x, b.y, b.z, b.w}, tt[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int k = 4 * j + e;
                    const float d = (n + k < p.n_valid) ? (v[k] + bb[e]) - tt[e] : 0.f;
                    lsum = fmaf(d, d, lsum);
                    a[k] = d * p.grad_scale;
                }
            }
            store_row_bf16(p.out, p.ld_out, row, n, a);
        } else if constexpr (EPI == kEpiDgrad) {
            static_assert(BN >= 128, "data gradients stage through 64-column boxes");
            if (half == 0) {  // this pair's SiLU derivatives have landed: into registers, then the next pair's load
                if (!__all_sync(0xffffffffu, umma::mbar_wait(dl.bar, dl.phase))) return false;
                dl.phase ^= 1;
                dl.pending = false;
#pragma unroll
                for (int j = 0; j < 8; j++)
                    dr[j] = *reinterpret_cast<const uint4*>(box1 + lane * 128 + ((j ^ (lane & 7)) << 4));
                umma::fence_async_shared();  // the reads above come before the next TMA write of the box
                __syncwarp();
                if (c + 64 < (h + 1) * (BN / 2)) d_issue(dl, rm, box1, lane, n0 + c + 64, m0 + q * 32);
                else if (nm0 >= 0) d_issue(dl, rm, box1, lane, nn0 + h * (BN / 2), nm0 + q * 32);
            }
            float a[32];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const uint4 w = half ? dr[4 + j] : dr[j];
                const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const __nv_bfloat162 b = *reinterpret_cast<const __nv_bfloat162*>(&ws[e]);
                    const int k = 8 * j + 2 * e;
                    a[k] = v[k] * __low2float(b);
                    a[k + 1] = v[k + 1] * __high2float(b);
                }
            }
            stage_row_half(box0, lane, half, a);
        }
        if constexpr (kTmaRows) {
            if (half == 1) {  // the box is complete: one TMA store per output
                umma::fence_async_shared();
                __syncwarp();
                if (lane == 0) {
                    const int x = n0 + c - 32, y = m0 + q * 32;
                    if (EPI == kEpiHidden) {
                        if (p.out) umma::tma_store_2d(&rm.out, smem_u32(box0), x, y);
                        umma::tma_store_2d(&rm.out2, smem_u32(box1), x, y);
                    } else {
                        umma::tma_store_2d(&rm.out, smem_u32(box0), x, y);
                    }
                    umma::bulk_commit();
                }
            }
        }
    }
    if constexpr (EPI == kEpiPartial) {  // bias-gradient partials, after the split's weight partials
        float* bp = p.outf + (size_t)z * p.split_stride + (size_t)p.M * p.ld_outf;
        if (p.bias_part == kBiasRows && h == 0 && n0 == 0)  // every column is the row sum: read one
            bp[row] = umma::tmem_ld1(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)BN);
        if (p.bias_part == kBiasCols && q == 0 && m0 == 0) {  // every row is the column sums: row 0 (lane 0)
#pragma unroll 1
            for (int c = h * (BN / 2); c < (h + 1) * (BN / 2); c += 32) {
                float v[32];
                umma::tmem_ld32(tmem + (uint32_t)(BN + c), v);
                if (lane == 0) {
                    float4* dst = reinterpret_cast<float4*>(bp + n0 + c);
#pragma unroll
                    for (int j = 0; j < 8; j++) dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                }
            }
        }
    }
    if constexpr (EPI == kEpiLoss) {  // one partial per warp: no barrier among the epilogue warps
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
        if (lane == 0) p.loss[mt * kEpiWarps + h * 4 + q] = lsum;
    }
    return true;
}

// Persistent: block b takes work items b, b + gridDim.x, ... (item = row tile + Mt (column tile + Nt
// split)). The ring's stage index and phase run on across items, and the accumulator alternates between
// two TMEM buffers, so that the producer and the MMA issuer start the next item while the epilogue
// warps drain the last one (acc_full[b]: MMAs of buffer b done; acc_empty[b]: its epilogue done).
// The weight-gradient items (kEpiPartial) read both operands MN-major: A = dZ^T and B = A_in^T straight
// from the row-major activations [rows][width] (the batch is K), 64 x 64 boxes (2 for A, BN / 64 for B).
// With bias_part, each K step also multiplies by a tile of ones into the TMEM columns after the
// accumulator: kBiasRows A times 16 columns of ones (N = 16, B K-major), each column of the product the
// row sums of A over the split; kBiasCols 128 rows of ones (A K-major) times B, each row the column sums
// of B^T. These items use one accumulator (a block takes one item on a full GPU).
template <int BN, int EPI>
__global__ void __launch_bounds__(kGemmThreads, 1)
    gemm_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, const GemmParams p,
                const __grid_constant__ RowMaps rm) {
    constexpr bool kMN = EPI == kEpiPartial;                  // A and B MN-major
    constexpr bool kBMN = kMN || EPI == kEpiDgrad;            // B MN-major (data gradients: B = W row-major)
    constexpr uint32_t kA = kBM * 128, kB = BN * 128, kStage = kA + kB;
    constexpr int STAGES = kGemmRing / (int)kStage;
    static_assert(STAGES >= 2, "operand ring needs two stages");
    constexpr int kBufs = kMN ? 1 : 2;  // accumulators in TMEM
    constexpr uint32_t kCols = 2u * BN;  // two accumulators, or one and the bias product (at most BN columns)
    extern __shared__ uint8_t dsm[];
    __shared__ uint64_t full[STAGES], empty[STAGES], acc_full[2], acc_empty[2], mma_done, zbar[kEpiWarps];
    __shared__ uint32_t tmem_s;
    const uint32_t base = (smem_u32(dsm) + 1023u) & ~1023u;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int Mt = p.M / kBM, Nt = p.N / BN;
    const int n_items = Mt * Nt * p.splits;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            umma::mbar_init(smem_u32(&full[s]), 1);
            umma::mbar_init(smem_u32(&empty[s]), 1);
        }
        for (int b = 0; b < 2; b++) {
            umma::mbar_init(smem_u32(&acc_full[b]), 1);
            umma::mbar_init(smem_u32(&acc_empty[b]), kEpiWarps);
        }
        umma::mbar_init(smem_u32(&mma_done), 1);
        for (int e = 0; e < kEpiWarps; e++) umma::mbar_init(smem_u32(&zbar[e]), 1);
        umma::fence_mbar_init();
    }
    if (warp == 1) {
        umma::tmem_alloc(smem_u32(&tmem_s), kCols);
        umma::tmem_relinquish();
    }
    const uint32_t ones = base + kGemmRing;  // weight-gradient items: 128 x 64 BF16 ones, K-major
    if (kMN && p.bias_part && warp >= 2) {
        uint4* o = reinterpret_cast<uint4*>(dsm + (ones - smem_u32(dsm)));
        for (int i = threadIdx.x - 64; i < kOnesTile / 16; i += kGemmThreads - 64)
            o[i] = make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
        umma::fence_async_shared();  // generic writes before the tensor core's reads
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_s;
    bool ok = true;
    if (warp == 0) {
        if (lane == 0) {  // TMA producer
            const int off = p.dyn ? *p.row0 : 0;
            int it = 0;  // k blocks issued by this block, over all its items
            for (int w = blockIdx.x; w < n_items && ok; w += gridDim.x) {
                const int mt = w % Mt, nt = (w / Mt) % Nt, z = w / (Mt * Nt);
                const int kb0 = (int)(((long long)z * p.k_blocks) / p.splits);
                const int nkb = (int)(((long long)(z + 1) * p.k_blocks) / p.splits) - kb0;
                const int a_off = (p.dyn & kDynAy) ? off : 0, b_off = (p.dyn & kDynBx) ? off : 0;
                for (int i = 0; i < nkb; i++, it++) {
                    const int s = it % STAGES;
                    if (it >= STAGES && !umma::mbar_wait(smem_u32(&empty[s]), ((it / STAGES) & 1) ^ 1)) {
                        ok = false;
                        break;
                    }
                    const uint32_t bar = smem_u32(&full[s]), sa = base + (uint32_t)s * kStage;
                    const int kx = (kb0 + i) * kBK;
                    umma::mbar_expect_tx(bar, kStage);
                    // MN-major: x = MN element (a multiple of 64), y = K row; K-major: x = K element, y = row
                    if constexpr (kMN) {
#pragma unroll
                        for (int j = 0; j < kBM / 64; j++)
                            umma::tma_load_2d(sa + j * umma::kMnBlockBytes, &ta, bar, mt * kBM + 64 * j, kx + a_off);
                    } else {
                        umma::tma_load_2d(sa, &ta, bar, kx, mt * kBM + a_off);
                    }
                    if constexpr (kBMN) {
#pragma unroll
                        for (int j = 0; j < BN / 64; j++)
                            umma::tma_load_2d(sa + kA + j * umma::kMnBlockBytes, &tb, bar, nt * BN + 64 * j,
                                              kx + b_off);
                    } else {
                        umma::tma_load_2d(sa + kA, &tb, bar, kx, nt * BN);
                    }
                }
            }
            if (!ok)  // let the copies already issued land before the block exits
                for (int i = it > STAGES ? it - STAGES : 0; i < it; i++)
                    umma::mbar_wait(smem_u32(&full[i % STAGES]), (i / STAGES) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            constexpr uint32_t idesc = umma::idesc_bf16_f32(kBM, BN, kMN, kBMN);
            constexpr uint32_t idesc_rows = umma::idesc_bf16_f32(kBM, 16, true, false);  // A (MN) x ones
            constexpr uint32_t idesc_cols = umma::idesc_bf16_f32(kBM, BN, false, true);  // ones x B (MN)
            const int bias = kMN ? p.bias_part : kBiasNone;
            int it = 0, t = 0;
            for (int w = blockIdx.x; w < n_items && ok; w += gridDim.x, t++) {
                const int z = w / (Mt * Nt);
                const int nkb = (int)(((long long)(z + 1) * p.k_blocks) / p.splits) -
                                (int)(((long long)z * p.k_blocks) / p.splits);
                const int b = t % kBufs;
                // buffer b is free once the epilogue of item t - kBufs has read it
                if (t >= kBufs && !umma::mbar_wait(smem_u32(&acc_empty[b]), ((t / kBufs) & 1) ^ 1)) {
                    ok = false;
                    break;
                }
                umma::fence_after_sync();
                const uint32_t acc = tmem + (uint32_t)(b * BN);
                for (int i = 0; i < nkb; i++, it++) {
                    const int s = it % STAGES;
                    if (!umma::mbar_wait(smem_u32(&full[s]), (it / STAGES) & 1)) {
                        ok = false;
                        break;
                    }
                    umma::fence_after_sync();
                    const uint32_t sa = base + (uint32_t)s * kStage, sb = sa + kA;
#pragma unroll
                    for (int k = 0; k < kBK / 16; k++) {
                        if constexpr (kMN) {  // 16 K rows = two 8-row swizzle atoms per step
                            const uint64_t ad = umma::sdesc_sw128_mn(sa + 2048u * k);
                            const uint64_t bd = umma::sdesc_sw128_mn(sb + 2048u * k);
                            umma::mma_bf16(acc, ad, bd, idesc, (i | k) != 0);
                            if (bias == kBiasRows)
                                umma::mma_bf16(acc + (uint32_t)BN, ad, umma::sdesc_sw128(ones + 32u * k), idesc_rows,
                                               (i | k) != 0);
                            else if (bias == kBiasCols)
                                umma::mma_bf16(acc + (uint32_t)BN, umma::sdesc_sw128(ones + 32u * k), bd, idesc_cols,
                                               (i | k) != 0);
                        } else if constexpr (kBMN) {  // A: 32 bytes of the row per step; B: two atoms
                            umma::mma_bf16(acc, umma::sdesc_sw128(sa + 32u * k), umma::sdesc_sw128_mn(sb + 2048u * k),
                                           idesc, (i | k) != 0);
                        } else {  // 16 K elements = 32 bytes of the 128-byte row per step
                            umma::mma_bf16(acc, umma::sdesc_sw128(sa + 32u * k), umma::sdesc_sw128(sb + 32u * k),
                                           idesc, (i | k) != 0);
                        }
                    }
                    umma::mma_commit(smem_u32(&empty[s]));  // frees the stage once these MMAs are done
                }
                if (ok) umma::mma_commit(smem_u32(&acc_full[b]));  // the item's MMAs have completed
            }
            // every MMA issued above has completed before tensor memory is freed
            umma::mma_commit(smem_u32(&mma_done));
            umma::mbar_wait(smem_u32(&mma_done), 0);
        }
    } else {  // epilogue warps (each wait's outcome made warp-uniform: tcgen05.ld needs the whole warp)
        uint8_t* after_ring = dsm + (base - smem_u32(dsm)) + kGemmRing;
        uint8_t* box0 = after_ring + (warp - 2) * 2 * kStageBox;  // 1024-byte aligned
        uint8_t* box1 = box0 + kStageBox;
        DLoad dl{smem_u32(&zbar[warp - 2]), 0u, false};
        const int q = warp & 3, h = (warp - 2) >> 2;
        if (EPI == kEpiDgrad && (int)blockIdx.x < n_items)  // the first pair of the first item
            d_issue(dl, rm, box1, lane, ((blockIdx.x / Mt) % Nt) * BN + h * (BN / 2), (blockIdx.x % Mt) * kBM + q * 32);
        int t = 0;
        for (int w = blockIdx.x; w < n_items; w += gridDim.x, t++) {
            const int mt = w % Mt, nt = (w / Mt) % Nt, z = w / (Mt * Nt);
            const int b = t % kBufs;
            ok = __all_sync(0xffffffffu, umma::mbar_wait(smem_u32(&acc_full[b]), (t / kBufs) & 1));
            if (!ok) break;
            umma::fence_after_sync();
            const int w2 = w + (int)gridDim.x;
            const bool more = w2 < n_items;
            ok = epilogue<BN, EPI>(p, rm, tmem + (uint32_t)(b * BN), warp, lane, mt * kBM, nt * BN, z, mt, box0, box1,
                                   dl, more ? (w2 % Mt) * kBM : -1, more ? ((w2 / Mt) % Nt) * BN : 0);
            if (!ok) break;
            umma::fence_before_sync();
            __syncwarp();
            if (lane == 0) umma::mbar_arrive(smem_u32(&acc_empty[b]));
        }
        if (dl.pending && lane == 0) umma::mbar_wait(dl.bar, dl.phase);  // a prefetch still in flight lands
        if (lane == 0) umma::bulk_wait_all();  // this warp's TMA stores have completed
    }
    if (!ok) atomicOr(p.status, kStatusGemmTimeout);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        umma::fence_after_sync();
        umma::tmem_dealloc(tmem, kCols);
    }
}

int sm_count_g() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

template <int BN, int EPI>
cudaError_t launch_gemm(const CUtensorMap& a, const CUtensorMap& b, const GemmParams& p, const RowMaps& rm,
                        cudaStream_t st) {
    const int items = (p.M / kBM) * (p.N / BN) * p.splits;  // one block per SM at most, persistent
    gemm_kernel<BN, EPI><<<items < sm_count_g() ? items : sm_count_g(), kGemmThreads, kGemmSmem, st>>>(a, b, p, rm);
    return cudaGetLastError();
}

template <int EPI>
cudaError_t gemm_bn(int BN, const CUtensorMap& a, const CUtensorMap& b, const GemmParams& p, const RowMaps& rm,
                    cudaStream_t st) {
    switch (BN) {
    case 64:  // the data-gradient epilogue stages 64-column boxes per half tile: BN >= 128 only
        if constexpr (EPI == kEpiDgrad) return cudaErrorInvalidValue;
        else return launch_gemm<64, EPI>(a, b, p, rm, st);
    case 128: return launch_gemm<128, EPI>(a, b, p, rm, st);
    case 256: return launch_gemm<256, EPI>(a, b, p, rm, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int EPI>
cudaError_t setup_epi() {
    cudaError_t e = cudaSuccess;
    if constexpr (EPI != kEpiDgrad)
        e = cudaFuncSetAttribute(gemm_kernel<64, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(gemm_kernel<128, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(gemm_kernel<256, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
    return e;
}

cudaError_t gemm_setup() {
    cudaError_t e = setup_epi<kEpiPartial>();
    if (e == cudaSuccess) e = setup_epi<kEpiHidden>();
    if (e == cudaSuccess) e = setup_epi<kEpiLoss>();
    if (e == cudaSuccess) e = setup_epi<kEpiDgrad>();
    if (e == cudaSuccess) e = setup_epi<kEpiLinear>();
    return e;
}

cudaError_t gemm(int BN, int epi, const CUtensorMap& a, const CUtensorMap& b, const GemmParams& p, cudaStream_t st,
                 const CUtensorMap* out_map, const CUtensorMap* out2_map, const CUtensorMap* dact_map) {
    if (p.M % kBM || p.N % BN || p.splits < 1 || p.splits > p.k_blocks) return cudaErrorInvalidValue;
    if (epi == kEpiDgrad && (BN < 128 || !dact_map || !out_map)) return cudaErrorInvalidValue;
    if (epi == kEpiPartial) {
        const long long nb = p.bias_part == kBiasRows ? p.M : p.bias_part == kBiasCols ? p.N : 0;
        if (p.split_stride < (long long)p.M * p.ld_outf + nb || (p.bias_part && p.ld_outf != p.N) ||
            p.bias_part < kBiasNone || p.bias_part > kBiasCols)
            return cudaErrorInvalidValue;
    }
    RowMaps rm;
    std::memset(&rm, 0, sizeof rm);
    if (BN >= 128 && (epi == kEpiHidden || epi == kEpiDgrad)) {  // these epilogues store through the maps
        if ((p.out && !out_map) || (epi == kEpiHidden && !out2_map)) return cudaErrorInvalidValue;
        if (out_map) rm.out = *out_map;
        if (out2_map) rm.out2 = *out2_map;
    }
    if (epi == kEpiDgrad) rm.dact = *dact_map;
    switch (epi) {
    case kEpiPartial: return gemm_bn<kEpiPartial>(BN, a, b, p, rm, st);
    case kEpiHidden: return gemm_bn<kEpiHidden>(BN, a, b, p, rm, st);
    case kEpiLoss: return gemm_bn<kEpiLoss>(BN, a, b, p, rm, st);
    case kEpiDgrad: return gemm_bn<kEpiDgrad>(BN, a, b, p, rm, st);
    case kEpiLinear: return gemm_bn<kEpiLinear>(BN, a, b, p, rm, st);
    default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------------------------------------------
// Weight-gradient partials summed over the K splits in a fixed order (deterministic gradients): a block
// covers 32 groups of four consecutive outputs (16-byte loads) with eight threads per group, thread g
// summing splits g, g + 8, ... in order; the eight sums are then added in g order. Many threads per
// output keep enough loads in flight: the partials are L2-resident and the sum is latency-bound. The
// outputs of one split are its M x N weight partials, then (nb > 0) its nb bias partials.
constexpr int kRedOut4 = 32, kRedGroups = 8;
__global__ void __launch_bounds__(kRedOut4 * kRedGroups)
    reduce_partials_kernel(const float* __restrict__ ws, int splits, long long stride4, int M, int N, int transpose,
                           float* __restrict__ grad_w, int nb, float* __restrict__ grad_b) {
    __shared__ float4 part[kRedGroups][kRedOut4];
    const size_t MN = (size_t)M * N, n4 = (MN + nb) / 4;
    const int o = threadIdx.x % kRedOut4, g = threadIdx.x / kRedOut4;
    const size_t i = (size_t)blockIdx.x * kRedOut4 + o;
    const float4* w4 = reinterpret_cast<const float4*>(ws);
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < n4) {
        int z = g;
        for (; z + 3 * kRedGroups < splits; z += 4 * kRedGroups) {
            float4 v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = w4[(size_t)(z + u * kRedGroups) * stride4 + i];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                s.x += v[u].x;
                s.y += v[u].y;
                s.z += v[u].z;
                s.w += v[u].w;
            }
        }
        for (; z < splits; z += kRedGroups) {
            const float4 v = w4[(size_t)z * stride4 + i];
            s.x += v.x;
            s.y += v.y;
            s.z += v.z;
            s.w += v.w;
        }
    }
    part[g][o] = s;
    __syncthreads();
    if (g == 0 && i < n4) {
        float4 t = part[0][o];
        for (int k = 1; k < kRedGroups; k++) {
            t.x += part[k][o].x;
            t.y += part[k][o].y;
            t.z += part[k][o].z;
            t.w += part[k][o].w;
        }
        const float r[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
        for (int h = 0; h < 4; h++) {
            const size_t e = 4 * i + h;
            if (e >= MN) {
                grad_b[e - MN] = r[h];
            } else {
                const size_t m = e / N, n = e % N;
                grad_w[transpose ? n * M + m : e] = r[h];
            }
        }
    }
}

cudaError_t reduce_partials(const float* ws, int splits, long long stride, int M, int N, bool transpose, float* grad_w,
                            int nb, float* grad_b, cudaStream_t st) {
    const size_t MN = (size_t)M * N;
    if (MN % 4 || nb % 4 || stride % 4 || stride < (long long)(MN + nb) || (nb && !grad_b)) return cudaErrorInvalidValue;
    const size_t blocks = ((MN + nb) / 4 + kRedOut4 - 1) / kRedOut4;
    reduce_partials_kernel<<<(unsigned)blocks, kRedOut4 * kRedGroups, 0, st>>>(ws, splits, stride / 4, M, N,
                                                                             transpose ? 1 : 0, grad_w, nb, grad_b);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------------
// Adam on the FP32 master parameters (weights of every layer, then biases), writing the BF16 weights that
// the GEMMs read (row-major [out][in]: the forward's K-major B, the data gradient's MN-major B). The step counter lives on the device (CUDA-graph replays).
__device__ __forceinline__ void write_bf16_weight(const AdamArgs& a, long long i, float w) {
    int l = 0;
    while (l + 1 < a.n_layers && i >= a.L[l + 1].w_off) l++;
    const AdamLayer& L = a.L[l];
    L.W[i - L.w_off] = __float2bfloat16_rn(w);
}

__global__ void adam_kernel(const AdamArgs a) {
    const int t = *a.step + 1;
    const float frac = a.total_steps > 1 ? fminf(1.f, (float)(t - 1) / (float)(a.total_steps - 1)) : 1.f;
    const float lr = a.lr_final + 0.5f * (a.lr - a.lr_final) * (1.f + cospif(frac));
    const float bc1 = 1.f - powf(a.b1, (float)t), bc2 = 1.f - powf(a.b2, (float)t);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n_params;
         i += (long long)gridDim.x * blockDim.x) {
        const float g = a.g[i];
        const float m = a.b1 * a.m[i] + (1.f - a.b1) * g;
        const float v = a.b2 * a.v[i] + (1.f - a.b2) * g * g;
        a.m[i] = m;
        a.v[i] = v;
        const float w = a.p[i] - lr * (m / bc1) / (sqrtf(v / bc2) + a.eps);
        a.p[i] = w;
        if (i < a.n_weights) write_bf16_weight(a, i, w);
    }
}

cudaError_t adam(const AdamArgs& a, cudaStream_t st) {
    adam_kernel<<<592, 256, 0, st>>>(a);
    return cudaGetLastError();
}

__global__ void cast_weights_kernel(const AdamArgs a) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n_weights;
         i += (long long)gridDim.x * blockDim.x)
        write_bf16_weight(a, i, a.p[i]);
}

cudaError_t cast_weights(const AdamArgs& a, cudaStream_t st) {
    cast_weights_kernel<<<592, 256, 0, st>>>(a);
    return cudaGetLastError();
}

// Mean squared error of the step (fixed summation order), next step number and batch position.
__global__ void finish_step_kernel(const float* loss_part, int n_part, float norm, float* losses, int* step,
                                   int* row0, int batch, int n_batches) {
    __shared__ float part[256];
    float s = 0.f;
    for (int i = threadIdx.x; i < n_part; i += 256) s += loss_part[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int t = *step;
        if (losses) losses[t] = part[0] * norm;
        *step = t + 1;
        *row0 = ((t + 1) % n_batches) * batch;
    }
}

cudaError_t finish_step(const float* loss_part, int n_part, float norm, float* losses, int* step, int* row0,
                        int batch, int n_batches, cudaStream_t st) {
    finish_step_kernel<<<1, 256, 0, st>>>(loss_part, n_part, norm, losses, step, row0, batch, n_batches);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------------
// Seeded cells on the device, the same counter-based draws as the host generator
// (combustion_gb300/synthetic.py): SplitMix64 uniforms per (seed, stream, counter), Box-Muller normals,
// Marsaglia-Tsang Gamma(alpha + 1) boosted by U^(1/alpha), mole fractions from normalised Gamma draws.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform_(uint64_t key, int stream, uint64_t idx) {
    const uint64_t base = key + ((uint64_t)(stream & 0xFFFFFF) << 40);
    return (double)(mix64(base + idx * 0x9E3779B97F4A7C15ull) >> 11) * (1.0 / 9007199254740992.0);
}
__device__ double normal_(uint64_t key, int stream, uint64_t idx) {
    const double u1 = uniform_(key, stream, 2 * idx), u2 = uniform_(key, stream, 2 * idx + 1);
    return sqrt(-2.0 * log1p(-u1)) * cos(2.0 * 3.141592653589793 * u2);
}
__device__ double gamma_(double alpha, uint64_t key, int stream, uint64_t idx) {
    const double a = alpha < 1.0 ? alpha + 1.0 : alpha;
    const double d = a - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * d);
    double out = 0.0;
    for (int rnd = 0; rnd < 64; rnd++) {  // bounded rejection loop (acceptance is above 95 %)
        const uint64_t sub = idx * 64 + rnd;
        const double x = normal_(key, stream, sub);
        const double u = uniform_(key, stream + 1, sub);
        const double b = 1.0 + c * x;
        const double v = b * b * b;
        if (v > 0 && log(fmax(u, 1e-300)) < 0.5 * x * x + d - d * v + d * log(v)) {
            out = d * v;
            break;
        }
    }
    if (alpha < 1.0) out *= pow(uniform_(key, stream + 2, idx), 1.0 / alpha);
    return out;
}

__global__ void generate_cells_kernel(const CellGenArgs a) {
    const uint64_t key = mix64(a.seed);
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.n; c += (size_t)gridDim.x * blockDim.x) {
        const uint64_t idx = a.offset + c;
        const double T = a.T_lo + (a.T_hi - a.T_lo) * uniform_(key, 1, idx);
        const double P = a.fixed_pressure ? a.P_fixed
                                          : 101325.0 * exp(a.lnP_lo + (a.lnP_hi - a.lnP_lo) * uniform_(key, 2, idx));
        const double pressure_R = P / a.R;
        double sum = 0.0;  // the bulk species' draw only enters the sum
        for (int k = 0; k < a.K; k++) {
            const double g = fmax(gamma_(a.alpha, key, 16 + 4 * k, idx), 1e-300);
            sum += g;
            if (k < a.K - 1) a.out[4 + k][c] = g;
        }
        const double total = pressure_R * 1.0 / T;
        for (int k = 0; k < a.K - 1; k++) a.out[4 + k][c] = a.out[4 + k][c] / sum * total;
        a.out[0][c] = pressure_R;
        a.out[1][c] = 1.0 / pressure_R;
        a.out[2][c] = T;
        a.out[3][c] = 1.0;
    }
}

cudaError_t generate_cells(const CellGenArgs& a, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    size_t grid = (a.n + 127) / 128;
    if (grid > 152 * 16) grid = 152 * 16;
    generate_cells_kernel<<<(unsigned)grid, 128, 0, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------------
// Order-preserving map of floats to ints (for atomic min / max).
__device__ __forceinline__ int ordered(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}

// Network inputs of one cell (rates layout): log(T/T0), log(P / 1 atm), mole fractions X_0 .. X_{K-1}
// with the bulk fraction from the total amount N = (P/R V) / T like the transport kernel's. FP32
// throughout (the inputs converted with integer instructions): the features end as BF16, and FP64
// arithmetic here would make the kernel FP64-pipe bound. Features come in order, so `s` accumulates the
// amounts read so far and the bulk (the last feature) is N - s: every input is read once.
__device__ __forceinline__ float raw_feature(const FeatureArgs& a, size_t c, int j, float logT, float logP,
                                             float N, float rN, float& s) {
    if (j == 0) return logT;
    if (j == 1) return logP;
    const int k = j - 2;
    if (k < a.K - 1) {
        const float x = dbl_to_flt(a.in[4 + k][c]);
        s += x;
        return x * rN;
    }
    return (N - s) * rN;
}

__global__ void features_kernel(const FeatureArgs a) {
    __shared__ int lo_s[kMaxOut], hi_s[kMaxOut];
    const bool hull = a.hull_lo != nullptr;
    if (hull) {
        for (int j = threadIdx.x; j < a.n_feat; j += blockDim.x) {
            lo_s[j] = 0x7fffffff;
            hi_s[j] = (int)0x80000000;
        }
        __syncthreads();
    }
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.rows; c += (size_t)gridDim.x * blockDim.x) {
        __nv_bfloat16* xr = a.X + (a.row0 + c) * a.n_in;
        if (c >= a.n) {  // padding row
            for (int j = 0; j < a.n_in; j += 8) *reinterpret_cast<uint4*>(xr + j) = make_uint4(0, 0, 0, 0);
            continue;
        }
        const float pR = dbl_to_flt(a.uniform_pressure ? a.in[0][0] : a.in[0][c]);
        const float T = dbl_to_flt(a.in[2][c]), V = dbl_to_flt(a.in[3][c]);
        const float N = pR * V / T, rN = 1.f / N;
        float s = 0.f;
        const float logT = logf(T / (float)a.T0), logP = logf(pR * (float)a.R_over_P0);
        bool inside = true;
        for (int j0 = 0; j0 < a.n_in; j0 += 8) {
            float x[8];
#pragma unroll
            for (int h = 0; h < 8; h++) {
                const int j = j0 + h;
                float f = 0.f;
                if (j < a.n_feat) {
                    f = raw_feature(a, c, j, logT, logP, N, rN, s);
                    if (a.raw) a.raw[c * a.n_feat + j] = f;
                    if (a.lo) inside &= (f >= a.lo[j]) & (f <= a.hi[j]);
                    if (hull) {
                        atomicMin(&lo_s[j], ordered(f));
                        atomicMax(&hi_s[j], ordered(f));
                    }
                    f = (f - a.mean[j]) * a.rstd[j];
                }
                x[h] = f;
            }
            *reinterpret_cast<uint4*>(xr + j0) =
                make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], x[5]), pack_bf16(x[6], x[7]));
        }
        if (a.outside) a.outside[a.idx_base + c] = inside ? 0 : 1;
        if (a.fail_idx) {
            const uint32_t cell = a.idx_base + (uint32_t)c;
            if (!inside) {
                a.fail_idx[atomicAdd(a.fail_count, 1u)] = cell;
            } else if (a.audit_stride && cell % a.audit_stride == a.audit_phase) {
                const uint32_t slot = atomicAdd(a.audit_count, 1u);
                if (slot < a.audit_cap) a.audit_idx[slot] = cell;
            }
        }
    }
    if (hull) {
        __syncthreads();
        for (int j = threadIdx.x; j < a.n_feat; j += blockDim.x) {
            atomicMin(&a.hull_lo[j], lo_s[j]);
            atomicMax(&a.hull_hi[j], hi_s[j]);
        }
    }
}

cudaError_t features(const FeatureArgs& a, cudaStream_t st) {
    if (a.rows == 0) return cudaSuccess;
    size_t grid = (a.rows + 127) / 128;
    if (grid > 152 * 8) grid = 152 * 8;
    features_kernel<<<(unsigned)grid, 128, 0, st>>>(a);
    return cudaGetLastError();
}

// Training targets: normalised logs of the plain kernel's transport outputs.
__global__ void targets_kernel(const TargetArgs a) {
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.n; c += (size_t)gridDim.x * blockDim.x) {
        float* y = a.Y + (a.row0 + c) * a.n_out;
        for (int j0 = 0; j0 < a.n_out; j0 += 4) {
            float t[4];
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const int j = j0 + h;
                float v = 0.f;
                if (j < a.n_feat) {
                    const float l = (float)log(a.out[j][c]);
                    if (a.raw) a.raw[c * a.n_feat + j] = l;
                    v = (l - a.mean[j]) * a.rstd[j];
                }
                t[h] = v;
            }
            *reinterpret_cast<float4*>(y + j0) = make_float4(t[0], t[1], t[2], t[3]);
        }
    }
}

cudaError_t targets(const TargetArgs& a, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    size_t grid = (a.n + 127) / 128;
    if (grid > 152 * 8) grid = 152 * 8;
    targets_kernel<<<(unsigned)grid, 128, 0, st>>>(a);
    return cudaGetLastError();
}

// Network outputs to transport properties: out_j = exp(mean_j + std_j y_j) in the plain kernel's layout.
__global__ void outputs_kernel(const OutputArgs a) {
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.n; c += (size_t)gridDim.x * blockDim.x) {
        const float* y = a.Y + c * a.ldY;
        for (int j0 = 0; j0 < a.n_feat; j0 += 4) {
            const float4 v = *reinterpret_cast<const float4*>(y + j0);
            const float vs[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const int j = j0 + h;
                if (j < a.n_feat) a.out[j][c] = (double)__expf(fmaf(a.std[j], vs[h], a.mean[j]));
            }
        }
    }
}

cudaError_t outputs(const OutputArgs& a, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    size_t grid = (a.n + 127) / 128;
    if (grid > 152 * 8) grid = 152 * 8;
    outputs_kernel<<<(unsigned)grid, 128, 0, st>>>(a);
    return cudaGetLastError();
}

// The ensemble: outputs exp((l_a + l_b) / 2) of the two networks' log outputs, the disagreement
// max_j |l_a,j - l_b,j| as the cell's error estimate, and the gate lists.
__global__ void combine_kernel(const CombineArgs a) {
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.n; c += (size_t)gridDim.x * blockDim.x) {
        const float* ya = a.Ya + c * a.ldY;
        const float* yb = a.Yb + c * a.ldY;
        float d = 0.f;
        for (int j0 = 0; j0 < a.n_feat; j0 += 4) {
            const float4 va = *reinterpret_cast<const float4*>(ya + j0);
            const float4 vb = *reinterpret_cast<const float4*>(yb + j0);
            const float as[4] = {va.x, va.y, va.z, va.w}, bs[4] = {vb.x, vb.y, vb.z, vb.w};
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const int j = j0 + h;
                if (j < a.n_feat) {
                    const float la = fmaf(a.std_a[j], as[h], a.mean_a[j]);
                    const float lb = fmaf(a.std_b[j], bs[h], a.mean_b[j]);
                    d = fmaxf(d, fabsf(la - lb));
                    a.out[j][c] = (double)__expf(0.5f * (la + lb));
                }
            }
        }
        const uint32_t cell = a.idx_base + (uint32_t)c;
        if (a.disagreement) a.disagreement[cell] = d;
        if (a.fail_idx) {
            const bool out = (a.outside && a.outside[cell]) || !(d <= a.threshold);
            if (out) {
                a.fail_idx[atomicAdd(a.fail_count, 1u)] = cell;
            } else if (a.audit_stride && cell % a.audit_stride == a.audit_phase) {
                const uint32_t slot = atomicAdd(a.audit_count, 1u);
                if (slot < a.audit_cap) a.audit_idx[slot] = cell;
            }
        }
    }
}

cudaError_t combine(const CombineArgs& a, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    size_t grid = (a.n + 127) / 128;
    if (grid > 152 * 8) grid = 152 * 8;
    combine_kernel<<<(unsigned)grid, 128, 0, st>>>(a);
    return cudaGetLastError();
}

// Audited cells: relative error of the surrogate against the plain kernel (per output group), then the
// plain values replace the surrogate's.
__global__ void audit_kernel(const AuditArgs a, size_t cap) {
    size_t n = *a.count;
    if (n > cap) n = cap;
    for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
        const size_t c = a.idx[j];
        float mx[3] = {0.f, 0.f, 0.f};
        double sq[3] = {0.0, 0.0, 0.0};
        for (int o = 0; o < a.n_feat; o++) {
            const double ref = a.plain[(size_t)o * a.cap + j];
            const double e = fabs(a.out[o][c] - ref) / fabs(ref);
            const int g = o < 2 ? o : 2;
            mx[g] = fmaxf(mx[g], (float)e);
            sq[g] += e * e;
            a.out[o][c] = ref;
        }
        for (int g = 0; g < 3; g++) {
            atomicMax(&a.max_err[g], __float_as_uint(mx[g]));
            atomicAdd(&a.sum_sq[g], sq[g]);
        }
    }
}

cudaError_t audit(const AuditArgs& a, size_t cap, cudaStream_t st) {
    if (cap == 0) return cudaSuccess;
    size_t grid = (cap + 127) / 128;
    if (grid > 1024) grid = 1024;
    audit_kernel<<<(unsigned)grid, 128, 0, st>>>(a, cap);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------------
// Fused inference: the whole network for pairs of 128-row tiles in one persistent kernel. Activations
// stay in shared memory between layers (written by the epilogue in the 128-byte-swizzled K-major layout
// the next layer's MMAs read); weights stream through a two-stage ring by TMA; the accumulators of the
// pair's two tiles live in the two halves of tensor memory, so that the epilogue of one tile overlaps
// the MMAs of the other. Shape: 64 inputs, hidden width 256, 64 outputs (up to 62 species).
//   warp 0: TMA producer (input tiles, weight chunks in the MMAs' order)
//   warp 1: TMEM owner and MMA issuer
//   warps 2-17: epilogue, four warps per TMEM lane quarter (64 columns each; the 64-wide output layer
//   takes two, 32 columns each): sixteen warps keep enough instructions in flight for a tile's epilogue
//   to take about as long as the other tile's MMAs
constexpr int kFusedEpiWarps = 16;
constexpr int kFusedThreads = 64 + 32 * kFusedEpiWarps;
constexpr int kFusedWidth = 256;
constexpr uint32_t kActChunk = kBM * 128;              // 16 KB: 128 rows x 64 BF16
constexpr uint32_t kActBytes = 4 * kActChunk;           // one tile's activations (256 columns)
constexpr uint32_t kWStage = kFusedWidth * 128;         // 32 KB: 256 weight rows x 64 BF16
constexpr int kWStages = 2;
constexpr int kFusedSmem = 2 * (int)kActBytes + kWStages * (int)kWStage + 1024;

__device__ __forceinline__ void store_act_bf16(uint32_t chunk_base, int r, int c, const float* a) {
    // 32 values of row r, columns [c, c + 32) of a 64-column chunk: four 16-byte pieces, swizzled
    const uint32_t row = chunk_base + (uint32_t)r * 128u;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int piece = ((c & 63) >> 3) + j;
        const uint32_t addr = row + (uint32_t)((piece ^ (r & 7)) << 4);
        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(pack_bf16(a[8 * j], a[8 * j + 1])),
                     "r"(pack_bf16(a[8 * j + 2], a[8 * j + 3])), "r"(pack_bf16(a[8 * j + 4], a[8 * j + 5])),
                     "r"(pack_bf16(a[8 * j + 6], a[8 * j + 7]))
                     : "memory");
    }
}

__global__ void __launch_bounds__(kFusedThreads, 1)
    mlp_infer_kernel(const __grid_constant__ CUtensorMap tx, const __grid_constant__ FusedMaps maps, const FusedParams p) {
    extern __shared__ uint8_t dsm[];
    __shared__ uint64_t w_full[kWStages], w_empty[kWStages], x_full[2], acc_full[2], act_ready[2], act_free[2], fin;
    __shared__ uint32_t tmem_s;
    // biases of every layer, the hidden layers' halved: silu(z) = h (1 + tanh h) with h = z / 2 = fma(1/2,
    // acc, b / 2), one FMA where z = acc + b and h = z / 2 took two (the same h: halving is exact)
    __shared__ __align__(16) float sbias[kMaxLayers * kFusedWidth];
    const uint32_t base = (smem_u32(dsm) + 1023u) & ~1023u;
    const uint32_t act0 = base, wring = base + 2 * kActBytes;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int L = p.L;
    for (int l = 0; l < L; l++)
        for (int c = threadIdx.x; c < p.dims[l + 1]; c += blockDim.x)
            sbias[l * kFusedWidth + c] = (l < L - 1 ? 0.5f : 1.0f) * p.bias[l][c];
    const int tiles = p.rows / kBM;
    const int pairs = (tiles + 1) / 2;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kWStages; s++) {
            umma::mbar_init(smem_u32(&w_full[s]), 1);
            umma::mbar_init(smem_u32(&w_empty[s]), 1);
        }
        for (int t = 0; t < 2; t++) {
            umma::mbar_init(smem_u32(&x_full[t]), 1);
            umma::mbar_init(smem_u32(&acc_full[t]), 1);
            umma::mbar_init(smem_u32(&act_ready[t]), kFusedEpiWarps);
            umma::mbar_init(smem_u32(&act_free[t]), 1);
        }
        umma::mbar_init(smem_u32(&fin), 1);
        umma::fence_mbar_init();
    }
    if (warp == 1) {
        umma::tmem_alloc(smem_u32(&tmem_s), 512);
        umma::tmem_relinquish();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_s;
    bool ok = true;
    // dims of layer l: K = p.dims[l], N = p.dims[l + 1]
    if (warp == 0) {
        if (lane == 0) {  // producer
            int g = 0;    // weight chunks issued so far
            int pi = 0;   // pairs done by this block
            for (int pr = blockIdx.x; pr < pairs && ok; pr += gridDim.x, pi++) {
                for (int t = 0; t < 2 && ok; t++) {
                    const int tile = 2 * pr + t;
                    if (tile >= tiles) break;
                    if (pi > 0 && !umma::mbar_wait(smem_u32(&act_free[t]), (pi - 1) & 1)) { ok = false; break; }
                    umma::mbar_expect_tx(smem_u32(&x_full[t]), kActChunk);
                    umma::tma_load_2d(act0 + t * kActBytes, &tx, smem_u32(&x_full[t]), 0, tile * kBM);
                }
                for (int l = 0; l < L && ok; l++) {
                    const int K = p.dims[l], N = p.dims[l + 1];
                    for (int t = 0; t < 2 && ok; t++) {
                        if (2 * pr + t >= tiles) break;
                        for (int kc = 0; kc < K / kBK; kc++, g++) {
                            const int s = g % kWStages;
                            if (g >= kWStages && !umma::mbar_wait(smem_u32(&w_empty[s]), ((g / kWStages) & 1) ^ 1)) {
                                ok = false;
                                break;
                            }
                            umma::mbar_expect_tx(smem_u32(&w_full[s]), (uint32_t)N * 128u);
                            umma::tma_load_2d(wring + s * kWStage, &maps.w[l], smem_u32(&w_full[s]), kc * kBK, 0);
                        }
                    }
                }
            }
            if (!ok)  // let the weight copies already issued land before the block exits
                for (int i = g > kWStages ? g - kWStages : 0; i < g; i++)
                    umma::mbar_wait(smem_u32(&w_full[i % kWStages]), (i / kWStages) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            int g = 0, pi = 0;
            for (int pr = blockIdx.x; pr < pairs && ok; pr += gridDim.x, pi++) {
                for (int l = 0; l < L && ok; l++) {
                    const int K = p.dims[l], N = p.dims[l + 1];
                    const uint32_t idesc = umma::idesc_bf16_f32(kBM, N);
                    for (int t = 0; t < 2 && ok; t++) {
                        if (2 * pr + t >= tiles) break;
                        const int use = pi * L + l;  // uses of this tile slot's barriers so far
                        if (l == 0) {
                            if (!umma::mbar_wait(smem_u32(&x_full[t]), pi & 1)) { ok = false; break; }
                            // the slot's accumulator was read by the previous pair's last epilogue
                            if (pi > 0 && !umma::mbar_wait(smem_u32(&act_ready[t]), (use - 1) & 1)) { ok = false; break; }
                        } else if (!umma::mbar_wait(smem_u32(&act_ready[t]), (use - 1) & 1)) {
                            ok = false;
                            break;
                        }
                        umma::fence_after_sync();
                        const uint32_t d = tmem + (uint32_t)(t * 256);
                        const uint32_t a_base = act0 + t * kActBytes;
                        for (int kc = 0; kc < K / kBK; kc++, g++) {
                            const int s = g % kWStages;
                            if (!umma::mbar_wait(smem_u32(&w_full[s]), (g / kWStages) & 1)) { ok = false; break; }
                            umma::fence_after_sync();
                            const uint32_t sa = a_base + kc * kActChunk, sb = wring + s * kWStage;
#pragma unroll
                            for (int k = 0; k < kBK / 16; k++)
                                umma::mma_bf16(d, umma::sdesc_sw128(sa + 32u * k), umma::sdesc_sw128(sb + 32u * k), idesc,
                                               (kc | k) != 0);
                            umma::mma_commit(smem_u32(&w_empty[s]));
                        }
                        umma::mma_commit(smem_u32(&acc_full[t]));
                        if (l == L - 1) umma::mma_commit(smem_u32(&act_free[t]));
                    }
                }
            }
            umma::mma_commit(smem_u32(&fin));  // every MMA issued here has completed before TMEM is freed
            umma::mbar_wait(smem_u32(&fin), 0);
        }
    } else {  // epilogue warps 2..17
        const int e = warp - 2;
        const int q = warp & 3;          // TMEM lane quarter
        const int quarter = e >> 2;      // column quarter
        const int r = q * 32 + lane;     // row within the tile
        int pi = 0;
        for (int pr = blockIdx.x; pr < pairs && ok; pr += gridDim.x, pi++) {
            for (int l = 0; l < L && ok; l++) {
                const int N = p.dims[l + 1];
                // this warp's columns: a quarter of N in chunks of 32 (N = 64: the first two quarters only)
                const int cols = N >= 128 ? N / 4 : 32;
                const int c_begin = quarter * cols < N ? quarter * cols : N;
                const float* bias = sbias + l * kFusedWidth;  // halved for the hidden layers
                for (int t = 0; t < 2 && ok; t++) {
                    const int tile = 2 * pr + t;
                    if (tile >= tiles) break;
                    const int use = pi * L + l;
                    if (!__all_sync(0xffffffffu, umma::mbar_wait(smem_u32(&acc_full[t]), use & 1))) {
                        ok = false;
                        break;
                    }
                    umma::fence_after_sync();
                    const uint32_t acc = tmem + (uint32_t)(t * 256) + ((uint32_t)(q * 32) << 16);
                    const uint32_t a_base = act0 + t * kActBytes;
#pragma unroll 1
                    for (int c = c_begin; c < c_begin + cols && c < N; c += 32) {
                        float v[32];
                        umma::tmem_ld32(acc + (uint32_t)c, v);
                        const float4* b4 = reinterpret_cast<const float4*>(bias + c);  // broadcast reads
                        if (l < L - 1) {
#pragma unroll
                            for (int j = 0; j < 8; j++) {
                                const float4 hb = b4[j];
                                const float hbb[4] = {hb.x, hb.y, hb.z, hb.w};
#pragma unroll
                                for (int e = 0; e < 4; e++) {
                                    const float h = fmaf(0.5f, v[4 * j + e], hbb[e]);
                                    v[4 * j + e] = fmaf(h, tanh_approx(h), h);
                                }
                            }
                            store_act_bf16(a_base + (uint32_t)(c >> 6) * kActChunk, r, c, v);
                        } else {
                            float4* dst = reinterpret_cast<float4*>(p.Y + ((size_t)tile * kBM + r) * p.ldY + c);
#pragma unroll
                            for (int j = 0; j < 8; j++) {
                                const float4 b = b4[j];
                                dst[j] = make_float4(v[4 * j] + b.x, v[4 * j + 1] + b.y, v[4 * j + 2] + b.z, v[4 * j + 3] + b.w);
                            }
                        }
                    }
                    // activations visible to the tensor core, accumulator reads complete: the MMAs of the
                    // slot's next layer (or next tile) may start
                    umma::fence_async_shared();
                    umma::fence_before_sync();
                    __syncwarp();
                    if (lane == 0) umma::mbar_arrive(smem_u32(&act_ready[t]));
                }
            }
        }
    }
    if (!ok) atomicOr(p.status, kStatusGemmTimeout);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        umma::fence_after_sync();
        umma::tmem_dealloc(tmem, 512);
    }
}

bool mlp_fused_shape(const int* dims, int L) {
    if (L < 2 || L > kMaxLayers || dims[0] != 64 || dims[L] != 64) return false;
    for (int l = 1; l < L; l++)
        if (dims[l] != kFusedWidth) return false;
    return true;
}

cudaError_t mlp_infer(const CUtensorMap& tx, const FusedMaps& maps, const FusedParams& p, cudaStream_t st) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaError_t e = cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kFusedSmem);
        if (e != cudaSuccess) return e;
    }
    if (p.rows % kBM || !mlp_fused_shape(p.dims, p.L)) return cudaErrorInvalidValue;
    const int pairs = (p.rows / kBM + 1) / 2;
    const int grid = pairs < sms ? pairs : sms;
    if (grid == 0) return cudaSuccess;
    mlp_infer_kernel<<<grid, kFusedThreads, kFusedSmem, st>>>(tx, maps, p);
    return cudaGetLastError();
}

}  // namespace sur
}  // namespace cbg
