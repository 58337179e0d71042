// Kernels of the learned transport surrogate: a BF16 tcgen05 GEMM with fused epilogues (bias + SiLU,
// MSE loss gradient, SiLU backward, split-K weight-gradient partials), and the element-wise kernels
// around it (cell generator, features, targets, outputs, gate audit, Adam).
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cbg {
namespace sur {

// warp 0: TMA producer, warp 1: TMEM owner + MMA issuer, warps 2-9: epilogue (two per TMEM lane quarter,
// each taking half of the tile's columns)
constexpr int kGemmThreads = 320;
constexpr int kEpiWarps = 8;       // loss partials per 128-row tile: one per epilogue warp
constexpr int kBM = 128;           // rows per tile (one M = 128 MMA, one TMEM lane per row)
constexpr int kBK = 64;            // K per pipeline stage: one 128-byte swizzle row of BF16
constexpr int kGemmRing = 144 * 1024;  // operand ring: stages x (A + B tile)
// Shared memory after the ring: per epilogue warp two 4 KB boxes (32 rows x 64 BF16, 128-byte swizzle)
// for the TMA stores of row-major outputs and the TMA loads of SiLU derivatives. The weight-gradient
// items, whose epilogue writes straight to global memory, keep a 128 x 64 BF16 tile of ones there instead
// (the extra operand of the bias-gradient MMAs).
constexpr int kStageBox = 4096, kOnesTile = 128 * 128;
constexpr int kGemmSmem = kGemmRing + 8 * 2 * kStageBox + 1024;  // + alignment; one block per SM
constexpr int kMaxIn = 259;        // rates-layout inputs for up to 256 species
constexpr int kMaxOut = 258;       // transport outputs for up to 256 species
constexpr int kMaxLayers = 8;

enum Epilogue : int {
    kEpiPartial = 0,  // FP32 accumulator tile to ws[split] (weight-gradient partials; A and B MN-major), and
                      // with bias_part the bias-gradient partials (row sums of A or column sums of B, by
                      // MMAs with a tile of ones)
    kEpiHidden = 1,   // z = acc + bias: silu(z) row-major, silu'(z) row-major (optional, for the backward)
    kEpiLoss = 2,     // y = acc + bias: d = y - target (valid columns), loss partial, d * scale row-major
    kEpiDgrad = 3,    // dz = acc * silu'(z) row-major
    kEpiLinear = 4,   // y = acc + bias to FP32 row-major
};

enum DynOffset : int { kDynAy = 1, kDynBx = 2, kDynTarget = 4 };
// Bias-gradient partials of a weight-gradient GEMM D = A B^T (A = dZ^T of a hidden layer, or A_in^T of the
// output layer with B = dY^T): kBiasRows = the row sums of A (M values, A times 16 columns of ones),
// kBiasCols = the column sums of B^T (N values, 128 rows of ones times B^T).
enum BiasPart : int { kBiasNone = 0, kBiasRows = 1, kBiasCols = 2 };

struct GemmParams {
    int M, N;               // output tile grid: M / 128 by N / BN blocks
    int k_blocks, splits;   // 64-wide K blocks in total; split z takes [z KB / S, (z + 1) KB / S)
    const int* row0;        // device row offset added where `dyn` says (training batch position): to the
    int dyn;                // rows of A (kDynAy) or to the K rows of the MN-major B (kDynBx)
    const float* bias;
    __nv_bfloat16* out;  int ld_out;   // row-major BF16 [M][ld]
    __nv_bfloat16* out2; int ld_out2;  // row-major BF16 [M][ld]
    long long split_stride;            // partials: floats from one split's [M][ld] block to the next
    int bias_part;                     // partials: kBiasRows / kBiasCols, after the split's [M][ld] block
    const float* target; int ld_target; int n_valid; float grad_scale;
    float* loss;            // one partial per epilogue warp: [row tile][kEpiWarps]
    float* outf; int ld_outf;  // FP32 output
    int* status;
};

// TMA maps of the epilogues' row-major BF16 matrices (boxes of 64 columns x 32 rows, 128-byte swizzle):
// the hidden-layer (silu'(Z), silu(Z)) and data-gradient (dZ) epilogues store through out / out2; the
// data-gradient epilogue loads the SiLU derivatives through dact.
struct RowMaps {
    CUtensorMap out, out2, dact;
};

enum SurStatus : int { kStatusGemmTimeout = 2 };

struct CellGenArgs {
    double* out[kMaxIn];  // P/R, R/P, T, V, n_0 .. n_{K-2}
    size_t n, offset;
    int K, fixed_pressure;
    uint64_t seed;
    double T_lo, T_hi, lnP_lo, lnP_hi, P_fixed, alpha, R;
};

struct FeatureArgs {
    const double* in[kMaxIn];  // rates layout
    size_t n, rows;            // cells; rows written (>= n, padding rows are zero)
    int K, n_feat, n_in;
    uint32_t uniform_pressure;
    double T0, R_over_P0;
    const float* mean; const float* rstd;  // normalisation of the raw features
    __nv_bfloat16* X; size_t row0;          // row-major [.][n_in], rows from row0
    float* raw;                             // raw features [n][n_feat] (optional, statistics)
    int* hull_lo; int* hull_hi;             // order-preserving integer min / max of raw features (optional)
    const float* lo; const float* hi;       // trust region (inference gate, optional)
    uint32_t* fail_idx; uint32_t* fail_count;  // cells idx_base + c outside the trust region
    uint32_t* audit_idx; uint32_t* audit_count; uint32_t audit_stride, audit_phase, audit_cap;
    uint32_t idx_base;
    uint8_t* outside;                       // per cell of the call: 1 outside the trust region (optional)
};

// Two networks' normalised outputs of the same cells -> transport properties (their mean in log space)
// and the ensemble gate: a cell falls back when it lies outside the trust region or when the networks'
// log outputs differ by more than `threshold` (max over outputs); every audit_stride-th other cell is
// audited.
struct CombineArgs {
    const float* Ya; const float* Yb; int ldY;
    size_t n;
    int n_feat;
    const float* mean_a; const float* std_a; const float* mean_b; const float* std_b;
    double* out[kMaxOut];
    float threshold;                  // +inf: the trust region alone; negative: every cell falls back
    const uint8_t* outside;           // per cell of the call (optional)
    float* disagreement;              // per cell of the call (optional)
    uint32_t* fail_idx; uint32_t* fail_count;
    uint32_t* audit_idx; uint32_t* audit_count; uint32_t audit_stride, audit_phase, audit_cap;
    uint32_t idx_base;
};

struct TargetArgs {
    const double* out[kMaxOut];  // plain transport outputs
    size_t n, row0;
    int n_feat, n_out;
    const float* mean; const float* rstd;
    float* Y;                    // [.][n_out] normalised log outputs
    float* raw;                  // [n][n_feat] log outputs (optional, statistics)
};

struct OutputArgs {
    const float* Y; int ldY;
    size_t n;
    int n_feat;
    const float* mean; const float* std;
    double* out[kMaxOut];
};

struct AuditArgs {
    const uint32_t* idx; const uint32_t* count;
    const double* plain; size_t cap;  // [n_feat][cap] plain outputs of the audited cells
    double* out[kMaxOut];
    int n_feat;
    unsigned* max_err;   // [3] FP32 bits (conductivity, viscosity, diffusion)
    double* sum_sq;      // [3]
};

struct AdamLayer {
    long long w_off;
    int n_out, n_in;
    __nv_bfloat16* W;
};
struct AdamArgs {
    AdamLayer L[kMaxLayers];
    int n_layers;
    long long n_weights, n_params;
    float lr, lr_final, b1, b2, eps;
    int total_steps;
    const int* step;
    float* p; const float* g; float* m; float* v;
};

// Fused inference (surrogate_kernels.cu): 64 -> 256 x (L - 1) -> 64, outputs FP32 [rows][ldY].
struct FusedMaps {
    CUtensorMap w[kMaxLayers];  // weights of layer l: [dims[l+1]][dims[l]], boxes of 64 columns x dims[l+1] rows
};
struct FusedParams {
    int rows, L;
    int dims[kMaxLayers + 1];
    const float* bias[kMaxLayers];
    float* Y;
    int ldY;
    int* status;
};
bool mlp_fused_shape(const int* dims, int L);
cudaError_t mlp_infer(const CUtensorMap& tx, const FusedMaps& maps, const FusedParams& p, cudaStream_t st);

// Launchers (surrogate_kernels.cu). gemm_setup() raises the GEMM's shared-memory limit on the current
// device; it runs before the first GEMM (and outside any stream capture).
cudaError_t gemm_setup();
// out_map / out2_map: store maps of p.out / p.out2 (required where the epilogue writes them: hidden layers
// and data gradients, whose width is a multiple of 256); dact_map: the data gradient's SiLU derivatives.
cudaError_t gemm(int BN, int epi, const CUtensorMap& a, const CUtensorMap& b, const GemmParams& p, cudaStream_t st,
                 const CUtensorMap* out_map = nullptr, const CUtensorMap* out2_map = nullptr,
                 const CUtensorMap* dact_map = nullptr);
// grad_w[m][n] (or [n][m] with transpose) = sum over z of ws[z * stride + m N + n]; with nb > 0 also
// grad_b[m] = sum over z of ws[z * stride + M N + m], m < nb. Fixed order.
cudaError_t reduce_partials(const float* ws, int splits, long long stride, int M, int N, bool transpose, float* grad_w,
                            int nb, float* grad_b, cudaStream_t st);

cudaError_t adam(const AdamArgs& a, cudaStream_t st);
cudaError_t finish_step(const float* loss_part, int n_part, float norm, float* losses, int* step, int* row0,
                        int batch, int n_batches, cudaStream_t st);
cudaError_t cast_weights(const AdamArgs& a, cudaStream_t st);
cudaError_t generate_cells(const CellGenArgs& a, cudaStream_t st);
cudaError_t features(const FeatureArgs& a, cudaStream_t st);
cudaError_t targets(const TargetArgs& a, cudaStream_t st);
cudaError_t outputs(const OutputArgs& a, cudaStream_t st);
cudaError_t combine(const CombineArgs& a, cudaStream_t st);
cudaError_t audit(const AuditArgs& a, size_t cap, cudaStream_t st);

}  // namespace sur
}  // namespace cbg
