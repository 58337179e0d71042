// Learned transport surrogate: host side (C ABI in include/combustion_gb300.h, kernels in
// surrogate_kernels.cu). No reference counterpart; the plain transport kernel (transport.rs:179-214)
// produces its training targets, takes the cells its trust gate rejects and audits a sample of the rest.
//
// Network: dims[0] = n_in (K + 2 features padded to 64) -> hidden layers of `width` (SiLU) -> dims[L] =
// n_out (K + 2 outputs padded to 64). Layer l computes Z = A_{l-1} W_l^T + b_l with W_l [dims[l+1]][dims[l]].
// Training step (one CUDA graph): forward GEMMs keep silu(Z) and silu'(Z) per hidden layer (row-major),
// the output GEMM's epilogue forms the MSE gradient; backward runs per layer a split-K weight-gradient
// GEMM that reads the row-major activations and gradients as MN-major operands and adds the bias-gradient
// partials (MMAs against a tile of ones), a deterministic reduction of both partials, and the
// data-gradient GEMM (row-major W as its MN-major B) whose epilogue multiplies by silu'(Z); Adam updates
// the FP32 master weights and rewrites the BF16 weights.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/combustion_gb300.h"
#include "capi_internal.h"
#include "kernels.h"
#include "surrogate_kernels.cuh"

using namespace cbg::sur;
using bf16 = __nv_bfloat16;

namespace {

constexpr double kR = 1.380649e-23 * 6.02214076e23;  // R = kB NA (model.rs:6-8)
constexpr size_t kInferChunk = (size_t)1 << 20;      // cells per inference pass
constexpr long long kMaxSteps = 1 << 20;             // training steps between two parameter resets

#define SUR_CUDA(call)                                              \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return cbi::cuda_fail(e_, #call);    \
    } while (0)
#define SUR_RC(call)              \
    do {                          \
        int rc_ = (call);         \
        if (rc_) return rc_;      \
    } while (0)

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 2-D BF16 tensor map over a row-major [outer][inner] matrix, boxes of 64 columns x box_rows rows with
// the 128-byte swizzle the MMA descriptors expect.
int make_map(CUtensorMap* m, const void* ptr, uint64_t inner, uint64_t outer, uint32_t box_rows) {
    auto fn = encode_fn();
    if (!fn) return cbi::fail(CB_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {inner * sizeof(bf16)};
    cuuint32_t box[2] = {64, box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cbi::fail(CB_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return CB_OK;
}

int bn_for(int N) { return N % 256 == 0 ? 256 : N % 128 == 0 ? 128 : 64; }
int pad64(int x) { return (x + 63) / 64 * 64; }

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <class T>
int dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return CB_OK;
    SUR_CUDA(cudaMalloc(p, count * sizeof(T)));
    return CB_OK;
}

}  // namespace

struct cb_surrogate {
    cb_mech* mech = nullptr;
    int device = 0, K = 0;
    int n_feat = 0, n_in = 0, n_out = 0, width = 0, hidden = 0, L = 0;
    int dims[kMaxLayers + 1] = {};
    int batch = 0;
    float lr = 1e-3f, lr_final = 1e-3f, b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    uint64_t seed = 0;
    long long n_weights = 0, n_params = 0, steps_done = 0;
    long long w_off[kMaxLayers] = {}, b_off[kMaxLayers] = {};
    float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;
    bf16* W[kMaxLayers] = {};
    CUtensorMap mW[kMaxLayers], mW_K[kMaxLayers];  // K-major B of the forward; MN-major B of the data gradient
    // normalisation (n_out floats each, zero beyond n_feat): in_mean, in_rstd, out_mean, out_rstd, out_std, lo, hi
    float* norm = nullptr;
    std::vector<float> h_norm;
    bool have_norm = false;
    // training set
    size_t n_train = 0;
    bf16* X = nullptr;
    float* Y = nullptr;
    CUtensorMap mX, mX_K;  // A operand of the first layer (128-row boxes); MN-major B of its weight gradient
    // per-step buffers (batch rows)
    bf16 *Sd[kMaxLayers] = {}, *Act[kMaxLayers] = {};  // silu'(Z_l) (backward) and silu(Z_l) of each hidden layer
    bf16 *dY = nullptr, *dZ[2] = {};
    CUtensorMap mAct_A[kMaxLayers], mdY_A, mdZ_A[2];         // K-major A operands (128-row boxes)
    CUtensorMap mAct_K[kMaxLayers], mdY_K, mdZ_K[2];         // MN-major weight-gradient operands (64-row boxes)
    CUtensorMap mSd_S[kMaxLayers], mAct_S[kMaxLayers], mdZ_S[2];  // TMA maps (32-row boxes) of the epilogues
    float* ws = nullptr;
    float* loss_part = nullptr;
    float* losses = nullptr;  // mean squared error of every step since the parameters were set
    int* counters = nullptr;  // [0] step, [1] batch row offset
    // evaluation scratch (rows <= batch)
    bf16* Xs = nullptr;
    float* Ys = nullptr;
    CUtensorMap mXs, mXs_K;
    // inference buffers
    bf16 *Xi = nullptr, *Hi[2] = {};
    float* Yi = nullptr;
    CUtensorMap mXi, mHi[2], mHi_S[2];
    uint32_t *fail_idx = nullptr, *audit_idx = nullptr, *gate_count = nullptr;
    double* audit_plain = nullptr;
    size_t fail_cap = 0, audit_cap = 0;  // grown to the largest call
    uint8_t* outside = nullptr;          // ensemble calls: trust-region flags of the call's cells
    float* disagreement = nullptr;       // ensemble calls: the networks' disagreement per cell
    size_t cell_cap = 0;
    unsigned* err_max = nullptr;
    double* err_sq = nullptr;
    int* status = nullptr;
    cudaStream_t stream = nullptr;
};

namespace {

GemmParams base_params(cb_surrogate* s) {
    GemmParams p;
    std::memset(&p, 0, sizeof p);
    p.splits = 1;
    p.status = s->status;
    return p;
}

AdamArgs adam_args(cb_surrogate* s, int total_steps) {
    AdamArgs a;
    std::memset(&a, 0, sizeof a);
    a.n_layers = s->L;
    for (int l = 0; l < s->L; l++) a.L[l] = AdamLayer{s->w_off[l], s->dims[l + 1], s->dims[l], s->W[l]};
    a.n_weights = s->n_weights;
    a.n_params = s->n_params;
    a.lr = s->lr;
    a.lr_final = s->lr_final;
    a.b1 = s->b1;
    a.b2 = s->b2;
    a.eps = s->eps;
    a.total_steps = total_steps;
    a.step = s->counters;
    a.p = s->p;
    a.g = s->g;
    a.m = s->m1;
    a.v = s->m2;
    return a;
}

// Splits of a weight-gradient GEMM: enough blocks to cover the GPU once.
int wgrad_splits(int M, int N, int BN, int k_blocks) {
    const int tiles = (M / kBM) * (N / BN);
    int s = std::max(1, 148 / std::max(1, tiles));
    return std::min(s, k_blocks);
}

// Forward (and, with `backward`, backward + optional Adam) over `rows` rows. mX: the first layer's input
// with 128-row boxes (A operand), mX_K: the same matrix with 64-row boxes (MN-major B operand of the first
// layer's weight gradient).
int run_pass(cb_surrogate* s, int rows, const CUtensorMap& mX, const CUtensorMap& mX_K, const float* Y, bool dyn,
             bool backward, bool update, int total_steps, cudaStream_t st) {
    const int L = s->L;
    // forward
    for (int l = 0; l < L; l++) {
        GemmParams p = base_params(s);
        p.M = rows;
        p.N = s->dims[l + 1];
        p.k_blocks = s->dims[l] / kBK;
        p.bias = s->p + s->b_off[l];
        if (l == 0 && dyn) {
            p.row0 = s->counters + 1;
            p.dyn = kDynAy;
        }
        int epi;
        if (l < L - 1) {
            epi = kEpiHidden;
            p.out = backward ? s->Sd[l] : nullptr;
            p.ld_out = s->width;
            p.out2 = s->Act[l];
            p.ld_out2 = s->width;
        } else if (backward) {
            epi = kEpiLoss;
            p.target = Y;
            p.ld_target = s->n_out;
            p.n_valid = s->n_feat;
            p.grad_scale = 2.0f / ((float)rows * (float)s->n_feat);
            p.out = s->dY;
            p.ld_out = s->n_out;
            p.loss = s->loss_part;
            if (dyn) {
                p.row0 = s->counters + 1;
                p.dyn |= kDynTarget;
            }
        } else {
            epi = kEpiLinear;
            p.outf = s->Yi;
            p.ld_outf = s->n_out;
        }
        const CUtensorMap& a = l == 0 ? mX : s->mAct_A[l - 1];
        if (epi == kEpiHidden)
            SUR_CUDA(gemm(bn_for(p.N), epi, a, s->mW[l], p, st, backward ? &s->mSd_S[l] : nullptr, &s->mAct_S[l]));
        else
            SUR_CUDA(gemm(bn_for(p.N), epi, a, s->mW[l], p, st));
    }
    if (!backward) return CB_OK;
    for (int l = L - 1; l >= 0; l--) {
        // weight gradient (split K over the rows, operands MN-major from the row-major activations) and
        // bias gradient (sums of the output gradient over the rows, by the tensor core), reduced in a fixed
        // order
        GemmParams p = base_params(s);
        const CUtensorMap *ma, *mb;
        bool transpose;
        if (l == L - 1) {  // W_L^T = A_{L-1}^T dY: M = width, N = n_out
            p.M = s->dims[l];
            p.N = s->dims[l + 1];
            ma = &s->mAct_K[l - 1];
            mb = &s->mdY_K;
            transpose = true;
            p.bias_part = kBiasCols;
        } else {  // W_l = dZ_l^T A_{l-1}: M = dims[l+1], N = dims[l]
            p.M = s->dims[l + 1];
            p.N = s->dims[l];
            ma = &s->mdZ_K[l % 2];
            mb = l == 0 ? &mX_K : &s->mAct_K[l - 1];
            transpose = false;
            p.bias_part = kBiasRows;
            if (l == 0 && dyn) {
                p.row0 = s->counters + 1;
                p.dyn = kDynBx;
            }
        }
        const int BN = bn_for(p.N);
        p.k_blocks = rows / kBK;
        p.splits = wgrad_splits(p.M, p.N, BN, p.k_blocks);
        p.outf = s->ws;
        p.ld_outf = p.N;
        const int nb = p.bias_part == kBiasRows ? p.M : p.N;
        p.split_stride = (long long)p.M * p.N + nb;
        SUR_CUDA(gemm(BN, kEpiPartial, *ma, *mb, p, st));
        SUR_CUDA(reduce_partials(s->ws, p.splits, p.split_stride, p.M, p.N, transpose, s->g + s->w_off[l], nb,
                                 s->g + s->b_off[l], st));
        if (l == 0) break;
        // data gradient through W_l, times silu'(Z_{l-1})
        GemmParams q = base_params(s);
        q.M = rows;
        q.N = s->dims[l];
        q.k_blocks = s->dims[l + 1] / kBK;
        q.out = s->dZ[(l - 1) % 2];
        q.ld_out = s->width;
        const CUtensorMap& a = l == L - 1 ? s->mdY_A : s->mdZ_A[l % 2];
        SUR_CUDA(gemm(bn_for(q.N), kEpiDgrad, a, s->mW_K[l], q, st, &s->mdZ_S[(l - 1) % 2], nullptr, &s->mSd_S[l - 1]));
    }
    if (update) {
        SUR_CUDA(adam(adam_args(s, total_steps), st));
        const int n_batches = (int)(s->n_train / s->batch);
        SUR_CUDA(finish_step(s->loss_part, kEpiWarps * rows / kBM, 1.0f / ((float)rows * (float)s->n_feat), s->losses, s->counters,
                             s->counters + 1, s->batch, n_batches, st));
    }
    return CB_OK;
}

int free_all(cb_surrogate* s) {
    void* ptrs[] = {s->p, s->g, s->m1, s->m2, s->norm, s->X, s->Y, s->dY, s->dZ[0], s->dZ[1],
                    s->ws, s->loss_part, s->losses, s->counters, s->Xs, s->Ys, s->Xi, s->Hi[0],
                    s->Hi[1], s->Yi, s->fail_idx, s->audit_idx, s->gate_count, s->audit_plain, s->err_max,
                    s->err_sq, s->status, s->outside, s->disagreement};
    for (void* q : ptrs) cudaFree(q);
    for (int l = 0; l < kMaxLayers; l++) {
        cudaFree(s->W[l]);
        cudaFree(s->Sd[l]);
        cudaFree(s->Act[l]);
    }
    if (s->stream) cudaStreamDestroy(s->stream);
    return CB_OK;
}

int check_device_status(cb_surrogate* s) {
    int st = 0;
    SUR_CUDA(cudaMemcpy(&st, s->status, sizeof st, cudaMemcpyDeviceToHost));
    if (st) {
        cudaMemset(s->status, 0, sizeof(int));
        return cbi::fail(CB_ERR_DEVICE, "a surrogate kernel reported status " + std::to_string(st) +
                                             " (a bounded wait ran out)");
    }
    return cbi::check_status(s->mech);
}

int ensure_inference(cb_surrogate* s, size_t rows) {
    if (s->Xi) return CB_OK;
    rows = kInferChunk;
    SUR_RC(dalloc(&s->Xi, rows * s->n_in));
    SUR_RC(dalloc(&s->Hi[0], rows * s->width));
    SUR_RC(dalloc(&s->Hi[1], rows * s->width));
    SUR_RC(dalloc(&s->Yi, rows * s->n_out));
    SUR_RC(dalloc(&s->gate_count, 2));
    SUR_RC(dalloc(&s->err_max, 3));
    SUR_RC(dalloc(&s->err_sq, 3));
    SUR_RC(make_map(&s->mXi, s->Xi, s->n_in, rows, kBM));
    SUR_RC(make_map(&s->mHi[0], s->Hi[0], s->width, rows, kBM));
    SUR_RC(make_map(&s->mHi[1], s->Hi[1], s->width, rows, kBM));
    SUR_RC(make_map(&s->mHi_S[0], s->Hi[0], s->width, rows, 32));
    SUR_RC(make_map(&s->mHi_S[1], s->Hi[1], s->width, rows, 32));
    return CB_OK;
}

// Inference forward over `rows` rows of Xi into Yi (FP32, normalised outputs): the fused kernel for the
// 64 -> 256 x n -> 64 shape, one GEMM per layer otherwise.
int infer_rows(cb_surrogate* s, int rows, const CUtensorMap& mX, cudaStream_t st) {
    if (mlp_fused_shape(s->dims, s->L)) {
        FusedMaps maps;
        std::memset(&maps, 0, sizeof maps);
        FusedParams p;
        std::memset(&p, 0, sizeof p);
        p.rows = rows;
        p.L = s->L;
        for (int l = 0; l <= s->L; l++) p.dims[l] = s->dims[l];
        for (int l = 0; l < s->L; l++) {
            maps.w[l] = s->mW[l];
            p.bias[l] = s->p + s->b_off[l];
        }
        p.Y = s->Yi;
        p.ldY = s->n_out;
        p.status = s->status;
        SUR_CUDA(mlp_infer(mX, maps, p, st));
        return CB_OK;
    }
    for (int l = 0; l < s->L; l++) {
        GemmParams p = base_params(s);
        p.M = rows;
        p.N = s->dims[l + 1];
        p.k_blocks = s->dims[l] / kBK;
        p.bias = s->p + s->b_off[l];
        int epi;
        if (l < s->L - 1) {
            epi = kEpiHidden;
            p.out2 = s->Hi[l % 2];
            p.ld_out2 = s->width;
        } else {
            epi = kEpiLinear;
            p.outf = s->Yi;
            p.ld_outf = s->n_out;
        }
        const CUtensorMap& a = l == 0 ? mX : s->mHi[(l - 1) % 2];
        if (epi == kEpiHidden)
            SUR_CUDA(gemm(bn_for(p.N), epi, a, s->mW[l], p, st, nullptr, &s->mHi_S[l % 2]));
        else
            SUR_CUDA(gemm(bn_for(p.N), epi, a, s->mW[l], p, st));
    }
    return CB_OK;
}

const float* nrm(const cb_surrogate* s, int which) { return s->norm + (size_t)which * s->n_out; }
enum { kInMean = 0, kInRstd, kOutMean, kOutRstd, kOutStd, kLo, kHi, kNormRows };

}  // namespace

extern "C" {

int cb_generate_cells(cb_mech* mech, size_t n, size_t offset, const cb_cell_distribution* d, double* const* outputs,
                      void* stream) {
    if (!mech || !d || !outputs) return cbi::fail(CB_ERR_INVALID, "null argument");
    const cbi::MechView v = cbi::view(mech);
    if (!(d->T_min > 0 && d->T_max >= d->T_min && d->P_min > 0 && d->P_max >= d->P_min && d->alpha > 0))
        return cbi::fail(CB_ERR_INVALID, "bad cell distribution");
    CellGenArgs a;
    std::memset(&a, 0, sizeof a);
    for (int q = 0; q < v.K + 3; q++) {
        if (!outputs[q]) return cbi::fail(CB_ERR_INVALID, "null output array");
        a.out[q] = outputs[q];
    }
    a.n = n;
    a.offset = offset;
    a.K = v.K;
    a.seed = d->seed;
    a.T_lo = d->T_min;
    a.T_hi = d->T_max;
    a.fixed_pressure = d->P_min == d->P_max;
    a.P_fixed = d->P_min * 101325.0;
    a.lnP_lo = std::log(d->P_min);
    a.lnP_hi = std::log(d->P_max);
    a.alpha = d->alpha;
    a.R = kR;
    SUR_CUDA(cudaSetDevice(v.device));
    SUR_CUDA(generate_cells(a, static_cast<cudaStream_t>(stream)));
    return CB_OK;
}

int cb_surrogate_create(cb_mech* mech, const cb_surrogate_desc* d, cb_surrogate** out) {
    if (!mech || !d || !out) return cbi::fail(CB_ERR_INVALID, "null argument");
    *out = nullptr;
    const cbi::MechView v = cbi::view(mech);
    if (d->width < 256 || d->width % 256 || d->hidden_layers < 1 || d->hidden_layers > 6 || d->batch < 128 ||
        d->batch % 128)
        return cbi::fail(CB_ERR_INVALID, "width must be a multiple of 256, 1..6 hidden layers, batch a multiple of 128");
    if (!(d->lr > 0) || !(d->lr_final >= 0) || !(d->beta1 >= 0 && d->beta1 < 1) || !(d->beta2 >= 0 && d->beta2 < 1) ||
        !(d->eps > 0))
        return cbi::fail(CB_ERR_INVALID, "bad optimiser settings");
    if (!v.transport_ready) return cbi::fail(CB_ERR_NOT_READY, "cb_transport_setup has not run");
    cb_surrogate* s = new cb_surrogate();
    s->mech = mech;
    s->device = v.device;
    s->K = v.K;
    s->n_feat = v.K + 2;
    s->n_in = pad64(s->n_feat);
    s->n_out = pad64(s->n_feat);
    s->width = d->width;
    s->hidden = d->hidden_layers;
    s->L = s->hidden + 1;
    s->batch = d->batch;
    s->lr = d->lr;
    s->lr_final = d->lr_final;
    s->b1 = d->beta1;
    s->b2 = d->beta2;
    s->eps = d->eps;
    s->seed = d->seed;
    s->dims[0] = s->n_in;
    for (int l = 1; l <= s->hidden; l++) s->dims[l] = s->width;
    s->dims[s->L] = s->n_out;
    long long off = 0;
    for (int l = 0; l < s->L; l++) {
        s->w_off[l] = off;
        off += (long long)s->dims[l] * s->dims[l + 1];
    }
    s->n_weights = off;
    for (int l = 0; l < s->L; l++) {
        s->b_off[l] = off;
        off += s->dims[l + 1];
    }
    s->n_params = off;
    auto fail_free = [&](int rc) {
        free_all(s);
        delete s;
        return rc;
    };
    cudaError_t e = cudaSetDevice(s->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = gemm_setup();
    if (e != cudaSuccess) return fail_free(cbi::cuda_fail(e, "surrogate stream"));
    int rc = CB_OK;
    const size_t B = s->batch, Wd = s->width;
    rc = rc ? rc : dalloc(&s->p, s->n_params);
    rc = rc ? rc : dalloc(&s->g, s->n_params);
    rc = rc ? rc : dalloc(&s->m1, s->n_params);
    rc = rc ? rc : dalloc(&s->m2, s->n_params);
    rc = rc ? rc : dalloc(&s->norm, (size_t)kNormRows * s->n_out);
    for (int l = 0; l < s->L && !rc; l++) {
        rc = dalloc(&s->W[l], (size_t)s->dims[l] * s->dims[l + 1]);
    }
    for (int l = 0; l < s->hidden && !rc; l++) {
        rc = dalloc(&s->Sd[l], B * Wd);
        rc = rc ? rc : dalloc(&s->Act[l], B * Wd);
    }
    rc = rc ? rc : dalloc(&s->dY, B * s->n_out);
    for (int h = 0; h < 2 && !rc; h++) rc = dalloc(&s->dZ[h], B * Wd);
    // weight-gradient partials: the largest splits x M x N of any layer
    size_t ws = 0;
    for (int l = 0; l < s->L; l++) {
        const int M = l == s->L - 1 ? s->dims[l] : s->dims[l + 1], N = l == s->L - 1 ? s->dims[l + 1] : s->dims[l];
        ws = std::max(ws, (size_t)wgrad_splits(M, N, bn_for(N), s->batch / kBK) * (M * N + std::max(M, N)));
    }
    rc = rc ? rc : dalloc(&s->ws, ws);
    rc = rc ? rc : dalloc(&s->losses, kMaxSteps);
    rc = rc ? rc : dalloc(&s->loss_part, kEpiWarps * B / kBM);
    rc = rc ? rc : dalloc(&s->counters, 2);
    rc = rc ? rc : dalloc(&s->Xs, B * s->n_in);
    rc = rc ? rc : dalloc(&s->Ys, B * s->n_out);
    rc = rc ? rc : dalloc(&s->status, 1);
    if (rc) return fail_free(rc);
    // tensor maps of the per-step buffers
    const int L = s->L;
    for (int l = 0; l < L && !rc; l++) {
        rc = make_map(&s->mW[l], s->W[l], s->dims[l], s->dims[l + 1], bn_for(s->dims[l + 1]));
        rc = rc ? rc : make_map(&s->mW_K[l], s->W[l], s->dims[l], s->dims[l + 1], kBK);
    }
    for (int l = 0; l < s->hidden && !rc; l++) {
        rc = make_map(&s->mAct_A[l], s->Act[l], Wd, B, kBM);
        rc = rc ? rc : make_map(&s->mAct_K[l], s->Act[l], Wd, B, kBK);
        rc = rc ? rc : make_map(&s->mSd_S[l], s->Sd[l], Wd, B, 32);
        rc = rc ? rc : make_map(&s->mAct_S[l], s->Act[l], Wd, B, 32);
    }
    rc = rc ? rc : make_map(&s->mdY_A, s->dY, s->n_out, B, kBM);
    rc = rc ? rc : make_map(&s->mdY_K, s->dY, s->n_out, B, kBK);
    for (int h = 0; h < 2 && !rc; h++) {
        rc = make_map(&s->mdZ_A[h], s->dZ[h], Wd, B, kBM);
        rc = rc ? rc : make_map(&s->mdZ_K[h], s->dZ[h], Wd, B, kBK);
        rc = rc ? rc : make_map(&s->mdZ_S[h], s->dZ[h], Wd, B, 32);
    }
    rc = rc ? rc : make_map(&s->mXs, s->Xs, s->n_in, B, kBM);
    rc = rc ? rc : make_map(&s->mXs_K, s->Xs, s->n_in, B, kBK);
    if (rc) return fail_free(rc);
    // He-uniform weights over the real fan-in, zero biases; padding rows / columns stay zero.
    std::vector<float> h(s->n_params, 0.f);
    uint64_t st = s->seed;
    for (int l = 0; l < L; l++) {
        const int fan_in = l == 0 ? s->n_feat : s->dims[l];
        const int rows = l == L - 1 ? s->n_feat : s->dims[l + 1];
        const int cols = l == 0 ? s->n_feat : s->dims[l];
        const double a = std::sqrt(6.0 / fan_in) * (l == L - 1 ? 0.5 : 1.0);
        for (int o = 0; o < rows; o++)
            for (int i = 0; i < cols; i++) {
                const double u = (double)(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
                h[s->w_off[l] + (size_t)o * s->dims[l] + i] = (float)((2.0 * u - 1.0) * a);
            }
    }
    rc = cb_surrogate_set_params(s, h.data());
    if (rc) return fail_free(rc);
    *out = s;
    return CB_OK;
}

int cb_surrogate_destroy(cb_surrogate* s) {
    if (!s) return CB_OK;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_all(s);
    delete s;
    return CB_OK;
}

int cb_surrogate_query(const cb_surrogate* s, cb_surrogate_info* info) {
    if (!s || !info) return cbi::fail(CB_ERR_INVALID, "null argument");
    std::memset(info, 0, sizeof *info);
    info->n_features = s->n_feat;
    info->n_in = s->n_in;
    info->n_out = s->n_out;
    info->width = s->width;
    info->hidden_layers = s->hidden;
    info->batch = s->batch;
    info->n_params = s->n_params;
    info->n_weights = s->n_weights;
    info->n_train = (int64_t)s->n_train;
    info->steps_done = s->steps_done;
    for (int l = 0; l < s->L; l++) {
        info->weight_offset[l] = s->w_off[l];
        info->bias_offset[l] = s->b_off[l];
    }
    for (int l = 0; l <= s->L; l++) info->dims[l] = s->dims[l];
    return CB_OK;
}

int cb_surrogate_get_params(const cb_surrogate* s, float* params) {
    if (!s || !params) return cbi::fail(CB_ERR_INVALID, "null argument");
    SUR_CUDA(cudaSetDevice(s->device));
    SUR_CUDA(cudaStreamSynchronize(s->stream));
    SUR_CUDA(cudaMemcpy(params, s->p, s->n_params * sizeof(float), cudaMemcpyDeviceToHost));
    return CB_OK;
}

int cb_surrogate_set_params(cb_surrogate* s, const float* params) {
    if (!s || !params) return cbi::fail(CB_ERR_INVALID, "null argument");
    SUR_CUDA(cudaSetDevice(s->device));
    SUR_CUDA(cudaStreamSynchronize(s->stream));
    SUR_CUDA(cudaMemcpy(s->p, params, s->n_params * sizeof(float), cudaMemcpyHostToDevice));
    SUR_CUDA(cudaMemset(s->m1, 0, s->n_params * sizeof(float)));
    SUR_CUDA(cudaMemset(s->m2, 0, s->n_params * sizeof(float)));
    SUR_CUDA(cudaMemset(s->counters, 0, 2 * sizeof(int)));
    SUR_CUDA(cudaMemset(s->status, 0, sizeof(int)));
    s->steps_done = 0;
    SUR_CUDA(cast_weights(adam_args(s, 1), s->stream));
    SUR_CUDA(cudaStreamSynchronize(s->stream));
    return CB_OK;
}

int cb_surrogate_normalisation(const cb_surrogate* s, float* in_mean, float* in_rstd, float* out_mean, float* out_std,
                               float* in_lo, float* in_hi) {
    if (!s) return cbi::fail(CB_ERR_INVALID, "null argument");
    if (!s->have_norm) return cbi::fail(CB_ERR_NOT_READY, "cb_surrogate_generate has not run");
    float* dst[] = {in_mean, in_rstd, out_mean, nullptr, out_std, in_lo, in_hi};
    for (int r = 0; r < kNormRows; r++)
        if (dst[r]) std::memcpy(dst[r], s->h_norm.data() + (size_t)r * s->n_out, s->n_feat * sizeof(float));
    return CB_OK;
}

int cb_surrogate_generate(cb_surrogate* s, size_t n_train, const cb_cell_distribution* dist) {
    if (!s || !dist) return cbi::fail(CB_ERR_INVALID, "null argument");
    n_train = n_train / s->batch * s->batch;
    if (n_train == 0) return cbi::fail(CB_ERR_INVALID, "fewer training cells than one batch");
    if (n_train > ((size_t)1 << 30)) return cbi::fail(CB_ERR_INVALID, "at most 2^30 training cells");
    SUR_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = s->stream;
    SUR_CUDA(cudaStreamSynchronize(st));
    cudaFree(s->X);
    cudaFree(s->Y);
    s->X = nullptr;
    s->Y = nullptr;
    s->n_train = 0;
    SUR_RC(dalloc(&s->X, n_train * s->n_in));
    SUR_RC(dalloc(&s->Y, n_train * s->n_out));
    SUR_RC(make_map(&s->mX, s->X, s->n_in, n_train, kBM));
    SUR_RC(make_map(&s->mX_K, s->X, s->n_in, n_train, kBK));
    const int K = s->K, nf = s->n_feat;
    const size_t C = std::min(n_train, (size_t)1 << 20);
    double* cells = nullptr;
    double* tout = nullptr;
    float *raw_in = nullptr, *raw_out = nullptr;
    int* hull = nullptr;
    auto cleanup = [&](int rc) {
        cudaFree(cells);
        cudaFree(tout);
        cudaFree(raw_in);
        cudaFree(raw_out);
        cudaFree(hull);
        return rc;
    };
    int rc = dalloc(&cells, (size_t)(K + 3) * C);
    rc = rc ? rc : dalloc(&tout, (size_t)(K + 2) * C);
    const size_t S = std::min(C, (size_t)65536);  // statistics sample
    rc = rc ? rc : dalloc(&raw_in, S * nf);
    rc = rc ? rc : dalloc(&raw_out, S * nf);
    rc = rc ? rc : dalloc(&hull, 2 * (size_t)nf);
    if (rc) return cleanup(rc);
    std::vector<double*> cin(K + 3), cout_(K + 2);
    for (int q = 0; q < K + 3; q++) cin[q] = cells + (size_t)q * C;
    for (int q = 0; q < K + 2; q++) cout_[q] = tout + (size_t)q * C;
    std::vector<int> hinit(2 * nf);
    for (int j = 0; j < nf; j++) {
        hinit[j] = 0x7fffffff;
        hinit[nf + j] = (int)0x80000000;
    }
    if (cudaMemcpy(hull, hinit.data(), hinit.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
        return cleanup(cbi::fail(CB_ERR_CUDA, "hull init"));
    const double T0 = cbi::view(s->mech).T0;
    std::vector<float> hn((size_t)kNormRows * s->n_out, 0.f);
    for (size_t lo = 0; lo < n_train; lo += C) {
        const size_t len = std::min(C, n_train - lo);
        rc = cb_generate_cells(s->mech, len, lo, dist, cin.data(), st);
        rc = rc ? rc : cbi::transport_gather(s->mech, len, cin.data(), cout_.data(), nullptr, nullptr, false, 0, st);
        if (rc) return cleanup(rc);
        if (lo == 0) {  // normalisation from the first cells: raw features and log outputs of S cells
            FeatureArgs f;
            std::memset(&f, 0, sizeof f);
            for (int q = 0; q < K + 3; q++) f.in[q] = cin[q];
            f.n = f.rows = S;
            f.K = K;
            f.n_feat = nf;
            f.n_in = s->n_in;
            f.T0 = T0;
            f.R_over_P0 = kR / 101325.0;
            f.mean = nrm(s, kInMean);  // zero until set: only the raw copy is used here
            f.rstd = nrm(s, kInRstd);
            f.X = s->X;
            f.raw = raw_in;
            TargetArgs t;
            std::memset(&t, 0, sizeof t);
            for (int q = 0; q < K + 2; q++) t.out[q] = cout_[q];
            t.n = S;
            t.n_feat = nf;
            t.n_out = s->n_out;
            t.mean = nrm(s, kOutMean);
            t.rstd = nrm(s, kOutRstd);
            t.Y = s->Y;
            t.raw = raw_out;
            if (cudaMemsetAsync(s->norm, 0, (size_t)kNormRows * s->n_out * sizeof(float), st) != cudaSuccess ||
                features(f, st) != cudaSuccess || targets(t, st) != cudaSuccess)
                return cleanup(cbi::fail(CB_ERR_CUDA, "normalisation sample"));
            std::vector<float> ri(S * nf), ro(S * nf);
            if (cudaMemcpyAsync(ri.data(), raw_in, ri.size() * sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaMemcpyAsync(ro.data(), raw_out, ro.size() * sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess)
                return cleanup(cbi::fail(CB_ERR_CUDA, "normalisation sample copy"));
            for (int j = 0; j < nf; j++) {
                double m_in = 0, m_out = 0;
                for (size_t c = 0; c < S; c++) {
                    m_in += ri[c * nf + j];
                    m_out += ro[c * nf + j];
                }
                m_in /= (double)S;
                m_out /= (double)S;
                double v_in = 0, v_out = 0;
                for (size_t c = 0; c < S; c++) {
                    v_in += (ri[c * nf + j] - m_in) * (ri[c * nf + j] - m_in);
                    v_out += (ro[c * nf + j] - m_out) * (ro[c * nf + j] - m_out);
                }
                const double sd_in = std::sqrt(v_in / (double)S), sd_out = std::sqrt(v_out / (double)S);
                if (!std::isfinite(m_out) || !std::isfinite(sd_out))
                    return cleanup(cbi::fail(CB_ERR_MECHANISM, "non-finite transport outputs in the training cells"));
                hn[(size_t)kInMean * s->n_out + j] = (float)m_in;
                hn[(size_t)kInRstd * s->n_out + j] = sd_in > 1e-12 ? (float)(1.0 / sd_in) : 1.f;
                hn[(size_t)kOutMean * s->n_out + j] = (float)m_out;
                hn[(size_t)kOutRstd * s->n_out + j] = sd_out > 1e-12 ? (float)(1.0 / sd_out) : 1.f;
                hn[(size_t)kOutStd * s->n_out + j] = sd_out > 1e-12 ? (float)sd_out : 1.f;
            }
            if (cudaMemcpyAsync(s->norm, hn.data(), hn.size() * sizeof(float), cudaMemcpyHostToDevice, st) != cudaSuccess)
                return cleanup(cbi::fail(CB_ERR_CUDA, "normalisation upload"));
        }
        FeatureArgs f;
        std::memset(&f, 0, sizeof f);
        for (int q = 0; q < K + 3; q++) f.in[q] = cin[q];
        f.n = f.rows = len;
        f.K = K;
        f.n_feat = nf;
        f.n_in = s->n_in;
        f.T0 = T0;
        f.R_over_P0 = kR / 101325.0;
        f.mean = nrm(s, kInMean);
        f.rstd = nrm(s, kInRstd);
        f.X = s->X;
        f.row0 = lo;
        f.hull_lo = hull;
        f.hull_hi = hull + nf;
        TargetArgs t;
        std::memset(&t, 0, sizeof t);
        for (int q = 0; q < K + 2; q++) t.out[q] = cout_[q];
        t.n = len;
        t.row0 = lo;
        t.n_feat = nf;
        t.n_out = s->n_out;
        t.mean = nrm(s, kOutMean);
        t.rstd = nrm(s, kOutRstd);
        t.Y = s->Y;
        if (features(f, st) != cudaSuccess || targets(t, st) != cudaSuccess)
            return cleanup(cbi::fail(CB_ERR_CUDA, "training features"));
    }
    std::vector<int> hh(2 * nf);
    if (cudaMemcpyAsync(hh.data(), hull, hh.size() * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return cleanup(cbi::fail(CB_ERR_CUDA, "training set"));
    for (int j = 0; j < nf; j++) {
        for (int side = 0; side < 2; side++) {
            int i = hh[side * nf + j];
            i = i >= 0 ? i : i ^ 0x7fffffff;
            float v;
            std::memcpy(&v, &i, sizeof v);
            hn[(size_t)(side ? kHi : kLo) * s->n_out + j] = v;
        }
    }
    if (cudaMemcpy(s->norm, hn.data(), hn.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
        return cleanup(cbi::fail(CB_ERR_CUDA, "trust region upload"));
    s->h_norm = hn;
    s->have_norm = true;
    s->n_train = n_train;
    SUR_CUDA(cudaMemset(s->counters + 1, 0, sizeof(int)));
    rc = check_device_status(s);
    return cleanup(rc);
}

int cb_surrogate_train(cb_surrogate* s, int32_t steps, float* losses) {
    if (!s) return cbi::fail(CB_ERR_INVALID, "null argument");
    if (!s->n_train) return cbi::fail(CB_ERR_NOT_READY, "cb_surrogate_generate has not run");
    if (steps <= 0) return CB_OK;
    if (s->steps_done + steps > kMaxSteps)
        return cbi::fail(CB_ERR_INVALID, "at most 2^20 training steps between parameter resets");
    SUR_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = s->stream;
    // the step counter restarts at the call's first step for the learning-rate schedule; Adam's bias
    // corrections use it as well (moments restart when the parameters are set)
    SUR_CUDA(cudaStreamSynchronize(st));
    // one training step as a CUDA graph: forward, backward, Adam, loss / step bookkeeping
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    SUR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = run_pass(s, s->batch, s->mX, s->mX_K, s->Y, true, true, true, (int)(s->steps_done + steps), st);
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return cbi::cuda_fail(e, "training step capture");
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cbi::cuda_fail(e, "training step graph");
    for (int i = 0; i < steps; i++) {
        e = cudaGraphLaunch(exec, st);
        if (e != cudaSuccess) break;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaGraphExecDestroy(exec);
    if (e != cudaSuccess) return cbi::cuda_fail(e, "training steps");
    const long long first = s->steps_done;
    s->steps_done += steps;
    if (losses) SUR_CUDA(cudaMemcpy(losses, s->losses + first, (size_t)steps * sizeof(float), cudaMemcpyDeviceToHost));
    return check_device_status(s);
}

int cb_surrogate_evaluate(cb_surrogate* s, int32_t rows, const float* features_h, const float* targets_h, float* loss,
                          float* grads, float* outputs_h) {
    if (!s || !features_h || !targets_h) return cbi::fail(CB_ERR_INVALID, "null argument");
    if (rows < 128 || rows % 128 || rows > s->batch) return cbi::fail(CB_ERR_INVALID, "rows: a multiple of 128, at most the batch");
    SUR_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = s->stream;
    const int n_in = s->n_in, n_out = s->n_out;
    std::vector<bf16> xb((size_t)rows * n_in);
    for (size_t e = 0; e < xb.size(); e++) xb[e] = __float2bfloat16(features_h[e]);
    SUR_CUDA(cudaMemcpyAsync(s->Xs, xb.data(), xb.size() * sizeof(bf16), cudaMemcpyHostToDevice, st));
    SUR_CUDA(cudaMemcpyAsync(s->Ys, targets_h, (size_t)rows * n_out * sizeof(float), cudaMemcpyHostToDevice, st));
    SUR_RC(run_pass(s, rows, s->mXs, s->mXs_K, s->Ys, false, true, false, 1, st));
    std::vector<float> lp(kEpiWarps * rows / kBM);
    SUR_CUDA(cudaMemcpyAsync(lp.data(), s->loss_part, lp.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (grads) SUR_CUDA(cudaMemcpyAsync(grads, s->g, s->n_params * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (outputs_h) {
        SUR_RC(ensure_inference(s, rows));
        SUR_RC(infer_rows(s, rows, s->mXs, st));
        SUR_CUDA(cudaMemcpyAsync(outputs_h, s->Yi, (size_t)rows * n_out * sizeof(float), cudaMemcpyDeviceToHost, st));
    }
    SUR_CUDA(cudaStreamSynchronize(st));
    if (loss) {
        double t = 0;
        for (float v : lp) t += v;
        *loss = (float)(t / ((double)rows * s->n_feat));
    }
    return check_device_status(s);
}

int cb_surrogate_transport(cb_surrogate* s, size_t n, const double* const* inputs, double* const* outputs,
                           uint32_t flags, uint32_t audit_stride, cb_surrogate_stats* stats, void* stream) {
    if (!s || !inputs || !outputs) return cbi::fail(CB_ERR_INVALID, "null argument");
    if (flags & ~(CB_UNIFORM_PRESSURE | CB_SURROGATE_NO_GATE | CB_SURROGATE_TIMING))
        return cbi::fail(CB_ERR_INVALID, "unknown flag");
    if (!s->have_norm) return cbi::fail(CB_ERR_NOT_READY, "cb_surrogate_generate has not run");
    if (n >= ((size_t)1 << 31)) return cbi::fail(CB_ERR_INVALID, "at most 2^31 - 1 cells per call");
    const int K = s->K, nf = s->n_feat;
    for (int q = 0; q < K + 3; q++)
        if (!inputs[q]) return cbi::fail(CB_ERR_INVALID, "null input array");
    for (int q = 0; q < K + 2; q++)
        if (!outputs[q]) return cbi::fail(CB_ERR_INVALID, "null output array");
    if (stats) std::memset(stats, 0, sizeof *stats);
    if (n == 0) return CB_OK;
    SUR_CUDA(cudaSetDevice(s->device));
    SUR_RC(ensure_inference(s, kInferChunk));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool gate = !(flags & CB_SURROGATE_NO_GATE);
    const bool uniform = flags & CB_UNIFORM_PRESSURE;
    const double T0 = cbi::view(s->mech).T0;
    // gate lists over the whole call: every cell may fall back; one audited cell per audit_stride
    const size_t audit_cap = gate && audit_stride ? n / audit_stride + 1 : 0;
    if (gate && n > s->fail_cap) {
        cudaFree(s->fail_idx);
        s->fail_idx = nullptr;
        s->fail_cap = 0;
        SUR_RC(dalloc(&s->fail_idx, n));
        s->fail_cap = n;
    }
    if (audit_cap > s->audit_cap) {
        cudaFree(s->audit_idx);
        cudaFree(s->audit_plain);
        s->audit_idx = nullptr;
        s->audit_plain = nullptr;
        s->audit_cap = 0;
        SUR_RC(dalloc(&s->audit_idx, audit_cap));
        SUR_RC(dalloc(&s->audit_plain, audit_cap * (size_t)(K + 2)));
        s->audit_cap = audit_cap;
    }
    // optional phase timing: features, network, outputs (summed over chunks), then the gate's plain work
    const bool timing = flags & CB_SURROGATE_TIMING;
    cudaEvent_t ev[5] = {};
    double ms[4] = {0, 0, 0, 0};
    struct EventGuard {
        cudaEvent_t* ev;
        ~EventGuard() {
            for (int i = 0; i < 5; i++)
                if (ev[i]) cudaEventDestroy(ev[i]);
        }
    } guard{ev};
    if (timing)
        for (auto& e : ev) SUR_CUDA(cudaEventCreate(&e));
    auto mark = [&](int i) { return timing ? cudaEventRecord(ev[i], st) : cudaSuccess; };
    auto elapsed = [&](int i, int j) -> cudaError_t {
        if (!timing) return cudaSuccess;
        cudaError_t e = cudaEventSynchronize(ev[j]);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev[i], ev[j]);
        ms[i] += t;
        return e;
    };
    SUR_CUDA(cudaMemsetAsync(s->err_max, 0, 3 * sizeof(unsigned), st));
    SUR_CUDA(cudaMemsetAsync(s->err_sq, 0, 3 * sizeof(double), st));
    if (gate) SUR_CUDA(cudaMemsetAsync(s->gate_count, 0, 2 * sizeof(uint32_t), st));
    std::vector<const double*> in(K + 3);
    std::vector<double*> out(K + 2);
    for (size_t lo = 0; lo < n; lo += kInferChunk) {
        const size_t len = std::min(kInferChunk, n - lo);
        const int rows = (int)((len + kBM - 1) / kBM * kBM);
        for (int q = 0; q < K + 3; q++) in[q] = (uniform && q < 2) ? inputs[q] : inputs[q] + lo;
        for (int q = 0; q < K + 2; q++) out[q] = outputs[q] + lo;
        FeatureArgs f;
        std::memset(&f, 0, sizeof f);
        for (int q = 0; q < K + 3; q++) f.in[q] = in[q];
        f.n = len;
        f.rows = rows;
        f.K = K;
        f.n_feat = nf;
        f.n_in = s->n_in;
        f.uniform_pressure = uniform;
        f.T0 = T0;
        f.R_over_P0 = kR / 101325.0;
        f.mean = nrm(s, kInMean);
        f.rstd = nrm(s, kInRstd);
        f.X = s->Xi;
        if (gate) {
            f.lo = nrm(s, kLo);
            f.hi = nrm(s, kHi);
            f.fail_idx = s->fail_idx;
            f.fail_count = s->gate_count;
            f.audit_idx = s->audit_idx;
            f.audit_count = s->gate_count + 1;
            f.audit_stride = audit_stride;
            f.audit_phase = audit_stride ? (uint32_t)(7919u % audit_stride) : 0u;
            f.audit_cap = (uint32_t)audit_cap;
            f.idx_base = (uint32_t)lo;
        }
        SUR_CUDA(mark(0));
        SUR_CUDA(features(f, st));
        SUR_CUDA(mark(1));
        SUR_RC(infer_rows(s, rows, s->mXi, st));
        SUR_CUDA(mark(2));
        OutputArgs o;
        std::memset(&o, 0, sizeof o);
        o.Y = s->Yi;
        o.ldY = s->n_out;
        o.n = len;
        o.n_feat = nf;
        o.mean = nrm(s, kOutMean);
        o.std = nrm(s, kOutStd);
        for (int q = 0; q < K + 2; q++) o.out[q] = out[q];
        SUR_CUDA(cbg::sur::outputs(o, st));
        SUR_CUDA(mark(3));
        SUR_CUDA(elapsed(0, 1));
        SUR_CUDA(elapsed(1, 2));
        SUR_CUDA(elapsed(2, 3));
    }
    uint64_t n_fail = 0, n_audit = 0;
    if (gate) {
        uint32_t cnt[2];
        SUR_CUDA(cudaMemcpyAsync(cnt, s->gate_count, sizeof cnt, cudaMemcpyDeviceToHost, st));
        SUR_CUDA(cudaStreamSynchronize(st));
        n_fail = cnt[0];
        n_audit = std::min<uint64_t>(cnt[1], audit_cap);
        SUR_CUDA(mark(3));
        const uint32_t pflags = uniform ? CB_UNIFORM_PRESSURE : 0;
        if (n_fail)  // the plain kernel writes the rejected cells' outputs in place
            SUR_RC(cbi::transport_gather(s->mech, n_fail, inputs, outputs, s->fail_idx, s->gate_count, false,
                                         pflags, st));
        if (n_audit) {
            std::vector<double*> aud(K + 2);
            for (int q = 0; q < K + 2; q++) aud[q] = s->audit_plain + (size_t)q * audit_cap;
            SUR_RC(cbi::transport_gather(s->mech, n_audit, inputs, aud.data(), s->audit_idx, s->gate_count + 1,
                                         true, pflags, st));
            AuditArgs a;
            std::memset(&a, 0, sizeof a);
            a.idx = s->audit_idx;
            a.count = s->gate_count + 1;
            a.plain = s->audit_plain;
            a.cap = audit_cap;
            for (int q = 0; q < K + 2; q++) a.out[q] = outputs[q];
            a.n_feat = nf;
            a.max_err = s->err_max;
            a.sum_sq = s->err_sq;
            SUR_CUDA(audit(a, n_audit, st));
        }
        SUR_CUDA(mark(4));
        SUR_CUDA(elapsed(3, 4));
    }
    unsigned em[3];
    double es[3];
    SUR_CUDA(cudaMemcpyAsync(em, s->err_max, sizeof em, cudaMemcpyDeviceToHost, st));
    SUR_CUDA(cudaMemcpyAsync(es, s->err_sq, sizeof es, cudaMemcpyDeviceToHost, st));
    SUR_CUDA(cudaStreamSynchronize(st));
    if (stats) {
        stats->cells = n;
        stats->fallback_cells = n_fail;
        stats->audited_cells = n_audit;
        const double counts[3] = {(double)n_audit, (double)n_audit, (double)n_audit * K};
        for (int gI = 0; gI < 3; gI++) {
            float v;
            std::memcpy(&v, &em[gI], sizeof v);
            stats->audit_max_rel_err[gI] = v;
            stats->audit_rms_rel_err[gI] = n_audit ? std::sqrt(es[gI] / counts[gI]) : 0.0;
        }
        stats->ms_features = ms[0];
        stats->ms_network = ms[1];
        stats->ms_outputs = ms[2];
        stats->ms_gate = ms[3];
    }
    return check_device_status(s);
}

int cb_surrogate_transport_pair(cb_surrogate* a, cb_surrogate* b, size_t n, const double* const* inputs,
                                double* const* outputs, uint32_t flags, const cb_surrogate_gate* gate,
                                cb_surrogate_stats* stats, void* stream) {
    if (!a || !b || !inputs || !outputs || !gate) return cbi::fail(CB_ERR_INVALID, "null argument");
    if (a == b) return cbi::fail(CB_ERR_INVALID, "the two networks must be different objects");
    if (flags & ~(CB_UNIFORM_PRESSURE | CB_SURROGATE_TIMING)) return cbi::fail(CB_ERR_INVALID, "unknown flag");
    if (a->mech != b->mech || a->n_feat != b->n_feat || a->n_in != b->n_in || a->n_out != b->n_out ||
        a->device != b->device)
        return cbi::fail(CB_ERR_INVALID, "the two networks must belong to the same mechanism and device");
    if (gate->fallback != CB_FALLBACK_MIXED && gate->fallback != CB_FALLBACK_PLAIN)
        return cbi::fail(CB_ERR_INVALID, "unknown fallback kernel");
    if (!a->have_norm || !b->have_norm) return cbi::fail(CB_ERR_NOT_READY, "cb_surrogate_generate has not run");
    if (n >= ((size_t)1 << 31)) return cbi::fail(CB_ERR_INVALID, "at most 2^31 - 1 cells per call");
    if (std::isnan(gate->threshold)) return cbi::fail(CB_ERR_INVALID, "NaN threshold");
    const int K = a->K, nf = a->n_feat;
    for (int q = 0; q < K + 3; q++)
        if (!inputs[q]) return cbi::fail(CB_ERR_INVALID, "null input array");
    for (int q = 0; q < K + 2; q++)
        if (!outputs[q]) return cbi::fail(CB_ERR_INVALID, "null output array");
    if (stats) std::memset(stats, 0, sizeof *stats);
    if (n == 0) return CB_OK;
    SUR_CUDA(cudaSetDevice(a->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool uniform = flags & CB_UNIFORM_PRESSURE;
    if (gate->threshold < 0.0) {  // every cell falls back: the fallback kernel alone, no network, no audit
        const uint32_t pflags = uniform ? CB_UNIFORM_PRESSURE : 0;
        if (gate->fallback == CB_FALLBACK_MIXED)
            SUR_RC(cbi::transport_gather_mixed(a->mech, n, inputs, outputs, nullptr, nullptr, false, pflags, st));
        else
            SUR_RC(cbi::transport_gather(a->mech, n, inputs, outputs, nullptr, nullptr, false, pflags, st));
        SUR_CUDA(cudaStreamSynchronize(st));
        if (stats) {
            stats->cells = n;
            stats->fallback_cells = n;
        }
        return cbi::check_status(a->mech);
    }
    SUR_RC(ensure_inference(a, kInferChunk));
    SUR_RC(ensure_inference(b, kInferChunk));
    const double T0 = cbi::view(a->mech).T0;
    const uint32_t audit_stride = gate->audit_stride;
    // Networks trained on the same cell distribution share their input normalisation: the features are
    // then computed once and both networks read them.
    const bool same_inputs =
        a->n_in == b->n_in && a->h_norm.size() == b->h_norm.size() &&
        std::memcmp(a->h_norm.data(), b->h_norm.data(), 2 * (size_t)a->n_out * sizeof(float)) == 0;
    const size_t audit_cap = audit_stride ? n / audit_stride + 1 : 0;
    // every cell may fall back; the lists and per-cell arrays live in the first network's object
    if (n > a->fail_cap) {
        cudaFree(a->fail_idx);
        a->fail_idx = nullptr;
        a->fail_cap = 0;
        SUR_RC(dalloc(&a->fail_idx, n));
        a->fail_cap = n;
    }
    if (n > a->cell_cap) {
        cudaFree(a->outside);
        cudaFree(a->disagreement);
        a->outside = nullptr;
        a->disagreement = nullptr;
        a->cell_cap = 0;
        SUR_RC(dalloc(&a->outside, n));
        SUR_RC(dalloc(&a->disagreement, n));
        a->cell_cap = n;
    }
    if (audit_cap > a->audit_cap) {
        cudaFree(a->audit_idx);
        cudaFree(a->audit_plain);
        a->audit_idx = nullptr;
        a->audit_plain = nullptr;
        a->audit_cap = 0;
        SUR_RC(dalloc(&a->audit_idx, audit_cap));
        SUR_RC(dalloc(&a->audit_plain, audit_cap * (size_t)(K + 2)));
        a->audit_cap = audit_cap;
    }
    const bool timing = flags & CB_SURROGATE_TIMING;
    cudaEvent_t ev[5] = {};
    double ms[4] = {0, 0, 0, 0};
    struct EventGuard {
        cudaEvent_t* ev;
        ~EventGuard() {
            for (int i = 0; i < 5; i++)
                if (ev[i]) cudaEventDestroy(ev[i]);
        }
    } guard{ev};
    if (timing)
        for (auto& e : ev) SUR_CUDA(cudaEventCreate(&e));
    auto mark = [&](int i) { return timing ? cudaEventRecord(ev[i], st) : cudaSuccess; };
    auto elapsed = [&](int i, int j) -> cudaError_t {
        if (!timing) return cudaSuccess;
        cudaError_t e = cudaEventSynchronize(ev[j]);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev[i], ev[j]);
        ms[i] += t;
        return e;
    };
    SUR_CUDA(cudaMemsetAsync(a->err_max, 0, 3 * sizeof(unsigned), st));
    SUR_CUDA(cudaMemsetAsync(a->err_sq, 0, 3 * sizeof(double), st));
    SUR_CUDA(cudaMemsetAsync(a->gate_count, 0, 2 * sizeof(uint32_t), st));
    for (size_t lo = 0; lo < n; lo += kInferChunk) {
        const size_t len = std::min(kInferChunk, n - lo);
        const int rows = (int)((len + kBM - 1) / kBM * kBM);
        SUR_CUDA(mark(0));
        for (cb_surrogate* s : {a, b}) {  // each network's own normalisation of the same cells
            if (s == b && same_inputs) break;
            FeatureArgs f;
            std::memset(&f, 0, sizeof f);
            for (int q = 0; q < K + 3; q++) f.in[q] = (uniform && q < 2) ? inputs[q] : inputs[q] + lo;
            f.n = len;
            f.rows = rows;
            f.K = K;
            f.n_feat = nf;
            f.n_in = s->n_in;
            f.uniform_pressure = uniform;
            f.T0 = T0;
            f.R_over_P0 = kR / 101325.0;
            f.mean = nrm(s, kInMean);
            f.rstd = nrm(s, kInRstd);
            f.X = s->Xi;
            if (s == a) {  // the first network's training range is the trust region
                f.lo = nrm(a, kLo);
                f.hi = nrm(a, kHi);
                f.outside = a->outside;
                f.idx_base = (uint32_t)lo;
            }
            SUR_CUDA(features(f, st));
        }
        SUR_CUDA(mark(1));
        SUR_RC(infer_rows(a, rows, a->mXi, st));
        SUR_RC(infer_rows(b, rows, same_inputs ? a->mXi : b->mXi, st));
        SUR_CUDA(mark(2));
        CombineArgs c;
        std::memset(&c, 0, sizeof c);
        c.Ya = a->Yi;
        c.Yb = b->Yi;
        c.ldY = a->n_out;
        c.n = len;
        c.n_feat = nf;
        c.mean_a = nrm(a, kOutMean);
        c.std_a = nrm(a, kOutStd);
        c.mean_b = nrm(b, kOutMean);
        c.std_b = nrm(b, kOutStd);
        for (int q = 0; q < K + 2; q++) c.out[q] = outputs[q] + lo;
        c.threshold = (float)gate->threshold;
        c.outside = a->outside;
        c.disagreement = a->disagreement;
        c.fail_idx = a->fail_idx;
        c.fail_count = a->gate_count;
        c.audit_idx = a->audit_idx;
        c.audit_count = a->gate_count + 1;
        c.audit_stride = audit_stride;
        c.audit_phase = audit_stride ? (uint32_t)(7919u % audit_stride) : 0u;
        c.audit_cap = (uint32_t)audit_cap;
        c.idx_base = (uint32_t)lo;
        SUR_CUDA(combine(c, st));
        SUR_CUDA(mark(3));
        SUR_CUDA(elapsed(0, 1));
        SUR_CUDA(elapsed(1, 2));
        SUR_CUDA(elapsed(2, 3));
    }
    if (gate->disagreement)
        SUR_CUDA(cudaMemcpyAsync(gate->disagreement, a->disagreement, n * sizeof(float), cudaMemcpyDeviceToDevice, st));
    uint32_t cnt[2];
    SUR_CUDA(cudaMemcpyAsync(cnt, a->gate_count, sizeof cnt, cudaMemcpyDeviceToHost, st));
    SUR_CUDA(cudaStreamSynchronize(st));
    const uint64_t n_fail = cnt[0], n_audit = std::min<uint64_t>(cnt[1], audit_cap);
    SUR_CUDA(mark(3));
    const uint32_t pflags = uniform ? CB_UNIFORM_PRESSURE : 0;
    if (n_fail) {  // the fallback kernel writes the rejected cells' outputs in place
        if (gate->fallback == CB_FALLBACK_MIXED)
            SUR_RC(cbi::transport_gather_mixed(a->mech, n_fail, inputs, outputs, a->fail_idx, a->gate_count, false,
                                               pflags, st));
        else
            SUR_RC(cbi::transport_gather(a->mech, n_fail, inputs, outputs, a->fail_idx, a->gate_count, false, pflags,
                                         st));
    }
    if (n_audit) {  // the audit's judge is the plain FP64 kernel
        std::vector<double*> aud(K + 2);
        for (int q = 0; q < K + 2; q++) aud[q] = a->audit_plain + (size_t)q * audit_cap;
        SUR_RC(cbi::transport_gather(a->mech, n_audit, inputs, aud.data(), a->audit_idx, a->gate_count + 1, true,
                                     pflags, st));
        AuditArgs au;
        std::memset(&au, 0, sizeof au);
        au.idx = a->audit_idx;
        au.count = a->gate_count + 1;
        au.plain = a->audit_plain;
        au.cap = audit_cap;
        for (int q = 0; q < K + 2; q++) au.out[q] = outputs[q];
        au.n_feat = nf;
        au.max_err = a->err_max;
        au.sum_sq = a->err_sq;
        SUR_CUDA(audit(au, n_audit, st));
    }
    SUR_CUDA(mark(4));
    SUR_CUDA(elapsed(3, 4));
    unsigned em[3];
    double es[3];
    SUR_CUDA(cudaMemcpyAsync(em, a->err_max, sizeof em, cudaMemcpyDeviceToHost, st));
    SUR_CUDA(cudaMemcpyAsync(es, a->err_sq, sizeof es, cudaMemcpyDeviceToHost, st));
    SUR_CUDA(cudaStreamSynchronize(st));
    if (stats) {
        stats->cells = n;
        stats->fallback_cells = n_fail;
        stats->audited_cells = n_audit;
        const double counts[3] = {(double)n_audit, (double)n_audit, (double)n_audit * K};
        for (int gI = 0; gI < 3; gI++) {
            float v;
            std::memcpy(&v, &em[gI], sizeof v);
            stats->audit_max_rel_err[gI] = v;
            stats->audit_rms_rel_err[gI] = n_audit ? std::sqrt(es[gI] / counts[gI]) : 0.0;
        }
        stats->ms_features = ms[0];
        stats->ms_network = ms[1];
        stats->ms_outputs = ms[2];
        stats->ms_gate = ms[3];
    }
    SUR_RC(check_device_status(b));
    return check_device_status(a);
}

}  // extern "C"
