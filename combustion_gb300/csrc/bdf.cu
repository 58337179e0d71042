// Batched constant-pressure reactors: a variable-order (1-5), variable-step BDF integrator in
// backward-difference form with Newton iterations on an analytic Jacobian, one warp per reactor.
//
// Role in the reference: the reactor loop of plot.rs:32-118 (state u = [T, V, n_active], du/dt = the
// rates function's outputs, reaction.rs:356-391) and the cvode crate's BDF (cvode/lib.rs:17-47: CV_BDF,
// dense linear solver, difference-quotient Jacobian). Here many reactors advance together: each warp
// owns one reactor at a time, taken from a work queue, and keeps its iteration matrix (LU with partial
// pivoting), difference array and rates scratch in shared memory, or in global memory (large mechanisms,
// or where the autotuner finds it faster: then each reactor keeps its own factorisation, made by panels,
// with a transposed copy for coalesced triangular solves); the rates program runs
// warp-cooperatively (lanes split species, third-body rows and reactions; per-species sums in the
// reactions' order). Launches are slices of at most `slice_steps` steps per reactor so that reactors of
// uneven stiffness rebalance between launches; a CUDA graph replays the slice sequence.
//
// Method (the published variable-step BDF of Shampine & Reichelt, "The MATLAB ODE suite", SIAM J. Sci.
// Comput. 18(1), 1997, with kappa = 0): predictor y_pred = sum_{j<=q} D_j, corrector
// d - c f(t_new, y_pred + d) + psi = 0 with c = h / gamma_q and psi = sum_{j=1..q} gamma_j D_j / gamma_q,
// solved by at most 4 Newton iterations on (I - c J); local error (1/(q+1)) d against atol + rtol |y|;
// step and order from the error norms of orders q-1, q, q+1 after q+1 steps of equal size; the
// difference array is rescaled by the R U matrices when h changes. J is recomputed only when Newton
// fails with a Jacobian from an earlier step; (I - c J) is refactorised after a step or order change
// and after a Newton failure, but kept after a rejected error test (Newton converged with it).
// Jacobian: species and volume columns analytic (mass action, third-body and falloff efficiencies with
// the Troe broadening held fixed), T and V rows by the chain rule through the energy equation, the
// temperature column by one forward difference.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/combustion_gb300.h"
#include "capi_internal.h"
#include "bdf_device.cuh"

namespace cbg {
namespace bdf {

// Evaluation hook: f and J at given states, one warp per state.
__global__ void eval_kernel(const __grid_constant__ Params p, int count) {
    const uint8_t* tab = p.tab;
    __shared__ uint64_t bar;
    if (p.smem_tables) {
        if (!stage_to_shared(cb_dsmem, p.tab, p.tab_bytes, &bar, p.status)) return;
        tab = cb_dsmem;
    } else {
        load_math(p.tab);
    }
    const Mech m(tab, p);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const Work w = carve(p, workspace_of(p, warp), (size_t)blockIdx.x * (blockDim.x >> 5) + warp);
    const int N = p.N;
    for (int s = blockIdx.x * (blockDim.x >> 5) + warp; s < count; s += gridDim.x * (blockDim.x >> 5)) {
        for (int i = lane; i < N; i += 32) w.y[i] = p.eval_y[(size_t)s * N + i];
        __syncwarp();
        jacobian_warp(p, m, w, p.pR[s], 1.0 / p.pR[s], w.y, p.eval_J + (size_t)s * N * N, w.LU, lane);
        if (p.mixed) rhs_warp_mixed(p, m, RatesMixedTables(p.tab_m), w, p.pR[s], 1.0 / p.pR[s], w.y, w.f, lane);
        for (int i = lane; i < N; i += 32) p.eval_f[(size_t)s * N + i] = w.f[i];
        __syncwarp();
    }
}

}  // namespace bdf
}  // namespace cbg

using namespace cbg::bdf;

struct cb_reactors {
    cb_mech* mech = nullptr;
    int device = 0;
    int K = 0, A = 0, R = 0, N = 0, LD = 0, n_eff = 0;
    size_t n = 0;         // reactors the launches cover (the autotuner lowers it while it calibrates)
    size_t capacity = 0;  // reactors of the batch: every per-reactor buffer holds this many
    cb_bdf_options opt{};
    std::vector<uint8_t> blob;
    int off_csr_start = 0, off_csr = 0, off_eff_t = 0;
    uint8_t* d_tab = nullptr;
    double* pR = nullptr;
    Head* head = nullptr;
    double* D = nullptr;
    double* J = nullptr;
    int* counters = nullptr;  // queue, done, status
    int warps = 0, smem_tables = -1;  // launch shape (0 / -1: autotune)
    bool have_state = false;
    cudaStream_t stream = nullptr;
    uint8_t* d_tab_m = nullptr;  // mixed-precision rates tables (CB_BDF_MIXED_RHS)
    // Workspaces in global memory (large mechanisms, CB_BDF_GLOBAL_MEMORY or the autotuner's choice):
    // ws_slots per-warp workspaces, and per reactor its factorisation, transpose, row order and 1 / U_kk.
    bool global = false;
    bool smem_ok = false;  // one workspace fits in shared memory and CB_BDF_GLOBAL_MEMORY is not set
    int regs = 64;         // global memory: the slice kernel's register cap (64: four blocks of 256 threads per
                           // SM, 80: three, 128: two)
    uint8_t* ws = nullptr;
    size_t ws_slots = 0;
    double *LUr = nullptr, *LUt = nullptr, *rdiag_r = nullptr;
    int* piv_r = nullptr;
    // Shared-memory workspaces: the Jacobian's per-reaction terms (kf, pK, sM) of every warp slot in
    // global memory instead, [jac_slots][3 R] (they are used by the Jacobian only).
    double* jac_ws = nullptr;
    size_t jac_slots = 0;
    // cb_reactors_set_outputs: trajectory [n][n_points][N] and the peak species' state [n][N]
    double* traj = nullptr;
    int n_points = 0, peak_k = -1;
    double* peak_state = nullptr;
};

namespace {

#define BDF_CUDA(call)                                           \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return cbi::cuda_fail(e_, #call); \
    } while (0)

uint32_t ws_bytes(const cb_reactors* s) {
    const size_t d = workspace_doubles(s->K, s->A, s->R, s->N, s->LD, s->n_eff, s->global);
    return (uint32_t)(((d * sizeof(double) + (size_t)s->N * sizeof(int)) + 127) & ~(size_t)127);
}

size_t smem_bytes(const cb_reactors* s, int warps, int tables) {
    const size_t tab = tables ? ((s->blob.size() + 127) & ~(size_t)127) : (size_t)cbg::kMathBytes;
    return tab + (s->global ? 0 : (size_t)warps * ws_bytes(s));
}

int max_smem() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v - 1024;
}

int sm_count() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
}

Params params(cb_reactors* s, int tables) {
    Params p;
    std::memset(&p, 0, sizeof p);
    p.tab = s->d_tab;
    p.tab_bytes = (uint32_t)s->blob.size();
    p.smem_tables = tables;
    p.off_csr_start = s->off_csr_start;
    p.off_csr = s->off_csr;
    p.off_eff_t = s->off_eff_t;
    p.K = s->K;
    p.A = s->A;
    p.R = s->R;
    p.N = s->N;
    p.LD = s->LD;
    p.n_eff = s->n_eff;
    p.ws_bytes = ws_bytes(s);
    p.n = (int)s->n;
    p.rtol = s->opt.rtol;
    p.atol = s->opt.atol;
    p.t_end = s->opt.t_end;
    p.h_min = 1e-20;
    p.max_steps = s->opt.max_steps;
    p.slice_steps = s->opt.slice_steps;
    p.pR = s->pR;
    p.head = s->head;
    p.D = s->D;
    p.J = s->J;
    p.queue = s->counters;
    p.done = s->counters + 1;
    p.status = s->counters + 2;
    p.tab_m = s->d_tab_m;
    p.traj = s->traj;
    p.n_points = s->n_points;
    p.peak_k = s->peak_k;
    p.peak_state = s->peak_state;
    p.mixed = (s->opt.flags & CB_BDF_MIXED_RHS) ? 1 : 0;
    p.reuse_lu = (s->opt.flags & CB_BDF_REUSE_LU) ? 1 : 0;
    p.lu32 = (s->global && (s->opt.flags & CB_BDF_LU32)) ? 1 : 0;
    p.jac_ws = s->global ? nullptr : s->jac_ws;
    if (s->global) {
        p.ws_global = s->ws;
        p.LUr = s->LUr;
        p.LUt = s->LUt;
        p.rdiag_r = s->rdiag_r;
        p.piv_r = s->piv_r;
    }
    return p;
}

// Global workspaces for at least `slots` warps in flight (outside any stream capture).
cudaError_t ensure_slots(cb_reactors* s, size_t slots) {
    if (!s->global || slots <= s->ws_slots) return cudaSuccess;
    if (s->ws) {
        cudaError_t e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return e;
        cudaFree(s->ws);
        s->ws = nullptr;
        s->ws_slots = 0;
    }
    cudaError_t e = cudaMalloc(&s->ws, slots * ws_bytes(s));
    if (e == cudaSuccess) s->ws_slots = slots;
    return e;
}

// Per-reactor factorisations and the evaluation hook's workspaces of the global-memory placement
// (s->global set; outside any stream capture).
cudaError_t ensure_global(cb_reactors* s) {
    cudaError_t e = cudaSuccess;
    if (!s->LUr) {  // all four or none: a partial allocation is released
        const size_t per = (size_t)s->N * s->LD, n = s->capacity;
        e = cudaMalloc(&s->LUr, n * per * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&s->LUt, n * per * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&s->rdiag_r, n * (size_t)s->N * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&s->piv_r, n * (size_t)s->N * sizeof(int));
        if (e != cudaSuccess) {
            cudaFree(s->LUr);
            cudaFree(s->LUt);
            cudaFree(s->rdiag_r);
            cudaFree(s->piv_r);
            s->LUr = s->LUt = s->rdiag_r = nullptr;
            s->piv_r = nullptr;
            return e;
        }
    }
    return ensure_slots(s, (size_t)sm_count());
}

// The slice kernel of the batch's variant: FP64 or mixed-precision first Newton iterations, workspaces
// in shared or global memory.
SliceFn slice_fn(const cb_reactors* s) {
    const bool mixed = (s->opt.flags & CB_BDF_MIXED_RHS) != 0;
    if (!s->global) return slice_kernel_fn(mixed);
    return s->regs == 128 ? slice_kernel_global_wide_fn(mixed)
                          : s->regs == 80 ? slice_kernel_global_mid_fn(mixed) : slice_kernel_global_fn(mixed);
}

// Shared-memory limit and grid of a launch shape (outside any stream capture).
cudaError_t prepare_slice(cb_reactors* s, int warps, int tables, int* grid) {
    const size_t smem = smem_bytes(s, warps, tables);
    const SliceFn fn = slice_fn(s);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 1;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * warps, smem);
    if (e != cudaSuccess) return e;
    *grid = sm_count() * (per_sm < 1 ? 1 : per_sm);
    if (!s->global && (size_t)*grid * warps > s->jac_slots) return cudaErrorInvalidConfiguration;
    return ensure_slots(s, (size_t)*grid * warps);
}

cudaError_t launch_slice(cb_reactors* s, int warps, int tables, int grid, cudaStream_t st) {
    slice_fn(s)<<<grid, 32 * warps, smem_bytes(s, warps, tables), st>>>(params(s, tables));
    return cudaGetLastError();
}

bool shape_fits(cb_reactors* s, int warps, int tables) { return (int)smem_bytes(s, warps, tables) <= max_smem(); }

// Scratch of cb_reactors_eval_noalloc, in the module's static device memory instead of cudaMalloc:
// states, pressures, du/dt and Jacobians of one call, at most kEvalScratchDoubles doubles (4 MiB; 173
// states at 53 species, N = 54). Its address is resolved once per device (cudaGetSymbolAddress) by the
// first call on that device and cached for the life of the process: a cudaDeviceReset (or anything else
// that destroys the device's primary context) invalidates it. Every element a call reads back is written
// by that call's kernel, so nothing in it has to start at zero; two calls in flight at once on one device
// share it and race.
constexpr size_t kEvalScratchDoubles = (size_t)1 << 19;
constexpr int kMaxDevices = 64;
static __device__ __align__(256) double g_eval_scratch[kEvalScratchDoubles];
std::mutex g_eval_scratch_mu;
double* g_eval_scratch_addr[kMaxDevices] = {};

}  // namespace

extern "C" {

int cb_reactors_create(cb_mech* mech, size_t n, const cb_bdf_options* opt, cb_reactors** out) {
    if (!mech || !opt || !out) return cbi::fail(CB_ERR_INVALID, "null argument");
    *out = nullptr;
    if (n == 0 || n > (1u << 30)) return cbi::fail(CB_ERR_INVALID, "reactor count out of range");
    if (!(opt->rtol > 0) || !(opt->atol > 0) || !(opt->t_end > 0) || opt->max_steps <= 0)
        return cbi::fail(CB_ERR_INVALID, "bad integrator options");
    const cbi::MechView v = cbi::view(mech);
    if (v.A != v.K - 1)
        return cbi::fail(CB_ERR_UNSUPPORTED, "reactors need every non-bulk species active (inert non-bulk species "
                                             "would be parameters, not state)");
    if (opt->flags & ~(CB_BDF_MIXED_RHS | CB_BDF_REUSE_LU | CB_BDF_GLOBAL_MEMORY | CB_BDF_LU32))
        return cbi::fail(CB_ERR_INVALID, "unknown integrator flag");
    cb_reactors* s = new cb_reactors();
    s->mech = mech;
    s->device = v.device;
    s->K = v.K;
    s->A = v.A;
    s->N = v.A + 2;
    s->LD = s->N | 1;
    s->n = n;
    s->capacity = n;
    s->opt = *opt;
    if (s->opt.slice_steps <= 0) s->opt.slice_steps = 256;
    s->warps = opt->warps_per_block;
    s->smem_tables = opt->tables_in_shared;
    // tables: the rates blob, then the per-species (reaction, coefficient) lists in reaction order
    const std::vector<uint8_t>& rb = *v.rates_blob;
    cbg::RatesHeader H;
    std::memcpy(&H, rb.data() + cbg::kMathBytes, sizeof H);
    s->R = H.R;
    s->n_eff = H.n_eff;
    std::vector<std::vector<int>> lists(s->A);
    for (int r = 0; r < H.R; r++) {
        cbg::Reaction x;
        std::memcpy(&x, rb.data() + H.off_reactions + (size_t)r * sizeof x, sizeof x);
        for (int q = 0; q < x.n_net; q++)
            if (x.net_k[q] < s->A) lists[x.net_k[q]].push_back((r << 8) | (x.net_n[q] & 0xff));
    }
    s->blob = rb;
    while (s->blob.size() % 16) s->blob.push_back(0);
    s->off_csr_start = (int)s->blob.size();
    std::vector<int> start(s->A + 1, 0), flat;
    for (int k = 0; k < s->A; k++) {
        start[k] = (int)flat.size();
        flat.insert(flat.end(), lists[k].begin(), lists[k].end());
    }
    start[s->A] = (int)flat.size();
    s->blob.resize(s->blob.size() + start.size() * 4);
    std::memcpy(s->blob.data() + s->off_csr_start, start.data(), start.size() * 4);
    while (s->blob.size() % 16) s->blob.push_back(0);
    s->off_csr = (int)s->blob.size();
    s->blob.resize(s->blob.size() + std::max<size_t>(flat.size(), 1) * 4);
    if (!flat.empty()) std::memcpy(s->blob.data() + s->off_csr, flat.data(), flat.size() * 4);
    while (s->blob.size() % 16) s->blob.push_back(0);
    // the third-body efficiencies transposed, [K][n_eff], so that the lanes of a warp (one row each)
    // read consecutive doubles
    s->off_eff_t = (int)s->blob.size();
    s->blob.resize(s->blob.size() + std::max<size_t>((size_t)s->K * s->n_eff, 1) * sizeof(double));
    for (int e = 0; e < s->n_eff; e++)
        for (int k = 0; k < s->K; k++)
            std::memcpy(s->blob.data() + s->off_eff_t + ((size_t)k * s->n_eff + e) * sizeof(double),
                        rb.data() + H.off_eff + ((size_t)e * s->K + k) * sizeof(double), sizeof(double));
    while (s->blob.size() % 16) s->blob.push_back(0);
    auto fail_free = [&](int rc) {
        cb_reactors_destroy(s);
        return rc;
    };
    cudaError_t e = cudaSetDevice(s->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_tab, s->blob.size());
    if (e == cudaSuccess) e = cudaMemcpy(s->d_tab, s->blob.data(), s->blob.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&s->pR, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->head, n * sizeof(Head));
    if (e == cudaSuccess) e = cudaMalloc(&s->D, n * kDRows * (size_t)s->N * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->J, n * (size_t)s->N * s->N * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->counters, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(s->counters, 0, 4 * sizeof(int));
    if (e == cudaSuccess && (s->opt.flags & CB_BDF_MIXED_RHS)) {
        const std::vector<uint8_t>& mb = *v.rates_mixed_blob;
        e = cudaMalloc(&s->d_tab_m, mb.size());
        if (e == cudaSuccess) e = cudaMemcpy(s->d_tab_m, mb.data(), mb.size(), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) return fail_free(cbi::cuda_fail(e, "reactor batch allocation"));
    // one warp's workspace beside the math tables in shared memory, or all of them in global memory (the
    // autotuner tries both placements when the first is possible)
    s->smem_ok = !(s->opt.flags & CB_BDF_GLOBAL_MEMORY) && shape_fits(s, 1, 0) && s->N <= cbg::bdf::kSmemMaxN;
    s->global = !s->smem_ok;
    if (s->global) {
        e = ensure_global(s);
        if (e != cudaSuccess) return fail_free(cbi::cuda_fail(e, "reactor workspaces in global memory"));
    } else {
        // as many warp slots as shared memory lets the SMs hold (every launch shape's grid fits)
        int dev = 0, smem_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        const size_t per_sm = std::max<size_t>(1, (size_t)smem_sm / ws_bytes(s));
        s->jac_slots = (size_t)sm_count() * per_sm;
        e = cudaMalloc(&s->jac_ws, s->jac_slots * 3 * (size_t)s->R * sizeof(double));
        if (e != cudaSuccess) return fail_free(cbi::cuda_fail(e, "reactor Jacobian scratch"));
    }
    *out = s;
    return CB_OK;
}

int cb_reactors_destroy(cb_reactors* s) {
    if (!s) return CB_OK;
    cudaSetDevice(s->device);
    if (s->stream) {
        cudaStreamSynchronize(s->stream);
        cudaStreamDestroy(s->stream);
    }
    cudaFree(s->d_tab);
    cudaFree(s->pR);
    cudaFree(s->head);
    cudaFree(s->D);
    cudaFree(s->J);
    cudaFree(s->counters);
    cudaFree(s->d_tab_m);
    cudaFree(s->ws);
    cudaFree(s->LUr);
    cudaFree(s->LUt);
    cudaFree(s->rdiag_r);
    cudaFree(s->piv_r);
    cudaFree(s->jac_ws);
    cudaFree(s->traj);
    cudaFree(s->peak_state);
    delete s;
    return CB_OK;
}

int cb_reactors_set_state(cb_reactors* s, const double* pressure_R, const double* T, const double* V,
                          const double* amounts) {
    if (!s || !pressure_R || !T || !V || !amounts) return cbi::fail(CB_ERR_INVALID, "null argument");
    const size_t n = s->n;
    const int N = s->N;
    std::vector<double> D(n * kDRows * (size_t)N, 0.0);
    for (size_t r = 0; r < n; r++) {
        if (!(T[r] > 0) || !(V[r] > 0) || !(pressure_R[r] > 0)) return cbi::fail(CB_ERR_INVALID, "non-positive T, V or P");
        double* y = D.data() + r * kDRows * N;
        y[0] = T[r];
        y[1] = V[r];
        for (int k = 0; k < s->A; k++) y[2 + k] = amounts[(size_t)k * n + r];
    }
    BDF_CUDA(cudaSetDevice(s->device));
    BDF_CUDA(cudaMemcpy(s->D, D.data(), D.size() * sizeof(double), cudaMemcpyHostToDevice));
    BDF_CUDA(cudaMemcpy(s->pR, pressure_R, n * sizeof(double), cudaMemcpyHostToDevice));
    BDF_CUDA(cudaMemset(s->head, 0, n * sizeof(Head)));
    BDF_CUDA(cudaMemset(s->counters, 0, 4 * sizeof(int)));
    // outputs not reached (a reactor that fails) read as NaN (all bits set)
    if (s->traj) BDF_CUDA(cudaMemset(s->traj, 0xff, n * (size_t)s->n_points * N * sizeof(double)));
    if (s->peak_state) BDF_CUDA(cudaMemset(s->peak_state, 0xff, n * (size_t)N * sizeof(double)));
    s->have_state = true;
    return CB_OK;
}

int cb_reactors_set_outputs(cb_reactors* s, int32_t n_points, int32_t peak_species) {
    if (!s) return cbi::fail(CB_ERR_INVALID, "null argument");
    if (n_points == 1 || n_points < 0) return cbi::fail(CB_ERR_INVALID, "n_points must be 0 (none) or at least 2");
    if (peak_species < -1 || peak_species >= s->A) return cbi::fail(CB_ERR_INVALID, "peak species out of range");
    BDF_CUDA(cudaSetDevice(s->device));
    BDF_CUDA(cudaStreamSynchronize(s->stream));
    cudaFree(s->traj);
    cudaFree(s->peak_state);
    s->traj = nullptr;
    s->peak_state = nullptr;
    s->n_points = 0;
    s->peak_k = -1;
    const size_t N = (size_t)s->N;
    if (n_points) {
        BDF_CUDA(cudaMalloc(&s->traj, s->n * (size_t)n_points * N * sizeof(double)));
        BDF_CUDA(cudaMemset(s->traj, 0xff, s->n * (size_t)n_points * N * sizeof(double)));
        s->n_points = n_points;
    }
    if (peak_species >= 0) {
        BDF_CUDA(cudaMalloc(&s->peak_state, s->n * N * sizeof(double)));
        BDF_CUDA(cudaMemset(s->peak_state, 0xff, s->n * N * sizeof(double)));
        s->peak_k = peak_species;
    }
    return CB_OK;
}

int cb_reactors_outputs(cb_reactors* s, double* times, double* trajectory, double* peak_time, double* peak_fraction,
                        double* peak_state) {
    if (!s) return cbi::fail(CB_ERR_INVALID, "null argument");
    if ((times || trajectory) && !s->traj) return cbi::fail(CB_ERR_NOT_READY, "no trajectory requested");
    if ((peak_time || peak_fraction || peak_state) && s->peak_k < 0)
        return cbi::fail(CB_ERR_NOT_READY, "no peak species requested");
    BDF_CUDA(cudaSetDevice(s->device));
    const size_t n = s->n, N = (size_t)s->N, P = (size_t)s->n_points;
    if (times)
        for (size_t j = 0; j < P; j++) times[j] = j == P - 1 ? s->opt.t_end : (double)j * (s->opt.t_end / (P - 1));
    if (trajectory) {  // device [n][P][N] -> host [P][N][n]
        std::vector<double> h(n * P * N);
        BDF_CUDA(cudaMemcpy(h.data(), s->traj, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (size_t r = 0; r < n; r++)
            for (size_t j = 0; j < P; j++)
                for (size_t i = 0; i < N; i++) trajectory[(j * N + i) * n + r] = h[(r * P + j) * N + i];
    }
    if (peak_time || peak_fraction) {
        std::vector<Head> h(n);
        BDF_CUDA(cudaMemcpy(h.data(), s->head, n * sizeof(Head), cudaMemcpyDeviceToHost));
        for (size_t r = 0; r < n; r++) {
            if (peak_time) peak_time[r] = h[r].peak_x >= 0.0 ? h[r].peak_t : NAN;
            if (peak_fraction) peak_fraction[r] = h[r].peak_x >= 0.0 ? h[r].peak_x : NAN;
        }
    }
    if (peak_state) {  // device [n][N] -> host [N][n]
        std::vector<double> h(n * N);
        BDF_CUDA(cudaMemcpy(h.data(), s->peak_state, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (size_t r = 0; r < n; r++)
            for (size_t i = 0; i < N; i++) peak_state[i * n + r] = h[r * N + i];
    }
    return CB_OK;
}

int cb_reactors_autotune(cb_reactors* s, int32_t calib_reactors, cb_reactor_tuning* out) {
    if (!s) return cbi::fail(CB_ERR_INVALID, "null argument");
    if (!s->have_state) return cbi::fail(CB_ERR_NOT_READY, "cb_reactors_set_state has not run");
    BDF_CUDA(cudaSetDevice(s->device));
    // candidates: workspaces in shared or global memory, reactors in flight per block, tables in shared
    // memory or read through L1
    struct Cand { int warps, tables, global, regs; };
    std::vector<Cand> cands;
    const bool placement = s->global;
    const int regs = s->regs;
    for (int g = s->smem_ok ? 0 : 1; g <= 1; g++) {
        s->global = g != 0;
        for (int tables = 1; tables >= 0; tables--)
            for (int w = 1; w <= 8; w++)
                if (shape_fits(s, w, tables) && (!g || (w & (w - 1)) == 0)) {
                    cands.push_back({w, tables, g, 64});
                    if (g && w >= 4) {  // 80 and 128 registers: full blocks only
                        cands.push_back({w, tables, g, 80});
                        cands.push_back({w, tables, g, 128});
                    }
                }
    }
    s->global = placement;
    if (cands.empty()) return cbi::fail(CB_ERR_UNSUPPORTED, "no launch shape fits");
    // calibrate on copies of the state: a few slices of the first reactors, then restore the state
    const size_t n_def = s->smem_ok ? 8192 : 512;
    const size_t n_cal = std::min<size_t>(s->n, calib_reactors > 0 ? (size_t)calib_reactors : n_def);
    const size_t hb = s->n * sizeof(Head), db = s->n * kDRows * (size_t)s->N * sizeof(double);
    std::vector<uint8_t> h0(hb), d0(db);
    BDF_CUDA(cudaMemcpy(h0.data(), s->head, hb, cudaMemcpyDeviceToHost));
    BDF_CUDA(cudaMemcpy(d0.data(), s->D, db, cudaMemcpyDeviceToHost));
    // the calibration runs the first n_cal reactors in 16-step slices and writes no outputs; the batch's
    // own settings come back on every path out of this function
    struct Restore {
        cb_reactors* s;
        size_t n;
        int steps, peak;
        double* traj;
        bool global;
        int regs;
        ~Restore() {
            s->n = n;
            s->opt.slice_steps = steps;
            s->traj = traj;
            s->peak_k = peak;
            s->global = global;
            s->regs = regs;
        }
    } restore{s, s->n, s->opt.slice_steps, s->peak_k, s->traj, placement, regs};
    s->traj = nullptr;
    s->peak_k = -1;
    s->n = n_cal;
    s->opt.slice_steps = 16;
    double best = 1e300;
    Cand pick = cands[0];
    cudaEvent_t a, b;
    BDF_CUDA(cudaEventCreate(&a));
    BDF_CUDA(cudaEventCreate(&b));
    int tried = 0;
    for (const Cand& c : cands) {
        cudaMemcpy(s->head, h0.data(), n_cal * sizeof(Head), cudaMemcpyHostToDevice);
        cudaMemcpy(s->D, d0.data(), n_cal * kDRows * (size_t)s->N * sizeof(double), cudaMemcpyHostToDevice);
        cudaMemset(s->counters, 0, 4 * sizeof(int));
        s->global = c.global != 0;
        s->regs = c.regs;
        if (s->global && ensure_global(s) != cudaSuccess) {
            cudaGetLastError();  // out of memory for the global placement: its candidates are skipped
            continue;
        }
        int grid = 0;
        if (prepare_slice(s, c.warps, c.tables, &grid) != cudaSuccess) continue;
        cudaEventRecord(a, s->stream);
        for (int rep = 0; rep < 2; rep++) {  // two slices: the first includes each reactor's start-up
            cudaMemsetAsync(s->counters, 0, sizeof(int), s->stream);
            if (launch_slice(s, c.warps, c.tables, grid, s->stream) != cudaSuccess) break;
        }
        cudaEventRecord(b, s->stream);
        if (cudaEventSynchronize(b) != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (out && tried < 32) {
            out->candidates[tried].warps_per_block = c.warps;
            out->candidates[tried].tables_in_shared = c.tables;
            out->candidates[tried].global_memory = c.global;
            out->candidates[tried].register_cap = c.global ? c.regs : 0;
            out->candidates[tried].ms = ms;
        }
        tried++;
        if (ms < best) {
            best = ms;
            pick = c;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    s->n = restore.n;
    s->opt.slice_steps = restore.steps;
    s->traj = restore.traj;
    s->peak_k = restore.peak;
    restore.global = pick.global != 0;
    restore.regs = pick.regs;
    s->global = restore.global;
    s->regs = restore.regs;
    BDF_CUDA(cudaMemcpy(s->head, h0.data(), hb, cudaMemcpyHostToDevice));
    BDF_CUDA(cudaMemcpy(s->D, d0.data(), db, cudaMemcpyHostToDevice));
    BDF_CUDA(cudaMemset(s->counters, 0, 4 * sizeof(int)));
    BDF_CUDA(cudaGetLastError());
    s->warps = pick.warps;
    s->smem_tables = pick.tables;
    if (out) {
        out->warps_per_block = pick.warps;
        out->tables_in_shared = pick.tables;
        out->global_memory = pick.global;
        out->register_cap = pick.global ? pick.regs : 0;
        out->n_candidates = std::min(tried, 32);
        out->calib_reactors = (int32_t)n_cal;
    }
    int st = 0;
    BDF_CUDA(cudaMemcpy(&st, s->counters + 2, sizeof st, cudaMemcpyDeviceToHost));
    if (st) return cbi::fail(CB_ERR_DEVICE, "table staging wait ran out during tuning");
    return CB_OK;
}

int cb_reactors_integrate(cb_reactors* s, cb_reactor_stats* stats) {
    if (!s) return cbi::fail(CB_ERR_INVALID, "null argument");
    if (!s->have_state) return cbi::fail(CB_ERR_NOT_READY, "cb_reactors_set_state has not run");
    BDF_CUDA(cudaSetDevice(s->device));
    if (s->warps <= 0 || s->smem_tables < 0) {
        int rc = cb_reactors_autotune(s, 0, nullptr);
        if (rc) return rc;
    }
    if (!shape_fits(s, s->warps, s->smem_tables)) return cbi::fail(CB_ERR_INVALID, "launch shape exceeds shared memory");
    cudaStream_t st = s->stream;
    int grid = 0;
    BDF_CUDA(prepare_slice(s, s->warps, s->smem_tables, &grid));
    // one graph: G slices, each a queue reset and a slice launch
    const int G = 4;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    BDF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int g = 0; g < G && e == cudaSuccess; g++) {
        e = cudaMemsetAsync(s->counters, 0, sizeof(int), st);
        if (e == cudaSuccess) e = launch_slice(s, s->warps, s->smem_tables, grid, st);
    }
    cudaError_t e2 = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cbi::cuda_fail(e != cudaSuccess ? e : e2, "reactor slice capture");
    }
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cbi::cuda_fail(e, "reactor slice graph");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, st);
    // every replay advances each unfinished reactor by up to G slices; bounded by the step limit
    const long long max_replays = (long long)s->opt.max_steps / ((long long)G * s->opt.slice_steps) + 4;
    int done = 0, replays = 0;
    for (long long rep = 0; rep < max_replays; rep++) {
        e = cudaGraphLaunch(exec, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&done, s->counters + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        replays++;
        if (e != cudaSuccess || done >= (int)s->n) break;
    }
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaGraphExecDestroy(exec);
    if (e != cudaSuccess) return cbi::cuda_fail(e, "reactor integration");
    int status = 0;
    BDF_CUDA(cudaMemcpy(&status, s->counters + 2, sizeof status, cudaMemcpyDeviceToHost));
    if (status) return cbi::fail(CB_ERR_DEVICE, "table staging wait ran out");
    if (stats) {
        std::memset(stats, 0, sizeof *stats);
        std::vector<Head> h(s->n);
        BDF_CUDA(cudaMemcpy(h.data(), s->head, s->n * sizeof(Head), cudaMemcpyDeviceToHost));
        for (const Head& x : h) {
            stats->steps += x.steps;
            stats->rhs_evals += x.rhs;
            stats->jacobians += x.jacs;
            stats->factorizations += x.lus;
            stats->newton_failures += x.newton_fail;
            stats->error_failures += x.err_fail;
            if (x.state == kDone) stats->finished++;
            else if (x.state != kRunning && x.state != kNew) stats->failed++;
        }
        stats->ms = ms;
        stats->warps_per_block = s->warps;
        stats->tables_in_shared = s->smem_tables;
        stats->global_memory = s->global ? 1 : 0;
        stats->register_cap = s->global ? s->regs : 0;
        stats->graph_replays = replays;
        stats->slices = replays * G;
    }
    return CB_OK;
}

int cb_reactors_results(cb_reactors* s, double* ignition_delay, double* state, int32_t* status, int32_t* steps) {
    if (!s) return cbi::fail(CB_ERR_INVALID, "null argument");
    BDF_CUDA(cudaSetDevice(s->device));
    const size_t n = s->n;
    const int N = s->N;
    std::vector<Head> h(n);
    BDF_CUDA(cudaMemcpy(h.data(), s->head, n * sizeof(Head), cudaMemcpyDeviceToHost));
    if (state) {
        std::vector<double> D(n * kDRows * (size_t)N);
        BDF_CUDA(cudaMemcpy(D.data(), s->D, D.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (size_t r = 0; r < n; r++)
            for (int i = 0; i < N; i++) state[(size_t)i * n + r] = D[r * kDRows * N + i];
    }
    for (size_t r = 0; r < n; r++) {
        const Head& x = h[r];
        if (ignition_delay) {
            // vertex of the parabola through the samples around the largest dT/dt
            double t = x.ign_t;
            if (std::isfinite(x.ta) && std::isfinite(x.tc) && x.tc > x.ign_t && x.ta < x.ign_t && !x.need_next) {
                const double d1 = x.ign_t - x.ta, d2 = x.ign_t - x.tc;
                const double num = d1 * d1 * (x.ign_g - x.gc) - d2 * d2 * (x.ign_g - x.ga);
                const double den = d1 * (x.ign_g - x.gc) - d2 * (x.ign_g - x.ga);
                if (den != 0.0) {
                    const double v = x.ign_t - 0.5 * num / den;
                    if (v > x.ta && v < x.tc) t = v;
                }
            }
            ignition_delay[r] = t;
        }
        if (status) status[r] = x.state;
        if (steps) steps[r] = x.steps;
    }
    return CB_OK;
}

int cb_reactors_eval(cb_reactors* s, int32_t m, const double* pressure_R, const double* states, double* f, double* J) {
    if (!s || !pressure_R || !states || !f || !J || m <= 0) return cbi::fail(CB_ERR_INVALID, "bad argument");
    BDF_CUDA(cudaSetDevice(s->device));
    const int N = s->N;
    double *dy = nullptr, *df = nullptr, *dJ = nullptr, *dp = nullptr;
    auto cleanup = [&](int rc) {
        cudaFree(dy);
        cudaFree(df);
        cudaFree(dJ);
        cudaFree(dp);
        return rc;
    };
    cudaError_t e = cudaMalloc(&dy, (size_t)m * N * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&df, (size_t)m * N * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dJ, (size_t)m * N * N * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dp, (size_t)m * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(dy, states, (size_t)m * N * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dp, pressure_R, (size_t)m * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cleanup(cbi::cuda_fail(e, "evaluation buffers"));
    // The staging-timeout status word is this call's own: a bit left by an earlier launch is cleared.
    if (e == cudaSuccess) e = cudaMemsetAsync(s->counters + 2, 0, sizeof(int), s->stream);
    if (e != cudaSuccess) return cleanup(cbi::cuda_fail(e, "evaluation status"));
    Params p = params(s, shape_fits(s, 1, 1) ? 1 : 0);
    p.pR = dp;
    p.eval_y = dy;
    p.eval_f = df;
    p.eval_J = dJ;
    const size_t smem = smem_bytes(s, 1, p.smem_tables);
    e = cudaFuncSetAttribute(eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) {
        eval_kernel<<<std::min(m, sm_count()), 32, smem, s->stream>>>(p, m);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(f, df, (size_t)m * N * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(J, dJ, (size_t)m * N * N * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cleanup(cbi::cuda_fail(e, "evaluation"));
    int st = 0;
    cudaMemcpy(&st, s->counters + 2, sizeof st, cudaMemcpyDeviceToHost);
    if (st) return cleanup(cbi::fail(CB_ERR_DEVICE, "table staging wait ran out"));
    return cleanup(CB_OK);
}

// No-allocation variant of cb_reactors_eval (same arguments and results): for callers that evaluate
// du/dt and Jacobians inside a time-critical loop (an implicit solver's Newton iterations on the host,
// a controller) and must not allocate per call: cudaMalloc and cudaFree cost tens of microseconds,
// cudaFree synchronises the whole device (stalling, e.g., a reactor integration running on another
// stream), and under a caching allocator that reserves the GPU's memory cudaMalloc can fail outright.
int cb_reactors_eval_noalloc(cb_reactors* s, int32_t m, const double* pressure_R, const double* states, double* f,
                             double* J) {
    if (!s || !pressure_R || !states || !f || !J || m <= 0) return cbi::fail(CB_ERR_INVALID, "bad argument");
    const int N = s->N;
    const size_t per_state = (size_t)N * N + 2 * (size_t)N + 1;
    const size_t max_states = kEvalScratchDoubles / per_state;
    if ((size_t)m > max_states)
        return cbi::fail(CB_ERR_INVALID, "cb_reactors_eval_noalloc: at most " + std::to_string(max_states) +
                                             " states per call for this mechanism (fixed 4 MiB device scratch)");
    if (s->device < 0 || s->device >= kMaxDevices) return cbi::fail(CB_ERR_UNSUPPORTED, "device index above 63");
    BDF_CUDA(cudaSetDevice(s->device));
    double* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_eval_scratch_mu);
        if (!g_eval_scratch_addr[s->device]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_eval_scratch);
            if (e != cudaSuccess) return cbi::cuda_fail(e, "cudaGetSymbolAddress(evaluation scratch)");
            g_eval_scratch_addr[s->device] = static_cast<double*>(p);
        }
        base = g_eval_scratch_addr[s->device];
    }
    double* dy = base;
    double* dp = dy + (size_t)m * N;
    double* df = dp + m;
    double* dJ = df + (size_t)m * N;
    cudaStream_t st = s->stream;
    BDF_CUDA(cudaMemcpyAsync(dy, states, (size_t)m * N * sizeof(double), cudaMemcpyHostToDevice, st));
    BDF_CUDA(cudaMemcpyAsync(dp, pressure_R, (size_t)m * sizeof(double), cudaMemcpyHostToDevice, st));
    BDF_CUDA(cudaMemsetAsync(s->counters + 2, 0, sizeof(int), st));  // this call's own staging status
    Params p = params(s, shape_fits(s, 1, 1) ? 1 : 0);
    p.pR = dp;
    p.eval_y = dy;
    p.eval_f = df;
    p.eval_J = dJ;
    const size_t smem = smem_bytes(s, 1, p.smem_tables);
    BDF_CUDA(cudaFuncSetAttribute(eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    eval_kernel<<<std::min(m, sm_count()), 32, smem, st>>>(p, m);
    BDF_CUDA(cudaGetLastError());
    BDF_CUDA(cudaMemcpyAsync(f, df, (size_t)m * N * sizeof(double), cudaMemcpyDeviceToHost, st));
    BDF_CUDA(cudaMemcpyAsync(J, dJ, (size_t)m * N * N * sizeof(double), cudaMemcpyDeviceToHost, st));
    BDF_CUDA(cudaStreamSynchronize(st));
    int status = 0;
    BDF_CUDA(cudaMemcpy(&status, s->counters + 2, sizeof status, cudaMemcpyDeviceToHost));
    if (status) return cbi::fail(CB_ERR_DEVICE, "table staging wait ran out");
    return CB_OK;
}

}  // extern "C"
