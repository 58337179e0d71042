// Device code of the batched reactors (bdf.cu): the integrator, its rates programs, factorisations and
// the slice kernels. Each slice-kernel variant is instantiated in its own translation unit
// (bdf_slice.cu, bdf_slice_global.cu) so that they compile in parallel; bdf.cu holds the host side and the
// evaluation hook.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/combustion_gb300.h"
#include "device_common.cuh"
#include "device_math.cuh"
#include "rates_core.cuh"
#include "rates_mixed_core.cuh"
#include "tables.h"
#include "tables_mixed.h"

namespace cbg {
namespace bdf {

constexpr int kMaxOrder = 5;
constexpr int kDRows = kMaxOrder + 3;
constexpr int kNewtonMaxIter = 4;
constexpr double kMinFactor = 0.2, kMaxFactor = 10.0;
constexpr int kPanel = 8;  // columns per panel of the blocked factorisation (global-memory matrices)
// 1 / n (n = 0..8, entry 0 unused), gamma_q = sum_{i=1..q} 1/i summed in increasing i, and 1 / gamma_q.
static __constant__ double kRcpInt[9] = {0.0, 1.0, 1.0 / 2, 1.0 / 3, 1.0 / 4, 1.0 / 5, 1.0 / 6, 1.0 / 7, 1.0 / 8};
static __constant__ double kGamma[7] = {0.0, 1.0, 1.0 + 1.0 / 2, 1.0 + 1.0 / 2 + 1.0 / 3, 1.0 + 1.0 / 2 + 1.0 / 3 + 1.0 / 4,
                                        1.0 + 1.0 / 2 + 1.0 / 3 + 1.0 / 4 + 1.0 / 5,
                                        1.0 + 1.0 / 2 + 1.0 / 3 + 1.0 / 4 + 1.0 / 5 + 1.0 / 6};
static __constant__ double kRcpGamma[7] = {0.0, 1.0 / 1.0, 1.0 / (1.0 + 1.0 / 2), 1.0 / (1.0 + 1.0 / 2 + 1.0 / 3),
                                           1.0 / (1.0 + 1.0 / 2 + 1.0 / 3 + 1.0 / 4),
                                           1.0 / (1.0 + 1.0 / 2 + 1.0 / 3 + 1.0 / 4 + 1.0 / 5),
                                           1.0 / (1.0 + 1.0 / 2 + 1.0 / 3 + 1.0 / 4 + 1.0 / 5 + 1.0 / 6)};
constexpr double kReuseSpread = 0.3;  // CB_BDF_REUSE_LU: largest |c / c_lu - 1| of a kept factorisation
constexpr int kReuseSteps = 20;       // CB_BDF_REUSE_LU: steps a factorisation is kept at most

enum State : int { kNew = 0, kRunning = 1, kDone = 2, kFailStep = 3, kFailSteps = 4, kFailLU = 5 };

struct Head {
    double t, h;
    double ign_t, ign_g, ta, ga, tc, gc, tp, gp;  // max dT/dt, its neighbours, the previous sample
    double c_lu;                                  // c of the factorisation kept between launches
    double peak_t, peak_x;                        // largest mole fraction of the peak species, its time
    int q, n_equal, state, jac_current;
    int steps, rhs, jacs, lus, newton_fail, err_fail, need_next, since_lu;
    int lu_have, lu_refresh;  // a kept factorisation exists; c changed since it was made
    int next_out, pad_out;    // next trajectory point to write
};

struct Params {
    const uint8_t* tab;
    uint32_t tab_bytes;
    int smem_tables;
    int off_csr_start, off_csr;  // per-species reaction lists inside the blob
    int off_eff_t;               // the third-body efficiencies transposed, [K][n_eff], inside the blob
    int K, A, R, N, LD, n_eff;
    uint32_t ws_bytes;           // per-warp workspace
    int n;
    double rtol, atol, t_end, h_min;
    int max_steps, slice_steps;
    const double* pR;  // P/R per reactor
    Head* head;
    double* D;  // [n][kDRows][N]
    double* J;  // [n][N][N]
    int* queue;
    int* done;
    int* status;
    // evaluation hook: states [m][N] -> f [m][N], J [m][N][N]
    const double* eval_y;
    double* eval_f;
    double* eval_J;
    const uint8_t* tab_m;  // mixed-precision rates tables (global memory): f(u) with CB_BDF_MIXED_RHS
    int mixed, reuse_lu, lu32;
    // Large states: per-warp workspaces in global memory (null: in shared memory), and per reactor its
    // factorisation [n][N][LD], the factors' transpose (coalesced triangular solves), pivots, 1 / U_kk.
    uint8_t* ws_global;
    double* LUr;
    double* LUt;
    double* rdiag_r;
    int* piv_r;
    // Outputs (cb_reactors_set_outputs): states at n_points uniform times [n][n_points][N] (null: none),
    // and the state where species peak_k's mole fraction among the active species peaks [n][N] (k < 0:
    // none).
    double* traj;
    int n_points, peak_k;
    double* peak_state;
    // Shared-memory workspaces: kf, pK, sM of the Jacobian per warp slot, [slots][3 R] (null: in the
    // workspace).
    double* jac_ws;
};


__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return __shfl_sync(0xffffffffu, v, 0);
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return __shfl_sync(0xffffffffu, v, 0);
}

// After an accepted step to t_new of size h at order q (backward differences D at t_new): the
// trajectory points in (t_new - h, t_new] from the interpolating polynomial through the last q + 1
// points (Newton's backward-difference form, y(t) = sum_j D_j prod_{m<j} (t - t_new + m h) / ((m+1) h),
// the dense output of the BDF method), and the peak of the chosen species' mole fraction.
static __device__ __noinline__ void record_outputs(const Params& p, Head& hd, int r, const double* D, double t_new, double h, int q,
                               int lane) {
    const int N = p.N;
    if (p.traj) {
        const double dt = p.t_end / (p.n_points - 1);
        while (hd.next_out < p.n_points) {
            const double tj = hd.next_out == p.n_points - 1 ? p.t_end : hd.next_out * dt;
            if (tj > t_new) break;
            double* out = p.traj + ((size_t)r * p.n_points + hd.next_out) * N;
            for (int i = lane; i < N; i += 32) {
                double y = D[i], pj = 1.0;
                for (int j = 1; j <= q; j++) {
                    pj *= (tj - t_new + (j - 1) * h) / (j * h);
                    y = fma(D[(size_t)j * N + i], pj, y);
                }
                out[i] = y;
            }
            hd.next_out++;
        }
    }
    if (p.peak_k >= 0) {  // mole fraction among the active species (the reference's plotted fractions)
        double s = 0.0;
        for (int i = 2 + lane; i < N; i += 32) s += D[i];
        s = warp_sum(s);
        const double x = D[2 + p.peak_k] / s;
        if (x > hd.peak_x) {
            hd.peak_x = x;
            hd.peak_t = t_new;
            for (int i = lane; i < N; i += 32) p.peak_state[(size_t)r * N + i] = D[i];
        }
    }
    __syncwarp();
}

// Concentrations, Gibbs exponentials and third-body sums in shared memory, viewed as a rates "cell".
struct WarpCell {
    Temps t;
    double C0, rcpC0, rcpC0sq;
    const double* C;
    const double* ex;
    const double* exn;
    const double* M;
};

struct Work {
    double *LU, *D, *ypred, *psi, *rscale, *y, *d, *f, *b, *tmp, *C, *ex, *exn, *M, *hk, *cpk, *cR, *kf, *pK, *sM, *rdiag;
    int* piv;
};

// Doubles of one warp's workspace; jac_parts: with the Jacobian's kf, pK, sM (global-memory workspaces).
__host__ __device__ inline size_t workspace_doubles(int K, int A, int R, int N, int LD, int n_eff, bool jac_parts) {
    return (size_t)N * LD + (size_t)kDRows * N + 8 * (size_t)N + K + 2 * (size_t)A + n_eff + A + K +
           (jac_parts ? 4 : 1) * (size_t)R + N;
}

// The workspace of warp slot `slot` at `base`.
__device__ inline Work carve(const Params& p, uint8_t* base, size_t slot) {
    Work w;
    double* q = reinterpret_cast<double*>(base);
    auto take = [&](size_t n) {
        double* r = q;
        q += n;
        return r;
    };
    const int N = p.N;
    w.LU = take((size_t)N * p.LD);
    w.D = take((size_t)kDRows * N);
    w.ypred = take(N);
    w.psi = take(N);
    w.rscale = take(N);
    w.y = take(N);
    w.d = take(N);
    w.f = take(N);
    w.b = take(N);
    w.tmp = take(N);
    w.C = take(p.K);
    w.ex = take(p.A);
    w.exn = take(p.A);
    w.M = take(p.n_eff);
    w.hk = take(p.A);
    w.cpk = take(p.K);
    w.cR = take(p.R);
    if (p.jac_ws) {
        double* j = p.jac_ws + slot * 3 * (size_t)p.R;
        w.kf = j;
        w.pK = j + p.R;
        w.sM = j + 2 * (size_t)p.R;
    } else {
        w.kf = take(p.R);
        w.pK = take(p.R);
        w.sM = take(p.R);
    }
    w.rdiag = take(N);
    w.piv = reinterpret_cast<int*>(q);
    return w;
}

struct Mech {
    RatesTables tb;
    const int* csr_start;
    const int* csr;
    const double* eff_t;  // [K][n_eff]
    __device__ Mech(const uint8_t* tab, const Params& p)
        : tb(tab), csr_start(reinterpret_cast<const int*>(tab + p.off_csr_start)),
          csr(reinterpret_cast<const int*>(tab + p.off_csr)),
          eff_t(reinterpret_cast<const double*>(tab + p.off_eff_t)) {}
};

struct RhsOut {
    double T, V, md, Ctot, S, E, Cp, dtE;
};

// Third-body sum e, sum_k E_ek C_k, from the transposed table Et [K][ld] (lanes on consecutive rows e
// read consecutive doubles), in four interleaved partial sums added pairwise at the end.
__device__ __forceinline__ double eff_dot(const double* Et, int ld, int e, const double* C, int K) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int k = 0;
    for (; k + 3 < K; k += 4) {
        s0 = fma(Et[(size_t)k * ld + e], C[k], s0);
        s1 = fma(Et[(size_t)(k + 1) * ld + e], C[k + 1], s1);
        s2 = fma(Et[(size_t)(k + 2) * ld + e], C[k + 2], s2);
        s3 = fma(Et[(size_t)(k + 3) * ld + e], C[k + 3], s3);
    }
    for (; k < K; k++) s0 = fma(Et[(size_t)k * ld + e], C[k], s0);
    return (s0 + s1) + (s2 + s3);
}

// The same in FP32 over the FP64 concentrations (the mixed program's third-body sums).
__device__ __forceinline__ float eff_dot_f32(const float* E, const double* C, int K) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int k = 0;
    for (; k + 3 < K; k += 4) {
        s0 = fmaf(E[k], dbl_to_flt(C[k]), s0);
        s1 = fmaf(E[k + 1], dbl_to_flt(C[k + 1]), s1);
        s2 = fmaf(E[k + 2], dbl_to_flt(C[k + 2]), s2);
        s3 = fmaf(E[k + 3], dbl_to_flt(C[k + 3]), s3);
    }
    for (; k < K; k++) s0 = fmaf(E[k], dbl_to_flt(C[k]), s0);
    return (s0 + s1) + (s2 + s3);
}

// Net production rate of species k, sum over its reactions of nu cR (reaction.rs:312-327), in two
// interleaved partial sums.
__device__ __forceinline__ double species_rate(const Mech& m, const double* cR, int k) {
    double w0 = 0.0, w1 = 0.0;
    int q = m.csr_start[k];
    const int qe = m.csr_start[k + 1];
    for (; q + 1 < qe; q += 2) {
        const int e0 = m.csr[q], e1 = m.csr[q + 1];
        w0 = fma(small_int_to_double((int)(int8_t)(e0 & 0xff)), cR[e0 >> 8], w0);
        w1 = fma(small_int_to_double((int)(int8_t)(e1 & 0xff)), cR[e1 >> 8], w1);
    }
    if (q < qe) {
        const int e = m.csr[q];
        w0 = fma(small_int_to_double((int)(int8_t)(e & 0xff)), cR[e >> 8], w0);
    }
    return w0 + w1;
}

// Rates of progress of the reactions of one model (the tables group reactions by model), lanes strided
// over the group, so that a warp never runs two models' programs under partial masks.
template <int MODEL, bool PARTS>
__device__ __forceinline__ void rates_group_warp(const Mech& m, const Work& w, const WarpCell& c, int lane) {
    const RatesHeader& H = *m.tb.H;
    const int end = H.group_end[MODEL];
    for (int r = (MODEL ? H.group_end[MODEL - 1] : 0) + lane; r < end; r += 32) {
        const Reaction& x = m.tb.reactions[r];
        ReactionParts pp;
        w.cR[r] = reaction_eval<MODEL, PARTS>(m.tb, x, c, MODEL >= 2 ? c.M[x.eff_row] : 0.0, &pp);
        if (PARTS) {
            w.kf[r] = pp.kf;
            w.pK[r] = pp.pK;
            w.sM[r] = pp.dkf_dM * pp.Rnet;
        }
    }
}

// du/dt of the reactor: the outputs of reaction.rs:356-391 at state y = [T, V, n_0 .. n_{A-1}].
template <bool PARTS>
__device__ __noinline__ RhsOut rhs_warp(const Params& p, const Mech& m, const Work& w, double pR, double rP, const double* y,
                           double* f, int lane) {
    const RatesHeader& H = *m.tb.H;
    const int K = p.K, A = p.A;
    RhsOut o;
    const double T = y[0], V = y[1];
    WarpCell c;
    c.t.T = T;
    c.t.rcpT = rcp64(T);
    c.t.lnT = log64(T);
    c.t.T2 = T * T;
    c.t.T3 = T * c.t.T2;
    c.t.T4 = c.t.T2 * c.t.T2;
    c.t.rcpT2 = c.t.rcpT * c.t.rcpT;
    const double md = rcp64(V);
    double s = 0.0;
    for (int k = lane; k < K - 1; k += 32) {
        const double ck = md * max0(y[2 + k]);
        w.C[k] = ck;
        s += ck;
    }
    s = warp_sum(s);
    const double Ctot = pR * c.t.rcpT;
    if (lane == 0) w.C[K - 1] = Ctot - s;
    c.C0 = H.C0 * c.t.rcpT;
    c.rcpC0 = H.rcp_C0 * T;
    c.rcpC0sq = c.rcpC0 * c.rcpC0;
    for (int k = lane; k < K; k += 32) {
        const Species& sp = m.tb.species[k];
        const int pc = piece_of(sp.split, T);
        const double* cp = sp.cp[pc];
        w.cpk[k] = fma(cp[4], c.t.T4, fma(cp[3], c.t.T3, fma(cp[2], c.t.T2, fma(cp[1], T, cp[0]))));
        if (k < A) {
            const double* h = sp.h[pc];
            w.hk[k] = fma(h[5], c.t.rcpT, fma(h[4], c.t.T4, fma(h[3], c.t.T3, fma(h[2], c.t.T2, fma(h[1], T, h[0])))));
            if (sp.need_exp | sp.need_exp_neg) {
                const double* g = sp.g[pc];
                const double x = fma(g[6], c.t.rcpT, fma(g[5], c.t.T4, fma(g[4], c.t.T3, fma(g[3], c.t.T2,
                                 fma(g[2], T, fma(g[1], c.t.lnT, g[0]))))));
                if (sp.need_exp) w.ex[k] = min_pos(H.M3, exp64(x));
                if (sp.need_exp_neg) w.exn[k] = min_pos(H.cbrt_max, exp64(-x));
            }
        }
    }
    __syncwarp();
    for (int e = lane; e < H.n_eff; e += 32) w.M[e] = Ctot + eff_dot(m.eff_t, H.n_eff, e, w.C, K);
    __syncwarp();
    c.C = w.C;
    c.ex = w.ex;
    c.exn = w.exn;
    c.M = w.M;
    rates_group_warp<0, PARTS>(m, w, c, lane);
    rates_group_warp<1, PARTS>(m, w, c, lane);
    rates_group_warp<2, PARTS>(m, w, c, lane);
    rates_group_warp<3, PARTS>(m, w, c, lane);
    rates_group_warp<4, PARTS>(m, w, c, lane);
    rates_group_warp<5, PARTS>(m, w, c, lane);
    __syncwarp();
    double E = 0.0, dtE = 0.0, Cp = 0.0;
    for (int k = lane; k < A; k += 32) {
        const double wk = species_rate(m, w.cR, k);
        f[2 + k] = wk;
        E = fma(wk, w.hk[k], E);
        dtE = fma(m.tb.species[k].dtE, wk, dtE);
    }
    for (int k = lane; k < K; k += 32) Cp = fma(w.cpk[k], w.C[k], Cp);
    E = warp_sum(E);
    dtE = warp_sum(dtE);
    Cp = warp_sum(Cp);
    const double dtT_T = div64(-E, Cp);
    if (lane == 0) {
        f[0] = T * dtT_T;
        f[1] = V * fma(rP * T, dtE, dtT_T);
    }
    __syncwarp();
    o.T = T;
    o.V = V;
    o.md = md;
    o.Ctot = Ctot;
    o.S = s;
    o.E = E;
    o.Cp = Cp;
    o.dtE = dtE;
    return o;
}

// The warp's cell for the mixed-precision rates program (reaction_rate_m).
struct WarpCellM {
    const double* C;
    const double* ex;
    const double* exn;
    const float* Mf;
    double C0, rcpC0, rcpC0sq;
    float Ctotf, Tf, lnTf, rcpTf;
};

// rates_group_warp for the mixed-precision program.
template <int MODEL>
__device__ __forceinline__ void rates_group_warp_m(const RatesMixedTables& tm, const Work& w, const WarpCellM& c, int lane) {
    const int end = tm.H->group_end[MODEL];
    for (int r = (MODEL ? tm.H->group_end[MODEL - 1] : 0) + lane; r < end; r += 32) {
        const ReactionF& x = tm.reactions[r];
        w.cR[r] = reaction_rate_m<MODEL>(tm, x, c, MODEL >= 2 ? c.Mf[x.eff_row] : 0.f);
    }
}

// du/dt by the mixed-precision rates program (the arithmetic of kernels_mixed.cu's rates_mixed_cell,
// warp-cooperative as rhs_warp): FP64 concentrations, Gibbs polynomials and exponentials, rates of
// progress, accumulation and energy sums; FP32 Arrhenius terms, third-body sums, falloff blending and
// h/RT, cp/R polynomials. w.M holds the FP32 third-body sums.
static __device__ __noinline__ void rhs_warp_mixed(const Params& p, const Mech& m, const RatesMixedTables& tm, const Work& w, double pR,
                               double rP, const double* y, double* f, int lane) {
    const RatesMixedHeader& H = *tm.H;
    const int K = p.K, A = p.A;
    const double T = y[0], V = y[1];
    const double rcpT = rcp64(T), lnT = log64(T);
    const double T2 = T * T, T3 = T * T2, T4 = T2 * T2;
    const double md = rcp64(V);
    double s = 0.0;
    for (int k = lane; k < K - 1; k += 32) {
        const double ck = md * max0(y[2 + k]);
        w.C[k] = ck;
        s += ck;
    }
    s = warp_sum(s);
    const double Ctot = pR * rcpT;
    if (lane == 0) w.C[K - 1] = Ctot - s;
    WarpCellM c;
    c.C0 = H.C0 * rcpT;
    c.rcpC0 = H.rcp_C0 * T;
    c.rcpC0sq = c.rcpC0 * c.rcpC0;
    c.Ctotf = dbl_to_flt(Ctot);
    c.Tf = dbl_to_flt(T);
    c.lnTf = dbl_to_flt(lnT);
    c.rcpTf = dbl_to_flt(rcpT);
    const float Tf = c.Tf, rcpTf = c.rcpTf;
    for (int k = lane; k < K; k += 32) {
        const SpeciesF& sp = tm.species[k];
        const int pc = piece_of_m(sp.split, T);
        const float* cp = sp.cp[pc];
        const float ck = fmaf(cp[4], Tf, cp[3]);
        w.cpk[k] = flt_to_dbl(fmaf(fmaf(fmaf(ck, Tf, cp[2]), Tf, cp[1]), Tf, cp[0]));
        if (k < A) {
            const float* h = sp.h[pc];
            w.hk[k] = flt_to_dbl(fmaf(h[5], rcpTf, fmaf(fmaf(fmaf(fmaf(h[4], Tf, h[3]), Tf, h[2]), Tf, h[1]), Tf, h[0])));
            if (sp.need_exp | sp.need_exp_neg) {
                const double* g = sp.g[pc];
                const double x = fma(g[6], rcpT, fma(g[5], T4, fma(g[4], T3, fma(g[3], T2, fma(g[2], T, fma(g[1], lnT, g[0]))))));
                gibbs_exps(x, sp.need_exp, sp.need_exp_neg, H.M3, H.cbrt_max, c.C0, c.rcpC0, w.ex[k], w.exn[k]);
            }
        }
    }
    __syncwarp();
    float* Mf = reinterpret_cast<float*>(w.M);
    for (int e = lane; e < H.n_eff; e += 32) Mf[e] = c.Ctotf + eff_dot_f32(tm.eff + (size_t)e * K, w.C, K);
    __syncwarp();
    c.C = w.C;
    c.ex = w.ex;
    c.exn = w.exn;
    c.Mf = Mf;
    rates_group_warp_m<0>(tm, w, c, lane);
    rates_group_warp_m<1>(tm, w, c, lane);
    rates_group_warp_m<2>(tm, w, c, lane);
    rates_group_warp_m<3>(tm, w, c, lane);
    rates_group_warp_m<4>(tm, w, c, lane);
    rates_group_warp_m<5>(tm, w, c, lane);
    __syncwarp();
    double E = 0.0, dtE = 0.0, Cp = 0.0;
    for (int k = lane; k < A; k += 32) {
        const double wk = species_rate(m, w.cR, k);
        f[2 + k] = wk;
        E = fma(wk, w.hk[k], E);
        dtE = fma(tm.species[k].dtE, wk, dtE);
    }
    for (int k = lane; k < K; k += 32) Cp = fma(w.cpk[k], w.C[k], Cp);
    E = warp_sum(E);
    dtE = warp_sum(dtE);
    Cp = warp_sum(Cp);
    const double dtT_T = -E * rcp64(Cp);
    if (lane == 0) {
        f[0] = T * dtT_T;
        f[1] = V * fma(rP * T, dtE, dtT_T);
    }
    __syncwarp();
}

// d/dC_{ks[i]} of prod_q C_{ks[q]}^{ns[q]}: one factor of species ks[i] removed, times its multiplicity.
__device__ __forceinline__ double deriv_product(const double* C, const uint16_t* ks, const int8_t* ns, int n, int i) {
    double p = small_int_to_double(ns[i]);
    for (int q = 0; q < n; q++) {
        const int mq = q == i ? ns[q] - 1 : ns[q];
        for (int t = 0; t < mq; t++) p *= C[ks[q]];
    }
    return p;
}

// Jacobian of du/dt at y into Jm (N rows of LD), also stored to Jg [N][N]; w.f receives f(y).
static __device__ __noinline__ void jacobian_warp(const Params& p, const Mech& m, const Work& w, double pR, double rP, const double* y,
                              double* Jg, double* Jm, int lane) {
    const int K = p.K, A = p.A, N = p.N, LD = p.LD;
    const RhsOut o = rhs_warp<true>(p, m, w, pR, rP, y, w.f, lane);
    // species rows: G[k][j] = d wdot_k / d C_j (bulk column kept in column 0 for now)
    for (int k = lane; k < A; k += 32) {
        double* row = Jm + (size_t)(2 + k) * LD;
        for (int j = 0; j < N; j++) row[j] = 0.0;
        for (int q = m.csr_start[k]; q < m.csr_start[k + 1]; q++) {
            const int e = m.csr[q];
            const int r = e >> 8;
            const double nu = small_int_to_double((int)(int8_t)(e & 0xff));
            const Reaction& x = m.tb.reactions[r];
            const double a = nu * w.kf[r];
            for (int i = 0; i < x.n_r; i++) {
                const int j = x.r_k[i];
                row[j == K - 1 ? 0 : 2 + j] += a * deriv_product(w.C, x.r_k, x.r_n, x.n_r, i);
            }
            if (x.model != 1) {
                const double b = -a * w.pK[r];
                for (int i = 0; i < x.n_p; i++) {
                    const int j = x.p_k[i];
                    row[j == K - 1 ? 0 : 2 + j] += b * deriv_product(w.C, x.p_k, x.p_n, x.n_p, i);
                }
            }
            if (x.eff_row >= 0) {  // M = C_total + sum (e_j - 1) C_j
                const double sm = nu * w.sM[r];
                const double* E = m.tb.eff + (size_t)x.eff_row * K;
                for (int j = 0; j < K - 1; j++) row[2 + j] = fma(sm, E[j], row[2 + j]);
                row[0] = fma(sm, E[K - 1], row[0]);
            }
        }
        // to the state variables: C_j = n_j / V (j < K-1), C_bulk = C_total - sum_j C_j
        const double gb = row[0];
        double sv = 0.0;
        for (int i = 0; i < K - 1; i++) {
            const double gi = row[2 + i];
            sv = fma(gi, w.C[i], sv);
            row[2 + i] = (gi - gb) * o.md;
        }
        row[1] = -o.md * fma(-gb, o.S, sv);
        row[0] = 0.0;
    }
    // d(C_p)/dV needs sum_{i<K-1} cp_i C_i
    double scp = 0.0;
    for (int i = lane; i < K - 1; i += 32) scp = fma(w.cpk[i], w.C[i], scp);
    scp = warp_sum(scp);
    __syncwarp();
    // T and V rows through dT/dt = -T E / Cp and dV/dt = V (dT/dt / T + R/P T dtE)
    const double rcpT = rcp64(o.T), rCp = rcp64(o.Cp);
    const double a0 = -o.T * rCp, b0 = (o.T * o.E) * (rCp * rCp);
    const double cpb = w.cpk[K - 1];
    for (int j = 1 + lane; j < N; j += 32) {
        double sh = 0.0, se = 0.0;
        for (int k = 0; k < A; k++) {
            const double jk = Jm[(size_t)(2 + k) * LD + j];
            sh = fma(w.hk[k], jk, sh);
            se = fma(m.tb.species[k].dtE, jk, se);
        }
        const double dCp = j == 1 ? -o.md * fma(-cpb, o.S, scp) : (w.cpk[j - 2] - cpb) * o.md;
        const double j0 = fma(a0, sh, b0 * dCp);
        double j1 = o.V * fma(rP * o.T, se, j0 * rcpT);
        if (j == 1) j1 += w.f[1] * o.md;
        Jm[j] = j0;
        Jm[(size_t)LD + j] = j1;
    }
    __syncwarp();
    // temperature column: forward difference
    const double dT = 1.4901161193847656e-8 * fmax(fabs(o.T), 1.0);
    for (int i = lane; i < N; i += 32) w.b[i] = y[i];
    __syncwarp();
    if (lane == 0) w.b[0] = y[0] + dT;
    __syncwarp();
    const double dTa = w.b[0] - y[0];  // the increment actually represented
    rhs_warp<false>(p, m, w, pR, rP, w.b, w.tmp, lane);
    const double rdT = 1.0 / dTa;
    for (int i = lane; i < N; i += 32) Jm[(size_t)i * LD] = (w.tmp[i] - w.f[i]) * rdT;
    __syncwarp();
    if (Jg)
        for (int idx = lane; idx < N * N; idx += 32) Jg[idx] = Jm[(size_t)(idx / N) * LD + idx % N];
    __syncwarp();
}

// In-place LU with partial pivoting (largest |A_ik|, lowest row on ties; whole rows swapped) of the
// N x N matrix in A (rows of LD), for matrices in shared memory; false on a zero or non-finite pivot.
// perm receives the row order: row i of the factors is row perm[i] of the input. The pivot is found on
// the bits of |A_ik| (non-negative doubles order as integers) by three warp reductions; the trailing
// update loads four rows before storing them, which keeps four FMAs in flight per lane.
__device__ inline bool lu_warp(double* A, int N, int LD, int* perm, double* rdiag, int lane) {
    for (int i = lane; i < N; i += 32) perm[i] = i;
    __syncwarp();
    for (int k = 0; k < N; k++) {
        unsigned long long best = 0ull;
        int bi = k;
        for (int i = k + lane; i < N; i += 32) {
            const unsigned long long v = (unsigned long long)__double_as_longlong(A[(size_t)i * LD + k]) & ~(1ull << 63);
            if (v > best) {
                best = v;
                bi = i;
            }
        }
        const unsigned hi = (unsigned)(best >> 32), lo = (unsigned)best;
        const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
        const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
        bi = (int)__reduce_min_sync(0xffffffffu, (hi == mhi && lo == mlo) ? (unsigned)bi : 0xffffffffu);
        const double bestd = __longlong_as_double((long long)(((unsigned long long)mhi << 32) | mlo));
        if (!(bestd > 0.0) || !(bestd < 1e300)) return false;
        if (bi != k) {
            for (int j = lane; j < N; j += 32) {
                const double t = A[(size_t)k * LD + j];
                A[(size_t)k * LD + j] = A[(size_t)bi * LD + j];
                A[(size_t)bi * LD + j] = t;
            }
            if (lane == 0) {
                const int t = perm[k];
                perm[k] = perm[bi];
                perm[bi] = t;
            }
        }
        __syncwarp();
        const double rp = 1.0 / A[(size_t)k * LD + k];
        if (lane == 0) rdiag[k] = rp;
        for (int i = k + 1 + lane; i < N; i += 32) A[(size_t)i * LD + k] *= rp;
        __syncwarp();
        for (int j = k + 1 + lane; j < N; j += 32) {
            const double akj = A[(size_t)k * LD + j];
            int i = k + 1;
            for (; i + 3 < N; i += 4) {
                double* r = A + (size_t)i * LD;
                const double l0 = r[k], l1 = r[LD + k], l2 = r[2 * LD + k], l3 = r[3 * LD + k];
                const double a0 = r[j], a1 = r[LD + j], a2 = r[2 * LD + j], a3 = r[3 * LD + j];
                r[j] = fma(-l0, akj, a0);
                r[LD + j] = fma(-l1, akj, a1);
                r[2 * LD + j] = fma(-l2, akj, a2);
                r[3 * LD + j] = fma(-l3, akj, a3);
            }
            for (; i < N; i++) A[(size_t)i * LD + j] = fma(-A[(size_t)i * LD + k], akj, A[(size_t)i * LD + j]);
        }
        __syncwarp();
    }
    return true;
}

// Rows of a lu_solve_warp right-hand side held per lane (row lane + 32 s in slot s) for N <= 32 S.
template <int S>
__device__ __forceinline__ double slot_value(const double (&x)[S], int k) {
    double v = x[0];
#pragma unroll
    for (int s = 1; s < S; s++)
        if (k >= 32 * s) v = x[s];
    return v;
}

// b <- U^-1 L^-1 (b permuted by perm) with the right-hand side in registers: the eliminated row's value
// reaches the other lanes by a shuffle, so a step waits for one FMA and one shuffle instead of a
// shared-memory round trip and a warp barrier. Same operations, in the same order, as the textbook
// column-oriented substitution (row k's value times column k subtracted from the rows below, then
// above, it).
template <int S>
__device__ inline void lu_solve_regs(const double* A, int N, int LD, const int* perm, const double* rdiag, double* b,
                                     int lane) {
    double x[S];
#pragma unroll
    for (int s = 0; s < S; s++) {
        const int i = lane + 32 * s;
        x[s] = i < N ? b[perm[i]] : 0.0;
    }
    __syncwarp();
    for (int k = 0; k < N - 1; k++) {
        const double xk = __shfl_sync(0xffffffffu, slot_value<S>(x, k), k & 31);
#pragma unroll
        for (int s = 0; s < S; s++) {
            if (32 * s + 31 <= k) continue;  // warp-uniform: the slot's rows are all at or above row k
            const int i = lane + 32 * s;
            if (i > k && i < N) x[s] = fma(-A[(size_t)i * LD + k], xk, x[s]);
        }
    }
    for (int k = N - 1; k >= 0; k--) {
        const double xk = __shfl_sync(0xffffffffu, slot_value<S>(x, k), k & 31) * rdiag[k];
#pragma unroll
        for (int s = 0; s < S; s++) {
            if (32 * s > k) continue;  // warp-uniform: the slot's rows are all below row k
            const int i = lane + 32 * s;
            if (i == k) x[s] = xk;
            else if (i < k) x[s] = fma(-A[(size_t)i * LD + k], xk, x[s]);
        }
    }
#pragma unroll
    for (int s = 0; s < S; s++) {
        const int i = lane + 32 * s;
        if (i < N) b[i] = x[s];
    }
    __syncwarp();
}

constexpr int kSmemMaxN = 160;  // largest state of the shared-memory path (lu_solve_warp's register slots)

__device__ inline void lu_solve_warp(const double* A, int N, int LD, const int* perm, const double* rdiag, double* b,
                                     int lane) {
    if (N <= 64) lu_solve_regs<2>(A, N, LD, perm, rdiag, b, lane);
    else if (N <= 96) lu_solve_regs<3>(A, N, LD, perm, rdiag, b, lane);
    else lu_solve_regs<5>(A, N, LD, perm, rdiag, b, lane);
}

// lu_warp by panels of kPanel columns, for matrices in global memory: inside a panel the pivot search,
// row swap (whole rows), scaling and update of the panel's own columns go column by column; then the
// panel's U rows right of it by forward substitution, and one rank-kPanel update of the trailing matrix,
// which so is read and written once per panel instead of once per column. Every element receives the
// same FMAs in the same order as in lu_warp, and perm the same row order. T = float: the FP32
// factorisation of CB_BDF_LU32 (1 / U_kk still stored as a double).
template <class T>
__device__ inline bool lu_warp_blocked(T* A, int N, int LD, int* perm, double* rdiag, int lane) {
    for (int i = lane; i < N; i += 32) perm[i] = i;
    __syncwarp();
    for (int kb = 0; kb < N; kb += kPanel) {
        const int ke = min(kb + kPanel, N);
        for (int k = kb; k < ke; k++) {
            T best = -1;
            int bi = k;
            for (int i = k + lane; i < N; i += 32) {
                const T v = fabs(A[(size_t)i * LD + k]);
                if (v > best) {
                    best = v;
                    bi = i;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const T ov = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov > best || (ov == best && oi < bi)) {
                    best = ov;
                    bi = oi;
                }
            }
            best = __shfl_sync(0xffffffffu, best, 0);
            bi = __shfl_sync(0xffffffffu, bi, 0);
            if (!(best > (T)0) || !(best < (sizeof(T) == 8 ? (T)1e300 : (T)1e38))) return false;
            if (bi != k) {
                for (int j = lane; j < N; j += 32) {
                    const T t = A[(size_t)k * LD + j];
                    A[(size_t)k * LD + j] = A[(size_t)bi * LD + j];
                    A[(size_t)bi * LD + j] = t;
                }
                if (lane == 0) {
                    const int t = perm[k];
                    perm[k] = perm[bi];
                    perm[bi] = t;
                }
            }
            __syncwarp();
            const T rp = (T)1 / A[(size_t)k * LD + k];
            if (lane == 0) rdiag[k] = (double)rp;
            for (int i = k + 1 + lane; i < N; i += 32) {
                T* Ai = A + (size_t)i * LD;
                const T l = Ai[k] * rp;
                Ai[k] = l;
                for (int j = k + 1; j < ke; j++) Ai[j] = fma(-l, A[(size_t)k * LD + j], Ai[j]);
            }
            __syncwarp();
        }
        if (ke == N) break;
        const int nb = ke - kb;
        // U rows of the panel, columns ke..N-1: forward substitution with the panel's unit lower L
        for (int j = ke + lane; j < N; j += 32) {
            T u[kPanel];
#pragma unroll
            for (int r = 0; r < kPanel; r++) {
                if (r < nb) {
                    T a = A[(size_t)(kb + r) * LD + j];
#pragma unroll
                    for (int t = 0; t < r; t++) a = fma(-A[(size_t)(kb + r) * LD + kb + t], u[t], a);
                    u[r] = a;
                    A[(size_t)(kb + r) * LD + j] = a;
                }
            }
        }
        __syncwarp();
        // trailing matrix: A[i][j] -= sum_t L[i][kb+t] U[kb+t][j], t in panel order
        for (int j = ke + lane; j < N; j += 32) {
            T u[kPanel];
#pragma unroll
            for (int t = 0; t < kPanel; t++) u[t] = t < nb ? A[(size_t)(kb + t) * LD + j] : (T)0;
#pragma unroll 2
            for (int i = ke; i < N; i++) {
                const T* Li = A + (size_t)i * LD + kb;
                T a = A[(size_t)i * LD + j];
#pragma unroll
                for (int t = 0; t < kPanel; t++)
                    if (t < nb) a = fma(-Li[t], u[t], a);
                A[(size_t)i * LD + j] = a;
            }
        }
        __syncwarp();
    }
    return true;
}

// At = A^T (both N x N with rows of LD), for the triangular solves below.
template <class T>
__device__ inline void transpose_warp(const T* A, T* At, int N, int LD, int lane) {
    for (int i = 0; i < N; i++)
        for (int j = lane; j < N; j += 32) At[(size_t)j * LD + i] = A[(size_t)i * LD + j];
    __syncwarp();
}

// A factor as a double: FP32 factors widened with integer instructions (off the FP64 pipe).
__device__ __forceinline__ double as_f64(double v) { return v; }
__device__ __forceinline__ double as_f64(float v) { return flt_to_dbl(v); }

// lu_solve_regs on the transposed factors: column k of L and U is row k of At, so every lane's reads of
// one elimination step fall in one contiguous row (global-memory matrices). Same operations and order;
// with FP32 factors (T = float) the right-hand side and its updates stay FP64.
template <int S, class T>
__device__ inline void lu_solve_t_regs(const T* At, int N, int LD, const int* perm, const double* rdiag, double* b,
                                       int lane) {
    double x[S];
#pragma unroll
    for (int s = 0; s < S; s++) {
        const int i = lane + 32 * s;
        x[s] = i < N ? b[perm[i]] : 0.0;
    }
    __syncwarp();
    for (int k = 0; k < N - 1; k++) {
        const double xk = __shfl_sync(0xffffffffu, slot_value<S>(x, k), k & 31);
        const T* col = At + (size_t)k * LD;
#pragma unroll
        for (int s = 0; s < S; s++) {
            if (32 * s + 31 <= k) continue;
            const int i = lane + 32 * s;
            if (i > k && i < N) x[s] = fma(-as_f64(col[i]), xk, x[s]);
        }
    }
    for (int k = N - 1; k >= 0; k--) {
        const double xk = __shfl_sync(0xffffffffu, slot_value<S>(x, k), k & 31) * rdiag[k];
        const T* col = At + (size_t)k * LD;
#pragma unroll
        for (int s = 0; s < S; s++) {
            if (32 * s > k) continue;
            const int i = lane + 32 * s;
            if (i == k) x[s] = xk;
            else if (i < k) x[s] = fma(-as_f64(col[i]), xk, x[s]);
        }
    }
#pragma unroll
    for (int s = 0; s < S; s++) {
        const int i = lane + 32 * s;
        if (i < N) b[i] = x[s];
    }
    __syncwarp();
}

// The same for any N with the right-hand side in memory (large mechanisms): b permuted through tmp, then
// one warp barrier per elimination step.
template <class T>
__device__ inline void lu_solve_t_mem(const T* At, int N, int LD, const int* perm, const double* rdiag, double* b,
                                      double* tmp, int lane) {
    for (int i = lane; i < N; i += 32) tmp[i] = b[perm[i]];
    __syncwarp();
    for (int i = lane; i < N; i += 32) b[i] = tmp[i];
    __syncwarp();
    for (int k = 0; k < N; k++) {
        const double bk = b[k];
        const T* col = At + (size_t)k * LD;
        for (int i = k + 1 + lane; i < N; i += 32) b[i] = fma(-as_f64(col[i]), bk, b[i]);
        __syncwarp();
    }
    for (int k = N - 1; k >= 0; k--) {
        const double bk = b[k] * rdiag[k];
        __syncwarp();
        if (lane == 0) b[k] = bk;
        const T* col = At + (size_t)k * LD;
        for (int i = lane; i < k; i += 32) b[i] = fma(-as_f64(col[i]), bk, b[i]);
        __syncwarp();
    }
}

template <class T>
__device__ inline void lu_solve_t_warp(const T* At, int N, int LD, const int* perm, const double* rdiag, double* b,
                                       double* tmp, int lane) {
    if (N <= 64) lu_solve_t_regs<2>(At, N, LD, perm, rdiag, b, lane);
    else if (N <= 96) lu_solve_t_regs<3>(At, N, LD, perm, rdiag, b, lane);
    else lu_solve_t_mem(At, N, LD, perm, rdiag, b, tmp, lane);
}

// I - c J (J in LU already when `fresh`, else from global) factorised in LU (pivots, 1 / U_kk); with
// per-reactor factorisations in global memory (GLOBAL), by panels, and its transpose into `LUt` for the
// solves. With CB_BDF_LU32 (GLOBAL only) the factors are FP32 and both they and their transpose live in
// LUt's bytes (LU stays the FP64 Jacobian scratch).
template <bool GLOBAL>
__device__ __noinline__ bool build_lu(const Params& p, double* LU, int* piv, double* rdiag, const double* Jg, double c, bool fresh,
                         double* LUt, int lane) {
    const int N = p.N, LD = p.LD;
    for (int idx = lane; idx < N * N; idx += 32) {
        const int i = idx / N, j = idx % N;
        const double Jij = fresh ? LU[(size_t)i * LD + j] : Jg[idx];
        LU[(size_t)i * LD + j] = (i == j ? 1.0 : 0.0) - c * Jij;
    }
    __syncwarp();
    if constexpr (!GLOBAL) {
        return lu_warp(LU, N, LD, piv, rdiag, lane);
    } else {
        if (p.lu32) {
            float* F = reinterpret_cast<float*>(LUt);
            for (int idx = lane; idx < N * N; idx += 32) {
                const int i = idx / N, j = idx % N;
                F[(size_t)i * LD + j] = (float)LU[(size_t)i * LD + j];
            }
            __syncwarp();
            if (!lu_warp_blocked(F, N, LD, piv, rdiag, lane)) return false;
            transpose_warp(F, F + (size_t)N * LD, N, LD, lane);
            return true;
        }
        if (!lu_warp_blocked(LU, N, LD, piv, rdiag, lane)) return false;
        transpose_warp(LU, LUt, N, LD, lane);
        return true;
    }
}

// Weighted RMS norm; rscale holds the reciprocal weights 1 / (atol + rtol |y_i|).
__device__ __forceinline__ double rms_scaled(const double* x, const double* rscale, int N, int lane) {
    double s = 0.0;
    for (int i = lane; i < N; i += 32) {
        const double v = x[i] * rscale[i];
        s = fma(v, v, s);
    }
    return sqrt(warp_sum(s) / N);
}

// D[0..q] <- (R U)^T D[0..q], R = R(q, factor), U = R(q, 1) (step size change by `factor`), in registers:
// lane j computes column j of R and of U (R[i][j] = R[i-1][j] ((i-1) - factor j) / i), then column j of
// R U from row i of R broadcast by shuffles; the columns of D then take (R U)[m][i] from lane i the same
// way. The products and sums are the textbook ones in the same order (sum over k, then over m, by FMAs).
// Loops are unrolled to the largest order with the entries beyond q masked out, so no array goes to
// local memory.
static __device__ __noinline__ void change_D(double* D, int N, int q, double factor, int lane) {
    const int j = lane;
    double Rc[kMaxOrder + 1], Uc[kMaxOrder + 1], RUc[kMaxOrder + 1];
    Rc[0] = 1.0;
    Uc[0] = 1.0;
#pragma unroll
    for (int i = 1; i <= kMaxOrder; i++) {
        const double mr = j == 0 ? 0.0 : ((double)(i - 1) - factor * j) * kRcpInt[i];
        const double mu = j == 0 ? 0.0 : ((double)(i - 1) - (double)j) * kRcpInt[i];
        Rc[i] = Rc[i - 1] * mr;
        Uc[i] = Uc[i - 1] * mu;
    }
#pragma unroll
    for (int i = 0; i <= kMaxOrder; i++) {  // lane j: (R U)[i][j] = sum_k R[i][k] U[k][j]
        double s = 0.0;
#pragma unroll
        for (int k = 0; k <= kMaxOrder; k++) {
            const double rik = __shfl_sync(0xffffffffu, Rc[i], k);
            if (k <= q) s = fma(rik, Uc[k], s);
        }
        RUc[i] = s;
    }
    for (int c0 = 0; c0 < N; c0 += 32) {  // warp-uniform loop: the shuffles need every lane
        const int col = c0 + lane;
        const bool in = col < N;
        double old[kMaxOrder + 1];
#pragma unroll
        for (int m = 0; m <= kMaxOrder; m++) old[m] = (in && m <= q) ? D[(size_t)m * N + col] : 0.0;
#pragma unroll
        for (int i = 0; i <= kMaxOrder; i++) {
            double s = 0.0;
#pragma unroll
            for (int m = 0; m <= kMaxOrder; m++) {
                const double rum = __shfl_sync(0xffffffffu, RUc[m], i);  // (R U)[m][i]
                if (m <= q) s = fma(rum, old[m], s);
            }
            if (in && i <= q) D[(size_t)i * N + col] = s;
        }
    }
    __syncwarp();
}

__device__ __forceinline__ double gamma_k(int k) { return kGamma[k]; }  // sum_{i=1..k} 1/i

// x^n for the small exponents of the Newton convergence test.
__device__ __forceinline__ double ipow(double x, int n) {
    double r = x;
    for (int i = 1; i < n; i++) r *= x;
    return r;
}

// x^(-1/n), x > 0 finite, for the step-size factors.
__device__ __forceinline__ double root_factor(double x, int n) { return exp64(-log64(x) * kRcpInt[n]); }

// One reactor for at most `budget` steps (warp-uniform control flow). MIXED: the first Newton iteration
// of each step on the mixed-precision f(u); GLOBAL: workspaces and per-reactor factorisations in global
// memory.
template <bool MIXED, bool GLOBAL>
__device__ inline void integrate(const Params& p, const Mech& m, const Work& w, int r, int lane) {
    const int N = p.N;
    Head hd = p.head[r];
    if (hd.state != kNew && hd.state != kRunning) return;
    double* Dg = p.D + (size_t)r * kDRows * N;
    double* Jg = p.J + (size_t)r * N * N;
    const double pR = p.pR[r], rP = 1.0 / pR;
    // the factorisation: the warp's workspace, or (GLOBAL) the reactor's own with its transpose
    double* LU = GLOBAL ? p.LUr + (size_t)r * N * p.LD : w.LU;
    int* piv = GLOBAL ? p.piv_r + (size_t)r * N : w.piv;
    double* rdiag = GLOBAL ? p.rdiag_r + (size_t)r * N : w.rdiag;
    double* LUt = GLOBAL ? p.LUt + (size_t)r * N * p.LD : nullptr;
    for (int i = lane; i < kDRows * N; i += 32) w.D[i] = Dg[i];
    __syncwarp();
    // lu_have: LU holds the factorisation of I - c_lu J; lu_refresh: c changed since (a step size or
    // order change), so it is made again before the next Newton iteration unless CB_BDF_REUSE_LU keeps
    // it. A launch starts with a fresh factorisation, except that with CB_BDF_REUSE_LU a reactor's own
    // (global memory) carries over.
    const bool carry = GLOBAL && p.reuse_lu;
    bool lu_have = carry ? hd.lu_have != 0 : false;
    bool lu_refresh = carry ? hd.lu_refresh != 0 : true;
    double c_lu = hd.c_lu;
    auto factorise = [&](double c, bool fresh) {
        lu_have = build_lu<GLOBAL>(p, LU, piv, rdiag, Jg, c, fresh, LUt, lane);
        c_lu = c;
        lu_refresh = false;
        hd.lus++;
        hd.since_lu = 0;
    };
    if (hd.state == kNew) {
        // f(y0), initial step (Hairer, Norsett and Wanner, Solving ODEs I, II.4), D_1 = h f(y0), J(y0)
        for (int i = lane; i < N; i += 32) w.y[i] = w.D[i];
        __syncwarp();
        rhs_warp<false>(p, m, w, pR, rP, w.y, w.f, lane);
        hd.rhs++;
        for (int i = lane; i < N; i += 32) w.rscale[i] = 1.0 / (p.atol + p.rtol * fabs(w.y[i]));
        __syncwarp();
        const double d0 = rms_scaled(w.y, w.rscale, N, lane), d1 = rms_scaled(w.f, w.rscale, N, lane);
        const double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
        for (int i = lane; i < N; i += 32) w.b[i] = fma(h0, w.f[i], w.y[i]);
        __syncwarp();
        rhs_warp<false>(p, m, w, pR, rP, w.b, w.tmp, lane);
        hd.rhs++;
        for (int i = lane; i < N; i += 32) w.b[i] = w.tmp[i] - w.f[i];
        __syncwarp();
        const double d2 = rms_scaled(w.b, w.rscale, N, lane) / h0;
        const double h1 = (d1 <= 1e-15 && d2 <= 1e-15) ? fmax(1e-6, h0 * 1e-3) : sqrt(0.01 / fmax(d1, d2));
        double h = fmin(100.0 * h0, h1);
        h = fmin(h, p.t_end);
        for (int i = lane; i < N; i += 32) {
            w.D[N + i] = h * w.f[i];
            for (int j = 2; j < kDRows; j++) w.D[(size_t)j * N + i] = 0.0;
        }
        __syncwarp();
        const double g0 = w.f[0];
        hd.t = 0.0;
        hd.h = h;
        hd.q = 1;
        hd.n_equal = 0;
        hd.ign_t = 0.0;
        hd.ign_g = g0;
        hd.ta = hd.ga = hd.tc = hd.gc = NAN;
        hd.tp = 0.0;
        hd.gp = g0;
        hd.need_next = 1;
        hd.next_out = 0;
        hd.peak_x = -1.0;
        record_outputs(p, hd, r, w.D, 0.0, h, 0, lane);  // the initial state: trajectory point 0
        jacobian_warp(p, m, w, pR, rP, w.y, Jg, LU, lane);
        hd.jacs++;
        hd.rhs += 2;
        hd.jac_current = 1;
        factorise(h / gamma_k(1), true);
        hd.state = kRunning;
    }
    const double newton_tol = fmax(10.0 * 2.220446049250313e-16 / p.rtol, fmin(0.03, sqrt(p.rtol)));
    int budget = p.slice_steps;
    // every rejected attempt shrinks h, so attempts are bounded; the cap only bounds one launch's length
    int attempts = 8 * p.slice_steps + 64;
    while (hd.state == kRunning && budget > 0 && attempts-- > 0) {
        if (hd.steps >= p.max_steps) {
            hd.state = kFailSteps;
            break;
        }
        int q = hd.q;
        double h = hd.h;
        if (hd.t + h > p.t_end) {  // land on t_end
            const double hn = p.t_end - hd.t;
            change_D(w.D, N, q, hn / h, lane);
            h = hn;
            hd.n_equal = 0;
            lu_refresh = true;
        }
        if (!(h >= p.h_min)) {
            hd.state = kFailStep;
            break;
        }
        const double t_new = hd.t + h;
        const double gq = gamma_k(q);
        const double c = h / gq;
        for (int i = lane; i < N; i += 32) {
            double yp = 0.0, ps = 0.0;
            for (int j = 0; j <= q; j++) yp += w.D[(size_t)j * N + i];
            for (int j = 1; j <= q; j++) ps = fma(gamma_k(j), w.D[(size_t)j * N + i], ps);
            w.ypred[i] = yp;
            w.psi[i] = ps * kRcpGamma[q];
            w.rscale[i] = 1.0 / (p.atol + p.rtol * fabs(yp));
            w.y[i] = yp;
            w.d[i] = 0.0;
        }
        __syncwarp();
        if (lu_have && lu_refresh && p.reuse_lu && fabs(c / c_lu - 1.0) <= kReuseSpread && hd.since_lu < kReuseSteps)
            lu_refresh = false;  // kept: the correction is scaled below
        if (!lu_have || lu_refresh) factorise(c, false);
        // a kept factorisation of I - c_lu J: Newton corrections scaled by 2 / (1 + c / c_lu)
        const double corr = (p.reuse_lu && c != c_lu) ? 2.0 / (1.0 + c / c_lu) : 1.0;
        // Newton iterations on d - c f(t_new, ypred + d) + psi = 0
        bool converged = false;
        int n_iter = 0;
        double dy_norm_old = -1.0;
        if (lu_have) {
            for (int k = 0; k < kNewtonMaxIter; k++) {
                // MIXED: the first iteration (the correction from the predictor) on the mixed-precision
                // f; the later ones, whose corrections decide convergence, in FP64
                if (MIXED && k == 0) rhs_warp_mixed(p, m, RatesMixedTables(p.tab_m), w, pR, rP, w.y, w.f, lane);
                else rhs_warp<false>(p, m, w, pR, rP, w.y, w.f, lane);
                hd.rhs++;
                n_iter = k + 1;
                bool finite = true;
                for (int i = lane; i < N; i += 32) {
                    const double fi = w.f[i];
                    finite &= (fabs(fi) < 1e300);
                    w.b[i] = fma(c, fi, -w.psi[i]) - w.d[i];
                }
                if (!__all_sync(0xffffffffu, finite)) break;
                __syncwarp();
                if constexpr (GLOBAL) {
                    if (p.lu32) {
                        const float* F = reinterpret_cast<const float*>(LUt);
                        lu_solve_t_warp(F + (size_t)N * p.LD, N, p.LD, piv, rdiag, w.b, w.tmp, lane);
                    } else {
                        lu_solve_t_warp(LUt, N, p.LD, piv, rdiag, w.b, w.tmp, lane);
                    }
                } else {
                    lu_solve_warp(LU, N, p.LD, piv, rdiag, w.b, lane);
                }
                if (corr != 1.0) {
                    for (int i = lane; i < N; i += 32) w.b[i] *= corr;
                    __syncwarp();
                }
                const double dy_norm = rms_scaled(w.b, w.rscale, N, lane);
                const double rate = dy_norm_old >= 0.0 ? dy_norm / dy_norm_old : -1.0;
                if (rate >= 0.0 && (rate >= 1.0 || ipow(rate, kNewtonMaxIter - k) / (1.0 - rate) * dy_norm > newton_tol))
                    break;
                for (int i = lane; i < N; i += 32) {
                    w.y[i] += w.b[i];
                    w.d[i] += w.b[i];
                }
                __syncwarp();
                // MIXED: the first FP64 correction follows the mixed one, whose size says nothing about
                // the FP64 iteration's rate; it is accepted when it is below the tolerance itself (the
                // first-iteration test of CVODE), and the rate is measured from it on.
                if (dy_norm == 0.0 || (rate >= 0.0 && rate / (1.0 - rate) * dy_norm < newton_tol) ||
                    (MIXED && k == 1 && dy_norm <= newton_tol)) {
                    converged = true;
                    break;
                }
                dy_norm_old = (MIXED && k == 0) ? -1.0 : dy_norm;
            }
        }
        if (!converged) {
            hd.newton_fail++;
            if (!hd.jac_current) {  // a fresh Jacobian at the predicted state, same step
                jacobian_warp(p, m, w, pR, rP, w.ypred, Jg, LU, lane);
                hd.jacs++;
                hd.rhs += 2;
                hd.jac_current = 1;
                factorise(c, true);
                hd.h = h;
                continue;
            }
            change_D(w.D, N, q, 0.5, lane);
            hd.h = 0.5 * h;
            hd.n_equal = 0;
            lu_refresh = true;
            continue;
        }
        const double safety = 0.9 * (2 * kNewtonMaxIter + 1) / (2 * kNewtonMaxIter + n_iter);
        for (int i = lane; i < N; i += 32) {
            w.rscale[i] = 1.0 / (p.atol + p.rtol * fabs(w.y[i]));
            w.b[i] = w.d[i] * kRcpInt[q + 1];  // error = error_const(q) d
        }
        __syncwarp();
        const double err_norm = rms_scaled(w.b, w.rscale, N, lane);
        if (err_norm > 1.0) {
            hd.err_fail++;
            const double factor = fmax(kMinFactor, safety * root_factor(err_norm, q + 1));
            change_D(w.D, N, q, factor, lane);
            hd.h = h * factor;
            hd.n_equal = 0;
            continue;  // the factorisation of the failed step is kept: Newton converged with it
        }
        // accepted
        hd.steps++;
        hd.since_lu++;
        budget--;
        hd.t = t_new;
        hd.jac_current = 0;
        for (int i = lane; i < N; i += 32) {
            const double di = w.d[i];
            w.D[(size_t)(q + 2) * N + i] = di - w.D[(size_t)(q + 1) * N + i];
            w.D[(size_t)(q + 1) * N + i] = di;
            for (int j = q; j >= 0; j--) w.D[(size_t)j * N + i] += w.D[(size_t)(j + 1) * N + i];
        }
        __syncwarp();
        hd.n_equal++;
        if (p.traj || p.peak_k >= 0) record_outputs(p, hd, r, w.D, t_new, h, q, lane);
        // dT/dt at the new point from the backward differences: h y' = sum_{j=1..q} D_j / j
        double g = 0.0;
        for (int j = 1; j <= q; j++) g += w.D[(size_t)j * N] * kRcpInt[j];
        g /= h;
        if (hd.need_next) {
            hd.tc = t_new;
            hd.gc = g;
            hd.need_next = 0;
        }
        if (g > hd.ign_g) {
            hd.ta = hd.tp;
            hd.ga = hd.gp;
            hd.ign_t = t_new;
            hd.ign_g = g;
            hd.need_next = 1;
        }
        hd.tp = t_new;
        hd.gp = g;
        if (t_new >= p.t_end) {
            hd.state = kDone;
            hd.h = h;
            break;
        }
        if (hd.n_equal < q + 1) {
            hd.h = h;
            continue;
        }
        // order and step size
        const double inf = 1e300;
        double em = inf, ep = inf;
        if (q > 1) {
            for (int i = lane; i < N; i += 32) w.b[i] = w.D[(size_t)q * N + i] * kRcpInt[q];
            __syncwarp();
            em = rms_scaled(w.b, w.rscale, N, lane);
        }
        if (q < kMaxOrder) {
            for (int i = lane; i < N; i += 32) w.b[i] = w.D[(size_t)(q + 2) * N + i] * kRcpInt[q + 2];
            __syncwarp();
            ep = rms_scaled(w.b, w.rscale, N, lane);
        }
        const double fm = em >= inf ? 0.0 : (em > 0.0 ? root_factor(em, q) : inf);
        const double fz = err_norm > 0.0 ? root_factor(err_norm, q + 1) : inf;
        const double fp = ep >= inf ? 0.0 : (ep > 0.0 ? root_factor(ep, q + 2) : inf);
        int dq = 0;
        double best = fz;
        if (fm > best) {
            best = fm;
            dq = -1;
        }
        if (fp > best) {
            best = fp;
            dq = 1;
        }
        q += dq;
        const double factor = fmin(kMaxFactor, safety * best);
        change_D(w.D, N, q, factor, lane);
        hd.q = q;
        hd.h = h * factor;
        hd.n_equal = 0;
        lu_refresh = true;
    }
    for (int i = lane; i < kDRows * N; i += 32) Dg[i] = w.D[i];
    hd.lu_have = (GLOBAL && lu_have) ? 1 : 0;  // only a reactor's own (global) factorisation outlives the launch
    hd.lu_refresh = lu_refresh ? 1 : 0;
    hd.c_lu = c_lu;
    if (lane == 0) {
        p.head[r] = hd;
        if (hd.state != kRunning) atomicAdd(p.done, 1);
    }
    __syncwarp();
}

// This warp's workspace: after the tables in shared memory, or its slot of the global workspaces.
__device__ __forceinline__ uint8_t* workspace_of(const Params& p, int warp) {
    if (p.ws_global) return p.ws_global + ((size_t)blockIdx.x * (blockDim.x >> 5) + warp) * p.ws_bytes;
    const size_t tab_smem = p.smem_tables ? ((p.tab_bytes + 127) & ~127u) : (size_t)kMathBytes;
    return cb_dsmem + tab_smem + (size_t)warp * p.ws_bytes;
}

template <bool MIXED, bool GLOBAL>
__device__ __forceinline__ void slice_body(const Params& p) {
    __shared__ uint64_t bar;
    const uint8_t* tab = p.tab;
    if (p.smem_tables) {
        if (!stage_to_shared(cb_dsmem, p.tab, p.tab_bytes, &bar, p.status)) return;
        tab = cb_dsmem;
    } else {
        load_math(p.tab);
    }
    const Mech m(tab, p);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const Work w = carve(p, workspace_of(p, warp), (size_t)blockIdx.x * (blockDim.x >> 5) + warp);
    for (;;) {
        int r = 0;
        if (lane == 0) r = atomicAdd(p.queue, 1);
        r = __shfl_sync(0xffffffffu, r, 0);
        if (r >= p.n) break;
        integrate<MIXED, GLOBAL>(p, m, w, r, lane);
    }
}

template <bool MIXED>
__global__ void slice_kernel(const __grid_constant__ Params p) {
    slice_body<MIXED, false>(p);
}

// Global-memory workspaces: four 256-thread blocks per SM (32 warps, 64 registers a thread) to hide the
// latency of workspaces that live in L2 and HBM (measured at 250 species, 4096 reactors: 17.3 s against
// 20.6 s with two blocks and 20.0 s with three).
template <bool MIXED>
__global__ void __launch_bounds__(256, 4) slice_kernel_global(const __grid_constant__ Params p) {
    slice_body<MIXED, true>(p);
}

// The same with two blocks per SM (128 registers a thread, fewer spills, half the warps).
template <bool MIXED>
__global__ void __launch_bounds__(256, 2) slice_kernel_global_wide(const __grid_constant__ Params p) {
    slice_body<MIXED, true>(p);
}

// And with three (80 registers a thread).
template <bool MIXED>
__global__ void __launch_bounds__(256, 3) slice_kernel_global_mid(const __grid_constant__ Params p) {
    slice_body<MIXED, true>(p);
}

using SliceFn = void (*)(Params);
SliceFn slice_kernel_fn(bool mixed);              // bdf_slice.cu: workspaces in shared memory
SliceFn slice_kernel_global_fn(bool mixed);       // bdf_slice_global.cu: workspaces in global memory
SliceFn slice_kernel_global_wide_fn(bool mixed);  // bdf_slice_global_wide.cu: the same, 128 registers
SliceFn slice_kernel_global_mid_fn(bool mixed);   // bdf_slice_global_mid.cu: the same, 80 registers

}  // namespace bdf
}  // namespace cbg
