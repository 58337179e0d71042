// Plain FP64 kernels: species production rates (reaction.rs:207-391), per-reaction rates of progress
// (reaction.rs:329-354) and mixture-averaged transport (transport.rs:141-210), one cell per thread.
//
// Every thread of a warp walks the same reaction / species / pair at the same time, so each table read
// is a broadcast; the per-cell working arrays (concentrations, Gibbs exponentials, accumulators) live in
// thread-local memory. The FP64 pipe is the bottleneck; nothing else here comes close to its limits.
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "device_math.cuh"
#include "kernels.h"
#include "rates_core.cuh"
#include "tables.h"

namespace cbg {

template <int KMAX>
struct Cell {
    Temps t;
    double Ctot, C0, rcpC0, rcpC0sq;
    double C[KMAX];              // concentrations, bulk last
    double ex[KMAX], exn[KMAX];  // min(M3, exp(g_k)), min(cbrt(f32::MAX), exp(-g_k))
};

// Prologue of reaction.rs:362-373 and the Gibbs exponentials of reaction.rs:234-263.
template <int KMAX>
__device__ __forceinline__ void cell_setup(const RatesTables& tb, double pressure_R, double T, double V,
                                           const double* const* amounts, size_t i, Cell<KMAX>& c) {
    const RatesHeader& H = *tb.H;
    const int K = H.K, A = H.A;
    const double md = rcp64(V);
    c.t.T = T;
    c.t.rcpT = rcp64(T);
    c.t.lnT = log64(T);
    c.t.T2 = T * T;
    c.t.T3 = T * c.t.T2;
    c.t.T4 = c.t.T2 * c.t.T2;
    c.t.rcpT2 = c.t.rcpT * c.t.rcpT;
    double sum = 0.0;
    for (int k = 0; k < K - 1; k++) {
        c.C[k] = md * max0(amounts[k][i]);
        sum += c.C[k];
    }
    c.Ctot = pressure_R * c.t.rcpT;
    c.C[K - 1] = c.Ctot - sum;
    c.C0 = H.C0 * c.t.rcpT;
    c.rcpC0 = H.rcp_C0 * T;
    c.rcpC0sq = c.rcpC0 * c.rcpC0;
    for (int k = 0; k < A; k++) {
        const Species& s = tb.species[k];
        if (!(s.need_exp | s.need_exp_neg)) continue;
        const double* g = s.g[piece_of(s.split, T)];
        const double x = fma(g[6], c.t.rcpT, fma(g[5], c.t.T4, fma(g[4], c.t.T3, fma(g[3], c.t.T2,
                         fma(g[2], T, fma(g[1], c.t.lnT, g[0]))))));
        if (s.need_exp) c.ex[k] = min_pos(H.M3, exp64(x));
        if (s.need_exp_neg) c.exn[k] = min_pos(H.cbrt_max, exp64(-x));
    }
}

// Reactions without a third body (models 0 and 1), one loop per model; emit(x, cR) takes each rate.
template <int KMAX, int MODEL, class Emit>
__device__ __forceinline__ void plain_group(const RatesTables& tb, const Cell<KMAX>& c, Emit emit) {
    for (int r = MODEL ? tb.H->group_end[MODEL - 1] : 0; r < tb.H->group_end[MODEL]; r++) {
        const Reaction& x = tb.reactions[r];
        emit(x, reaction_rate<MODEL>(tb, x, c, 0.0));
    }
}

// Reactions with a third body (models 2-5: consecutive in the tables, efficiency row e for reaction
// group_end[1] + e). The third-body sums efficiency() (reaction.rs:141-145) of four consecutive rows
// (padded to a multiple of 4) take one pass over the concentrations, one local load of C_k per four
// FMAs, just before their reactions: no array of sums is kept. The model branch is uniform across the
// warp (every lane is at the same reaction).
template <int KMAX, class Emit>
__device__ __forceinline__ void third_body_groups(const RatesTables& tb, const Cell<KMAX>& c, Emit emit) {
    const RatesHeader& H = *tb.H;
    const int K = H.K, r_begin = H.group_end[1], r_end = H.group_end[5];
    for (int r0 = r_begin; r0 < r_end; r0 += 4) {
        const double* E = tb.eff + (size_t)(r0 - r_begin) * K;
        double s[4] = {0.0, 0.0, 0.0, 0.0};
        for (int k = 0; k < K; k++) {
            const double ck = c.C[k];
#pragma unroll
            for (int q = 0; q < 4; q++) s[q] = fma(E[q * K + k], ck, s[q]);
        }
        const double M0 = c.Ctot + s[0], M1 = c.Ctot + s[1], M2 = c.Ctot + s[2], M3 = c.Ctot + s[3];
        const int rq = min(r_end - r0, 4);
#pragma unroll 1
        for (int q = 0; q < rq; q++) {
            const int r = r0 + q;
            const double M = q == 0 ? M0 : q == 1 ? M1 : q == 2 ? M2 : M3;  // integer selects
            const Reaction& x = tb.reactions[r];
            double cR;
            if (r < H.group_end[2]) cR = reaction_rate<2>(tb, x, c, M);
            else if (r < H.group_end[3]) cR = reaction_rate<3>(tb, x, c, M);
            else if (r < H.group_end[4]) cR = reaction_rate<4>(tb, x, c, M);
            else cR = reaction_rate<5>(tb, x, c, M);
            emit(x, cR);
        }
    }
}

template <int KMAX>
__device__ void rates_cell(const RatesTables& tb, const RatesArgs<KMAX>& io, size_t i) {
    const RatesHeader& H = *tb.H;
    const int K = H.K, A = H.A;
    const bool uniform = io.flags & kUniformPressure;
    const double pressure_R = uniform ? io.in[0][0] : io.in[0][i];
    const double rcp_pressure_R = uniform ? io.in[1][0] : io.in[1][i];
    const double T = io.in[2][i], V = io.in[3][i];
    Cell<KMAX> c;
    cell_setup<KMAX>(tb, pressure_R, T, V, io.in + 4, i, c);
    double wdot[KMAX];
    for (int k = 0; k < A; k++) wdot[k] = 0.0;
    // species_rates (reaction.rs:312-327), reactions grouped by model
    // read-modify-writes in pairs, the two reads issued together (net species are distinct)
    auto accumulate = [&](const Reaction& x, double cR) {
#pragma unroll 1
        for (int q = 0; q < x.n_net; q += 2) {
            const int k0 = x.net_k[q], k1 = x.net_k[q + 1 < x.n_net ? q + 1 : q];
            const double w0 = wdot[k0], w1 = wdot[k1];
            wdot[k0] = fma(small_int_to_double(x.net_n[q]), cR, w0);
            if (q + 1 < x.n_net) wdot[k1] = fma(small_int_to_double(x.net_n[q + 1]), cR, w1);
        }
    };
    plain_group<KMAX, 0>(tb, c, accumulate);
    plain_group<KMAX, 1>(tb, c, accumulate);
    third_body_groups<KMAX>(tb, c, accumulate);
    // Energy and volume (reaction.rs:375-384).
    double E = 0.0;
    for (int k = 0; k < A; k++) {
        const Species& s = tb.species[k];
        const double* h = s.h[piece_of(s.split, T)];
        const double hk = fma(h[5], c.t.rcpT, fma(h[4], c.t.T4, fma(h[3], c.t.T3, fma(h[2], c.t.T2, fma(h[1], T, h[0])))));
        E = fma(wdot[k], hk, E);
    }
    double Cp = 0.0;
    for (int k = 0; k < K; k++) {
        const Species& s = tb.species[k];
        const double* cp = s.cp[piece_of(s.split, T)];
        const double ck = fma(cp[4], c.t.T4, fma(cp[3], c.t.T3, fma(cp[2], c.t.T2, fma(cp[1], T, cp[0]))));
        Cp = fma(ck, c.C[k], Cp);
    }
    const double dtT_T = div64(-E, Cp);
    double dtE = 0.0;
    for (int k = 0; k < A; k++) dtE = fma(tb.species[k].dtE, wdot[k], dtE);
    io.out[0][i] = T * dtT_T;
    io.out[1][i] = V * fma(rcp_pressure_R * T, dtE, dtT_T);
    for (int k = 0; k < A; k++) io.out[2 + k][i] = wdot[k];
}

template <int KMAX>
__device__ void reaction_rates_cell(const RatesTables& tb, const ReactionRatesArgs<KMAX>& io, size_t i) {
    Cell<KMAX> c;
    cell_setup<KMAX>(tb, io.in[0][i], io.in[1][i], io.in[2][i], io.in + 3, i, c);
    auto store = [&](const Reaction& x, double cR) { io.out[x.orig][i] = cR; };
    plain_group<KMAX, 0>(tb, c, store);
    plain_group<KMAX, 1>(tb, c, store);
    third_body_groups<KMAX>(tb, c, store);
}

template <int KMAX, bool SMEM>
__global__ void __launch_bounds__(kBlock) rates_kernel(const uint8_t* __restrict__ gtab, uint32_t tab_bytes,
                                                      const __grid_constant__ RatesArgs<KMAX> io, size_t n,
                                                      int* status) {
    __shared__ uint64_t bar;
    const uint8_t* tab = gtab;
    if (SMEM) {  // the whole blob, math tables first, into dynamic shared memory
        if (!stage_to_shared(cb_dsmem, gtab, tab_bytes, &bar, status)) return;
        tab = cb_dsmem;
    } else {  // tables read from global memory; only the math tables go to shared memory
        load_math(gtab);
    }
    const RatesTables tb(tab);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        rates_cell<KMAX>(tb, io, i);
}

template <int KMAX, bool SMEM>
__global__ void __launch_bounds__(kBlock) reaction_rates_kernel(const uint8_t* __restrict__ gtab, uint32_t tab_bytes,
                                                               const __grid_constant__ ReactionRatesArgs<KMAX> io,
                                                               size_t n, int* status) {
    __shared__ uint64_t bar;
    const uint8_t* tab = gtab;
    if (SMEM) {  // the whole blob, math tables first, into dynamic shared memory
        if (!stage_to_shared(cb_dsmem, gtab, tab_bytes, &bar, status)) return;
        tab = cb_dsmem;
    } else {  // tables read from global memory; only the math tables go to shared memory
        load_math(gtab);
    }
    const RatesTables tb(tab);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        reaction_rates_cell<KMAX>(tb, io, i);
}

// ---------------------------------------------------------------------------------------------------
// Pieces shared by the thread-per-cell and warp-per-cell transport kernels, so that both evaluate the
// same expressions: a cell's sum n, T/T0 and amount arrays (transport.rs:179-190), the conductivity of
// its two mixing sums (transport.rs:141-146) and one species' mixture diffusion (transport.rs:176).
template <class Args>
__device__ __forceinline__ const double* const* transport_inputs(const TransportHeader& H, const Args& io,
                                                                 size_t i, double& N, double& Tn) {
    if (io.flags & kFromRates) {  // sum n = (P/R V) / T and T/T0 of a rates-layout cell
        const double pressure_R = (io.flags & kUniformPressure) ? io.in[0][0] : io.in[0][i];
        const double T = io.in[2][i];
        N = div64(pressure_R * io.in[3][i], T);
        Tn = div64(T, H.T0);
        return io.in + 4;
    }
    N = io.in[0][i];
    Tn = io.in[1][i];
    return io.in + 2;
}
// Products here are rounded on their own (never fused into the next add, as in the reference's own
// arithmetic), so that the two kernels cannot differ by where the compiler contracts.
__device__ __forceinline__ double conductivity_of(double Ac, double Bc, double N, double VT) {
    return __dmul_rn(__dadd_rn(div64(Ac, N), div64(N, Bc)), VT);
}
__device__ __forceinline__ double diffusion_of(double MVTN, double VT, double W, double X, double S) {
    return div64(__dsub_rn(MVTN, __dmul_rn(__dmul_rn(VT, W), X)), S);
}

// Rows k0 .. k0 + Q - 1 of Wilke's mixing sums (transport.rs:148-158, the square expanded), each summed
// over j in order, and their terms of mu added in row order.
template <int Q>
__device__ __forceinline__ double wilke_rows(const double* A2, const double* AB, const double* B2, int K, int k0,
                                             const double* X, const double* Y, const double* Z, const double* v,
                                             double mu) {
    const double* a2 = A2 + (size_t)k0 * K;
    const double* ab = AB + (size_t)k0 * K;
    const double* b2 = B2 + (size_t)k0 * K;
    double s1[Q], s2[Q], s3[Q];
#pragma unroll
    for (int q = 0; q < Q; q++) s1[q] = s2[q] = s3[q] = 0.0;
    for (int j = 0; j < K; j++) {
        const double xj = X[j], yj = Y[j], zj = Z[j];
#pragma unroll
        for (int q = 0; q < Q; q++) {
            s1[q] = fma(a2[q * K + j], xj, s1[q]);
            s2[q] = fma(ab[q * K + j], yj, s2[q]);
            s3[q] = fma(b2[q * K + j], zj, s3[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int k = k0 + q;
        const double den = fma(v[k], fma(v[k], s3[q], s2[q]), s1[q]);
        mu = fma(X[k] * (v[k] * v[k]), rcp64(den), mu);
    }
    return mu;
}

template <int KMAX>
__device__ void transport_cell(const uint8_t* tab, const TransportArgs<KMAX>& io, size_t i, size_t o) {
    // i: the cell's index in the inputs, o: in the outputs (they differ for gathered cells)
    const TransportHeader& H = *reinterpret_cast<const TransportHeader*>(tab + kMathBytes);
    const double* cond = reinterpret_cast<const double*>(tab + H.off_cond);
    const double* visc = reinterpret_cast<const double*>(tab + H.off_visc);
    const double* W = reinterpret_cast<const double*>(tab + H.off_W);
    const double* diff = reinterpret_cast<const double*>(tab + H.off_diff);
    const double* A2 = reinterpret_cast<const double*>(tab + H.off_A2);
    const double* AB = reinterpret_cast<const double*>(tab + H.off_AB);
    const double* B2 = reinterpret_cast<const double*>(tab + H.off_B2);
    const int K = H.K;
    double N, Tn;
    const double* const* amounts = transport_inputs(H, io, i, N, Tn);
    const double L1 = log64(Tn), L2 = L1 * L1, L3 = L2 * L1, L4 = L3 * L1;
    auto poly = [&](const double* P) { return fma(P[4], L4, fma(P[3], L3, fma(P[2], L2, fma(P[1], L1, P[0])))); };

    double X[KMAX], v[KMAX], Y[KMAX], Z[KMAX];
    double s = 0.0;
    for (int k = 0; k < K - 1; k++) {
        X[k] = amounts[k][i];
        s += X[k];
    }
    X[K - 1] = N - s;
    const double VT = sqrt(Tn);
    double MN = 0.0;
    for (int k = 0; k < K; k++) MN = fma(W[k], X[k], MN);
    const double MVTN = MN * VT;

    // Conductivity (transport.rs:141-146).
    double Ac = 0.0, Bc = 0.0;
    for (int k = 0; k < K; k++) {
        const double c = poly(cond + 5 * k);
        Ac = fma(X[k], c, Ac);
        Bc = fma(X[k], rcp64(c), Bc);
    }
    io.out[0][o] = conductivity_of(Ac, Bc, N, VT);

    // Viscosity, Wilke mixing (transport.rs:148-158) with the square expanded:
    // sum_j X_j (a + b v_k/v_j)^2 = sum_j a^2 X_j + v_k sum_j 2ab X_j/v_j + v_k^2 sum_j b^2 X_j/v_j^2.
    for (int k = 0; k < K; k++) {
        v[k] = poly(visc + 5 * k);
        const double r = rcp64(v[k]);
        Y[k] = X[k] * r;
        Z[k] = Y[k] * r;
    }
    // Four rows per pass over j: 12 independent FMA chains per thread and one load of X_j, Y_j, Z_j per
    // 12 FMAs; the last K % 4 rows in a pass of their own size (no FMAs on padding rows).
    double mu = 0.0;
    int k0 = 0;
    for (; k0 + 4 <= K; k0 += 4) mu = wilke_rows<4>(A2, AB, B2, K, k0, X, Y, Z, v, mu);
    if (K - k0 >= 2) {
        mu = wilke_rows<2>(A2, AB, B2, K, k0, X, Y, Z, v, mu);
        k0 += 2;
    }
    if (K - k0 == 1) mu = wilke_rows<1>(A2, AB, B2, K, k0, X, Y, Z, v, mu);
    io.out[1][o] = VT * mu;

    // Mixture-averaged diffusion (transport.rs:162-177); S reuses Y.
    double* S = Y;
    for (int k = 0; k < K; k++) S[k] = 0.0;
    // Two pairs per iteration: two independent polynomial + reciprocal chains.
    const double* P = diff;
    for (int k = 1; k < K; k++) {
        const double xk = X[k];
        double sa = 0.0, sb = 0.0;
        int j = 0;
        for (; j + 1 < k; j += 2, P += 10) {
            const double Ra = rcp64(poly(P)), Rb = rcp64(poly(P + 5));
            sa = fma(X[j], Ra, sa);
            sb = fma(X[j + 1], Rb, sb);
            S[j] = fma(xk, Ra, S[j]);
            S[j + 1] = fma(xk, Rb, S[j + 1]);
        }
        if (j < k) {
            const double R = rcp64(poly(P));
            sa = fma(X[j], R, sa);
            S[j] = fma(xk, R, S[j]);
            P += 5;
        }
        S[k] += sa + sb;
    }
    for (int k = 0; k < K; k++) io.out[2 + k][o] = diffusion_of(MVTN, VT, W[k], X[k], S[k]);
}

template <int KMAX, bool SMEM>
__global__ void __launch_bounds__(kTransportBlock) transport_kernel(const uint8_t* __restrict__ gtab, uint32_t tab_bytes,
                                                          const __grid_constant__ TransportArgs<KMAX> io,
                                                          size_t n, int* status) {
    __shared__ uint64_t bar;
    const uint8_t* tab = gtab;
    if (SMEM) {  // the whole blob, math tables first, into dynamic shared memory
        if (!stage_to_shared(cb_dsmem, gtab, tab_bytes, &bar, status)) return;
        tab = cb_dsmem;
    } else {  // tables read from global memory; only the math tables go to shared memory
        load_math(gtab);
    }
    if (io.count) n = min(n, (size_t)*io.count);  // gathered cells: the count is known on the device only
    for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
        const size_t i = io.index ? (size_t)(io.index[j] & kIndexMask) : j;
        transport_cell<KMAX>(tab, io, i, (io.flags & kCompactOut) ? j : i);
    }
}

// ---------------------------------------------------------------------------------------------------
// Warp-per-cell transport for small gathered launches (the surrogate gate's fallback and audit cells):
// the 32 lanes share one cell's species rows, so a few hundred cells still spread over every SM. Each
// sum is evaluated in the order transport_cell uses, which makes the two kernels' outputs identical bit
// for bit:
//  - per-species terms (polynomials, reciprocals) and the per-row viscosity sums run lane-parallel;
//  - the chains over species (sum n, mean molar mass, conductivity sums, viscosity) run on one lane each;
//  - the diffusion pair matrix goes by blocks of 32 rows: lane q walks the pairs of row 32b+q left to
//    right (its even/odd-column sums, as transport_cell's two chains) and leaves the reciprocals of
//    each 32-column chunk in a shared tile; lane c then adds that chunk's rows, in row order, to column
//    sum S[32t+c], which is first seeded with its row's own sum, exactly when transport_cell does.
constexpr int kWarpCellWarps = 8;  // cells (warps) per block
// Shared memory ahead of the warps' scratch: the staged blob or the math tables, rounded to 16 bytes.
__host__ __device__ __forceinline__ size_t warp_table_bytes(bool staged, uint32_t tab_bytes) {
    return ((staged ? (size_t)tab_bytes : (size_t)kMathBytes) + 15) & ~(size_t)15;
}
template <int KMAX>
constexpr int kWarpScratch = 4 * KMAX + 32 * 33;  // doubles per warp: X, v, Y, Z and a 32 x 33 tile

template <int KMAX>
__device__ void transport_cell_warp(const uint8_t* tab, const TransportArgs<KMAX>& io, size_t i, size_t o,
                                    double* sh) {
    static_assert(2 * KMAX <= 32 * 33, "the viscosity terms reuse the tile");
    const int lane = threadIdx.x & 31;
    const TransportHeader& H = *reinterpret_cast<const TransportHeader*>(tab + kMathBytes);
    const double* cond = reinterpret_cast<const double*>(tab + H.off_cond);
    const double* visc = reinterpret_cast<const double*>(tab + H.off_visc);
    const double* W = reinterpret_cast<const double*>(tab + H.off_W);
    const double* diff = reinterpret_cast<const double*>(tab + H.off_diff);
    const double* A2 = reinterpret_cast<const double*>(tab + H.off_A2);
    const double* AB = reinterpret_cast<const double*>(tab + H.off_AB);
    const double* B2 = reinterpret_cast<const double*>(tab + H.off_B2);
    const int K = H.K;
    double N, Tn;
    const double* const* amounts = transport_inputs(H, io, i, N, Tn);
    const double L1 = log64(Tn), L2 = L1 * L1, L3 = L2 * L1, L4 = L3 * L1;
    auto poly = [&](const double* P) { return fma(P[4], L4, fma(P[3], L3, fma(P[2], L2, fma(P[1], L1, P[0])))); };
    double* X = sh;
    double* v = sh + KMAX;
    double* Y = sh + 2 * KMAX;
    double* Z = sh + 3 * KMAX;
    double* T = sh + 4 * KMAX;

    for (int k = lane; k < K - 1; k += 32) X[k] = amounts[k][i];
    __syncwarp();
    if (lane == 0) {
        double s = 0.0;
        for (int k = 0; k < K - 1; k++) s += X[k];
        X[K - 1] = N - s;
    }
    __syncwarp();
    const double VT = sqrt(Tn);

    // Conductivity: species polynomials and reciprocals lane-parallel (in v, Y), then three chains on
    // lanes 0-2: the mean molar mass and the two mixing sums.
    for (int k = lane; k < K; k += 32) {
        const double c = poly(cond + 5 * k);
        v[k] = c;
        Y[k] = rcp64(c);
    }
    __syncwarp();
    double acc = 0.0;
    if (lane < 3) {
        const double* src = lane == 0 ? W : lane == 1 ? v : Y;
#pragma unroll 1
        for (int k = 0; k < K; k++) acc = fma(src[k], X[k], acc);
    }
    const double MN = __shfl_sync(0xffffffffu, acc, 0);
    const double Ac = __shfl_sync(0xffffffffu, acc, 1);
    const double Bc = __shfl_sync(0xffffffffu, acc, 2);
    __syncwarp();  // lanes 0-2 are done with v and Y
    if (lane == 0) io.out[0][o] = conductivity_of(Ac, Bc, N, VT);
    const double MVTN = MN * VT;

    // Viscosity: one row of the expanded Wilke sums per lane, each over j in order; the products and
    // reciprocals of the rows go to the tile, the sum over rows to lane 0.
    for (int k = lane; k < K; k += 32) {
        v[k] = poly(visc + 5 * k);
        const double r = rcp64(v[k]);
        Y[k] = X[k] * r;
        Z[k] = Y[k] * r;
    }
    __syncwarp();
#pragma unroll 1
    for (int k = lane; k < K; k += 32) {
        const double* a2 = A2 + (size_t)k * K;
        const double* ab = AB + (size_t)k * K;
        const double* b2 = B2 + (size_t)k * K;
        double s1 = 0.0, s2 = 0.0, s3 = 0.0;
#pragma unroll 4
        for (int j = 0; j < K; j++) {
            s1 = fma(a2[j], X[j], s1);
            s2 = fma(ab[j], Y[j], s2);
            s3 = fma(b2[j], Z[j], s3);
        }
        const double den = fma(v[k], fma(v[k], s3, s2), s1);
        T[2 * k] = X[k] * (v[k] * v[k]);
        T[2 * k + 1] = rcp64(den);
    }
    __syncwarp();
    if (lane == 0) {
        double mu = 0.0;
#pragma unroll 1
        for (int k = 0; k < K; k++) mu = fma(T[2 * k], T[2 * k + 1], mu);
        io.out[1][o] = VT * mu;
    }
    __syncwarp();

    // Mixture-averaged diffusion; S reuses Y.
    double* S = Y;
#pragma unroll 1
    for (int b = 0; 32 * b < K; b++) {
        const int r = 32 * b + lane;
        const double* P = diff + 5 * ((size_t)r * (size_t)(r > 0 ? r - 1 : 0) / 2);  // pair (r, 0)
        const int rows = min(32, K - 32 * b);
        double sa = 0.0, sb = 0.0;
#pragma unroll 1
        for (int t = 0; t <= b; t++) {
            const int j0 = 32 * t;
            const int j1 = r < K ? min(j0 + 32, r) : j0;
            int j = j0;
            double* Trow = T + 33 * lane;  // this row's reciprocals, column j at Trow[j - j0]
#pragma unroll 1
            for (; j + 1 < j1; j += 2) {  // j0 is even: sa takes the even columns, sb the odd ones
                const double Ra = rcp64(poly(P + 5 * j)), Rb = rcp64(poly(P + 5 * (j + 1)));
                sa = fma(X[j], Ra, sa);
                sb = fma(X[j + 1], Rb, sb);
                Trow[j - j0] = Ra;
                Trow[j + 1 - j0] = Rb;
            }
            if (j < j1) {
                const double R = rcp64(poly(P + 5 * j));
                sa = fma(X[j], R, sa);
                Trow[j - j0] = R;
            }
            if (t == b && r < K) S[r] = 0.0 + (sa + sb);
            __syncwarp();
            const int jc = j0 + lane;
            if (jc < K) {
                double s = S[jc];
#pragma unroll 1
                for (int q = t == b ? lane + 1 : 0; q < rows; q++) s = fma(X[32 * b + q], T[33 * q + lane], s);
                S[jc] = s;
            }
            __syncwarp();
        }
    }
    for (int k = lane; k < K; k += 32) io.out[2 + k][o] = diffusion_of(MVTN, VT, W[k], X[k], S[k]);
    __syncwarp();  // the scratch is reused by the warp's next cell
}

template <int KMAX, bool SMEM>
__global__ void __launch_bounds__(32 * kWarpCellWarps) transport_warp_kernel(const uint8_t* __restrict__ gtab,
                                                                           uint32_t tab_bytes,
                                                                           const __grid_constant__ TransportArgs<KMAX> io,
                                                                           size_t n, int* status) {
    __shared__ uint64_t bar;
    const uint8_t* tab = gtab;
    if (SMEM) {
        if (!stage_to_shared(cb_dsmem, gtab, tab_bytes, &bar, status)) return;
        tab = cb_dsmem;
    } else {
        load_math(gtab);
    }
    const size_t table_bytes = warp_table_bytes(SMEM, tab_bytes);
    double* sh = reinterpret_cast<double*>(cb_dsmem + table_bytes) + (size_t)(threadIdx.x >> 5) * kWarpScratch<KMAX>;
    if (io.count) n = min(n, (size_t)*io.count);
    const size_t warps = (size_t)gridDim.x * kWarpCellWarps;
    for (size_t j = (size_t)blockIdx.x * kWarpCellWarps + (threadIdx.x >> 5); j < n; j += warps) {
        const size_t i = io.index[j] & kIndexMask;
        transport_cell_warp<KMAX>(tab, io, i, (io.flags & kCompactOut) ? j : i, sh);
    }
}

// ---------------------------------------------------------------------------------------------------
namespace {
int sm_count() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

template <class Args>
bool gathered(const Args&) { return false; }
template <int KMAX>
bool gathered(const TransportArgs<KMAX>& io) { return io.index != nullptr; }

// Persistent grid: as many blocks as fit on the GPU at once (each stages the tables once), never more
// than the cells need. Tables go to shared memory when they fit, else they are read through L1/L2.
template <int BLOCK, class Args, class KS, class KG>
cudaError_t launch_table_kernel(KS ksmem, KG kglobal, const uint8_t* tab, uint32_t tab_bytes, const Args& io,
                                size_t n, cudaStream_t st, int* status) {
    const bool smem = (int)tab_bytes <= max_table_smem();
    // Gathered cells are few (a trust gate's fallback or audit): one warp per block spreads them over
    // every SM instead of filling a few blocks.
    const int block = gathered(io) ? 32 : BLOCK;
    int per_sm = 1;
    const size_t want = (n + block - 1) / block;
    cudaError_t e = table_kernel_occupancy(ksmem, kglobal, block, tab_bytes, kMathBytes, smem, &per_sm);
    if (e != cudaSuccess) return e;
    size_t grid = (size_t)sm_count() * per_sm;
    if (want < grid) grid = want ? want : 1;
    if (smem) ksmem<<<(unsigned)grid, block, tab_bytes, st>>>(tab, tab_bytes, io, n, status);
    else kglobal<<<(unsigned)grid, block, kMathBytes, st>>>(tab, tab_bytes, io, n, status);
    return cudaGetLastError();
}
template <int BLOCK, class KS, class KG>
size_t wave_of(KS ksmem, KG kglobal, uint32_t tab_bytes) {
    int per_sm = 1;
    if (table_kernel_occupancy(ksmem, kglobal, BLOCK, tab_bytes, kMathBytes, (int)tab_bytes <= max_table_smem(),
                               &per_sm) != cudaSuccess)
        return 0;
    return (size_t)sm_count() * per_sm * BLOCK;
}
}  // namespace

// Non-finite values by exponent bits (all ones): integer instructions only.
__global__ void count_nonfinite_kernel(const __grid_constant__ CountArgs args, size_t n, unsigned long long* count) {
    unsigned long long c = 0;
    for (int q = 0; q < args.m; q++)
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
            c += (__double2hiint(args.a[q][i]) & 0x7ff00000) == 0x7ff00000;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

cudaError_t launch_count_nonfinite(const CountArgs& args, size_t n, unsigned long long* count, cudaStream_t st) {
    if (n == 0 || args.m == 0) return cudaSuccess;
    size_t grid = (n + 255) / 256;
    if (grid > (size_t)sm_count() * 8) grid = (size_t)sm_count() * 8;
    count_nonfinite_kernel<<<(unsigned)grid, 256, 0, st>>>(args, n, count);
    return cudaGetLastError();
}

// The elementary functions of the plain path on device arrays (which: 0 exp, 1 log, 2 reciprocal), for
// accuracy checks against CUDA's own functions.
__global__ void math_check_kernel(const uint8_t* math, int which, const double* x, double* y, size_t n) {
    load_math(math);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double v = x[i];
        y[i] = which == 0 ? exp64(v) : which == 1 ? log64(v) : rcp64(v);
    }
}

cudaError_t launch_math_check(const uint8_t* math, int which, const double* x, double* y, size_t n,
                              cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    size_t grid = (n + 255) / 256;
    if (grid > 4096) grid = 4096;
    math_check_kernel<<<(unsigned)grid, 256, kMathBytes, st>>>(math, which, x, y, n);
    return cudaGetLastError();
}

// Test hook: polls of the first staging wait of this file's kernels (negative: the default limit).
cudaError_t set_stage_wait_polls(long long polls) {
    const long long v = polls < 0 ? kWaitLimit : polls;
    return cudaMemcpyToSymbol(g_stage_wait_polls, &v, sizeof v);
}

int max_table_smem() {
    static int v = -1;
    if (v < 0) {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        v = optin - 1024;  // room for the static shared variables
    }
    return v;
}

#define CB_DISPATCH(FN, KERNEL, ARGS, BLOCK)                                                               \
    cudaError_t FN(int kmax, const uint8_t* tab, uint32_t tab_bytes, const void* args, size_t n,            \
                   cudaStream_t st, int* status) {                                                         \
        switch (kmax) {                                                                                    \
        case 16: return launch_table_kernel<BLOCK>(KERNEL<16, true>, KERNEL<16, false>, tab, tab_bytes,    \
                                                   *static_cast<const ARGS<16>*>(args), n, st, status);    \
        case 64: return launch_table_kernel<BLOCK>(KERNEL<64, true>, KERNEL<64, false>, tab, tab_bytes,    \
                                                   *static_cast<const ARGS<64>*>(args), n, st, status);    \
        case 256: return launch_table_kernel<BLOCK>(KERNEL<256, true>, KERNEL<256, false>, tab, tab_bytes, \
                                                    *static_cast<const ARGS<256>*>(args), n, st, status);  \
        default: return cudaErrorInvalidValue;                                                             \
        }                                                                                                  \
    }
CB_DISPATCH(launch_rates, rates_kernel, RatesArgs, kBlock)
CB_DISPATCH(launch_reaction_rates, reaction_rates_kernel, ReactionRatesArgs, kBlock)
#undef CB_DISPATCH

#define CB_WAVE(FN, KERNEL, BLOCK)                                                     \
    size_t FN(int kmax, uint32_t tab_bytes) {                                          \
        switch (kmax) {                                                                \
        case 16: return wave_of<BLOCK>(KERNEL<16, true>, KERNEL<16, false>, tab_bytes);    \
        case 64: return wave_of<BLOCK>(KERNEL<64, true>, KERNEL<64, false>, tab_bytes);    \
        case 256: return wave_of<BLOCK>(KERNEL<256, true>, KERNEL<256, false>, tab_bytes); \
        default: return 0;                                                             \
        }                                                                              \
    }
CB_WAVE(wave_rates, rates_kernel, kBlock)
CB_WAVE(wave_reaction_rates, reaction_rates_kernel, kBlock)
CB_WAVE(wave_transport, transport_kernel, kTransportBlock)
#undef CB_WAVE

namespace {
// Gathered launches of up to this many cells per SM go warp-per-cell (above 16 species): one cell per
// thread would leave most SMs idle and the rest latency-bound; beyond it, one per thread keeps every
// lane busy without the warp form's serial chains.
constexpr size_t kWarpCellsPerSm = 128;

template <int KMAX>
cudaError_t launch_transport_k(const uint8_t* tab, uint32_t tab_bytes, const TransportArgs<KMAX>& io, size_t n,
                               cudaStream_t st, int* status) {
    if constexpr (KMAX >= 64) {
        if (io.index && n <= (size_t)sm_count() * kWarpCellsPerSm) {
            const size_t scratch = (size_t)kWarpCellWarps * kWarpScratch<KMAX> * sizeof(double);
            const bool smem = warp_table_bytes(true, tab_bytes) + scratch <= (size_t)max_table_smem();
            const size_t bytes = warp_table_bytes(smem, tab_bytes) + scratch;
            auto kern = smem ? transport_warp_kernel<KMAX, true> : transport_warp_kernel<KMAX, false>;
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
            if (e != cudaSuccess) return e;
            int per_sm = 1;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * kWarpCellWarps, bytes);
            if (per_sm < 1) per_sm = 1;
            size_t grid = (size_t)sm_count() * per_sm;
            const size_t want = (n + kWarpCellWarps - 1) / kWarpCellWarps;
            if (want < grid) grid = want ? want : 1;
            kern<<<(unsigned)grid, 32 * kWarpCellWarps, bytes, st>>>(tab, tab_bytes, io, n, status);
            return cudaGetLastError();
        }
    }
    return launch_table_kernel<kTransportBlock>(transport_kernel<KMAX, true>, transport_kernel<KMAX, false>, tab,
                                                tab_bytes, io, n, st, status);
}
}  // namespace

cudaError_t launch_transport(int kmax, const uint8_t* tab, uint32_t tab_bytes, const void* args, size_t n,
                             cudaStream_t st, int* status) {
    switch (kmax) {
    case 16: return launch_transport_k<16>(tab, tab_bytes, *static_cast<const TransportArgs<16>*>(args), n, st, status);
    case 64: return launch_transport_k<64>(tab, tab_bytes, *static_cast<const TransportArgs<64>*>(args), n, st, status);
    case 256:
        return launch_transport_k<256>(tab, tab_bytes, *static_cast<const TransportArgs<256>*>(args), n, st, status);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace cbg
