// Mixed-precision kernels: the same programs as kernels.cu (reaction.rs:207-391, transport.rs:141-210)
// with FP64 kept only where the reference's values cancel:
//   FP64  Gibbs polynomials and exponentials of the equilibrium constant, the forward-minus-reverse rate
//         of progress, the accumulation into species rates (and the energy dot products over them)
//   FP32  Arrhenius exponentials (argument and exponential; the result stored as a double so that it
//         keeps the full range), third-body sums, falloff blending, h/RT and cp/R polynomials, and all of
//         transport (polynomial fits, Wilke mixing, conductivity, mixture diffusion)
// Conversions between the two formats use integer instructions (device_math.cuh): the FP64 pipe is the
// bottleneck of the rates kernel and the FP32 pipe that of transport.
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "device_math.cuh"
#include "kernels.h"
#include "rates_mixed_core.cuh"
#include "tables_mixed.h"

namespace cbg {

// Per-cell working state of the mixed rates program.
template <int KMAX>
struct CellM {
    double C[KMAX];              // FP64 concentrations, bulk last
    double ex[KMAX], exn[KMAX];  // FP64 Gibbs exponentials
    float Mf[4 * KMAX];          // FP32 third-body concentrations, one per efficiency row
    double C0, rcpC0, rcpC0sq;
    float Ctotf, Tf, lnTf, rcpTf;
};

// Accumulation into the species rates (reaction.rs:312-327), one reaction model.
template <int KMAX, int MODEL>
__device__ __forceinline__ void accumulate_group_m(const RatesMixedTables& tb, const CellM<KMAX>& c, double* wdot) {
    for (int r = MODEL ? tb.H->group_end[MODEL - 1] : 0; r < tb.H->group_end[MODEL]; r++) {
        const ReactionF& x = tb.reactions[r];
        const double cR = reaction_rate_m<MODEL>(tb, x, c, MODEL >= 2 ? c.Mf[x.eff_row] : 0.f);
        // read-modify-writes in pairs, the two reads issued together (net species are distinct)
#pragma unroll 1
        for (int q = 0; q < x.n_net; q += 2) {
            const int k0 = x.net_k[q], k1 = x.net_k[q + 1 < x.n_net ? q + 1 : q];
            const double w0 = wdot[k0], w1 = wdot[k1];
            wdot[k0] = fma(small_int_to_double(x.net_n[q]), cR, w0);
            if (q + 1 < x.n_net) wdot[k1] = fma(small_int_to_double(x.net_n[q + 1]), cR, w1);
        }
    }
}

template <int KMAX>
__device__ void rates_mixed_cell(const RatesMixedTables& tb, const RatesArgs<KMAX>& io, size_t i) {
    const RatesMixedHeader& H = *tb.H;
    const int K = H.K, A = H.A;
    const bool uniform = io.flags & kUniformPressure;
    const double pressure_R = uniform ? io.in[0][0] : io.in[0][i];
    const double rcp_pressure_R = uniform ? io.in[1][0] : io.in[1][i];
    const double T = io.in[2][i], V = io.in[3][i];
    CellM<KMAX> c;
    // FP64 prologue (reaction.rs:362-373): temperatures for the Gibbs polynomials, concentrations for
    // the rates of progress.
    const double md = rcp64(V), rcpT = rcp64(T), lnT = log64(T);
    const double T2 = T * T, T3 = T * T2, T4 = T2 * T2;
    double sum = 0.0;
    for (int k = 0; k < K - 1; k++) {
        c.C[k] = md * max0(io.in[4 + k][i]);
        sum += c.C[k];
    }
    const double Ctot = pressure_R * rcpT;
    c.C[K - 1] = Ctot - sum;
    c.Ctotf = dbl_to_flt(Ctot);
    c.Tf = dbl_to_flt(T);
    c.lnTf = dbl_to_flt(lnT);
    c.rcpTf = dbl_to_flt(rcpT);
    c.C0 = H.C0 * rcpT;
    c.rcpC0 = H.rcp_C0 * T;
    c.rcpC0sq = c.rcpC0 * c.rcpC0;

    // FP64 Gibbs exponentials (reaction.rs:234-263).
    for (int k = 0; k < A; k++) {
        const SpeciesF& s = tb.species[k];
        if (!(s.need_exp | s.need_exp_neg)) continue;
        const double* g = s.g[piece_of_m(s.split, T)];
        const double x = fma(g[6], rcpT, fma(g[5], T4, fma(g[4], T3, fma(g[3], T2, fma(g[2], T, fma(g[1], lnT, g[0]))))));
        gibbs_exps(x, s.need_exp, s.need_exp_neg, H.M3, H.cbrt_max, c.C0, c.rcpC0, c.ex[k], c.exn[k]);
    }
    // FP32 third-body sums, four rows per pass (rows in reaction-group order, padded to a multiple of 4).
    for (int e0 = 0; e0 < H.n_eff; e0 += 4) {
        const float* E = tb.eff + (size_t)e0 * K;
        float s[4] = {0.f, 0.f, 0.f, 0.f};
        for (int k = 0; k < K; k++) {
            const float ck = dbl_to_flt(c.C[k]);  // integer ops, recomputed per pass (no FP32 copy kept)
#pragma unroll
            for (int q = 0; q < 4; q++) s[q] = fmaf(E[q * K + k], ck, s[q]);
        }
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (e0 + q < H.n_eff) c.Mf[e0 + q] = c.Ctotf + s[q];
    }

    double wdot[KMAX];
    for (int k = 0; k < A; k++) wdot[k] = 0.0;
    accumulate_group_m<KMAX, 0>(tb, c, wdot);
    accumulate_group_m<KMAX, 1>(tb, c, wdot);
    accumulate_group_m<KMAX, 2>(tb, c, wdot);
    accumulate_group_m<KMAX, 3>(tb, c, wdot);
    accumulate_group_m<KMAX, 4>(tb, c, wdot);
    accumulate_group_m<KMAX, 5>(tb, c, wdot);
    // Energy (reaction.rs:375-384): FP32 polynomials, FP64 sums over the FP64 species rates.
    const float Tf = c.Tf, rcpTf = c.rcpTf;
    double E = 0.0, Cp = 0.0, dtE = 0.0;
    for (int k = 0; k < K; k++) {
        const SpeciesF& s = tb.species[k];
        const int p = piece_of_m(s.split, T);
        const float* cp = s.cp[p];
        const float ck = fmaf(cp[4], Tf, cp[3]);
        const float cpk = fmaf(fmaf(fmaf(ck, Tf, cp[2]), Tf, cp[1]), Tf, cp[0]);
        Cp = fma(flt_to_dbl(cpk), c.C[k], Cp);
        if (k < A) {
            const float* h = s.h[p];
            const float hk = fmaf(h[5], rcpTf, fmaf(fmaf(fmaf(fmaf(h[4], Tf, h[3]), Tf, h[2]), Tf, h[1]), Tf, h[0]));
            E = fma(wdot[k], flt_to_dbl(hk), E);
            dtE = fma(s.dtE, wdot[k], dtE);
        }
    }
    const double dtT_T = -E * rcp64(Cp);
    io.out[0][i] = T * dtT_T;
    io.out[1][i] = V * fma(rcp_pressure_R * T, dtE, dtT_T);
    for (int k = 0; k < A; k++) io.out[2 + k][i] = wdot[k];
}

template <int KMAX, bool SMEM>
__global__ void __launch_bounds__(kBlock, 2) rates_mixed_kernel(const uint8_t* __restrict__ gtab, uint32_t tab_bytes,
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
    const RatesMixedTables tb(tab);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        rates_mixed_cell<KMAX>(tb, io, i);
}

// ---------------------------------------------------------------------------------------------------
// i: the cell's index in the inputs, o: in the outputs (they differ for gathered cells).
template <int KMAX>
__device__ void transport_mixed_cell(const uint8_t* tab, const TransportArgs<KMAX>& io, size_t i, size_t o) {
    const TransportMixedHeader& H = *reinterpret_cast<const TransportMixedHeader*>(tab + kMathBytes);
    const float* cond = reinterpret_cast<const float*>(tab + H.off_cond);
    const float* visc = reinterpret_cast<const float*>(tab + H.off_visc);
    const float* W = reinterpret_cast<const float*>(tab + H.off_W);
    const float4* diff = reinterpret_cast<const float4*>(tab + H.off_diff);   // two per species pair
    const float4* wil = reinterpret_cast<const float4*>(tab + H.off_wilke);   // {a^2, 2ab, b^2, 0}
    const int K = H.K;
    float N, Tn;
    const double* const* amounts;
    if (io.flags & kFromRates) {
        const double pressure_R = (io.flags & kUniformPressure) ? io.in[0][0] : io.in[0][i];
        const float T = dbl_to_flt(io.in[2][i]);
        N = __fdividef(dbl_to_flt(pressure_R) * dbl_to_flt(io.in[3][i]), T);
        Tn = T / (float)H.T0;
        amounts = io.in + 4;
    } else {
        N = dbl_to_flt(io.in[0][i]);
        Tn = dbl_to_flt(io.in[1][i]);
        amounts = io.in + 2;
    }
    const float L1 = logf(Tn), L2 = L1 * L1, L3 = L2 * L1, L4 = L3 * L1;
    auto poly = [&](const float* P) { return fmaf(P[4], L4, fmaf(P[3], L3, fmaf(P[2], L2, fmaf(P[1], L1, P[0])))); };

    float X[KMAX], v[KMAX], Y[KMAX], Z[KMAX];
    // sum of the non-bulk amounts with an error term (Kahan): the bulk amount is a difference
    float s = 0.f, comp = 0.f;
    for (int k = 0; k < K - 1; k++) {
        X[k] = dbl_to_flt(amounts[k][i]);
        const float y = X[k] - comp, t = s + y;
        comp = (t - s) - y;
        s = t;
    }
    X[K - 1] = (N - s) + comp;
    const float VT = sqrtf(Tn);
    float MN = 0.f;
    for (int k = 0; k < K; k++) MN = fmaf(W[k], X[k], MN);
    const float MVTN = MN * VT;

    float Ac = 0.f, Bc = 0.f;
    for (int k = 0; k < K; k++) {
        const float c = poly(cond + 5 * k);
        Ac = fmaf(X[k], c, Ac);
        Bc = fmaf(X[k], rcp_f32(c), Bc);
    }
    io.out[0][o] = flt_to_dbl((__fdividef(Ac, N) + __fdividef(N, Bc)) * VT);

    for (int k = 0; k < K; k++) {
        v[k] = poly(visc + 5 * k);
        const float r = rcp_f32(v[k]);
        Y[k] = X[k] * r;
        Z[k] = Y[k] * r;
    }
    float mu = 0.f;
    for (int k0 = 0; k0 < K; k0 += 4) {
        const float4* w = wil + (size_t)k0 * K;
        float s1[4] = {0.f, 0.f, 0.f, 0.f}, s2[4] = {0.f, 0.f, 0.f, 0.f}, s3[4] = {0.f, 0.f, 0.f, 0.f};
        for (int j = 0; j < K; j++) {
            const float xj = X[j], yj = Y[j], zj = Z[j];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float4 c = w[q * K + j];
                s1[q] = fmaf(c.x, xj, s1[q]);
                s2[q] = fmaf(c.y, yj, s2[q]);
                s3[q] = fmaf(c.z, zj, s3[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int k = k0 + q;
            if (k < K) mu = fmaf(X[k] * (v[k] * v[k]), rcp_f32(fmaf(v[k], fmaf(v[k], s3[q], s2[q]), s1[q])), mu);
        }
    }
    io.out[1][o] = flt_to_dbl(VT * mu);

    float* S = Y;
    for (int k = 0; k < K; k++) S[k] = 0.f;
    // a pair's fit: float4 {P0, P1, P2, P3} then {P4, 0, 0, 0}
    auto poly4 = [&](const float4* Q) {
        const float4 a = Q[0];
        const float p4 = Q[1].x;
        return fmaf(p4, L4, fmaf(a.w, L3, fmaf(a.z, L2, fmaf(a.y, L1, a.x))));
    };
    const float4* P = diff;
    for (int k = 1; k < K; k++) {
        const float xk = X[k];
        float sa = 0.f, sb = 0.f;
        int j = 0;
        for (; j + 1 < k; j += 2, P += 4) {
            const float Ra = rcp_f32(poly4(P)), Rb = rcp_f32(poly4(P + 2));
            sa = fmaf(X[j], Ra, sa);
            sb = fmaf(X[j + 1], Rb, sb);
            S[j] = fmaf(xk, Ra, S[j]);
            S[j + 1] = fmaf(xk, Rb, S[j + 1]);
        }
        if (j < k) {
            const float R = rcp_f32(poly4(P));
            sa = fmaf(X[j], R, sa);
            S[j] = fmaf(xk, R, S[j]);
            P += 2;
        }
        S[k] += sa + sb;
    }
    for (int k = 0; k < K; k++) io.out[2 + k][o] = flt_to_dbl(__fdividef(fmaf(-(VT * W[k]), X[k], MVTN), S[k]));
}

template <int KMAX, bool SMEM>
__global__ void __launch_bounds__(kTransportMixedBlock) transport_mixed_kernel(const uint8_t* __restrict__ gtab,
                                                                         uint32_t tab_bytes,
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
        transport_mixed_cell<KMAX>(tab, io, i, (io.flags & kCompactOut) ? j : i);
    }
}

// ---------------------------------------------------------------------------------------------------
namespace {
int sm_count_m() {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

template <int BLOCK, class KS, class KG>
size_t wave_of_m(KS ksmem, KG kglobal, uint32_t tab_bytes) {
    int per_sm = 1;
    if (table_kernel_occupancy(ksmem, kglobal, BLOCK, tab_bytes, kMathBytes, (int)tab_bytes <= max_table_smem(),
                               &per_sm) != cudaSuccess)
        return 0;
    return (size_t)sm_count_m() * per_sm * BLOCK;
}

template <class Args>
bool gathered_m(const Args&) { return false; }
template <int KMAX>
bool gathered_m(const TransportArgs<KMAX>& io) { return io.index != nullptr; }

template <int BLOCK, class Args, class KS, class KG>
cudaError_t launch_mixed(KS ksmem, KG kglobal, const uint8_t* tab, uint32_t tab_bytes, const Args& io, size_t n,
                         cudaStream_t st, int* status) {
    const bool smem = (int)tab_bytes <= max_table_smem();
    // A gathered launch of fewer cells than one wave of full blocks (a trust gate's fallback) spreads
    // them over every SM in one-warp blocks.
    int block = BLOCK, per_sm = 1;
    cudaError_t e = table_kernel_occupancy(ksmem, kglobal, BLOCK, tab_bytes, kMathBytes, smem, &per_sm);
    if (e != cudaSuccess) return e;
    if (gathered_m(io) && n < (size_t)sm_count_m() * per_sm * BLOCK) {
        block = 32;
        e = table_kernel_occupancy(ksmem, kglobal, block, tab_bytes, kMathBytes, smem, &per_sm);
        if (e != cudaSuccess) return e;
    }
    const size_t want = (n + block - 1) / block;
    size_t grid = (size_t)sm_count_m() * per_sm;
    if (want < grid) grid = want ? want : 1;
    if (smem) ksmem<<<(unsigned)grid, block, tab_bytes, st>>>(tab, tab_bytes, io, n, status);
    else kglobal<<<(unsigned)grid, block, kMathBytes, st>>>(tab, tab_bytes, io, n, status);
    return cudaGetLastError();
}
}  // namespace

#define CB_DISPATCH_M(FN, KERNEL, ARGS, BLOCK)                                                             \
    cudaError_t FN(int kmax, const uint8_t* tab, uint32_t tab_bytes, const void* args, size_t n,            \
                   cudaStream_t st, int* status) {                                                         \
        switch (kmax) {                                                                                    \
        case 16: return launch_mixed<BLOCK>(KERNEL<16, true>, KERNEL<16, false>, tab, tab_bytes,           \
                                            *static_cast<const ARGS<16>*>(args), n, st, status);           \
        case 64: return launch_mixed<BLOCK>(KERNEL<64, true>, KERNEL<64, false>, tab, tab_bytes,           \
                                            *static_cast<const ARGS<64>*>(args), n, st, status);           \
        case 256: return launch_mixed<BLOCK>(KERNEL<256, true>, KERNEL<256, false>, tab, tab_bytes,        \
                                             *static_cast<const ARGS<256>*>(args), n, st, status);         \
        default: return cudaErrorInvalidValue;                                                             \
        }                                                                                                  \
    }
CB_DISPATCH_M(launch_rates_mixed, rates_mixed_kernel, RatesArgs, kBlock)
CB_DISPATCH_M(launch_transport_mixed, transport_mixed_kernel, TransportArgs, kTransportMixedBlock)
#undef CB_DISPATCH_M

#define CB_WAVE_M(FN, KERNEL, BLOCK)                                                        \
    size_t FN(int kmax, uint32_t tab_bytes) {                                               \
        switch (kmax) {                                                                     \
        case 16: return wave_of_m<BLOCK>(KERNEL<16, true>, KERNEL<16, false>, tab_bytes);    \
        case 64: return wave_of_m<BLOCK>(KERNEL<64, true>, KERNEL<64, false>, tab_bytes);    \
        case 256: return wave_of_m<BLOCK>(KERNEL<256, true>, KERNEL<256, false>, tab_bytes); \
        default: return 0;                                                                  \
        }                                                                                   \
    }
CB_WAVE_M(wave_rates_mixed, rates_mixed_kernel, kBlock)
CB_WAVE_M(wave_transport_mixed, transport_mixed_kernel, kTransportMixedBlock)
#undef CB_WAVE_M

}  // namespace cbg
