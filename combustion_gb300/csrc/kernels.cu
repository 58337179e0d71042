// Plain FP64 kernels: species production rates (reaction.rs:207-391) and mixture-averaged transport
// (transport.rs:141-210), one cell per thread.
//
// Every thread of a warp walks the same reaction / species / pair at the same time, so each table read
// is a broadcast; the per-cell working arrays (concentrations, Gibbs exponentials, accumulators) live in
// thread-local memory. The FP64 pipe is the bottleneck; nothing else here comes close to its limits.
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "fp64_math.cuh"
#include "kernels.h"
#include "tables.h"

namespace cbg {

constexpr double kF32Max = 3.4028234663852886e+38;       // f32::MAX as f64
constexpr double kF32MinPos = 1.1754943508222875e-38;    // f32::MIN_POSITIVE as f64

struct Temps {
    double lnT, T, T2, T3, T4, rcpT, rcpT2;
};

__device__ __forceinline__ double factor_of(int f, const Temps& t) {
    switch (f) {
    case kRcpT2: return t.rcpT2;
    case kRcpT: return t.rcpT;
    case kT4: return t.T4;
    case kT3: return t.T3;
    case kT2: return t.T2;
    case kT: return t.T;
    default: return 1.0;
    }
}

// arrhenius() of reaction.rs:113-139; the has_x and factor branches are uniform across the warp.
__device__ __forceinline__ double arrhenius(const Arrhenius& a, const Temps& t) {
    double k;
    if (a.has_x) {
        double x = fma(a.beta, t.lnT, fma(a.mEa, t.rcpT, a.lnA));
        k = exp64(x);
        if (a.factor != kNone) k = factor_of(a.factor, t) * k;
    } else {
        k = a.factor != kNone ? factor_of(a.factor, t) * a.A : a.A;
    }
    return min_pos(kF32Max, k);
}

// Piece 0 for T <= split (lib.rs:15); NaN splits (one piece) select piece 0 as well.
__device__ __forceinline__ int piece_of(double split, double T) { return bits(T) <= bits(split) ? 0 : 1; }

template <int KMAX>
__device__ void rates_cell(const uint8_t* tab, const RatesArgs<KMAX>& io, size_t i) {
    const RatesHeader& H = *reinterpret_cast<const RatesHeader*>(tab);
    const Species* species = reinterpret_cast<const Species*>(tab + H.off_species);
    const Reaction* reactions = reinterpret_cast<const Reaction*>(tab + H.off_reactions);
    const Falloff* falloff = reinterpret_cast<const Falloff*>(tab + H.off_falloff);
    const double* eff = reinterpret_cast<const double*>(tab + H.off_eff);
    const int K = H.K, A = H.A;
    const bool uniform = io.flags & 2u;
    const double pressure_R = uniform ? io.in[0][0] : io.in[0][i];
    const double rcp_pressure_R = uniform ? io.in[1][0] : io.in[1][i];
    const double T = io.in[2][i], V = io.in[3][i];

    // Prologue (reaction.rs:362-373).
    double C[KMAX];
    Temps t;
    const double md = rcp64(V);
    t.T = T;
    t.rcpT = rcp64(T);
    t.lnT = log64(T);
    t.T2 = T * T;
    t.T3 = T * t.T2;
    t.T4 = t.T2 * t.T2;
    t.rcpT2 = t.rcpT * t.rcpT;
    double sum = 0.0;
    for (int k = 0; k < K - 1; k++) {
        C[k] = md * max0(io.in[4 + k][i]);
        sum += C[k];
    }
    const double Ctot = pressure_R * t.rcpT;
    C[K - 1] = Ctot - sum;

    // Gibbs exponentials of the active species (reaction.rs:234-263).
    double ex[KMAX], exn[KMAX];
    for (int k = 0; k < A; k++) {
        const Species& s = species[k];
        if (!(s.need_exp | s.need_exp_neg)) continue;
        const double* g = s.g[piece_of(s.split, T)];
        double x = fma(g[6], t.rcpT, fma(g[5], t.T4, fma(g[4], t.T3, fma(g[3], t.T2, fma(g[2], T, fma(g[1], t.lnT, g[0]))))));
        if (s.need_exp) ex[k] = min_pos(H.M3, exp64(x));
        if (s.need_exp_neg) exn[k] = min_pos(H.cbrt_max, exp64(-x));
    }

    double wdot[KMAX];
    for (int k = 0; k < A; k++) wdot[k] = 0.0;
    const double C0 = H.C0 * t.rcpT, rcpC0 = H.rcp_C0 * T;

    for (int r = 0; r < H.R; r++) {
        const Reaction& x = reactions[r];
        double M = Ctot;
        if (x.eff_row >= 0) {  // efficiency() (reaction.rs:141-145)
            const double* e = eff + (size_t)x.eff_row * K;
            double s = 0.0;
            for (int k = 0; k < K; k++) s = fma(e[k], C[k], s);
            M = Ctot + s;
        }
        double num, den = 1.0;
        bool ratio = false;
        if (x.model == 4) {  // Troe (reaction.rs:160-193)
            const Falloff& f = falloff[x.falloff];
            const double k0 = arrhenius(f.k0, t);
            double Pr, kinf;
            if (f.flags & kKinfConst) {
                Pr = M * k0;
                kinf = f.ainf;
            } else {
                const double ki = arrhenius(x.k, t);
                Pr = div64(M * k0, ki + kF32MinPos);
                kinf = f.ainf * ki;
            }
            double lnF;
            if (f.flags & kFcentConst) lnF = f.ln_fcent;
            else {
                double F = 0.0;
                if (f.flags & kTermT3) F = f.c1mA * exp64(T * f.c3);
                if (f.flags & kTermT1) F += f.cA * exp64(T * f.c1);
                if (f.flags & kTermAConst) F += f.cA;
                if (f.flags & kTermT2) F += exp64(f.cmT2 * t.rcpT);
                lnF = log64(F);
            }
            const double Cc = fma(-0.67, lnF, -H.ln10_04);
            const double Nn = fma(-1.27, lnF, H.ln10_075);
            const double lnPrC = log64(Pr + kF32MinPos) + Cc;
            const double f1 = div64(lnPrC, fma(-0.14, lnPrC, Nn));
            const double Fb = exp64(div64(lnF, fma(f1, f1, 1.0)));
            num = (Fb * kinf) * Pr;
            den = Pr + 1.0;
            ratio = true;
        } else if (x.model == 3) {  // Lindemann (reaction.rs:153-159)
            const Falloff& f = falloff[x.falloff];
            const double Ck0 = M * arrhenius(f.k0, t);
            const double ki = arrhenius(x.k, t);
            num = Ck0 * ki;
            den = (Ck0 + ki) + kF32MinPos;
            ratio = true;
        } else {
            num = arrhenius(x.k, t);
            if (x.model == 2) num *= M;  // three-body (reaction.rs:152)
        }
        // Rate of progress (reaction.rs:269-306).
        double Rf = 1.0;
        for (int q = 0; q < x.n_r; q++)
            for (int n = 0; n < x.r_n[q]; n++) Rf *= C[x.r_k[q]];
        double Rnet = Rf;
        if (x.model != 1) {
            double p = 1.0;
            for (int q = 0; q < x.n_net; q++) {
                const int nu = x.net_n[q], k = x.net_k[q];
                const double tt = nu > 0 ? ex[k] : exn[k];
                for (int n = 0; n < (nu > 0 ? nu : -nu); n++) p *= tt;
            }
            switch (x.minus_sigma_net) {
            case 1: p = C0 * p; break;
            case -1: p = rcpC0 * p; break;
            case -2: p = (rcpC0 * rcpC0) * p; break;
            default: break;
            }
            double Rr = 1.0;
            for (int q = 0; q < x.n_p; q++)
                for (int n = 0; n < x.p_n[q]; n++) Rr *= C[x.p_k[q]];
            Rnet = Rf - p * Rr;
        }
        const double cR = ratio ? div64(Rnet * num, den) : Rnet * num;
        for (int q = 0; q < x.n_net; q++) wdot[x.net_k[q]] = fma((double)x.net_n[q], cR, wdot[x.net_k[q]]);
    }

    // Energy and volume (reaction.rs:375-384).
    double E = 0.0;
    for (int k = 0; k < A; k++) {
        const Species& s = species[k];
        const double* h = s.h[piece_of(s.split, T)];
        const double hk = fma(h[5], t.rcpT, fma(h[4], t.T4, fma(h[3], t.T3, fma(h[2], t.T2, fma(h[1], T, h[0])))));
        E = fma(wdot[k], hk, E);
    }
    double Cp = 0.0;
    for (int k = 0; k < K; k++) {
        const Species& s = species[k];
        const double* c = s.cp[piece_of(s.split, T)];
        const double ck = fma(c[4], t.T4, fma(c[3], t.T3, fma(c[2], t.T2, fma(c[1], T, c[0]))));
        Cp = fma(ck, C[k], Cp);
    }
    const double dtT_T = div64(-E, Cp);
    double dtE = 0.0;
    for (int k = 0; k < A; k++) dtE = fma(species[k].dtE, wdot[k], dtE);
    io.out[0][i] = T * dtT_T;
    io.out[1][i] = V * fma(rcp_pressure_R * T, dtE, dtT_T);
    for (int k = 0; k < A; k++) io.out[2 + k][i] = wdot[k];
}

template <int KMAX, bool SMEM>
__global__ void __launch_bounds__(kBlock) rates_kernel(const uint8_t* __restrict__ gtab, uint32_t tab_bytes,
                                                      const __grid_constant__ RatesArgs<KMAX> io, size_t n,
                                                      int* status) {
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ uint64_t bar;
    const uint8_t* tab = gtab;
    if (SMEM) {
        if (!stage_to_shared(smem, gtab, tab_bytes, &bar, status)) return;
        tab = smem;
    }
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        rates_cell<KMAX>(tab, io, i);
}

// ---------------------------------------------------------------------------------------------------
template <int KMAX>
__device__ void transport_cell(const uint8_t* tab, const TransportArgs<KMAX>& io, size_t i) {
    const TransportHeader& H = *reinterpret_cast<const TransportHeader*>(tab);
    const double* cond = reinterpret_cast<const double*>(tab + H.off_cond);
    const double* visc = reinterpret_cast<const double*>(tab + H.off_visc);
    const double* W = reinterpret_cast<const double*>(tab + H.off_W);
    const double* diff = reinterpret_cast<const double*>(tab + H.off_diff);
    const double* A2 = reinterpret_cast<const double*>(tab + H.off_A2);
    const double* AB = reinterpret_cast<const double*>(tab + H.off_AB);
    const double* B2 = reinterpret_cast<const double*>(tab + H.off_B2);
    const int K = H.K;
    const double N = io.in[0][i], Tn = io.in[1][i];
    const double L1 = log64(Tn), L2 = L1 * L1, L3 = L2 * L1, L4 = L3 * L1;
    auto poly = [&](const double* P) { return fma(P[4], L4, fma(P[3], L3, fma(P[2], L2, fma(P[1], L1, P[0])))); };

    double X[KMAX], v[KMAX], Y[KMAX], Z[KMAX];
    double s = 0.0;
    for (int k = 0; k < K - 1; k++) {
        X[k] = io.in[2 + k][i];
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
    io.out[0][i] = (div64(Ac, N) + div64(N, Bc)) * VT;

    // Viscosity, Wilke mixing (transport.rs:148-158) with the square expanded:
    // sum_j X_j (a + b v_k/v_j)^2 = sum_j a^2 X_j + v_k sum_j 2ab X_j/v_j + v_k^2 sum_j b^2 X_j/v_j^2.
    for (int k = 0; k < K; k++) {
        v[k] = poly(visc + 5 * k);
        const double r = rcp64(v[k]);
        Y[k] = X[k] * r;
        Z[k] = Y[k] * r;
    }
    double mu = 0.0;
    for (int k = 0; k < K; k++) {
        const double* a2 = A2 + (size_t)k * K;
        const double* ab = AB + (size_t)k * K;
        const double* b2 = B2 + (size_t)k * K;
        double s1 = 0.0, s2 = 0.0, s3 = 0.0;
        for (int j = 0; j < K; j++) {
            s1 = fma(a2[j], X[j], s1);
            s2 = fma(ab[j], Y[j], s2);
            s3 = fma(b2[j], Z[j], s3);
        }
        const double den = fma(v[k], fma(v[k], s3, s2), s1);
        mu = fma(X[k] * (v[k] * v[k]), rcp64(den), mu);
    }
    io.out[1][i] = VT * mu;

    // Mixture-averaged diffusion (transport.rs:162-177); S reuses Y.
    double* S = Y;
    for (int k = 0; k < K; k++) S[k] = 0.0;
    const double* P = diff;
    for (int k = 1; k < K; k++) {
        const double xk = X[k];
        double sk = 0.0;
        for (int j = 0; j < k; j++, P += 5) {
            const double R = rcp64(poly(P));
            sk = fma(X[j], R, sk);
            S[j] = fma(xk, R, S[j]);
        }
        S[k] += sk;
    }
    for (int k = 0; k < K; k++) io.out[2 + k][i] = div64(MVTN - (VT * W[k]) * X[k], S[k]);
}

template <int KMAX, bool SMEM>
__global__ void __launch_bounds__(kBlock) transport_kernel(const uint8_t* __restrict__ gtab, uint32_t tab_bytes,
                                                          const __grid_constant__ TransportArgs<KMAX> io,
                                                          size_t n, int* status) {
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ uint64_t bar;
    const uint8_t* tab = gtab;
    if (SMEM) {
        if (!stage_to_shared(smem, gtab, tab_bytes, &bar, status)) return;
        tab = smem;
    }
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        transport_cell<KMAX>(tab, io, i);
}

// ---------------------------------------------------------------------------------------------------
namespace {
int g_sms = 0;
int sm_count() {
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 1;
    }
    return g_sms;
}

template <int KMAX>
cudaError_t launch_rates_k(const uint8_t* tab, uint32_t tab_bytes, const RatesArgs<KMAX>& io, size_t n,
                           cudaStream_t st, int* status, int max_smem) {
    const bool smem = (int)tab_bytes <= max_smem;
    int blocks_per_sm = 1;
    if (smem) {
        auto k = rates_kernel<KMAX, true>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tab_bytes);
        if (e != cudaSuccess) return e;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k, kBlock, tab_bytes);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
        size_t want = (n + kBlock - 1) / kBlock, grid = (size_t)sm_count() * blocks_per_sm;
        if (want < grid) grid = want ? want : 1;
        k<<<(unsigned)grid, kBlock, tab_bytes, st>>>(tab, tab_bytes, io, n, status);
    } else {
        auto k = rates_kernel<KMAX, false>;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k, kBlock, 0);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
        size_t want = (n + kBlock - 1) / kBlock, grid = (size_t)sm_count() * blocks_per_sm;
        if (want < grid) grid = want ? want : 1;
        k<<<(unsigned)grid, kBlock, 0, st>>>(tab, tab_bytes, io, n, status);
    }
    return cudaGetLastError();
}

template <int KMAX>
cudaError_t launch_transport_k(const uint8_t* tab, uint32_t tab_bytes, const TransportArgs<KMAX>& io, size_t n,
                               cudaStream_t st, int* status, int max_smem) {
    const bool smem = (int)tab_bytes <= max_smem;
    int blocks_per_sm = 1;
    if (smem) {
        auto k = transport_kernel<KMAX, true>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tab_bytes);
        if (e != cudaSuccess) return e;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k, kBlock, tab_bytes);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
        size_t want = (n + kBlock - 1) / kBlock, grid = (size_t)sm_count() * blocks_per_sm;
        if (want < grid) grid = want ? want : 1;
        k<<<(unsigned)grid, kBlock, tab_bytes, st>>>(tab, tab_bytes, io, n, status);
    } else {
        auto k = transport_kernel<KMAX, false>;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k, kBlock, 0);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
        size_t want = (n + kBlock - 1) / kBlock, grid = (size_t)sm_count() * blocks_per_sm;
        if (want < grid) grid = want ? want : 1;
        k<<<(unsigned)grid, kBlock, 0, st>>>(tab, tab_bytes, io, n, status);
    }
    return cudaGetLastError();
}
}  // namespace

int max_table_smem() {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return optin - 1024;  // leave room for the static shared variables
}

cudaError_t launch_rates(int kmax, const uint8_t* tab, uint32_t tab_bytes, const void* args, size_t n,
                         cudaStream_t st, int* status) {
    const int ms = max_table_smem();
    switch (kmax) {
    case 16: return launch_rates_k<16>(tab, tab_bytes, *static_cast<const RatesArgs<16>*>(args), n, st, status, ms);
    case 64: return launch_rates_k<64>(tab, tab_bytes, *static_cast<const RatesArgs<64>*>(args), n, st, status, ms);
    case 256: return launch_rates_k<256>(tab, tab_bytes, *static_cast<const RatesArgs<256>*>(args), n, st, status, ms);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_transport(int kmax, const uint8_t* tab, uint32_t tab_bytes, const void* args, size_t n,
                             cudaStream_t st, int* status) {
    const int ms = max_table_smem();
    switch (kmax) {
    case 16: return launch_transport_k<16>(tab, tab_bytes, *static_cast<const TransportArgs<16>*>(args), n, st, status, ms);
    case 64: return launch_transport_k<64>(tab, tab_bytes, *static_cast<const TransportArgs<64>*>(args), n, st, status, ms);
    case 256: return launch_transport_k<256>(tab, tab_bytes, *static_cast<const TransportArgs<256>*>(args), n, st, status, ms);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace cbg
