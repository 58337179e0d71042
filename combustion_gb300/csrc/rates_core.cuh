// Rates program pieces shared by the one-cell-per-thread kernels (kernels.cu) and the warp-per-reactor
// integrator (bdf.cu): temperature powers, Arrhenius rate constants, table views, concentration
// products and the evaluation of one reaction (reaction.rs:113-309). A "cell" type provides C[]
// (concentrations, bulk last), ex[] / exn[] (clamped Gibbs exponentials), t (Temps) and the scalars C0,
// rcpC0, rcpC0sq; arrays in thread-local memory and pointers into shared memory both fit. The third-body
// concentration of a reaction that has one comes as an argument (the caller keeps it where it suits).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "device_common.cuh"
#include "device_math.cuh"
#include "tables.h"

namespace cbg {

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
        k = exp64(x);  // beta includes the power of T (tables.h)
    } else {
        k = a.factor != kNone ? factor_of(a.factor, t) * a.A : a.A;
    }
    return min_pos(kF32Max, k);
}

// Piece 0 for T <= split (lib.rs:15); NaN splits (one piece) select piece 0 as well.
__device__ __forceinline__ int piece_of(double split, double T) { return bits(T) <= bits(split) ? 0 : 1; }

struct RatesTables {
    const RatesHeader* H;
    const Species* species;
    const Reaction* reactions;
    const Falloff* falloff;
    const double* eff;
    __device__ explicit RatesTables(const uint8_t* tab)
        : H(reinterpret_cast<const RatesHeader*>(tab + kMathBytes)),
          species(reinterpret_cast<const Species*>(tab + H->off_species)),
          reactions(reinterpret_cast<const Reaction*>(tab + H->off_reactions)),
          falloff(reinterpret_cast<const Falloff*>(tab + H->off_falloff)),
          eff(reinterpret_cast<const double*>(tab + H->off_eff)) {}
};

// (double)v for a small integer with integer instructions only (no FP64 conversion on the FP64 pipe).
__device__ __forceinline__ double small_int_to_double(int v) {
    if (v == 0) return 0.0;
    const unsigned a = v < 0 ? (unsigned)(-v) : (unsigned)v;
    const int e = 31 - __clz(a);
    const unsigned long long mant = (unsigned long long)(a ^ (1u << e)) << (52 - e);
    const unsigned long long sign = v < 0 ? (1ull << 63) : 0ull;
    return __longlong_as_double((long long)(sign | ((unsigned long long)(1023 + e) << 52) | mant));
}

// Product of concentrations with multiplicities (product_of_exponentiations, reaction.rs:53-63),
// seeded with the first factor. BATCH (a thread's own cell, arrays in thread-local memory): the loads
// (kMaxSide slots, absent ones skipped) are issued together before the first multiply, so that the reads
// overlap instead of each waiting for the previous factor. Otherwise (a warp's cell in shared memory,
// one reaction per lane) one load per factor, fewer registers. The multiplication order is the same.
template <bool BATCH>
__device__ __forceinline__ double conc_product(const double* C, const uint16_t* ks, const int8_t* ns, int n) {
    if constexpr (BATCH) {
        double v[kMaxSide];
#pragma unroll
        for (int q = 0; q < kMaxSide; q++) v[q] = q < n ? C[ks[q]] : 1.0;
        double p = v[0];
#pragma unroll 1
        for (int m = 1; m < ns[0]; m++) p *= v[0];
#pragma unroll
        for (int q = 1; q < kMaxSide; q++) {
            if (q < n) {
#pragma unroll 1
                for (int m = 0; m < ns[q]; m++) p *= v[q];
            }
        }
        return p;
    } else {
        double p = C[ks[0]];
#pragma unroll 1
        for (int m = 1; m < ns[0]; m++) p *= C[ks[0]];
#pragma unroll 1
        for (int q = 1; q < n; q++)
#pragma unroll 1
            for (int m = 0; m < ns[q]; m++) p *= C[ks[q]];
        return p;
    }
}

// 1/Kc without its standard-state factor: the cached Gibbs exponentials of the net species, |nu| times
// each, in species order; with BATCH four loads issued together per batch, as in conc_product.
template <bool BATCH, class Rx, class CellT>
__device__ __forceinline__ double gibbs_product(const Rx& x, const CellT& c) {
    if constexpr (BATCH) {
        double p = 1.0;
#pragma unroll
        for (int q0 = 0; q0 < kMaxNet; q0 += 4) {
            if (q0 >= x.n_net) break;
            double v[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int q = q0 + j;
                v[j] = q < x.n_net ? (x.net_n[q] > 0 ? c.ex[x.net_k[q]] : c.exn[x.net_k[q]]) : 1.0;
            }
            int j0 = 0;
            if (q0 == 0) {  // seeded with the first factor
                p = v[0];
                const int nu0 = x.net_n[0];
#pragma unroll 1
                for (int m = 1; m < (nu0 > 0 ? nu0 : -nu0); m++) p *= v[0];
                j0 = 1;
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (j >= j0 && q0 + j < x.n_net) {
                    const int nu = x.net_n[q0 + j];
#pragma unroll 1
                    for (int m = 0; m < (nu > 0 ? nu : -nu); m++) p *= v[j];
                }
            }
        }
        return p;
    } else {
        const int nu0 = x.net_n[0];
        const double t0 = nu0 > 0 ? c.ex[x.net_k[0]] : c.exn[x.net_k[0]];
        double p = t0;
#pragma unroll 1
        for (int n = 1; n < (nu0 > 0 ? nu0 : -nu0); n++) p *= t0;
#pragma unroll 1
        for (int q = 1; q < x.n_net; q++) {
            const int nu = x.net_n[q], k = x.net_k[q];
            const double tt = nu > 0 ? c.ex[k] : c.exn[k];
#pragma unroll 1
            for (int n = 0; n < (nu > 0 ? nu : -nu); n++) p *= tt;
        }
        return p;
    }
}

// Cells whose arrays are the thread's own (thread-local memory) batch their loads.
template <class CellT>
constexpr bool kBatchLoads = std::is_array<decltype(CellT::C)>::value;

// Pieces of one reaction's rate of progress, for the analytic Jacobian: cR = kf * Rnet with
// Rnet = Rf - pK * Pp, and dkf/dM the forward coefficient's derivative in the third-body concentration.
struct ReactionParts {
    double kf, Rf, pK, Pp, Rnet, dkf_dM;
};

// cR of one reaction (reaction.rs:149-309): forward rate constant (with third-body efficiency and
// falloff), rate of progress against the equilibrium constant, and their product. M: the reaction's
// third-body concentration C + sum (e_k - 1) C_k (reaction.rs:141-145), unused by models 0 and 1.
// MODEL is a compile-time constant: reactions are grouped by model, so no model branch (and no
// predicated FP64 instruction of another model) is executed per reaction.
template <int MODEL, bool PARTS, class CellT>
__device__ __forceinline__ double reaction_eval(const RatesTables& tb, const Reaction& x, const CellT& c, double M,
                                                ReactionParts* parts) {
    const RatesHeader& H = *tb.H;
    const Temps& t = c.t;
    double kf;  // forward rate coefficient: k, k M, or the falloff-blended value
    if constexpr (MODEL == 4) {  // Troe (reaction.rs:160-193)
        const Falloff& f = tb.falloff[x.falloff];
        const double k0 = arrhenius(f.k0, t);
        double Pr, kinf, dPr_dM;
        if (f.flags & kKinfConst) {
            Pr = M * k0;
            kinf = f.ainf;
            dPr_dM = k0;
        } else {
            const double ki = arrhenius(x.k, t);
            Pr = div64(M * k0, ki + kF32MinPos);
            kinf = f.ainf * ki;
            dPr_dM = PARTS ? div64(k0, ki + kF32MinPos) : 0.0;
        }
        double lnF;
        if (f.flags & kFcentConst) {
            lnF = f.ln_fcent;
        } else {
            double F = 0.0;
            if (f.flags & kTermT3) F = f.c1mA * exp64(t.T * f.c3);
            if (f.flags & kTermT1) F += f.cA * exp64(t.T * f.c1);
            if (f.flags & kTermAConst) F += f.cA;
            if (f.flags & kTermT2) F += exp64(f.cmT2 * t.rcpT);
            lnF = log64(F);
        }
        const double Cc = fma(-0.67, lnF, -H.ln10_04);
        const double Nn = fma(-1.27, lnF, H.ln10_075);
        const double lnPrC = log64(Pr + kF32MinPos) + Cc;
        const double f1 = div64(lnPrC, fma(-0.14, lnPrC, Nn));
        const double Fb = exp64(div64(lnF, fma(f1, f1, 1.0)));
        kf = div64((Fb * kinf) * Pr, Pr + 1.0);
        if constexpr (PARTS) {  // the broadening factor is held constant (its Pr dependence is dropped)
            const double r1 = rcp64(Pr + 1.0);
            parts->dkf_dM = ((Fb * kinf) * dPr_dM) * (r1 * r1);
        }
    } else if constexpr (MODEL == 3) {  // Lindemann (reaction.rs:153-159)
        const Falloff& f = tb.falloff[x.falloff];
        const double k0 = arrhenius(f.k0, t);
        const double Ck0 = M * k0;
        const double ki = arrhenius(x.k, t);
        kf = div64(Ck0 * ki, (Ck0 + ki) + kF32MinPos);
        if constexpr (PARTS) {
            const double q = div64(ki, (Ck0 + ki) + kF32MinPos);
            parts->dkf_dM = k0 * (q * q);
        }
    } else if constexpr (MODEL == 5) {  // SRI: the commented formula of reaction.rs:194-203
        const Falloff& f = tb.falloff[x.falloff];
        const double k0 = arrhenius(f.k0, t);
        const double ki = arrhenius(x.k, t);
        const double Pr = div64(M * k0, ki + kF32MinPos);
        const double lP = log64(Pr + kF32MinPos);
        double base = exp64(f.smrC * t.T);
        if (f.sri_flags & kSriA) base = fma(f.sA, exp64(f.smB * t.rcpT), base);
        double F = exp64(log64(base) * rcp64(fma(lP, lP, 1.0)));
        if (f.sri_flags & kSriD) F = f.sD * F;
        if (f.sri_flags & kSriE) F *= exp64(f.sE * t.lnT);
        kf = div64((F * ki) * Pr, Pr + 1.0);
        if constexpr (PARTS) {  // F held constant, as for Troe
            const double r1 = rcp64(Pr + 1.0);
            parts->dkf_dM = ((F * ki) * div64(k0, ki + kF32MinPos)) * (r1 * r1);
        }
    } else if constexpr (MODEL == 2) {  // three-body (reaction.rs:152)
        const double k = arrhenius(x.k, t);
        kf = k * M;
        if constexpr (PARTS) parts->dkf_dM = k;
    } else {  // elementary, irreversible
        kf = arrhenius(x.k, t);
        if constexpr (PARTS) parts->dkf_dM = 0.0;
    }
    // Rate of progress (reaction.rs:269-306).
    constexpr bool B = kBatchLoads<CellT>;
    const double Rf = conc_product<B>(c.C, x.r_k, x.r_n, x.n_r);
    double Rnet = Rf;
    if constexpr (PARTS) {
        parts->kf = kf;
        parts->Rf = Rf;
        parts->pK = 0.0;
        parts->Pp = 0.0;
    }
    if constexpr (MODEL != 1) {
        // 1/Kc: product of the cached Gibbs exponentials, repeated |nu| times, in species order.
        double p = gibbs_product<B>(x, c);
        // (P0/RT)^(-sum nu): the factor chosen with integer selects, one multiply for every reaction.
        const int msn = x.minus_sigma_net;
        const double cfac = msn == 1 ? c.C0 : msn == -1 ? c.rcpC0 : msn == -2 ? c.rcpC0sq : 1.0;
        p *= cfac;
        const double Pp = conc_product<B>(c.C, x.p_k, x.p_n, x.n_p);
        Rnet = fma(-p, Pp, Rf);
        if constexpr (PARTS) {
            parts->pK = p;
            parts->Pp = Pp;
        }
    }
    if constexpr (PARTS) parts->Rnet = Rnet;
    return kf * Rnet;
}

template <int MODEL, class CellT>
__device__ __forceinline__ double reaction_rate(const RatesTables& tb, const Reaction& x, const CellT& c, double M) {
    return reaction_eval<MODEL, false>(tb, x, c, M, nullptr);
}

}  // namespace cbg
