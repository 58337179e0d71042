// Mixed-precision rate of progress of one reaction (reaction.rs:113-309 with FP32 Arrhenius exponentials,
// third-body sums and falloff blending; FP64 equilibrium constant, forward-minus-reverse rate and the
// product with the forward coefficient), shared by the per-cell kernels (kernels_mixed.cu) and the
// batched reactors' mixed right-hand side (bdf.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "device_math.cuh"
#include "rates_core.cuh"
#include "tables_mixed.h"

namespace cbg {

struct RatesMixedTables {
    const RatesMixedHeader* H;
    const SpeciesF* species;
    const ReactionF* reactions;
    const FalloffF* falloff;
    const float* eff;
    __device__ explicit RatesMixedTables(const uint8_t* tab)
        : H(reinterpret_cast<const RatesMixedHeader*>(tab + kMathBytes)),
          species(reinterpret_cast<const SpeciesF*>(tab + H->off_species)),
          reactions(reinterpret_cast<const ReactionF*>(tab + H->off_reactions)),
          falloff(reinterpret_cast<const FalloffF*>(tab + H->off_falloff)),
          eff(reinterpret_cast<const float*>(tab + H->off_eff)) {}
};

__device__ __forceinline__ int piece_of_m(double split, double T) {
    return __double_as_longlong(T) <= __double_as_longlong(split) ? 0 : 1;
}

// min(f32::MAX, k) of reaction.rs:138 with k = exp(b lnT - Ea/T + ln A) evaluated in FP32.
__device__ __forceinline__ double arrhenius_f(const ArrheniusF& a, float lnT, float rcpT) {
    if (!a.has_x) return min_pos(kF32Max, a.A);
    return min_pos(kF32Max, exp_f32x(fmaf(a.b, lnT, fmaf(a.mEa, rcpT, a.lnA))));
}

// The products of the rate of progress are the FP64 path's (rates_core.cuh: conc_product, gibbs_product).

// e^x and e^-x of an FP64 argument to FP32 relative accuracy (a few 1e-8) over the FP64 range: x = n ln2
// + r with n = rint(x / ln2) and r formed in FP64 (three FP64 instructions; the reduction error is
// below 1e-13 for |x| < 708), e^r and e^-r in FP32 (exp2f of r log2(e)), then 2^n and 2^-n added to the
// exponent fields with integer instructions (|n| <= 1021 keeps both results normal). Beyond |x| = 708,
// infinities and NaN: the FP64 exponential and its reciprocal.
__device__ __forceinline__ void exp_pair_mixed(double x, double& ep, double& em) {
    const int hi = __double2hiint(x);
    if ((hi & 0x7fffffff) >= 0x40862000) {
        ep = exp64(x);
        em = rcp64(ep);
        return;
    }
    const double t = fma(x, 0x1.71547652b82fep+0, 0x1.8p52);  // x / ln2 + 1.5 * 2^52: n in the low word
    const int n = __double2loint(t);
    const double r = fma(t - 0x1.8p52, -0x1.62e42fefa39efp-1, x);
    const float rl = dbl_to_flt(r) * 0x1.715476p+0f;  // r log2(e), |r| <= ln2 / 2
    const long long bp = __double_as_longlong(flt_to_dbl(exp2f(rl)));
    const long long bm = __double_as_longlong(flt_to_dbl(exp2f(-rl)));
    ep = __longlong_as_double(bp + ((long long)n << 52));
    em = __longlong_as_double(bm - ((long long)n << 52));
}

// The cached Gibbs exponentials of the mixed program for exponent x (reaction.rs:234-263), with the
// standard-state factor of the equilibrium constant folded in: ex = min(M3, e^x) RT/P0 and
// exn = min(cbrt(f32::MAX), e^-x) P0/RT, so that a reaction's product of |nu| factors per net species
// carries (P0/RT)^(-sum nu) without a multiply per reaction. Both exponentials to FP32 relative accuracy
// (exp_pair_mixed: 3 FP64 operations where an FP64 exponential and reciprocal take 12).
__device__ __forceinline__ void gibbs_exps(double x, bool need_exp, bool need_exp_neg, double M3, double cbrt_max,
                                           double C0, double rcpC0, double& ex, double& exn) {
    double ep, em;
    exp_pair_mixed(x, ep, em);
    if (need_exp) ex = min_pos(M3, ep) * rcpC0;
    if (need_exp_neg) exn = min_pos(cbrt_max, em) * C0;
}

// cR of one reaction. MODEL is a compile-time constant (reactions are grouped by model), so no
// predicated FP64 instruction of another model's branch is executed.
// CellT: any cell view with C, ex, exn (FP64, indexable, from gibbs_exps), C0, rcpC0, rcpC0sq and the FP32
// temperatures Ctotf, Tf, lnTf, rcpTf (one thread's cell here, one warp's cell in the batched reactors).
// Mf: the reaction's FP32 third-body concentration (unused by models 0 and 1).
template <int MODEL, class CellT>
__device__ __forceinline__ double reaction_rate_m(const RatesMixedTables& tb, const ReactionF& x, const CellT& c,
                                                  float Mf) {
    const RatesMixedHeader& H = *tb.H;
    double kf;  // forward rate coefficient including third body and falloff
    if constexpr (MODEL == 4) {  // Troe, blending in FP32 (reaction.rs:160-193)
        const FalloffF& f = tb.falloff[x.falloff];
        const double k0 = arrhenius_f(f.k0, c.lnTf, c.rcpTf);
        const double Md = flt_to_dbl(Mf);
        double Pr, kinf;
        if (f.flags & kKinfConst) {
            Pr = Md * k0;
            kinf = f.ainf;
        } else {
            const double ki = arrhenius_f(x.k, c.lnTf, c.rcpTf);
            Pr = (Md * k0) * rcp64(ki + kF32MinPos);
            kinf = f.ainf * ki;
        }
        float lnF;
        if (f.flags & kFcentConst) {
            lnF = f.ln_fcent;
        } else {
            float F = 0.f;
            if (f.flags & kTermT3) F = f.c1mA * expf(c.Tf * f.c3);
            if (f.flags & kTermT1) F += f.cA * expf(c.Tf * f.c1);
            if (f.flags & kTermAConst) F += f.cA;
            if (f.flags & kTermT2) F += expf(f.cmT2 * c.rcpTf);
            lnF = logf(F);
        }
        const float Cc = fmaf(-0.67f, lnF, -H.ln10_04);
        const float Nn = fmaf(-1.27f, lnF, H.ln10_075);
        const float lnPrC = log_dbl_f32(Pr + kF32MinPos) + Cc;
        const float f1 = __fdividef(lnPrC, fmaf(-0.14f, lnPrC, Nn));
        const float Fb = expf(__fdividef(lnF, fmaf(f1, f1, 1.f)));
        kf = (flt_to_dbl(Fb) * kinf) * (Pr * rcp64(Pr + 1.0));
    } else if constexpr (MODEL == 3) {  // Lindemann (reaction.rs:153-159)
        const FalloffF& f = tb.falloff[x.falloff];
        const double Ck0 = flt_to_dbl(Mf) * arrhenius_f(f.k0, c.lnTf, c.rcpTf);
        const double ki = arrhenius_f(x.k, c.lnTf, c.rcpTf);
        kf = (Ck0 * ki) * rcp64((Ck0 + ki) + kF32MinPos);
    } else if constexpr (MODEL == 5) {  // SRI (reaction.rs:194-203, commented formula), blending in FP32
        const FalloffF& f = tb.falloff[x.falloff];
        const double k0 = arrhenius_f(f.k0, c.lnTf, c.rcpTf);
        const double ki = arrhenius_f(x.k, c.lnTf, c.rcpTf);
        const double Pr = (flt_to_dbl(Mf) * k0) * rcp64(ki + kF32MinPos);
        const float lP = log_dbl_f32(Pr + kF32MinPos);
        float base = expf(f.smrC * c.Tf);
        if (f.sri_flags & kSriA) base = fmaf(f.sA, expf(f.smB * c.rcpTf), base);
        float F = expf(__fdividef(logf(base), fmaf(lP, lP, 1.f)));
        if (f.sri_flags & kSriD) F *= f.sD;
        if (f.sri_flags & kSriE) F *= expf(f.sE * c.lnTf);
        kf = (flt_to_dbl(F) * ki) * (Pr * rcp64(Pr + 1.0));
    } else if constexpr (MODEL == 2) {  // three-body (reaction.rs:152)
        kf = arrhenius_f(x.k, c.lnTf, c.rcpTf) * flt_to_dbl(Mf);
    } else {
        kf = arrhenius_f(x.k, c.lnTf, c.rcpTf);
    }
    // FP64 rate of progress (reaction.rs:269-306).
    constexpr bool B = kBatchLoads<CellT>;
    const double Rf = conc_product<B>(c.C, x.r_k, x.r_n, x.n_r);
    double Rnet = Rf;
    if constexpr (MODEL != 1) {
        // (P0/RT)^(-sum nu) is folded into the cell's exponentials (gibbs_exps), one factor per use
        const double p = gibbs_product<B>(x, c);
        Rnet = fma(-p, conc_product<B>(c.C, x.p_k, x.p_n, x.n_p), Rf);
    }
    return kf * Rnet;
}

}  // namespace cbg
