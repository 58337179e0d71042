// Tables of the mixed-precision form (kernels_mixed.cu), built by mechanism.cpp next to the FP64 ones.
//
// FP64 stays where the reference's values cancel: the Gibbs polynomials and exponentials of the
// equilibrium constant, the forward-minus-reverse rate of progress and the accumulation into species
// rates. Everything else (Arrhenius exponentials, third-body sums, falloff blending, enthalpy and heat
// capacity polynomials, all of transport) is FP32.
#pragma once
#include <stdint.h>

#include "tables.h"

namespace cbg {

// k = min(f32::MAX, exp(b lnT + mEa / T + lnA)) with the whole temperature exponent b in the argument
// (arrhenius() of reaction.rs:113-139 without the power-of-T split, which only serves FP32 range).
struct ArrheniusF {
    float b, mEa, lnA;
    int32_t has_x;  // 0: k = A exactly (no temperature dependence); then A holds lnA's value
    double A;
};

struct FalloffF {
    ArrheniusF k0;
    double ainf;                    // A_inf (FP64: k_inf can exceed the FP32 range)
    float c1mA, cA, c3, c1, cmT2, ln_fcent;
    int32_t flags, sri_flags;
    float sA, smB, smrC, sD, sE, pad;  // SRI constants (tables.h)
};

struct ReactionF {
    int32_t model, minus_sigma_net, eff_row, falloff;
    int32_t n_r, n_p, n_net, orig;
    uint16_t r_k[kMaxSide], p_k[kMaxSide], net_k[kMaxNet];
    int8_t r_n[kMaxSide], p_n[kMaxSide], net_n[kMaxNet];
    ArrheniusF k;
};

struct SpeciesF {
    double split;
    double g[2][7];     // Gibbs polynomial, FP64
    float h[2][6];      // enthalpy_RT, FP32
    float cp[2][5];     // cp/R, FP32
    float pad0;
    double dtE;
    int32_t need_exp, need_exp_neg;
};

struct RatesMixedHeader {
    int32_t K, A, R, n_eff, n_falloff, total_bytes;
    int32_t off_species, off_reactions, off_falloff, off_eff, off_math, pad;
    int32_t group_end[6], pad1[2];  // as RatesHeader::group_end
    double M3, cbrt_max, C0, rcp_C0;
    float ln10_04, ln10_075, pad2[2];
};

struct TransportMixedHeader {
    int32_t K, n_pairs, total_bytes, off_math;
    // off_diff: per species pair (k, j < k) its 5 fit coefficients padded to 8 floats (two 16-byte
    // loads); off_wilke: per (k, j) of the rows padded to a multiple of 4, {a^2, 2ab, b^2, 0} (one 16-byte
    // load for the three Wilke terms)
    int32_t off_cond, off_visc, off_W, off_diff, off_wilke, pad_w[3];
    double T0, pad3;
};

}  // namespace cbg
