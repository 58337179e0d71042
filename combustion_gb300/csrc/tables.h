// Packed mechanism tables, shared by the host builder (mechanism.cpp) and the kernels (kernels.cu).
//
// The reference compiles each mechanism into straight-line code with the constants folded in
// (reaction.rs:356-391, transport.rs:179-214). Here the mechanism stays data: one contiguous blob per
// path, read by every thread of a warp at the same address (a broadcast), staged into shared memory
// with a bulk TMA copy when it fits. All constants are already canonicalised the way the reference's
// expression builder folds them (ast/lib.rs:195-232), so the kernels evaluate plain arithmetic.
#pragma once
#include <stdint.h>

namespace cbg {

constexpr int kMaxSide = 4;  // distinct species on one side of a reaction
constexpr int kMaxNet = 8;   // active species with a non-zero net coefficient
constexpr int kAlign = 16;   // section alignment inside a blob (bulk TMA granularity)

// Temperature factor of arrhenius() (reaction.rs:117-125).
enum Factor : int32_t { kNone = 0, kRcpT2, kRcpT, kT4, kT3, kT2, kT };

// k = min(f32::MAX, exp(beta*lnT + mEa*rcpT + lnA))  when has_x, where beta = b' + m also carries the
//     integer power T^m that reaction.rs:117-125 peels off (exp(m lnT) = T^m to a few ulps),
//     min(f32::MAX, factor * A)                          otherwise (A alone without factor).
struct Arrhenius {
    double beta, mEa, lnA, A;
    int32_t factor, has_x, has_beta_rem, pad1;  // has_beta_rem: the reference program has a b' lnT term
};

enum FalloffFlags : int32_t {
    kKinfConst = 1,    // Troe k_inf has b = Ea = 0: k_inf is the constant ainf (reaction.rs:172-174)
    kTermT3 = 2,       // (1-A) exp(-T/T3) term present
    kTermT1 = 4,       // A exp(-T/T1) term present (T1 < 1e30)
    kTermAConst = 8,   // constant A term (T1 >= 1e30)
    kTermT2 = 16,      // exp(-T2/T) term present
    kFcentConst = 32,  // Fcent has no runtime term: lnFcent = ln_fcent
};

// SRI blending F = D (A exp(-B/T) + exp(-T/C))^(1/(1 + ln(Pr)^2)) T^E (the reference's commented
// formula, reaction.rs:194-203): which optional factors are present.
enum SriFlags : int32_t { kSriA = 1, kSriD = 2, kSriE = 4 };

struct Falloff {
    Arrhenius k0;                       // low-pressure rate constant (Troe: A divided by A_inf)
    double ainf;                        // canonical A_inf multiplying the Troe k_inf
    double c1mA, cA, c3, c1, cmT2;      // canonical (1-A), A, -1/T3, -1/T1, -T2
    double ln_fcent;                    // lnFcent when constant
    int32_t flags, sri_flags;
    double sA, smB, smrC, sD, sE;       // SRI: canonical A, -B, -1/C, D, E
};

// Reactions are stored grouped by model (RatesHeader::group_end), each group in the mechanism's order;
// orig is the reaction's index in the mechanism (per-reaction outputs).
struct Reaction {
    int32_t model, minus_sigma_net, eff_row, falloff;  // eff_row/falloff: -1 when absent
    int32_t n_r, n_p, n_net, orig;
    uint16_t r_k[kMaxSide], p_k[kMaxSide], net_k[kMaxNet];
    int8_t r_n[kMaxSide], p_n[kMaxSide], net_n[kMaxNet];
    Arrhenius k;                        // forward / high-pressure rate constant
};

// Per species thermodynamics: piece 0 for T <= split (lib.rs:15).
struct Species {
    double split;      // NaN: single piece (both pieces equal)
    double g[2][7];    // Gibbs0_RT coefficients times [1, lnT, T, T2, T3, T4, 1/T] (reaction.rs:78-81)
    double h[2][6];    // enthalpy_RT: a0, a1/2, a2/3, a3/4, a4/5, a5 times [1, T, T2, T3, T4, 1/T]
    double cp[2][5];   // cp/R: a0..a4 times [1, T, T2, T3, T4]
    double dtE;        // canonical 1 - W_k / W_bulk (reaction.rs:382)
    int32_t need_exp, need_exp_neg;  // Gibbs exponentials some reversible reaction uses
    int32_t pad[2];
};

// Tables of the FP64 elementary functions (fp64_math.cuh), staged with every blob: lookups use a
// different index in every lane, which shared memory serves and the constant cache would serialise.
struct MathTables {
    double exp2j[256];   // 2^(j/256), correctly rounded
    double log_hi[257];  // ln(1 + j/256) as a double-double (log_hi[256] + log_lo[256] = ln 2 split
    double log_lo[257];  //   exactly like the ln 2 constant of log_fast)
    double rcp[257];     // 1 / (1 + j/256), rounded
    double pad;
};

// Every blob starts with its MathTables, so that a kernel finds them at the base of its dynamic shared
// memory whether the rest of the blob is staged there or read from global memory; the blob's header
// follows at kMathBytes.
constexpr int kMathBytes = (int)sizeof(MathTables);
static_assert(kMathBytes % kAlign == 0, "math tables must keep the blob sections aligned");

struct RatesHeader {
    int32_t K, A, R, n_eff, n_falloff, total_bytes;
    int32_t off_species, off_reactions, off_falloff, off_eff, off_math, pad;
    int32_t group_end[6], pad1[2];  // reactions [group_end[m-1], group_end[m]) have model m
    double M3, cbrt_max, C0, rcp_C0, ln10_04, ln10_075, pad2[2];
};

struct TransportHeader {
    int32_t K, n_pairs, total_bytes, off_math;
    int32_t off_cond, off_visc, off_W, off_diff, off_A2, off_AB, off_B2, pad2;
    double T0, pad3;  // temperature normalisation (inputs from the rates layout are divided by it)
};

}  // namespace cbg
