/* FP64 CPU oracle for the per-cell chemistry path (rates + mixture-averaged transport).
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker that the CUDA path is compared against, and the
 * timed CPU baseline. Nothing in the product library may include, link or call it.
 *
 * It restates, in plain C and with no FMA contraction, the evaluation semantics of the
 * reference's FP64 interpreter (ast/interpret.rs:52-148) applied to the straight-line programs
 * that reaction.rs:356-391 (species rates), reaction.rs:329-354 (per-reaction rates) and
 * transport.rs:179-214 (transport properties) build, including the constant folding that the
 * expression builder performs while it builds them (ast/lib.rs:195-232, 337-347).
 * Parity is unpinned: the reference has no tests or golden vectors for this path and cannot be
 * built here (no Rust toolchain), so this restatement is checked against an independent numpy
 * restatement and against physics known-answer tests instead. */
#ifndef COMBUSTION_ORACLE_H
#define COMBUSTION_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_mech or_mech;

/* Mechanism in SI units, species ordered active-first with the inert bulk species last
 * (lib.rs:127-140). Arrays are row-major: nasa7 [K][2][7], reactants/products/efficiencies
 * [R][K], rate/k0 [R][3] = (A, b, activation temperature), troe [R][4] = (A, T3, T1, T2),
 * sri [R][5]. model codes: 0 elementary, 1 irreversible, 2 three-body, 3 Lindemann, 4 Troe, 5 SRI. */
or_mech* or_mech_new(int K, int R, const double* molar_mass, const double* nasa7_split, const double* nasa7,
                     const int32_t* geometry, const double* diameter, const double* well_depth,
                     const double* polarizability, const double* dipole, const double* rotational_relaxation,
                     const uint8_t* reactants, const uint8_t* products, const int32_t* model, const double* rate,
                     const double* k0, const double* troe, const double* sri, const double* efficiencies);
void or_mech_free(or_mech* m);
int or_active(const or_mech* m);
/* Non-zero when the reference's builder would have rejected the mechanism (panics in reaction.rs /
 * lib.rs); the message is copied to msg. */
int or_check(const or_mech* m, char* msg, size_t len);

/* transport.rs:119-138: the 50 temperatures, x = ln(T/T0), and the fitted quantities for every species
 * (conductivity/sqrt(T), sqrt(viscosity/sqrt(T))) and ordered pair (diffusivity/T^1.5). */
int or_transport_samples(const or_mech* m, double T0, double* x /*[50]*/, double* y_cond /*[K][50]*/,
                         double* y_visc /*[K][50]*/, double* y_diff /*[K*K][50]*/);
/* Weighted least-squares fits of those samples (weights 1/y^2, degree 4), long-double Householder QR. */
int or_transport_fit(const or_mech* m, double T0, double* cond /*[K][5]*/, double* visc /*[K][5]*/,
                     double* diff /*[K*K][5]*/);
/* Per-species physics at one temperature (transport.rs:97-116), for known-answer tests. */
double or_viscosity(const or_mech* m, int k, double T);
double or_conductivity(const or_mech* m, int k, double T);
double or_diffusivity(const or_mech* m, int a, int b, double T);
double or_omega22(const or_mech* m, int a, int b, double T);

/* Install raw (unscaled) fit coefficients and the normalisation of transport.rs:180-182. */
void or_set_transport(or_mech* m, double T0, double viscosity0, double conductivity0, const double* cond,
                      const double* visc, const double* diff);

/* One cell. rates: in [K+3] = (P/R, R/P, T, V, n_0..n_{K-2}), out [A+2] = (dT/dt, dV/dt, wdot_0..).
 * reaction_rates: in [K+2] = (P/R, T, V, n_0..n_{K-2}), out [R].
 * transport: in [K+1] = (sum n, T/T0, n_0..n_{K-2}), out [K+2] = (lambda/lambda0, mu/mu0, rhoD_k/mu0).
 * scale (optional, same length as out): the sum of magnitudes of the terms each output accumulates,
 * the denominator of the conditioning-aware relative error used by the parity tests. */
void or_rates(const or_mech* m, const double* in, double* out, double* scale);
void or_reaction_rates(const or_mech* m, const double* in, double* out);
void or_transport(const or_mech* m, const double* in, double* out, double* scale);

/* Struct-of-arrays batches over n cells on nthreads POSIX threads; in/out/scale are arrays of
 * pointers, one per input/output (scale may be NULL). Returns 0. */
int or_rates_batch(const or_mech* m, size_t n, const double* const* in, double* const* out,
                   double* const* scale, int nthreads);
int or_reaction_rates_batch(const or_mech* m, size_t n, const double* const* in, double* const* out,
                            double* const* scale, int nthreads);
int or_transport_batch(const or_mech* m, size_t n, const double* const* in, double* const* out,
                       double* const* scale, int nthreads);
/* Rates + transport of the same cells, transport inputs derived as sum n = (P/R * V) / T, T' = T / T0. */
int or_fused_batch(const or_mech* m, size_t n, const double* const* in, double* const* out_rates,
                   double* const* out_transport, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
