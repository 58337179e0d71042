/* combustion_gb300: GB300 (sm_103a) per-cell chemistry kernels behind a C ABI.
 *
 * Drop-in for the per-cell path of Matthias-Fauconneau/combustion: the reference builds one
 * straight-line program per mechanism (reaction::rates, reaction.rs:356-391; reaction::reactions_rates,
 * reaction.rs:329-354; transport::properties, transport.rs:179-214) and runs it once per cell through
 * device::assemble (device.rs:25-49 on the CPU, device.rs:59-96 on a GPU), whose call takes uniform
 * constants plus one struct-of-arrays slice per input and returns one array per output. Here a
 * mechanism handle holds the same mechanism as tables on the GPU, and each cb_*_f64 call is that
 * assembled function's call: same inputs, same outputs, same order.
 *
 * Conventions
 *  - Every function returns CB_OK (0) or a CB_ERR_* code; cb_last_error() describes the last failure
 *    of the calling thread. Nothing aborts, traps or prints.
 *  - Arrays are caller-owned. Pointer arrays (inputs/outputs) are read on the host during the call.
 *  - Device-memory calls are asynchronous on the given CUDA stream (cudaStream_t passed as void*,
 *    NULL = legacy default stream). With CB_HOST_MEMORY the call copies host arrays through
 *    library-owned device buffers and returns when the outputs are on the host.
 *  - A mechanism handle may be used from one host thread at a time.
 */
#ifndef COMBUSTION_GB300_H
#define COMBUSTION_GB300_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum cb_status {
    CB_OK = 0,
    CB_ERR_INVALID = 1,    /* null pointer, bad size or flag */
    CB_ERR_MECHANISM = 2,  /* mechanism rejected (the reference's loader or builder would panic) */
    CB_ERR_CUDA = 3,       /* CUDA runtime error */
    CB_ERR_NOT_READY = 4,  /* transport requested before cb_transport_setup */
    CB_ERR_UNSUPPORTED = 5,/* feature outside this build (e.g. SRI falloff, more species than supported) */
    CB_ERR_DEVICE = 6      /* a kernel reported a failure (e.g. a bounded wait ran out) */
};

/* Reaction models (lib.rs:238-245). */
enum cb_reaction_model {
    CB_ELEMENTARY = 0, CB_IRREVERSIBLE = 1, CB_THREE_BODY = 2, CB_LINDEMANN = 3, CB_TROE = 4, CB_SRI = 5
};
/* Species geometry (model.rs:15-19). */
enum cb_geometry { CB_ATOM = 0, CB_LINEAR = 1, CB_NONLINEAR = 2 };

/* Call flags. */
#define CB_HOST_MEMORY 1u       /* inputs/outputs are host arrays (copied through device buffers) */
#define CB_UNIFORM_PRESSURE 2u  /* rates: inputs[0] (P/R) and inputs[1] (R/P) each point to ONE value,
                                   the reference's uniform "constants" (device.rs:31-32) */

/* A mechanism in SI units, species ordered active first and the inert bulk species last: the output
 * of the reference's loader (yaml.rs:54-171) and of combustion::new (lib.rs:127-140).
 * Row-major arrays: nasa7 [K][2][7] (piece 0 for T <= split), reactants/products/efficiencies [R][K],
 * rate and k0 [R][3] = (A [SI], temperature exponent b, activation temperature Ea/R [K]),
 * troe [R][4] = (A, T3, T1, T2; T2 = +inf when absent), sri [R][5] (may be NULL without SRI).
 * Transport: diameter [m], well_depth [J], polarizability [m^3], dipole [C.m] (lib.rs:40-59). */
typedef struct cb_mech_desc {
    int32_t n_species;
    int32_t n_reactions;
    const double* molar_mass;            /* [K] kg/mol */
    const double* nasa7_split;           /* [K] K; NaN: one piece */
    const double* nasa7;                 /* [K][2][7] */
    const int32_t* geometry;             /* [K] cb_geometry */
    const double* diameter;              /* [K] */
    const double* well_depth;            /* [K] */
    const double* polarizability;        /* [K] */
    const double* dipole;                /* [K] */
    const double* rotational_relaxation; /* [K] */
    const uint8_t* reactants;            /* [R][K] */
    const uint8_t* products;             /* [R][K] */
    const int32_t* model;                /* [R] cb_reaction_model */
    const double* rate;                  /* [R][3] */
    const double* k0;                    /* [R][3] (falloff models; may be NULL otherwise) */
    const double* troe;                  /* [R][4] (may be NULL without Troe reactions) */
    const double* sri;                   /* [R][5] (may be NULL) */
    const double* efficiencies;          /* [R][K] (may be NULL: all 1) */
} cb_mech_desc;

typedef struct cb_mech cb_mech;

typedef struct cb_mech_info {
    int32_t n_species;        /* K */
    int32_t n_active;         /* A: species whose amount some reaction changes (lib.rs:130-135) */
    int32_t n_reactions;      /* R */
    int32_t transport_ready;  /* cb_transport_setup done */
    double T0, viscosity0, conductivity0; /* transport normalisation (transport.rs:180-182) */
    int32_t rates_inputs;     /* K+3 */
    int32_t rates_outputs;    /* A+2 */
    int32_t transport_inputs; /* K+1 */
    int32_t transport_outputs;/* K+2 */
    size_t device_table_bytes;
} cb_mech_info;

/* Algorithmic work per cell (the roofline numerator): FP64 flops counted with FMA = 2, plus the number
 * of exp, log, division/reciprocal and sqrt evaluations, and DRAM bytes in/out (per-cell pressure). */
typedef struct cb_work {
    double flops;
    double exps, logs, divs, sqrts;
    double bytes_in, bytes_out;
} cb_work;

/* Replaces combustion::new (lib.rs:127-140) plus the table-building half of reaction::rates
 * (reaction.rs:356-391): validates the mechanism exactly as the reference's builder would (active
 * species prefix, net order, unimplemented SRI) and uploads its tables to the current CUDA device. */
int cb_mech_create(const cb_mech_desc* desc, cb_mech** out);
/* Host only, no device needed: the validation of cb_mech_create (combustion::new, lib.rs:127-140),
 * filling info (species, active species, reactions, table size) without uploading anything. */
int cb_mech_validate(const cb_mech_desc* desc, cb_mech_info* info);
int cb_mech_destroy(cb_mech* mech);
int cb_mech_query(const cb_mech* mech, cb_mech_info* info);

/* Replaces transport::properties::<5> (transport.rs:212-214): fits the 50-point collision-integral
 * species properties (transport.rs:119-138) and uploads the scaled polynomials (transport.rs:180-182)
 * for a normalisation (T0, viscosity0, conductivity0) chosen by the caller (cantera.rs:60-76). */
int cb_transport_setup(cb_mech* mech, double T0, double viscosity0, double conductivity0);
/* Host only: the fits of transport::Polynomials::new (transport.rs:125-136) for temperature
 * normalisation T0, without a device: cond [K][5], visc [K][5], diff [K*K][5] (any may be NULL). */
int cb_transport_fit(const cb_mech_desc* desc, double T0, double* cond, double* visc, double* diff);
/* Raw fitted coefficients (before the transport.rs:180-182 scaling): cond [K][5], visc [K][5],
 * diff [K*K][5] (every ordered pair; only j < k is used). Any pointer may be NULL. */
int cb_transport_coefficients(const cb_mech* mech, double* cond, double* visc, double* diff);

/* Replaces device::assemble(reaction::rates(...)) called as f(constants, inputs) (device.rs:30-47).
 * inputs  [K+3]: P/R, R/P, T [K], V [m^3], n_0 .. n_{K-2} [mol] (n arrays of length n)
 * outputs [A+2]: dT/dt [K/s], dV/dt [m^3/s], wdot_0 .. wdot_{A-1} [mol/m^3/s] */
int cb_rates_f64(cb_mech* mech, size_t n, const double* const* inputs, double* const* outputs,
                 uint32_t flags, void* stream);
/* Replaces reaction::reactions_rates (reaction.rs:329-354):
 * inputs [K+2]: P/R, T, V, n_0 .. n_{K-2};  outputs [R]: rate of progress of each reaction. */
int cb_reaction_rates_f64(cb_mech* mech, size_t n, const double* const* inputs, double* const* outputs,
                          uint32_t flags, void* stream);
/* Replaces device::assemble(transport::properties::<5>(...)) (transport.rs:179-214):
 * inputs  [K+1]: sum of amounts n [mol], T/T0, n_0 .. n_{K-2}
 * outputs [K+2]: lambda/lambda0, mu/mu0, rhoD_0/mu0 .. rhoD_{K-1}/mu0 */
int cb_transport_f64(cb_mech* mech, size_t n, const double* const* inputs, double* const* outputs,
                     uint32_t flags, void* stream);
/* Both on the same cells: rates inputs as cb_rates_f64, and transport evaluated at
 * sum n = (P/R * V) / T and T/T0 (the ideal-gas total of the same cell). */
int cb_rates_transport_f64(cb_mech* mech, size_t n, const double* const* inputs, double* const* rates_out,
                           double* const* transport_out, uint32_t flags, void* stream);

/* Number of non-finite values (NaN or infinity) in n_arrays arrays of n doubles each, e.g. a call's
 * outputs: the reference's CPU path asserts finite inputs and outputs around every evaluation
 * (plot.rs:41-46); here the caller checks when it wants to. Device arrays (stream-ordered; *count is
 * written when the call returns, which synchronises the stream) or, with CB_HOST_MEMORY, host arrays. */
int cb_count_nonfinite(cb_mech* mech, size_t n, int32_t n_arrays, const double* const* arrays, uint64_t* count,
                       uint32_t flags, void* stream);

/* Mixed-precision forms of the three calls above (same inputs, outputs and flags). FP64 is kept for the
 * Gibbs polynomials and exponentials of the equilibrium constant (reaction.rs:234-304), the
 * forward-minus-reverse rate of progress (reaction.rs:305-306) and the accumulation into species rates
 * (reaction.rs:312-327); Arrhenius exponentials, third-body sums, falloff blending, the h/RT and cp/R
 * polynomials and all of transport run in FP32. No reference counterpart: the reference's FP64 path is
 * cb_*_f64. Its error against that path is measured by the tests (below 1e-4, condition-scaled). */
int cb_rates_mixed(cb_mech* mech, size_t n, const double* const* inputs, double* const* outputs,
                   uint32_t flags, void* stream);
int cb_transport_mixed(cb_mech* mech, size_t n, const double* const* inputs, double* const* outputs,
                       uint32_t flags, void* stream);
int cb_rates_transport_mixed(cb_mech* mech, size_t n, const double* const* inputs, double* const* rates_out,
                             double* const* transport_out, uint32_t flags, void* stream);

int cb_work_model(const cb_mech* mech, cb_work* rates, cb_work* transport);

/* Diagnostic: FP64 fused multiply-adds per second the current GPU issues (8 independent chains per
 * thread, 8 blocks of 256 threads per SM, best of 3): the peak of the FP64-bound kernels' roofline. */
int cb_device_fp64_peak(double* fma_per_second);

/* Diagnostic: the FP64 elementary functions the kernels use (which: 0 exp, 1 natural log, 2 reciprocal)
 * evaluated on n device doubles, synchronously on `stream`. */
int cb_fp64_math(int which, const double* x, double* y, size_t n, void* stream);

/* Blocks until the mechanism's work on `stream` is done and reports any kernel-side failure. */
int cb_synchronize(cb_mech* mech, void* stream);

/* Test hook, no reference counterpart: the number of polls of the first bounded wait with which the
 * plain FP64 kernels (rates, per-reaction rates, transport) wait for their table staging copy; negative
 * restores the default. At 0 that wait runs out at once: the kernels set the staging-timeout status and
 * wait again, with the full limit, for the copy to land, then return without computing, and the next
 * synchronising call reports CB_ERR_DEVICE (and clears the status). For tests of that error path. */
int cb_debug_stage_wait_polls(int64_t polls);

/* ---- Seeded synthetic cells on the device ----------------------------------------------------------
 * No reference counterpart (the reference reads states from Cantera or its own reactor). T uniform on
 * [T_min, T_max] K, P log-uniform on [P_min, P_max] atm (fixed when equal), V = 1 m^3, mole fractions
 * Dirichlet(alpha) over all K species, n_k = X_k P V / (R T): the counter-based SplitMix64 draws of the
 * package's host generator (cell `offset + i` of the seeded sequence). Outputs: K + 3 device arrays of
 * n doubles in the rates layout. */
typedef struct cb_cell_distribution {
    double T_min, T_max;
    double P_min, P_max;
    double alpha;
    uint64_t seed;
} cb_cell_distribution;
int cb_generate_cells(cb_mech* mech, size_t n, size_t offset, const cb_cell_distribution* dist,
                      double* const* outputs, void* stream);

/* ---- Learned transport surrogate -------------------------------------------------------------------
 * No reference counterpart. A multilayer perceptron maps (log T/T0, log P/atm, X_0 .. X_{K-1}) to the
 * logs of the plain transport outputs (lambda/lambda0, mu/mu0, rhoD_k/mu0), normalised per column.
 * BF16 weights and activations, FP32 accumulation on the tcgen05 tensor cores, SiLU hidden layers,
 * FP32 master weights trained by Adam on the MSE of the normalised outputs, with a cosine learning-rate
 * decay from lr to lr_final. Training cells come from cb_generate_cells and their targets from the
 * plain FP64 transport kernel. A per-cell trust gate (raw inputs inside the per-column range of the
 * training cells) sends other cells to the plain kernel, and a sampled audit recomputes every
 * audit_stride-th cell with the plain kernel, reports the surrogate's error on it and keeps the plain
 * values. Inputs of every call: rates-layout device arrays (P/R, R/P, T, V, n_0 .. n_{K-2}). */
typedef struct cb_surrogate cb_surrogate;
typedef struct cb_surrogate_desc {
    int32_t width;          /* hidden width, a multiple of 256 */
    int32_t hidden_layers;  /* 1 .. 6 */
    int32_t batch;          /* training rows per step, a multiple of 128 */
    float lr, lr_final, beta1, beta2, eps;
    uint64_t seed;          /* weight initialisation */
} cb_surrogate_desc;
typedef struct cb_surrogate_info {
    int32_t n_features, n_in, n_out, width, hidden_layers, batch;
    int64_t n_params, n_weights, n_train, steps_done;
    int64_t weight_offset[8], bias_offset[8];  /* layer l: weights [dims[l+1]][dims[l]], then biases */
    int32_t dims[9];
} cb_surrogate_info;
typedef struct cb_surrogate_stats {
    uint64_t cells, fallback_cells, audited_cells;
    double audit_max_rel_err[3];  /* conductivity, viscosity, diffusion coefficients */
    double audit_rms_rel_err[3];
    /* with CB_SURROGATE_TIMING: device milliseconds of the phases (CUDA events on the call's stream) */
    double ms_features, ms_network, ms_outputs, ms_gate;
} cb_surrogate_stats;
#define CB_SURROGATE_NO_GATE 8u  /* network outputs for every cell: no trust gate, no audit */
#define CB_SURROGATE_TIMING 16u  /* time the phases of the call */

int cb_surrogate_create(cb_mech* mech, const cb_surrogate_desc* desc, cb_surrogate** out);
int cb_surrogate_destroy(cb_surrogate* s);
int cb_surrogate_query(const cb_surrogate* s, cb_surrogate_info* info);
/* Training set: n_train cells (rounded down to whole batches) from `dist`, their plain transport outputs,
 * the normalisation of inputs and outputs and the trust region. Synchronous. */
int cb_surrogate_generate(cb_surrogate* s, size_t n_train, const cb_cell_distribution* dist);
/* `steps` Adam steps over the training set, replayed as one captured CUDA graph per step; losses (host,
 * `steps` floats, may be NULL) receives each step's mean squared error. Synchronous. */
int cb_surrogate_train(cb_surrogate* s, int32_t steps, float* losses);
/* Transport outputs (K + 2 device arrays) of n cells: network, then gate fallback and audit. Flags:
 * CB_UNIFORM_PRESSURE, CB_SURROGATE_NO_GATE. Returns when the outputs and `stats` (may be NULL) are
 * final. */
int cb_surrogate_transport(cb_surrogate* s, size_t n, const double* const* inputs, double* const* outputs,
                           uint32_t flags, uint32_t audit_stride, cb_surrogate_stats* stats, void* stream);
/* Ensemble-gated transport (no reference counterpart): two networks of the same mechanism and shape,
 * trained from different initial weights, evaluate every cell; the outputs are the mean of their logs.
 * Their disagreement max_j |ln y_a,j - ln y_b,j| is the cell's error estimate: a cell whose
 * disagreement exceeds `threshold`, or whose raw inputs leave the first network's training range, is
 * recomputed by the fallback kernel (CB_FALLBACK_MIXED: the mixed-precision transport kernel, about 1e-6;
 * CB_FALLBACK_PLAIN: the plain FP64 kernel). threshold = +inf gates on the training range alone; a
 * negative threshold sends every cell to the fallback kernel, which then runs alone (no network, no
 * audit, `disagreement` untouched). Every
 * audit_stride-th other cell is recomputed by the plain kernel, which judges the reported error, and
 * keeps the plain values. `disagreement` (device, n floats, may be NULL) receives every cell's estimate,
 * from which a caller calibrates the threshold for a stated error on cells of its own. Flags:
 * CB_UNIFORM_PRESSURE, CB_SURROGATE_TIMING. Returns when the outputs and `stats` are final. */
typedef struct cb_surrogate_gate {
    double threshold;
    uint32_t audit_stride;  /* 0: no audit */
    uint32_t fallback;      /* CB_FALLBACK_MIXED or CB_FALLBACK_PLAIN */
    float* disagreement;
} cb_surrogate_gate;
#define CB_FALLBACK_MIXED 0u
#define CB_FALLBACK_PLAIN 1u
int cb_surrogate_transport_pair(cb_surrogate* a, cb_surrogate* b, size_t n, const double* const* inputs,
                                double* const* outputs, uint32_t flags, const cb_surrogate_gate* gate,
                                cb_surrogate_stats* stats, void* stream);
/* Parameters (FP32 master copy, layout of cb_surrogate_info) and normalisation (host arrays of
 * n_features floats each; any may be NULL). Setting parameters resets the Adam moments. */
int cb_surrogate_get_params(const cb_surrogate* s, float* params);
int cb_surrogate_set_params(cb_surrogate* s, const float* params);
int cb_surrogate_normalisation(const cb_surrogate* s, float* in_mean, float* in_rstd, float* out_mean,
                               float* out_std, float* in_lo, float* in_hi);
/* One forward and backward pass on `rows` given rows (a multiple of 128, at most the batch): normalised
 * features [rows][n_in] and targets [rows][n_out] (host, FP32; features are rounded to BF16). Returns
 * the mean squared error, the gradient of every parameter (n_params floats) and, when `outputs` is not
 * NULL, the network outputs [rows][n_out]. Host arrays, synchronous; no parameter is changed. */
int cb_surrogate_evaluate(cb_surrogate* s, int32_t rows, const float* features, const float* targets,
                          float* loss, float* grads, float* outputs);
const char* cb_last_error(void);
const char* cb_version(void);

/* ---- Cantera-YAML mechanisms ------------------------------------------------------------------------
 * Replaces the reference's loader and builder front end (yaml.rs:54-171 + lib.rs:20-140): reads a
 * Cantera YAML mechanism (units cm/s/mol, activation energy K or cal/mol; elementary, irreversible,
 * three-body, falloff with Troe / SRI / Lindemann, single-rate pressure-dependent-Arrhenius) into SI
 * arrays with the species some reaction changes first. cb_yaml_desc fills a cb_mech_desc whose pointers
 * stay valid until cb_yaml_free; cb_yaml_species_name returns the k-th species' name in that order. */
typedef struct cb_yaml_mech cb_yaml_mech;
int cb_yaml_load(const char* text, size_t length, cb_yaml_mech** out);
int cb_yaml_desc(const cb_yaml_mech* mech, cb_mech_desc* desc);
const char* cb_yaml_species_name(const cb_yaml_mech* mech, int32_t k);
int cb_yaml_free(cb_yaml_mech* mech);

/* ---- Batched constant-pressure reactors (variable-order BDF) ----------------------------------------
 * Replaces the reactor loop of plot.rs:32-118 with the cvode crate's role (cvode/lib.rs:17-47: BDF,
 * dense Newton): state u = [T, V, n_0 .. n_{A-1}] at fixed P/R, du/dt = the outputs of cb_rates_f64 for
 * that state (reaction.rs:356-391). Needs every non-bulk species active (A = K - 1). Up to 65 species a
 * reactor's workspace fits in shared memory, and the autotuner chooses between that placement and global
 * memory (at 53 species it picks global: more warps per SM); above, always global memory (24 (K + 1)^2
 * bytes per reactor for its Jacobian and factorisation, plus about 0.6 MB per reactor in flight at 250
 * species).
 * Every reactor is integrated from t = 0 to t_end with its own step size and order (1-5) against
 * atol + rtol |u_i| for every component; its ignition delay is the time of the largest dT/dt (the
 * vertex of a parabola through the samples around it). The host side is synchronous. */
typedef struct cb_reactors cb_reactors;
typedef struct cb_bdf_options {
    double rtol, atol;
    double t_end;               /* s */
    int32_t max_steps;          /* per reactor; reactors that need more end with status 4 */
    int32_t slice_steps;        /* steps per reactor per kernel launch (0: 256) */
    int32_t warps_per_block;    /* reactors in flight per block (0: autotuned) */
    int32_t tables_in_shared;   /* 1: mechanism tables in shared memory, 0: through L1, -1: autotuned */
    int32_t flags;              /* CB_BDF_* below (0: FP64 right-hand side, factorisation at every change) */
} cb_bdf_options;
/* The first Newton iteration of every step (the correction from the predictor) evaluates f(u) by the
 * mixed-precision rates program (FP32 Arrhenius, third-body and falloff terms; FP64 equilibrium
 * constants, rates of progress and accumulation); the later iterations, which decide convergence (the
 * FP64 Newton correction), the initial step's f, the Jacobian and the factorisation stay FP64. Newton on
 * the mixed f alone cannot meet an absolute tolerance below its rounding noise. */
#define CB_BDF_MIXED_RHS 1u
/* Keep the factorisation of I - c J while c = h / gamma_q stays within 30 % of the factorised value and
 * for at most 20 steps (the Newton correction is then scaled by 2 / (1 + c / c_lu), as in CVODE); the
 * factorisation also carries over between launches when it lives in global memory. */
#define CB_BDF_REUSE_LU 2u
/* Workspaces and factorisations in global memory only, even when one reactor's fit in shared memory
 * (without this flag the autotuner times both placements; large mechanisms always use global memory;
 * without CB_BDF_REUSE_LU the integration takes the same steps either way). */
#define CB_BDF_GLOBAL_MEMORY 4u
/* With workspaces in global memory: factorise I - c J in FP32 (the FP32 pipe is many times the FP64 one
 * on this GPU). The Newton residuals, corrections and triangular-solve accumulations stay FP64, so a
 * converged step meets the same tolerances; only the convergence rate depends on the factorisation's
 * accuracy. Ignored when the workspaces are in shared memory. */
#define CB_BDF_LU32 8u
typedef struct cb_reactor_stats {
    uint64_t steps, rhs_evals, jacobians, factorizations, newton_failures, error_failures;
    uint64_t finished, failed;
    double ms;                  /* device time of the integration */
    int32_t warps_per_block, tables_in_shared, graph_replays, slices;
    int32_t global_memory;       /* workspaces in global (1) or shared (0) memory */
    int32_t register_cap;        /* global memory: the kernel's registers a thread, 64, 80 or 128 */
} cb_reactor_stats;
typedef struct cb_reactor_tuning {
    int32_t warps_per_block, tables_in_shared, n_candidates, calib_reactors;
    int32_t global_memory, register_cap;
    struct { int32_t warps_per_block, tables_in_shared, global_memory, register_cap; double ms; } candidates[32];
} cb_reactor_tuning;
int cb_reactors_create(cb_mech* mech, size_t n, const cb_bdf_options* options, cb_reactors** out);
int cb_reactors_destroy(cb_reactors* batch);
/* Initial states (host arrays): pressure_R [n], T [n], V [n], amounts [A][n] (active species). */
int cb_reactors_set_state(cb_reactors* batch, const double* pressure_R, const double* T, const double* V,
                          const double* amounts);
/* Times the launch shapes that fit (reactors per block, table placement, workspaces in shared or global
 * memory, and for global memory the kernel's register cap; global only with CB_BDF_GLOBAL_MEMORY or when
 * one workspace does not fit in shared memory) on copies of the first calib_reactors reactors (0: 8192,
 * or 512 with global memory only) and keeps the fastest; the state is left as it was. */
int cb_reactors_autotune(cb_reactors* batch, int32_t calib_reactors, cb_reactor_tuning* result);
/* Integrates every reactor to t_end (autotuning first when the shape is not set). */
int cb_reactors_integrate(cb_reactors* batch, cb_reactor_stats* stats);
/* Per reactor (host arrays, any may be NULL): ignition delay [n] (s), final state [A+2][n],
 * status [n] (2 done, 3 step size underflow, 4 step limit, 1 unfinished), accepted steps [n]. */
int cb_reactors_results(cb_reactors* batch, double* ignition_delay, double* state, int32_t* status,
                        int32_t* steps);
/* Outputs of the following integrations, headless (the role of plot.rs:76-138, which samples the state
 * at uniform times and reports where the OH mole fraction peaks): n_points states per reactor at
 * t_j = j t_end / (n_points - 1), from the integrator's interpolating polynomial (0: none, else >= 2),
 * and for active species peak_species (-1: none) the largest mole fraction among the active species
 * over the accepted steps, its time and the state there. Allocates device memory; call before
 * cb_reactors_integrate (cb_reactors_set_state resets the outputs). */
int cb_reactors_set_outputs(cb_reactors* batch, int32_t n_points, int32_t peak_species);
/* Host arrays, any may be NULL: times [n_points], trajectory [n_points][A+2][n], peak_time [n],
 * peak_fraction [n], peak_state [A+2][n]. Points a failed reactor did not reach are NaN. */
int cb_reactors_outputs(cb_reactors* batch, double* times, double* trajectory, double* peak_time,
                        double* peak_fraction, double* peak_state);
/* The integrator's du/dt and Jacobian at m given states (host): pressure_R [m], states [m][A+2] ->
 * f [m][A+2], J [m][A+2][A+2] (row i: d f_i / d u_j). Synchronous. */
int cb_reactors_eval(cb_reactors* batch, int32_t m, const double* pressure_R, const double* states, double* f,
                     double* J);
/* cb_reactors_eval without any device allocation; no reference counterpart. For callers that evaluate
 * du/dt and Jacobians inside a time-critical host loop and must not allocate per call (cudaFree
 * synchronises the whole device; under a caching allocator cudaMalloc can fail). Device staging is a
 * fixed 4 MiB static buffer of the library: m is limited to 2^19 / (N^2 + 2N + 1) states (173 at 53
 * species, N = 54; larger m fails with CB_ERR_INVALID). The first call on a device resolves that
 * buffer's address (cudaGetSymbolAddress) and keeps it for the life of the process: make that call
 * before any stream capture, and not across a cudaDeviceReset (which invalidates the kept address).
 * Calls in flight at the same time on one device share the buffer and race. */
int cb_reactors_eval_noalloc(cb_reactors* batch, int32_t m, const double* pressure_R, const double* states,
                             double* f, double* J);

#ifdef __cplusplus
}
#endif
#endif
