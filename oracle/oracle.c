/* FP64 CPU oracle: restatement of the reference interpreter's semantics for reaction.rs and
 * transport.rs. TEST INFRASTRUCTURE ONLY (see oracle.h). Build with -ffp-contract=off and without
 * -ffast-math so that every operation rounds exactly once, as ast/interpret.rs:52-112 does.
 *
 * Constant folding. The reference builds each per-cell program with simplifying constructors
 * (ast/lib.rs:195-232): a constant c combined with a runtime value x gives
 *   add/sub:  x unchanged when (f32)c == 0
 *   mul:      0 when (f32)c == 0, x when (f32)c == 1, -x when (f32)c == -1, c*x otherwise
 *   div:      x * (1/c), then the mul rules
 * and sums drop constant zero terms (ast/lib.rs:337-339). Because x+0, 1*x and -1*x are exact, each
 * rule is reproduced here by canonicalising the mechanism constant once (canon_add / canon_mul) and
 * then evaluating plainly in the builder's operation order. */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../combustion_gb300/csrc/collision_integrals.h"

#define F32MAX ((double)FLT_MAX)   /* f32::MAX as f64 (reaction.rs:138) */
#define F32MINPOS ((double)FLT_MIN) /* f32::MIN_POSITIVE as f64 (reaction.rs:158,177,189) */

static const double kB = 1.380649e-23, NA = 6.02214076e23; /* model.rs:6-7 */
#define RGAS (kB * NA)                                      /* model.rs:8 */

/* ---- folding helpers ---------------------------------------------------------------------- */
static float as_f32(double c) { return fabs(c) < 1e38 ? (float)c : (c > 0 ? INFINITY : -INFINITY); }
static double canon_add(double c) { return as_f32(c) == 0.0f ? 0.0 : c; }
static double canon_mul(double c) {
    float f = as_f32(c);
    if (f == 0.0f) return 0.0;
    if (f == 1.0f) return 1.0;
    if (f == -1.0f) return -1.0;
    return c;
}

/* ---- mechanism ---------------------------------------------------------------------------- */
enum { ELEMENTARY = 0, IRREVERSIBLE = 1, THREE_BODY = 2, LINDEMANN = 3, TROE = 4, SRI = 5 };
enum { F_NONE = 0, F_RCPT2, F_RCPT, F_T4, F_T3, F_T2, F_T };

typedef struct { /* arrhenius() of reaction.rs:113-139 after folding */
    int factor;    /* temperature factor */
    int has_x;     /* the exp() term is present */
    double beta;   /* canonical b' (0 when (f32)b' == 0) */
    double mEa;    /* canonical -Ea (0 when Ea == 0) */
    double lnA;    /* canonical ln A added to the exponent (0: folded away) */
    double A;      /* no exponent: canonical A multiplying the factor, or A itself */
} arrh_t;

typedef struct {
    int model;
    arrh_t k, k0;         /* forward (or high-pressure) and low-pressure rate constants */
    int kinf_const;       /* Troe with b = Ea = 0 for k_inf: k_inf is the constant A_inf */
    double ainf;          /* canonical A_inf factored out of the Troe k_inf (reaction.rs:163-170) */
    double troe_1mA, troe_A, troe_c3, troe_c1, troe_mT2; /* canonical Fcent constants */
    int troe_t1, troe_t2; /* T1 < 1e30, T2 finite */
    int fcent_const; double fcent_value;
    double sri_A, sri_mB, sri_mrC, sri_D, sri_E; /* canonical SRI constants: A, -B, -1/C, D, E */
    int n_eff; int* eff_k; double* eff_c; /* non-unit efficiencies: species and (e-1) (0 => plain C_k) */
    int n_r; int* r_k; int* r_n;          /* reactant species and multiplicities */
    int n_p; int* p_k; int* p_n;          /* product species and multiplicities */
    int n_net; int* net_k; int* net_n;    /* active species with non-zero net stoichiometry */
    int sigma_net;                        /* products - reactants, all species */
} reaction_t;

struct or_mech {
    int K, R, A;
    double* molar_mass; double* split; double* nasa7; int32_t* geometry;
    double* diameter; double* well_depth; double* polarizability; double* dipole; double* rot; double* dof;
    uint8_t* reactants; uint8_t* products; int32_t* model; double* rate; double* k0; double* troe; double* sri;
    double* eff;
    reaction_t* rx;
    /* per-species thermodynamic constants after folding */
    double* h_c;   /* [K][2][6] enthalpy_RT coefficients: a0, a1/2, a2/3, a3/4, a4/5, a5 (canonical) */
    double* cp_c;  /* [K][2][5] cp/R coefficients (canonical) */
    double* g_c;   /* [K][2][7] Gibbs0_RT coefficients (canonical only for one-piece species) */
    double* dtE_c; /* [A] canonical 1 - W_k/W_bulk */
    double M3, CBRT, C0c, rcpC0c, ln10_04, ln10_075;
    int err; char msg[256];
    /* transport */
    int has_transport; double T0, mu0, lambda0;
    double* tc_cond; double* tc_visc; double* tc_diff; /* scaled + canonical [K][5], [K][5], [K*K][5] */
    double* wilke_va; double* wilke_b;                 /* [K][K] canonical Va_kj (add) and b_kj (mul) */
    double* W_c;                                       /* canonical molar masses (mul) */
};

static void fail(or_mech* m, const char* s) {
    if (!m->err) { m->err = 1; snprintf(m->msg, sizeof m->msg, "%s", s); }
}

static void arrh_build(arrh_t* a, double A, double b, double Ea) {
    double br;
    /* reaction.rs:117-125 */
    if (b <= -1.5) { a->factor = F_RCPT2; br = b + 2.; }
    else if (b <= -0.5) { a->factor = F_RCPT; br = b + 1.; }
    else if (b >= 3.5) { a->factor = F_T4; br = b - 4.; }
    else if (b >= 2.5) { a->factor = F_T3; br = b - 3.; }
    else if (b >= 1.5) { a->factor = F_T2; br = b - 2.; }
    else if (b >= 0.5) { a->factor = F_T; br = b - 1.; }
    else { a->factor = F_NONE; br = b; }
    a->beta = (as_f32(br) != 0.0f) ? canon_mul(br) : 0.0; /* (f32)b'==1 gives lnT itself: canon 1 */
    a->mEa = (Ea != 0.0) ? canon_mul(-Ea) : 0.0;
    a->has_x = (a->beta != 0.0) || (a->mEa != 0.0);
    a->lnA = canon_add(log(A));
    a->A = a->factor ? canon_mul(A) : A;
}

typedef struct { double lnT, T, T2, T3, T4, rcpT, rcpT2; } temps_t;

static double factor_value(int f, const temps_t* t) {
    switch (f) {
    case F_RCPT2: return t->rcpT2; case F_RCPT: return t->rcpT; case F_T4: return t->T4;
    case F_T3: return t->T3; case F_T2: return t->T2; case F_T: return t->T; default: return 1.0;
    }
}

static double arrh_eval(const arrh_t* a, const temps_t* t) {
    double k;
    if (a->has_x) {
        double x;
        if (a->beta != 0.0 && a->mEa != 0.0) x = a->beta * t->lnT + a->mEa * t->rcpT;
        else if (a->beta != 0.0) x = a->beta * t->lnT;
        else x = a->mEa * t->rcpT;
        if (a->lnA != 0.0) x = x + a->lnA;
        double e = exp(x);
        k = a->factor ? factor_value(a->factor, t) * e : e;
    } else {
        k = a->factor ? factor_value(a->factor, t) * a->A : a->A;
    }
    return fmin(F32MAX, k); /* min(f32::MAX, k): NaN-ignoring like f64::min */
}

static double* dupd(const double* p, size_t n) {
    double* q = malloc(n * sizeof *q);
    if (p) memcpy(q, p, n * sizeof *q); else memset(q, 0, n * sizeof *q);
    return q;
}

or_mech* or_mech_new(int K, int R, const double* molar_mass, const double* nasa7_split, const double* nasa7,
                     const int32_t* geometry, const double* diameter, const double* well_depth,
                     const double* polarizability, const double* dipole, const double* rotational_relaxation,
                     const uint8_t* reactants, const uint8_t* products, const int32_t* model, const double* rate,
                     const double* k0, const double* troe, const double* sri, const double* efficiencies) {
    or_mech* m = calloc(1, sizeof *m);
    m->K = K; m->R = R;
    m->molar_mass = dupd(molar_mass, K); m->split = dupd(nasa7_split, K); m->nasa7 = dupd(nasa7, (size_t)K * 14);
    m->geometry = malloc(K * sizeof(int32_t)); memcpy(m->geometry, geometry, K * sizeof(int32_t));
    m->diameter = dupd(diameter, K); m->well_depth = dupd(well_depth, K); m->polarizability = dupd(polarizability, K);
    m->dipole = dupd(dipole, K); m->rot = dupd(rotational_relaxation, K);
    m->dof = malloc(K * sizeof(double));
    for (int k = 0; k < K; k++) m->dof[k] = geometry[k] == 0 ? 0. : geometry[k] == 1 ? 1. : 3. / 2.; /* lib.rs:58 */
    m->reactants = malloc((size_t)R * K); memcpy(m->reactants, reactants, (size_t)R * K);
    m->products = malloc((size_t)R * K); memcpy(m->products, products, (size_t)R * K);
    m->model = malloc(R * sizeof(int32_t)); memcpy(m->model, model, R * sizeof(int32_t));
    m->rate = dupd(rate, (size_t)R * 3); m->k0 = dupd(k0, (size_t)R * 3); m->troe = dupd(troe, (size_t)R * 4);
    m->sri = dupd(sri, (size_t)R * 5); m->eff = dupd(efficiencies, (size_t)R * K);

    /* active species: prefix of species whose amount some reaction changes (lib.rs:130-135) */
    int A = 0;
    {
        int* changes = calloc(K, sizeof(int));
        for (int r = 0; r < R; r++)
            for (int k = 0; k < K; k++)
                if (reactants[(size_t)r * K + k] != products[(size_t)r * K + k]) changes[k] = 1;
        while (A < K && changes[A]) A++;
        for (int k = A; k < K; k++) if (changes[k]) fail(m, "active species do not form a prefix");
        free(changes);
    }
    m->A = A;
    if (A == 0 || A == K) fail(m, "the mechanism needs at least one active and one inert (bulk) species");

    m->M3 = 0; {
        float mx = cbrtf(FLT_MAX); /* reaction.rs:244-251, in f32 arithmetic */
        while (mx * mx * mx > FLT_MAX) mx = nextafterf(mx, -INFINITY);
        m->M3 = (double)mx;
    }
    m->CBRT = (double)cbrtf(FLT_MAX);
    const double P0 = 101325. / RGAS; /* NASA7::reference_pressure, lib.rs:14 */
    m->C0c = canon_mul(P0);
    m->rcpC0c = canon_mul(1. / P0);
    m->ln10_04 = 0.4 * log(10.);
    m->ln10_075 = 0.75 * log(10.);

    m->rx = calloc(R, sizeof(reaction_t));
    for (int r = 0; r < R; r++) {
        reaction_t* x = &m->rx[r];
        const double* rc = &m->rate[r * 3];
        x->model = model[r];
        const uint8_t* re = &reactants[(size_t)r * K];
        const uint8_t* pr = &products[(size_t)r * K];
        x->r_k = malloc(K * sizeof(int)); x->r_n = malloc(K * sizeof(int));
        x->p_k = malloc(K * sizeof(int)); x->p_n = malloc(K * sizeof(int));
        x->net_k = malloc(K * sizeof(int)); x->net_n = malloc(K * sizeof(int));
        int sr = 0, sp = 0;
        for (int k = 0; k < K; k++) {
            if (re[k]) { x->r_k[x->n_r] = k; x->r_n[x->n_r++] = re[k]; }
            if (pr[k]) { x->p_k[x->n_p] = k; x->p_n[x->n_p++] = pr[k]; }
            sr += re[k]; sp += pr[k];
            if (k < A && pr[k] != re[k]) { x->net_k[x->n_net] = k; x->net_n[x->n_net++] = (int)pr[k] - (int)re[k]; }
        }
        x->sigma_net = sp - sr;
        if (x->n_r == 0) fail(m, "reaction without reactants");
        if (x->model != IRREVERSIBLE) {
            if (x->n_p == 0) fail(m, "reversible reaction without products");
            if (x->n_net == 0) fail(m, "reversible reaction without net change of an active species");
            if (-x->sigma_net < -2 || -x->sigma_net > 1) fail(m, "unsupported net order (reaction.rs:298-303)");
        }
        if (x->model == THREE_BODY || x->model == LINDEMANN || x->model == TROE || x->model == SRI) {
            const double* e = &m->eff[(size_t)r * K];
            x->eff_k = malloc(K * sizeof(int)); x->eff_c = malloc(K * sizeof(double));
            for (int k = 0; k < K; k++) {
                if (e[k] == 1.) continue;           /* reaction.rs:143 */
                double c = e[k] - 1.;
                double cc = (c == 1.) ? 0.0 : canon_mul(c); /* 0.0 marks "plain C_k" */
                if (c != 1. && cc == 1.) cc = 0.0;  /* (f32)(e-1)==1: the builder yields C_k itself */
                if (c != 1. && as_f32(c) == 0.0f) continue; /* the reference would panic; no term */
                x->eff_k[x->n_eff] = k; x->eff_c[x->n_eff++] = cc;
            }
        }
        if (x->model == TROE) {
            const double* kk0 = &m->k0[r * 3];
            double ainf = rc[0];
            arrh_build(&x->k0, kk0[0] / ainf, kk0[1], kk0[2]); /* reaction.rs:163-170 */
            x->kinf_const = (rc[1] == 0. && rc[2] == 0.);
            if (!x->kinf_const) arrh_build(&x->k, 1.0, rc[1], rc[2]);
            x->ainf = canon_mul(ainf);
            const double* t = &m->troe[r * 4];
            double Atroe = t[0], T3 = t[1], T1 = t[2], T2 = t[3];
            x->troe_1mA = canon_mul(1. - Atroe);
            x->troe_c3 = canon_mul(1. / (-T3));
            x->troe_t1 = T1 < 1e30;
            x->troe_A = x->troe_t1 ? canon_mul(Atroe) : canon_add(Atroe);
            x->troe_c1 = canon_mul(1. / (-T1));
            x->troe_t2 = isfinite(T2);
            x->troe_mT2 = canon_mul(-T2);
            /* Fcent is a constant when neither exponential term survives */
            x->fcent_const = (x->troe_1mA == 0.0) && !x->troe_t1 && !x->troe_t2;
            if (x->fcent_const) x->fcent_value = x->troe_A;
        } else if (x->model == LINDEMANN) {
            arrh_build(&x->k0, m->k0[r * 3], m->k0[r * 3 + 1], m->k0[r * 3 + 2]);
            arrh_build(&x->k, rc[0], rc[1], rc[2]);
        } else if (x->model == SRI) {
            /* the reference leaves SRI unimplemented; its commented formula (reaction.rs:194-203) uses
               the unscaled k0 and k_inf and F = D (A exp(-B/T) + exp(-T/C))^(1/(1 + ln(Pr)^2)) T^E */
            const double* s = &m->sri[r * 5];
            if (!(s[2] != 0.) || !(s[3] > 0.)) fail(m, "SRI needs C != 0 and D > 0");
            arrh_build(&x->k0, m->k0[r * 3], m->k0[r * 3 + 1], m->k0[r * 3 + 2]);
            arrh_build(&x->k, rc[0], rc[1], rc[2]);
            x->sri_A = canon_mul(s[0]);
            x->sri_mB = canon_mul(-s[1]);
            x->sri_mrC = canon_mul(-1. / s[2]);
            x->sri_D = canon_mul(s[3]);
            x->sri_E = canon_mul(s[4]);
        } else {
            arrh_build(&x->k, rc[0], rc[1], rc[2]);
        }
    }

    /* thermodynamic constants (reaction.rs:75-81) */
    m->h_c = calloc((size_t)K * 12, sizeof(double));
    m->cp_c = calloc((size_t)K * 10, sizeof(double));
    m->g_c = calloc((size_t)K * 14, sizeof(double));
    for (int k = 0; k < K; k++) {
        for (int p = 0; p < 2; p++) {
            const double* a = &m->nasa7[k * 14 + p * 7];
            double* h = &m->h_c[k * 12 + p * 6];
            h[0] = canon_add(a[0]); h[1] = canon_mul(a[1] / 2.); h[2] = canon_mul(a[2] / 3.);
            h[3] = canon_mul(a[3] / 4.); h[4] = canon_mul(a[4] / 5.); h[5] = canon_mul(a[5]);
            double* c = &m->cp_c[k * 10 + p * 5];
            c[0] = canon_add(a[0]);
            for (int i = 1; i < 5; i++) c[i] = canon_mul(a[i]);
            double* g = &m->g_c[k * 14 + p * 7];
            double gr[7] = {a[0] - a[6], -a[0], -a[1] / 2., (1. / 3. - 1. / 2.) * a[2], (1. / 4. - 1. / 3.) * a[3],
                            (1. / 5. - 1. / 4.) * a[4], a[5]};
            int one_piece = isnan(m->split[k]);
            for (int i = 0; i < 7; i++) g[i] = one_piece ? (i == 0 ? canon_add(gr[i]) : canon_mul(gr[i])) : gr[i];
        }
    }
    m->dtE_c = calloc(K, sizeof(double));
    for (int k = 0; k < A; k++) m->dtE_c[k] = canon_mul(1. - m->molar_mass[k] / m->molar_mass[K - 1]);
    m->W_c = calloc(K, sizeof(double));
    for (int k = 0; k < K; k++) m->W_c[k] = canon_mul(m->molar_mass[k]);
    return m;
}

void or_mech_free(or_mech* m) {
    if (!m) return;
    for (int r = 0; r < m->R; r++) {
        reaction_t* x = &m->rx[r];
        free(x->r_k); free(x->r_n); free(x->p_k); free(x->p_n); free(x->net_k); free(x->net_n);
        free(x->eff_k); free(x->eff_c);
    }
    free(m->rx);
    free(m->molar_mass); free(m->split); free(m->nasa7); free(m->geometry); free(m->diameter); free(m->well_depth);
    free(m->polarizability); free(m->dipole); free(m->rot); free(m->dof); free(m->reactants); free(m->products);
    free(m->model); free(m->rate); free(m->k0); free(m->troe); free(m->sri); free(m->eff); free(m->h_c);
    free(m->cp_c); free(m->g_c); free(m->dtE_c); free(m->W_c);
    free(m->tc_cond); free(m->tc_visc); free(m->tc_diff); free(m->wilke_va); free(m->wilke_b);
    free(m);
}

int or_active(const or_mech* m) { return m->A; }

int or_check(const or_mech* m, char* msg, size_t len) {
    if (m->err && msg && len) snprintf(msg, len, "%s", m->msg);
    return m->err;
}

/* ---- rates (reaction.rs:207-327, 356-391) -------------------------------------------------- */
static int piece(const or_mech* m, int k, double T) { return (T <= m->split[k]) ? 0 : 1; } /* lib.rs:15 */

static double gibbs_RT(const or_mech* m, int k, const temps_t* t) {
    /* thermodynamic(): ((((((g0 + g1 lnT) + g2 T) + g3 T2) + g4 T3) + g5 T4) + g6 rcpT) */
    const double* g = &m->g_c[k * 14 + (isnan(m->split[k]) ? 0 : piece(m, k, t->T)) * 7];
    double s = g[0];
    s = s + g[1] * t->lnT; s = s + g[2] * t->T; s = s + g[3] * t->T2; s = s + g[4] * t->T3;
    s = s + g[5] * t->T4; s = s + g[6] * t->rcpT;
    return s;
}

static double enthalpy_RT(const or_mech* m, int k, const temps_t* t) {
    const double* h = &m->h_c[k * 12 + (isnan(m->split[k]) ? 0 : piece(m, k, t->T)) * 6];
    double s = h[0];
    if (h[1] != 0.) s = s + h[1] * t->T;
    if (h[2] != 0.) s = s + h[2] * t->T2;
    if (h[3] != 0.) s = s + h[3] * t->T3;
    if (h[4] != 0.) s = s + h[4] * t->T4;
    if (h[5] != 0.) s = s + h[5] * t->rcpT;
    return s;
}

static double cp_R(const or_mech* m, int k, const temps_t* t) {
    const double* c = &m->cp_c[k * 10 + (isnan(m->split[k]) ? 0 : piece(m, k, t->T)) * 5];
    double s = c[0];
    if (c[1] != 0.) s = s + c[1] * t->T;
    if (c[2] != 0.) s = s + c[2] * t->T2;
    if (c[3] != 0.) s = s + c[3] * t->T3;
    if (c[4] != 0.) s = s + c[4] * t->T4;
    return s;
}

typedef struct {
    temps_t t;
    double C;      /* total concentration */
    double* Ck;    /* [K] concentrations, bulk last */
    double* ex; double* exn; char* has_ex; char* has_exn; /* Gibbs exponential caches */
} cell_t;

static double efficiency(const reaction_t* x, const cell_t* c) {
    /* reaction.rs:141-145: C + (((t0 + t1) + t2) + ...) */
    if (x->n_eff == 0) return c->C;
    double s = 0.;
    for (int i = 0; i < x->n_eff; i++) {
        double ck = c->Ck[x->eff_k[i]];
        double term = (x->eff_c[i] == 0.0) ? ck : x->eff_c[i] * ck;
        s = (i == 0) ? term : s + term;
    }
    return c->C + s;
}

static double prod_pow(const int* ks, const int* ns, int n, const double* C) {
    /* product_of_exponentiations (reaction.rs:53-63): repeated multiplication, species order */
    double p = 0.; int first = 1;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < ns[i]; j++) {
            if (first) { p = C[ks[i]]; first = 0; } else p = p * C[ks[i]];
        }
    return p;
}

/* cR of one reaction (reaction.rs:269-309). mag receives |cR_forward| + |cR_reverse|. */
static double reaction_cR(const or_mech* m, const reaction_t* x, cell_t* c, double* mag) {
    const temps_t* t = &c->t;
    double n, d = 1.0; int has_d = 0;
    switch (x->model) {
    case ELEMENTARY: case IRREVERSIBLE:
        n = arrh_eval(&x->k, t);
        break;
    case THREE_BODY:
        n = arrh_eval(&x->k, t) * efficiency(x, c);
        break;
    case LINDEMANN: {
        double M = efficiency(x, c);
        double k0 = arrh_eval(&x->k0, t);
        double Ck0 = M * k0;
        double kinf = arrh_eval(&x->k, t);
        n = Ck0 * kinf;
        d = (Ck0 + kinf) + F32MINPOS; has_d = 1;
        break;
    }
    case TROE: {
        double M = efficiency(x, c);
        double k0 = arrh_eval(&x->k0, t);
        double Pr, kinf_e;
        if (x->kinf_const) { Pr = M * k0; kinf_e = x->ainf; }
        else {
            double kinf = arrh_eval(&x->k, t);
            Pr = (M * k0) / (kinf + F32MINPOS);
            kinf_e = x->ainf * kinf;
        }
        double lnFcent;
        if (x->fcent_const) lnFcent = log(x->fcent_value);
        else {
            double F = 0.; int first = 1;
            if (x->troe_1mA != 0.) { double e = x->troe_1mA * exp(t->T * x->troe_c3); F = e; first = 0; }
            if (x->troe_t1) {
                if (x->troe_A != 0.) { double e = x->troe_A * exp(t->T * x->troe_c1); F = first ? e : F + e; first = 0; }
            } else if (x->troe_A != 0.) { F = first ? x->troe_A : F + x->troe_A; first = 0; }
            if (x->troe_t2) { double e = exp(x->troe_mT2 * t->rcpT); F = first ? e : F + e; first = 0; }
            lnFcent = log(F);
        }
        double Cc = -0.67 * lnFcent - m->ln10_04;
        double Nn = -1.27 * lnFcent + m->ln10_075;
        double lnPrC = log(Pr + F32MINPOS) + Cc;
        double f1 = lnPrC / (-0.14 * lnPrC + Nn);
        double Fb = exp(lnFcent / (f1 * f1 + 1.));
        n = (Fb * kinf_e) * Pr;
        d = Pr + 1.; has_d = 1;
        break;
    }
    case SRI: {
        double M = efficiency(x, c);
        double k0 = arrh_eval(&x->k0, t);
        double kinf = arrh_eval(&x->k, t);
        double Pr = (M * k0) / (kinf + F32MINPOS);
        double lP = log(Pr + F32MINPOS);
        double base = exp(x->sri_mrC * t->T);
        if (x->sri_A != 0.) base = x->sri_A * exp(x->sri_mB * t->rcpT) + base;
        double F = exp(log(base) * (1. / (1. + lP * lP)));
        if (x->sri_D != 1.) F = x->sri_D * F;
        if (x->sri_E != 0.) F = F * exp(x->sri_E * t->lnT);
        n = (F * kinf) * Pr;
        d = Pr + 1.; has_d = 1;
        break;
    }
    default:
        *mag = NAN; return NAN;
    }
    double Rf = prod_pow(x->r_k, x->r_n, x->n_r, c->Ck);
    double Rnet, RrK = 0.;
    if (x->model == IRREVERSIBLE) Rnet = Rf;
    else {
        double p = 0.; int first = 1;
        for (int i = 0; i < x->n_net; i++) {
            int k = x->net_k[i], nu = x->net_n[i];
            double tt;
            if (nu > 0) {
                if (!c->has_ex[k]) { c->ex[k] = fmin(m->M3, exp(gibbs_RT(m, k, t))); c->has_ex[k] = 1; }
                tt = c->ex[k];
            } else {
                if (!c->has_exn[k]) { c->exn[k] = fmin(m->CBRT, exp(-gibbs_RT(m, k, t))); c->has_exn[k] = 1; }
                tt = c->exn[k];
            }
            for (int j = 0; j < abs(nu); j++) { if (first) { p = tt; first = 0; } else p = p * tt; }
        }
        double rK;
        switch (-x->sigma_net) {
        case 0: rK = p; break;
        case 1: rK = (m->C0c * t->rcpT) * p; break;
        case -1: rK = (m->rcpC0c * t->T) * p; break;
        default: { double rc0 = m->rcpC0c * t->T; rK = (rc0 * rc0) * p; }
        }
        double Rr = prod_pow(x->p_k, x->p_n, x->n_p, c->Ck);
        RrK = rK * Rr;
        Rnet = Rf - RrK;
    }
    double cR = has_d ? (Rnet * n) / d : Rnet * n;
    if (mag) *mag = fabs(has_d ? (Rf * n) / d : Rf * n) + fabs(has_d ? (RrK * n) / d : RrK * n);
    return cR;
}

static void cell_prologue(const or_mech* m, double pressure_R, double T, double V, const double* n, cell_t* c) {
    int K = m->K;
    double md = 1. / V;
    c->t.rcpT = 1. / T;
    c->t.lnT = log(T);
    c->t.T = T;
    c->t.T2 = T * T;
    for (int k = 0; k < K - 1; k++) c->Ck[k] = md * fmax(0., n[k]);
    c->t.T3 = T * c->t.T2;
    c->C = pressure_R * c->t.rcpT;
    c->t.rcpT2 = c->t.rcpT * c->t.rcpT;
    c->t.T4 = c->t.T2 * c->t.T2;
    double s = 0.;
    for (int k = 0; k < K - 1; k++) s = (k == 0) ? c->Ck[k] : s + c->Ck[k];
    c->Ck[K - 1] = c->C - s;
    memset(c->has_ex, 0, K); memset(c->has_exn, 0, K);
}

typedef struct { double* Ck; double* ex; double* exn; char* has_ex; char* has_exn; double* wdot; double* wmag;
                 char* winit; double* cR; double* cRmag; } work_t;

static void work_alloc(const or_mech* m, work_t* w) {
    int K = m->K, R = m->R;
    w->Ck = malloc(K * sizeof(double)); w->ex = malloc(K * sizeof(double)); w->exn = malloc(K * sizeof(double));
    w->has_ex = malloc(K); w->has_exn = malloc(K); w->wdot = malloc(K * sizeof(double));
    w->wmag = malloc(K * sizeof(double)); w->winit = malloc(K); w->cR = malloc(R * sizeof(double));
    w->cRmag = malloc(R * sizeof(double));
}
static void work_free(work_t* w) {
    free(w->Ck); free(w->ex); free(w->exn); free(w->has_ex); free(w->has_exn); free(w->wdot); free(w->wmag);
    free(w->winit); free(w->cR); free(w->cRmag);
}

static void rates_cell(const or_mech* m, const double* in, double* out, double* scale, work_t* w) {
    int K = m->K, A = m->A;
    cell_t c = {.Ck = w->Ck, .ex = w->ex, .exn = w->exn, .has_ex = w->has_ex, .has_exn = w->has_exn};
    double pressure_R = in[0], rcp_pressure_R = in[1], T = in[2], V = in[3];
    cell_prologue(m, pressure_R, T, V, in + 4, &c);
    memset(w->winit, 0, A);
    for (int k = 0; k < A; k++) w->wmag[k] = 0.;
    for (int r = 0; r < m->R; r++) {
        const reaction_t* x = &m->rx[r];
        double mag;
        double cR = reaction_cR(m, x, &c, &mag);
        for (int i = 0; i < x->n_net; i++) {
            int k = x->net_k[i], nu = x->net_n[i];
            double s = w->wdot[k];
            if (nu == 1) s = w->winit[k] ? s + cR : cR;
            else if (nu == -1) s = w->winit[k] ? s - cR : -cR;
            else { double v = (double)nu * cR; s = w->winit[k] ? s + v : v; }
            w->wdot[k] = s; w->winit[k] = 1;
            w->wmag[k] += abs(nu) * mag;
        }
    }
    /* energy (reaction.rs:375-384) */
    double E = 0., Emag = 0.;
    for (int k = 0; k < A; k++) {
        double h = enthalpy_RT(m, k, &c.t);
        double term = w->wdot[k] * h;
        E = (k == 0) ? term : E + term;
        Emag += w->wmag[k] * fabs(h);
    }
    double Cp = 0., Cpmag = 0.;
    for (int k = 0; k < K; k++) {
        double term = cp_R(m, k, &c.t) * c.Ck[k];
        Cp = (k == 0) ? term : Cp + term;
        Cpmag += fabs(term);
    }
    double dtT_T = -E / Cp;
    double dtE = 0., dtEmag = 0.; int first = 1;
    for (int k = 0; k < A; k++) {
        if (m->dtE_c[k] == 0.) continue;
        double term = m->dtE_c[k] * w->wdot[k];
        dtE = first ? term : dtE + term; first = 0;
        dtEmag += fabs(m->dtE_c[k]) * w->wmag[k];
    }
    double dtV = V * (dtT_T + rcp_pressure_R * T * dtE);
    out[0] = T * dtT_T;
    out[1] = dtV;
    for (int k = 0; k < A; k++) out[2 + k] = w->wdot[k];
    if (scale) {
        double sT = Emag / fabs(Cp); /* |dT/dt / T| bound */
        scale[0] = fabs(T) * sT;
        scale[1] = fabs(V) * (sT + fabs(rcp_pressure_R * T) * dtEmag);
        for (int k = 0; k < A; k++) scale[2 + k] = w->wmag[k];
        (void)Cpmag;
    }
}

void or_rates(const or_mech* m, const double* in, double* out, double* scale) {
    work_t w; work_alloc(m, &w);
    rates_cell(m, in, out, scale, &w);
    work_free(&w);
}

static void reaction_rates_cell(const or_mech* m, const double* in, double* out, double* scale, work_t* w) {
    cell_t c = {.Ck = w->Ck, .ex = w->ex, .exn = w->exn, .has_ex = w->has_ex, .has_exn = w->has_exn};
    cell_prologue(m, in[0], in[1], in[2], in + 3, &c);
    for (int r = 0; r < m->R; r++) {
        double mag;
        out[r] = reaction_cR(m, &m->rx[r], &c, &mag);
        if (scale) scale[r] = mag;
    }
}

void or_reaction_rates(const or_mech* m, const double* in, double* out) {
    work_t w; work_alloc(m, &w);
    reaction_rates_cell(m, in, out, NULL, &w);
    work_free(&w);
}

/* ---- transport physics (transport.rs:14-117) ---------------------------------------------- */
static double sq(double x) { return x * x; }
static double cb(double x) { return x * x * x; }

static const double fine_structure = 7.2973525693e-3, Planck = 6.62607015e-34, electron_charge = 1.602176634e-19,
                    light_speed = 299792458.;
static double mu0_vac(void) { return 2. * fine_structure * Planck / (electron_charge * electron_charge * light_speed); }
static double eps0_vac(void) { return 1. / (light_speed * light_speed * mu0_vac()); }

/* Householder least squares in long double: minimise |A x - b|, A m x n row-major (m >= n). */
static void lsq(int mm, int n, const double* A, const double* b, double* x) {
    long double* Q = malloc(sizeof(long double) * mm * n);
    long double* y = malloc(sizeof(long double) * mm);
    for (int i = 0; i < mm * n; i++) Q[i] = A[i];
    for (int i = 0; i < mm; i++) y[i] = b[i];
    for (int j = 0; j < n; j++) {
        long double nrm = 0;
        for (int i = j; i < mm; i++) nrm += Q[i * n + j] * Q[i * n + j];
        nrm = sqrtl(nrm);
        long double alpha = Q[j * n + j] > 0 ? -nrm : nrm;
        long double v0 = Q[j * n + j] - alpha;
        /* v = (v0, Q[j+1..][j]) ; H = I - 2 v v^T / (v^T v) */
        long double vtv = v0 * v0;
        for (int i = j + 1; i < mm; i++) vtv += Q[i * n + j] * Q[i * n + j];
        if (vtv == 0) continue;
        for (int c = j + 1; c < n; c++) {
            long double s = v0 * Q[j * n + c];
            for (int i = j + 1; i < mm; i++) s += Q[i * n + j] * Q[i * n + c];
            s = 2 * s / vtv;
            Q[j * n + c] -= s * v0;
            for (int i = j + 1; i < mm; i++) Q[i * n + c] -= s * Q[i * n + j];
        }
        long double s = v0 * y[j];
        for (int i = j + 1; i < mm; i++) s += Q[i * n + j] * y[i];
        s = 2 * s / vtv;
        y[j] -= s * v0;
        for (int i = j + 1; i < mm; i++) y[i] -= s * Q[i * n + j];
        Q[j * n + j] = alpha;
    }
    for (int j = n - 1; j >= 0; j--) {
        long double s = y[j];
        for (int c = j + 1; c < n; c++) s -= Q[j * n + c] * (long double)x[c];
        x[j] = (double)(s / Q[j * n + j]);
    }
    free(Q); free(y);
}

/* Degree-6 fits of each T* row over delta*, truncated to degree 5 (transport.rs:48-51). */
static double omega22_fit[37][6], astar_fit[39][6];
static pthread_once_t fit_once = PTHREAD_ONCE_INIT;
static void fit_rows(int n, const double (*table)[8], double (*fit)[6]) {
    for (int r = 0; r < n; r++) {
        double A[8 * 7], x[7];
        for (int i = 0; i < 8; i++) { double p = 1.; for (int k = 0; k < 7; k++) { A[i * 7 + k] = p; p *= cb_header_delta[i]; } }
        lsq(8, 7, A, table[r], x);
        for (int k = 0; k < 6; k++) fit[r][k] = x[k];
    }
}
static void init_fits(void) { fit_rows(37, cb_omega22, omega22_fit); fit_rows(39, cb_astar, astar_fit); }

static double chi(const or_mech* m, int a, int b) {
    if ((m->dipole[a] > 0.) == (m->dipole[b] > 0.)) return 1.;
    int polar = m->dipole[a] != 0. ? a : b, non_polar = m->dipole[a] != 0. ? b : a;
    return 1. + 1. / 4. * m->polarizability[non_polar] / cb(m->diameter[non_polar]) *
                    sq(m->dipole[polar] / sqrt(4. * M_PI * eps0_vac() * m->well_depth[polar] * cb(m->diameter[polar]))) *
                    sqrt(m->well_depth[polar] / m->well_depth[non_polar]);
}
static double interaction_well_depth(const or_mech* m, int a, int b) {
    return sqrt(m->well_depth[a] * m->well_depth[b]) * sq(chi(m, a, b));
}
static double Tstar(const or_mech* m, int a, int b, double T) { return T * kB / interaction_well_depth(m, a, b); }
static double reduced_dipole(const or_mech* m, int a, int b) {
    return m->dipole[a] * m->dipole[b] /
           (8. * M_PI * eps0_vac() * sqrt(m->well_depth[a] * m->well_depth[b]) * cb((m->diameter[a] + m->diameter[b]) / 2.));
}
static double reduced_mass(const or_mech* m, int a, int b) {
    const double* W = m->molar_mass;
    return W[a] / NA * W[b] / NA / (W[a] / NA + W[b] / NA);
}
static double reduced_diameter(const or_mech* m, int a, int b) {
    return (m->diameter[a] + m->diameter[b]) / 2. * pow(chi(m, a, b), -1. / 6.);
}
static double quadratic_interpolation(const double x[3], const double y[3], double x0) {
    return ((x[1] - x[0]) * (y[2] - y[1]) - (y[1] - y[0]) * (x[2] - x[1])) / ((x[1] - x[0]) * (x[2] - x[0]) * (x[2] - x[1])) *
               (x0 - x[0]) * (x0 - x[1]) +
           ((y[1] - y[0]) / (x[1] - x[0])) * (x0 - x[1]) + y[1];
}
static double collision_integral(const or_mech* m, int I0, int N, const double (*table)[8], const double (*fit)[6],
                                 int a, int b, double T) {
    pthread_once(&fit_once, init_fits);
    double lnTs = log(Tstar(m, a, b, T));
    double hl[39];
    for (int i = 0; i < 39; i++) hl[i] = log(cb_header_Tstar[i]);
    int first = -1;
    for (int i = 1; i < 39; i++) if (lnTs < hl[i]) { first = i; break; }
    if (first < 0) return NAN; /* T* beyond the table: the reference panics (transport.rs:85) */
    int start = first - 1;
    if (start > I0 + N - 3) start = I0 + N - 3;
    if (start < I0) return NAN; /* below the table start: the reference's index underflows */
    double xs[3] = {hl[start], hl[start + 1], hl[start + 2]};
    if (!(xs[0] <= lnTs && lnTs <= xs[2])) return NAN;
    double ds = reduced_dipole(m, a, b);
    double y[3];
    for (int i = 0; i < 3; i++) {
        if (ds == 0.) y[i] = table[start - I0 + i][0];
        else {
            const double* P = fit[start - I0 + i];
            double s = 0., p = 1.;
            for (int k = 0; k < 6; k++) { s += P[k] * p; p *= ds; }
            y[i] = s;
        }
    }
    return quadratic_interpolation(xs, y, lnTs);
}
double or_omega22(const or_mech* m, int a, int b, double T) {
    return collision_integral(m, 1, 37, cb_omega22, (const double (*)[6])omega22_fit, a, b, T);
}
static double astar(const or_mech* m, int a, int b, double T) {
    return collision_integral(m, 0, 39, cb_astar, (const double (*)[6])astar_fit, a, b, T);
}
double or_viscosity(const or_mech* m, int k, double T) {
    return 5. / 16. * sqrt(M_PI * m->molar_mass[k] / NA * kB * T) / (or_omega22(m, k, k, T) * M_PI * sq(m->diameter[k]));
}
static double omega11(const or_mech* m, int a, int b, double T) { return or_omega22(m, a, b, T) / astar(m, a, b, T); }
double or_diffusivity(const or_mech* m, int a, int b, double T) {
    return 3. / 16. * sqrt(2. * M_PI / reduced_mass(m, a, b)) * pow(kB * T, 3. / 2.) /
           (M_PI * sq(reduced_diameter(m, a, b)) * omega11(m, a, b, T));
}
static double cp_R_T(const or_mech* m, int k, double T) { /* lib.rs:16 */
    const double* a = &m->nasa7[k * 14 + ((T <= m->split[k]) || isnan(m->split[k]) ? 0 : 1) * 7];
    return a[0] + a[1] * T + a[2] * T * T + a[3] * T * T * T + a[4] * T * T * T * T;
}
static double fz(double Ts) { return 1. + pow(M_PI, 3. / 2.) / sqrt(Ts) * (1. / 2. + 1. / Ts) + (1. / 4. * sq(M_PI) + 2.) / Ts; }
double or_conductivity(const or_mech* m, int k, double T) {
    double W = m->molar_mass[k];
    double f_internal = W / NA / (kB * T) * or_diffusivity(m, k, k, T) / or_viscosity(m, k, T);
    double c1 = 2. / M_PI * (5. / 2. - f_internal) /
                (m->rot[k] * fz(Tstar(m, k, k, 298.)) / fz(Tstar(m, k, k, T)) + 2. / M_PI * (5. / 3. * m->dof[k] + f_internal));
    double f_translation = 5. / 2. * (1. - c1 * m->dof[k] / (3. / 2.));
    double f_rotation = f_internal * (1. + c1);
    double Cv_internal = cp_R_T(m, k, T) - 5. / 2. - m->dof[k];
    return (or_viscosity(m, k, T) / (W / NA)) * kB * (f_translation * 3. / 2. + f_rotation * m->dof[k] + f_internal * Cv_internal);
}

int or_transport_samples(const or_mech* m, double T0, double* x, double* y_cond, double* y_visc, double* y_diff) {
    const int N = 50, K = m->K;
    for (int n = 0; n < N; n++) {
        double T = 300. + (double)n / (double)(N - 1) * (3000. - 300.);
        x[n] = log(T / T0);
        for (int k = 0; k < K; k++) {
            if (y_cond) y_cond[k * N + n] = or_conductivity(m, k, T) / sqrt(T);
            if (y_visc) y_visc[k * N + n] = sqrt(or_viscosity(m, k, T) / sqrt(T));
        }
        if (y_diff)
            for (int k = 0; k < K; k++)
                for (int j = 0; j < K; j++) y_diff[((size_t)k * K + j) * N + n] = or_diffusivity(m, k, j, T) / (T * sqrt(T));
    }
    return 0;
}

static void fit_one(const double* x, const double* y, double* P) {
    /* regression(): weights 1/y^2 on the rows of the Vandermonde system (transport.rs:24-34) */
    double A[50 * 5], b[50];
    for (int n = 0; n < 50; n++) {
        double w = 1. / sq(y[n]);
        double p = 1.;
        for (int k = 0; k < 5; k++) { A[n * 5 + k] = w * p; p *= x[n]; }
        b[n] = w * y[n];
    }
    lsq(50, 5, A, b, P);
}

int or_transport_fit(const or_mech* m, double T0, double* cond, double* visc, double* diff) {
    int K = m->K;
    double x[50];
    double* yc = malloc(sizeof(double) * K * 50);
    double* yv = malloc(sizeof(double) * K * 50);
    double* yd = malloc(sizeof(double) * (size_t)K * K * 50);
    or_transport_samples(m, T0, x, yc, yv, yd);
    for (int k = 0; k < K; k++) { fit_one(x, yc + k * 50, cond + k * 5); fit_one(x, yv + k * 50, visc + k * 5); }
    for (size_t p = 0; p < (size_t)K * K; p++) fit_one(x, yd + p * 50, diff + p * 5);
    free(yc); free(yv); free(yd);
    return 0;
}

void or_set_transport(or_mech* m, double T0, double viscosity0, double conductivity0, const double* cond,
                      const double* visc, const double* diff) {
    int K = m->K;
    m->has_transport = 1; m->T0 = T0; m->mu0 = viscosity0; m->lambda0 = conductivity0;
    free(m->tc_cond); free(m->tc_visc); free(m->tc_diff); free(m->wilke_va); free(m->wilke_b);
    m->tc_cond = malloc(sizeof(double) * K * 5); m->tc_visc = malloc(sizeof(double) * K * 5);
    m->tc_diff = malloc(sizeof(double) * (size_t)K * K * 5);
    double sv = sqrt(sqrt(T0)) / sqrt(viscosity0), sc = sqrt(T0) / (2. * conductivity0), sd = sqrt(T0) / (RGAS * viscosity0);
    for (int k = 0; k < K * 5; k++) {
        double c = sc * cond[k], v = sv * visc[k];
        m->tc_cond[k] = (k % 5 == 0) ? canon_add(c) : canon_mul(c);
        m->tc_visc[k] = (k % 5 == 0) ? canon_add(v) : canon_mul(v);
    }
    for (size_t p = 0; p < (size_t)K * K * 5; p++) { double d = sd * diff[p]; m->tc_diff[p] = (p % 5 == 0) ? canon_add(d) : canon_mul(d); }
    m->wilke_va = malloc(sizeof(double) * K * K); m->wilke_b = malloc(sizeof(double) * K * K);
    const double* W = m->molar_mass;
    for (int k = 0; k < K; k++)
        for (int j = 0; j < K; j++) {
            double Va = sqrt(1. / sqrt(8.) * 1. / sqrt(1. + W[k] / W[j])); /* transport.rs:154 */
            m->wilke_va[k * K + j] = canon_add(Va);
            m->wilke_b[k * K + j] = canon_mul(Va * sqrt(sqrt(W[j] / W[k])));
        }
}

static double poly5(const double* P, const double* L) {
    /* P.dot(lnT): ((((p0 + p1 L1) + p2 L2) + p3 L3) + p4 L4), zero terms dropped */
    double s = P[0];
    for (int i = 1; i < 5; i++) if (P[i] != 0.) s = s + P[i] * L[i];
    return s;
}

static void transport_cell(const or_mech* m, const double* in, double* out, double* scale, double* X, double* v,
                           double* rv, double* S, char* Sinit) {
    int K = m->K;
    double N = in[0], T = in[1];
    double lnT = log(T);
    double L[5];
    L[0] = 1.; L[1] = lnT; L[2] = L[1] * lnT; L[3] = L[2] * lnT; L[4] = L[3] * lnT;
    double s = 0.;
    for (int k = 0; k < K - 1; k++) { X[k] = in[2 + k]; s = (k == 0) ? X[k] : s + X[k]; }
    X[K - 1] = N - s;
    double VT = sqrt(T);
    double MN = 0.; int first = 1;
    for (int k = 0; k < K; k++) {
        if (m->W_c[k] == 0.) continue;
        double t = m->W_c[k] * X[k];
        MN = first ? t : MN + t; first = 0;
    }
    double MVTN = MN * VT;
    /* conductivityNIVT (transport.rs:141-146) */
    double Acc = 0., Bcc = 0.;
    for (int k = 0; k < K; k++) {
        double c = poly5(&m->tc_cond[k * 5], L);
        double a = X[k] * c, b = X[k] / c;
        if (k == 0) { Acc = a; Bcc = b; } else { Acc = Acc + a; Bcc = Bcc + b; }
    }
    out[0] = (Acc / N + N / Bcc) * VT;
    /* viscosityIVT (transport.rs:148-158) */
    for (int k = 0; k < K; k++) { v[k] = poly5(&m->tc_visc[k * 5], L); rv[k] = 1. / v[k]; }
    double mu = 0.;
    for (int k = 0; k < K; k++) {
        double den = 0.;
        for (int j = 0; j < K; j++) {
            double b = m->wilke_b[k * K + j], va = m->wilke_va[k * K + j];
            double q = (b * v[k]) * rv[j];
            double t = (va != 0.) ? va + q : q;
            double term = X[j] * (t * t);
            den = (j == 0) ? term : den + term;
        }
        double term = (X[k] * (v[k] * v[k])) / den;
        mu = (k == 0) ? term : mu + term;
    }
    out[1] = VT * mu;
    /* density_diffusivity (transport.rs:162-177) */
    for (int k = 0; k < K; k++) Sinit[k] = 0;
    for (int k = 0; k < K; k++)
        for (int j = 0; j < k; j++) {
            double y = poly5(&m->tc_diff[((size_t)k * K + j) * 5], L);
            double Rkj = 1. / y;
            double t = X[j] * Rkj;
            S[k] = Sinit[k] ? S[k] + t : t; Sinit[k] = 1;
            t = X[k] * Rkj;
            S[j] = Sinit[j] ? S[j] + t : t; Sinit[j] = 1;
        }
    for (int k = 0; k < K; k++) {
        double sub = (VT * m->W_c[k]) * X[k];
        out[2 + k] = (MVTN - sub) / S[k];
        if (scale) scale[2 + k] = (fabs(MVTN) + fabs(sub)) / fabs(S[k]);
    }
    if (scale) { scale[0] = fabs(out[0]); scale[1] = fabs(out[1]); }
}

void or_transport(const or_mech* m, const double* in, double* out, double* scale) {
    int K = m->K;
    double* X = malloc(sizeof(double) * K * 4);
    char* Si = malloc(K);
    transport_cell(m, in, out, scale, X, X + K, X + 2 * K, X + 3 * K, Si);
    free(X); free(Si);
}

/* ---- batches ------------------------------------------------------------------------------ */
typedef struct {
    const or_mech* m; size_t lo, hi; int kind;
    const double* const* in; double* const* out; double* const* scale; double* const* out2;
} job_t;

static void* run_job(void* p) {
    job_t* j = p;
    const or_mech* m = j->m;
    int K = m->K, A = m->A, R = m->R;
    work_t w; work_alloc(m, &w);
    double* tin = malloc(sizeof(double) * (K + 3));
    double* tout = malloc(sizeof(double) * (K + 2 > R ? K + 2 : R));
    double* tsc = malloc(sizeof(double) * (K + 2));
    double* X = malloc(sizeof(double) * K * 4);
    char* Si = malloc(K);
    double* tout2 = malloc(sizeof(double) * (K + 2));
    for (size_t i = j->lo; i < j->hi; i++) {
        if (j->kind == 0) { /* rates */
            for (int q = 0; q < K + 3; q++) tin[q] = j->in[q][i];
            rates_cell(m, tin, tout, j->scale ? tsc : NULL, &w);
            for (int q = 0; q < A + 2; q++) { j->out[q][i] = tout[q]; if (j->scale) j->scale[q][i] = tsc[q]; }
        } else if (j->kind == 1) { /* reaction rates */
            for (int q = 0; q < K + 2; q++) tin[q] = j->in[q][i];
            double* rsc = j->scale ? malloc(sizeof(double) * R) : NULL;
            reaction_rates_cell(m, tin, tout, rsc, &w);
            for (int q = 0; q < R; q++) { j->out[q][i] = tout[q]; if (rsc) j->scale[q][i] = rsc[q]; }
            free(rsc);
        } else if (j->kind == 2) { /* transport */
            for (int q = 0; q < K + 1; q++) tin[q] = j->in[q][i];
            transport_cell(m, tin, tout, j->scale ? tsc : NULL, X, X + K, X + 2 * K, X + 3 * K, Si);
            for (int q = 0; q < K + 2; q++) { j->out[q][i] = tout[q]; if (j->scale) j->scale[q][i] = tsc[q]; }
        } else { /* fused */
            for (int q = 0; q < K + 3; q++) tin[q] = j->in[q][i];
            rates_cell(m, tin, tout, NULL, &w);
            for (int q = 0; q < A + 2; q++) j->out[q][i] = tout[q];
            double tr[1];
            (void)tr;
            double* tin2 = tsc; /* reuse: K+1 entries */
            tin2[0] = (tin[0] * tin[3]) / tin[2];
            tin2[1] = tin[2] / m->T0;
            for (int q = 0; q < K - 1; q++) tin2[2 + q] = tin[4 + q];
            transport_cell(m, tin2, tout2, NULL, X, X + K, X + 2 * K, X + 3 * K, Si);
            for (int q = 0; q < K + 2; q++) j->out2[q][i] = tout2[q];
        }
    }
    free(tin); free(tout); free(tsc); free(X); free(Si); free(tout2);
    work_free(&w);
    return NULL;
}

static int run_batch(const or_mech* m, size_t n, int kind, const double* const* in, double* const* out,
                     double* const* scale, double* const* out2, int nthreads) {
    if (m->err) return 1;
    if ((kind == 2 || kind == 3) && !m->has_transport) return 2;
    if (nthreads < 1) nthreads = 1;
    if ((size_t)nthreads > n) nthreads = n ? (int)n : 1;
    pthread_t* th = malloc(sizeof(pthread_t) * nthreads);
    job_t* jobs = malloc(sizeof(job_t) * nthreads);
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = (job_t){m, n * t / nthreads, n * (t + 1) / nthreads, kind, in, out, scale, out2};
        if (nthreads == 1) run_job(&jobs[t]);
        else pthread_create(&th[t], NULL, run_job, &jobs[t]);
    }
    if (nthreads > 1) for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th); free(jobs);
    return 0;
}

int or_rates_batch(const or_mech* m, size_t n, const double* const* in, double* const* out, double* const* scale,
                   int nthreads) {
    return run_batch(m, n, 0, in, out, scale, NULL, nthreads);
}
int or_reaction_rates_batch(const or_mech* m, size_t n, const double* const* in, double* const* out,
                            double* const* scale, int nthreads) {
    return run_batch(m, n, 1, in, out, scale, NULL, nthreads);
}
int or_transport_batch(const or_mech* m, size_t n, const double* const* in, double* const* out, double* const* scale,
                       int nthreads) {
    return run_batch(m, n, 2, in, out, scale, NULL, nthreads);
}
int or_fused_batch(const or_mech* m, size_t n, const double* const* in, double* const* out_rates,
                   double* const* out_transport, int nthreads) {
    return run_batch(m, n, 3, in, out_rates, NULL, out_transport, nthreads);
}
