// Host side of a mechanism: validation, canonical constants, transport fits and packed tables.
#include "mechanism.hpp"

#include <cfloat>
#include <cmath>
#include <cstring>
#include <algorithm>
#include <mutex>

#include "collision_integrals.h"
#include "tables.h"
#include "tables_mixed.h"

namespace cbg {

namespace {

constexpr double kB = 1.380649e-23;   // model.rs:6
constexpr double NA = 6.02214076e23;  // model.rs:7
const double Rgas = kB * NA;          // model.rs:8
constexpr double PI = 3.141592653589793;

// The reference's expression builder folds a constant c that meets a runtime value
// (ast/lib.rs:195-232): additions drop c when (f32)c == 0; multiplications give 0, x or -x when
// (f32)c is 0, 1 or -1. Since x + 0, 1 * x and -1 * x are exact, replacing c by its canonical value
// and computing plainly gives the builder's result.
float to_f32(double c) { return std::fabs(c) < 1e38 ? (float)c : (c > 0 ? INFINITY : -INFINITY); }
double fold_add(double c) { return to_f32(c) == 0.0f ? 0.0 : c; }
double fold_mul(double c) {
    float f = to_f32(c);
    if (f == 0.0f) return 0.0;
    if (f == 1.0f) return 1.0;
    if (f == -1.0f) return -1.0;
    return c;
}

Arrhenius make_arrhenius(double A, double b, double Ea) {
    // reaction.rs:113-139: peel an integer power of T off b, keep the remainder in the exponent.
    Arrhenius a{};
    double rem;
    if (b <= -1.5) { a.factor = kRcpT2; rem = b + 2.; }
    else if (b <= -0.5) { a.factor = kRcpT; rem = b + 1.; }
    else if (b >= 3.5) { a.factor = kT4; rem = b - 4.; }
    else if (b >= 2.5) { a.factor = kT3; rem = b - 3.; }
    else if (b >= 1.5) { a.factor = kT2; rem = b - 2.; }
    else if (b >= 0.5) { a.factor = kT; rem = b - 1.; }
    else { a.factor = kNone; rem = b; }
    const double brem = to_f32(rem) != 0.0f ? fold_mul(rem) : 0.0;
    a.mEa = Ea != 0.0 ? fold_mul(-Ea) : 0.0;
    a.has_x = (brem != 0.0 || a.mEa != 0.0) ? 1 : 0;
    a.has_beta_rem = brem != 0.0;
    // The kernel folds the peeled power T^m back into the exponent: beta = b' + m (exact in FP64).
    static const double power[] = {0., -2., -1., 4., 3., 2., 1.};
    a.beta = brem + power[a.factor];
    a.lnA = fold_add(std::log(A));
    a.A = a.factor != kNone ? fold_mul(A) : A;
    return a;
}

template <class T>
void append(std::vector<uint8_t>& blob, const T* p, size_t n) {
    size_t at = blob.size();
    blob.resize(at + n * sizeof(T));
    std::memcpy(blob.data() + at, p, n * sizeof(T));
}
int32_t align_blob(std::vector<uint8_t>& blob) {
    while (blob.size() % kAlign) blob.push_back(0);
    return (int32_t)blob.size();
}

// A blob is [MathTables][header][sections...]; offsets in the header are from the blob's start.
template <class H>
void begin_blob(std::vector<uint8_t>& blob, const H& h) {
    blob.clear();
    MathTables mt = make_math_tables();
    append(blob, &mt, 1);
    append(blob, &h, 1);
}
template <class H>
void finish_blob(std::vector<uint8_t>& blob, H& h) {
    h.total_bytes = align_blob(blob);
    h.off_math = 0;
    std::memcpy(blob.data() + kMathBytes, &h, sizeof h);
}

// Least squares min |A x - b| by Householder QR in long double (A is m x n, row-major, m >= n).
std::vector<double> least_squares(int m, int n, std::vector<long double> A, std::vector<long double> b) {
    for (int j = 0; j < n; j++) {
        long double norm = 0;
        for (int i = j; i < m; i++) norm += A[i * n + j] * A[i * n + j];
        norm = std::sqrt(norm);
        if (norm == 0) continue;
        long double alpha = A[j * n + j] > 0 ? -norm : norm;
        std::vector<long double> v(m - j);
        v[0] = A[j * n + j] - alpha;
        for (int i = j + 1; i < m; i++) v[i - j] = A[i * n + j];
        long double vv = 0;
        for (auto x : v) vv += x * x;
        for (int c = j; c < n; c++) {
            long double s = 0;
            for (int i = j; i < m; i++) s += v[i - j] * A[i * n + c];
            s = 2 * s / vv;
            for (int i = j; i < m; i++) A[i * n + c] -= s * v[i - j];
        }
        long double s = 0;
        for (int i = j; i < m; i++) s += v[i - j] * b[i];
        s = 2 * s / vv;
        for (int i = j; i < m; i++) b[i] -= s * v[i - j];
    }
    std::vector<long double> x(n);
    for (int j = n - 1; j >= 0; j--) {
        long double s = b[j];
        for (int c = j + 1; c < n; c++) s -= A[j * n + c] * x[c];
        x[j] = s / A[j * n + j];
    }
    return std::vector<double>(x.begin(), x.end());
}

// Degree-6 least-squares fit of every T* row of a table over the 8 delta* columns, keeping degrees
// 0..5 (transport.rs:48-51).
struct DeltaFits {
    double omega22[37][6];
    double astar[39][6];
};
const DeltaFits& delta_fits() {
    static DeltaFits f;
    static std::once_flag once;
    std::call_once(once, [] {
        auto fit = [](const double* row, double* out) {
            std::vector<long double> A(8 * 7), b(8);
            for (int i = 0; i < 8; i++) {
                long double p = 1;
                for (int k = 0; k < 7; k++) { A[i * 7 + k] = p; p *= cb_header_delta[i]; }
                b[i] = row[i];
            }
            auto x = least_squares(8, 7, A, b);
            for (int k = 0; k < 6; k++) out[k] = x[k];
        };
        for (int r = 0; r < 37; r++) fit(cb_omega22[r], f.omega22[r]);
        for (int r = 0; r < 39; r++) fit(cb_astar[r], f.astar[r]);
    });
    return f;
}

// --- species transport physics (transport.rs:57-117) ---------------------------------------------
constexpr double fine_structure = 7.2973525693e-3, planck = 6.62607015e-34, charge = 1.602176634e-19,
                 light = 299792458.;
double vacuum_permittivity() {
    double mu0 = 2. * fine_structure * planck / (charge * charge * light);
    return 1. / (light * light * mu0);
}

struct Pair {
    double well_depth;      // interaction well depth (J)
    double reduced_dipole;  // delta*
    double diameter;        // reduced collision diameter (m)
    double mass;            // reduced mass (kg)
};

Pair pair_of(const HostMechanism& m, int a, int b) {
    const double* mu = m.dipole.data();
    double chi = 1.;  // polar / non-polar correction (transport.rs:62-68)
    if ((mu[a] > 0.) != (mu[b] > 0.)) {
        int p = mu[a] != 0. ? a : b, q = mu[a] != 0. ? b : a;
        double dp = m.diameter[p], dq = m.diameter[q];
        double red = mu[p] / std::sqrt(4. * PI * vacuum_permittivity() * m.well_depth[p] * (dp * dp * dp));
        chi = 1. + 1. / 4. * m.polarizability[q] / (dq * dq * dq) * (red * red) *
                       std::sqrt(m.well_depth[p] / m.well_depth[q]);
    }
    Pair r;
    r.well_depth = std::sqrt(m.well_depth[a] * m.well_depth[b]) * (chi * chi);
    double s = (m.diameter[a] + m.diameter[b]) / 2.;
    r.reduced_dipole = mu[a] * mu[b] / (8. * PI * vacuum_permittivity() * std::sqrt(m.well_depth[a] * m.well_depth[b]) * (s * s * s));
    r.diameter = (m.diameter[a] + m.diameter[b]) / 2. * std::pow(chi, -1. / 6.);
    r.mass = m.W[a] / NA * m.W[b] / NA / (m.W[a] / NA + m.W[b] / NA);
    return r;
}

// Quadratic interpolation in ln T* over three table rows starting at the row after the last header
// entry not above ln T* (transport.rs:14-17, 82-96). first_row: header index of the table's row 0.
double collision_integral(const Pair& p, double T, int first_row, int rows, const double (*table)[8],
                          const double (*fits)[6]) {
    double lnTs = std::log(T * kB / p.well_depth);
    int above = -1;
    for (int i = 1; i < 39; i++)
        if (lnTs < std::log(cb_header_Tstar[i])) { above = i; break; }
    if (above < 0) return NAN;
    int start = above - 1;
    if (start > first_row + rows - 3) start = first_row + rows - 3;
    if (start < first_row) return NAN;
    double x[3], y[3];
    for (int i = 0; i < 3; i++) {
        x[i] = std::log(cb_header_Tstar[start + i]);
        int row = start - first_row + i;
        if (p.reduced_dipole == 0.) y[i] = table[row][0];
        else {
            double s = 0., d = 1.;
            for (int k = 0; k < 6; k++) { s += fits[row][k] * d; d *= p.reduced_dipole; }
            y[i] = s;
        }
    }
    if (!(x[0] <= lnTs && lnTs <= x[2])) return NAN;
    double curvature = ((x[1] - x[0]) * (y[2] - y[1]) - (y[1] - y[0]) * (x[2] - x[1])) /
                       ((x[1] - x[0]) * (x[2] - x[0]) * (x[2] - x[1]));
    return curvature * (lnTs - x[0]) * (lnTs - x[1]) + ((y[1] - y[0]) / (x[1] - x[0])) * (lnTs - x[1]) + y[1];
}

double omega22(const Pair& p, double T) {
    return collision_integral(p, T, 1, 37, cb_omega22, delta_fits().omega22);
}
double omega11(const Pair& p, double T) {
    return omega22(p, T) / collision_integral(p, T, 0, 39, cb_astar, delta_fits().astar);
}

double cp_R_at(const HostMechanism& m, int k, double T) {  // lib.rs:16
    const double* a = &m.nasa7[k * 14 + ((T <= m.split[k] || std::isnan(m.split[k])) ? 0 : 7)];
    return a[0] + a[1] * T + a[2] * T * T + a[3] * T * T * T + a[4] * T * T * T * T;
}

double rotational_scaling(double Ts) {  // fz of transport.rs:109
    return 1. + std::pow(PI, 3. / 2.) / std::sqrt(Ts) * (1. / 2. + 1. / Ts) + (1. / 4. * (PI * PI) + 2.) / Ts;
}

}  // namespace

// Tables of fp64_math.cuh, computed in long double and rounded once.
MathTables make_math_tables() {
    MathTables t;
    std::memset(&t, 0, sizeof t);
    for (int j = 0; j < 256; j++) t.exp2j[j] = (double)std::exp2((long double)j / 256.0L);
    for (int j = 0; j <= 256; j++) {
        long double c = 1.0L + (long double)j / 256.0L;
        long double l = std::log(c);
        t.log_hi[j] = (double)l;
        t.log_lo[j] = (double)(l - (long double)t.log_hi[j]);
        t.rcp[j] = (double)(1.0L / c);
    }
    // ln 2 split exactly as in log_fast so that e ln2 + ln c cancels exactly just below x = 1.
    t.log_hi[256] = 0x1.62e42fefa4000p-1;
    t.log_lo[256] = -0x1.8432a1b0e2634p-43;
    t.log_hi[0] = 0.0;
    t.log_lo[0] = 0.0;
    return t;
}

namespace {

void add_work(Work& w, double flops, double exps = 0, double logs = 0, double divs = 0, double sqrts = 0) {
    w.flops += flops; w.exps += exps; w.logs += logs; w.divs += divs; w.sqrts += sqrts;
}

}  // namespace

double species_viscosity(const HostMechanism& m, int k, double T) {
    Pair p = pair_of(m, k, k);
    double d = m.diameter[k];
    return 5. / 16. * std::sqrt(PI * m.W[k] / NA * kB * T) / (omega22(p, T) * PI * (d * d));
}

double pair_diffusivity(const HostMechanism& m, int a, int b, double T) {
    Pair p = pair_of(m, a, b);
    return 3. / 16. * std::sqrt(2. * PI / p.mass) * std::pow(kB * T, 3. / 2.) / (PI * (p.diameter * p.diameter) * omega11(p, T));
}

double species_conductivity(const HostMechanism& m, int k, double T) {
    // Warnatz model with temperature-scaled rotational relaxation (transport.rs:106-116).
    double W = m.W[k], dof = m.dof[k];
    double mu = species_viscosity(m, k, T);
    double f_int = W / NA / (kB * T) * pair_diffusivity(m, k, k, T) / mu;
    double eps = pair_of(m, k, k).well_depth;
    double c1 = 2. / PI * (5. / 2. - f_int) /
                (m.rot[k] * rotational_scaling(298. * kB / eps) / rotational_scaling(T * kB / eps) +
                 2. / PI * (5. / 3. * dof + f_int));
    double f_trans = 5. / 2. * (1. - c1 * dof / (3. / 2.));
    double f_rot = f_int * (1. + c1);
    double cv_int = cp_R_at(m, k, T) - 5. / 2. - dof;
    return (mu / (W / NA)) * kB * (f_trans * 3. / 2. + f_rot * dof + f_int * cv_int);
}

int build_mechanism(const cb_mech_desc* d, HostMechanism& m, std::string& err) {
    if (!d) { err = "null mechanism description"; return CB_ERR_INVALID; }
    const int K = d->n_species, R = d->n_reactions;
    if (K < 2 || R < 1) { err = "a mechanism needs at least 2 species and 1 reaction"; return CB_ERR_INVALID; }
    if (K > 65535) { err = "too many species"; return CB_ERR_UNSUPPORTED; }
    if (!d->molar_mass || !d->nasa7_split || !d->nasa7 || !d->geometry || !d->diameter || !d->well_depth ||
        !d->polarizability || !d->dipole || !d->rotational_relaxation || !d->reactants || !d->products ||
        !d->model || !d->rate) {
        err = "a required mechanism array is null"; return CB_ERR_INVALID;
    }
    m.K = K; m.R = R;
    auto cp = [](const double* p, size_t n) { return std::vector<double>(p, p + n); };
    m.W = cp(d->molar_mass, K); m.split = cp(d->nasa7_split, K); m.nasa7 = cp(d->nasa7, (size_t)K * 14);
    m.geometry.assign(d->geometry, d->geometry + K);
    m.diameter = cp(d->diameter, K); m.well_depth = cp(d->well_depth, K);
    m.polarizability = cp(d->polarizability, K); m.dipole = cp(d->dipole, K);
    m.rot = cp(d->rotational_relaxation, K);
    m.dof.resize(K);
    for (int k = 0; k < K; k++) {
        if (m.geometry[k] < CB_ATOM || m.geometry[k] > CB_NONLINEAR) { err = "bad species geometry"; return CB_ERR_INVALID; }
        m.dof[k] = m.geometry[k] == CB_ATOM ? 0. : m.geometry[k] == CB_LINEAR ? 1. : 3. / 2.;  // lib.rs:58
        if (!(m.W[k] > 0.)) { err = "molar masses must be positive"; return CB_ERR_MECHANISM; }
    }
    m.reactants.assign(d->reactants, d->reactants + (size_t)R * K);
    m.products.assign(d->products, d->products + (size_t)R * K);
    m.model.assign(d->model, d->model + R);
    m.rate = cp(d->rate, (size_t)R * 3);
    m.k0 = d->k0 ? cp(d->k0, (size_t)R * 3) : std::vector<double>((size_t)R * 3, 0.);
    m.troe = d->troe ? cp(d->troe, (size_t)R * 4) : std::vector<double>((size_t)R * 4, 0.);
    m.sri = d->sri ? cp(d->sri, (size_t)R * 5) : std::vector<double>((size_t)R * 5, 0.);
    m.eff = d->efficiencies ? cp(d->efficiencies, (size_t)R * K) : std::vector<double>((size_t)R * K, 1.);

    // Active species: those whose amount some reaction changes; they must come first (lib.rs:130-135).
    std::vector<char> changes(K, 0);
    for (int r = 0; r < R; r++)
        for (int k = 0; k < K; k++)
            if (m.reactants[(size_t)r * K + k] != m.products[(size_t)r * K + k]) changes[k] = 1;
    int A = 0;
    while (A < K && changes[A]) A++;
    for (int k = A; k < K; k++)
        if (changes[k]) { err = "active species must precede inert species (lib.rs:130-135)"; return CB_ERR_MECHANISM; }
    if (A == K) { err = "the last species must be inert: it is the bulk species"; return CB_ERR_MECHANISM; }
    if (A == 0) { err = "no reaction changes any species"; return CB_ERR_MECHANISM; }
    m.A = A;

    // ---- rates tables ------------------------------------------------------------------------
    std::vector<Species> species(K);
    std::vector<Reaction> reactions(R);
    std::vector<Falloff> falloff;
    std::vector<double> eff_rows;
    for (int k = 0; k < K; k++) {
        Species& s = species[k];
        std::memset(&s, 0, sizeof s);
        s.split = m.split[k];
        bool one_piece = std::isnan(m.split[k]);
        for (int p = 0; p < 2; p++) {
            const double* a = &m.nasa7[k * 14 + p * 7];
            // Gibbs0_RT (reaction.rs:78): constant only for single-piece species, where the builder folds.
            double g[7] = {a[0] - a[6], -a[0], -a[1] / 2., (1. / 3. - 1. / 2.) * a[2], (1. / 4. - 1. / 3.) * a[3],
                           (1. / 5. - 1. / 4.) * a[4], a[5]};
            for (int i = 0; i < 7; i++) s.g[p][i] = one_piece ? (i == 0 ? fold_add(g[i]) : fold_mul(g[i])) : g[i];
            s.h[p][0] = fold_add(a[0]);
            s.h[p][1] = fold_mul(a[1] / 2.); s.h[p][2] = fold_mul(a[2] / 3.); s.h[p][3] = fold_mul(a[3] / 4.);
            s.h[p][4] = fold_mul(a[4] / 5.); s.h[p][5] = fold_mul(a[5]);
            s.cp[p][0] = fold_add(a[0]);
            for (int i = 1; i < 5; i++) s.cp[p][i] = fold_mul(a[i]);
        }
        s.dtE = k < A ? fold_mul(1. - m.W[k] / m.W[K - 1]) : 0.;
    }
    for (int r = 0; r < R; r++) {
        Reaction& x = reactions[r];
        std::memset(&x, 0, sizeof x);
        x.model = m.model[r];
        x.eff_row = -1; x.falloff = -1;
        if (x.model < CB_ELEMENTARY || x.model > CB_SRI) { err = "bad reaction model"; return CB_ERR_INVALID; }
        const uint8_t* re = &m.reactants[(size_t)r * K];
        const uint8_t* pr = &m.products[(size_t)r * K];
        int sum_r = 0, sum_p = 0;
        for (int k = 0; k < K; k++) {
            sum_r += re[k]; sum_p += pr[k];
            if (re[k]) {
                if (x.n_r == kMaxSide) { err = "more than 4 distinct reactants"; return CB_ERR_UNSUPPORTED; }
                x.r_k[x.n_r] = (uint16_t)k; x.r_n[x.n_r++] = (int8_t)re[k];
            }
            if (pr[k]) {
                if (x.n_p == kMaxSide) { err = "more than 4 distinct products"; return CB_ERR_UNSUPPORTED; }
                x.p_k[x.n_p] = (uint16_t)k; x.p_n[x.n_p++] = (int8_t)pr[k];
            }
            if (k < A && re[k] != pr[k]) {
                if (x.n_net == kMaxNet) { err = "more than 8 species change in one reaction"; return CB_ERR_UNSUPPORTED; }
                x.net_k[x.n_net] = (uint16_t)k; x.net_n[x.n_net++] = (int8_t)((int)pr[k] - (int)re[k]);
            }
        }
        x.minus_sigma_net = sum_r - sum_p;
        if (x.n_r == 0) { err = "a reaction has no reactants"; return CB_ERR_MECHANISM; }
        if (x.model != CB_IRREVERSIBLE) {
            // reaction.rs:290-305: a reversible reaction needs products and a net change (the product
            // of Gibbs factors is unwrapped) and a net order the equilibrium constant covers.
            if (x.n_p == 0 || x.n_net == 0) { err = "a reversible reaction has no products or no net change"; return CB_ERR_MECHANISM; }
            if (x.minus_sigma_net < -2 || x.minus_sigma_net > 1) { err = "net reaction order outside -2..1 (reaction.rs:298-303)"; return CB_ERR_UNSUPPORTED; }
            for (int i = 0; i < x.n_net; i++) {
                if (x.net_n[i] > 0) species[x.net_k[i]].need_exp = 1; else species[x.net_k[i]].need_exp_neg = 1;
            }
        }
        const double* rc = &m.rate[r * 3];
        if (!(rc[0] > 0.)) { err = "pre-exponential factors must be positive"; return CB_ERR_MECHANISM; }
        if (x.model == CB_THREE_BODY || x.model == CB_LINDEMANN || x.model == CB_TROE || x.model == CB_SRI) {
            x.eff_row = (int32_t)(eff_rows.size() / K);
            const double* e = &m.eff[(size_t)r * K];
            for (int k = 0; k < K; k++) {
                // efficiency(): C + sum over e != 1 of (e-1) C_k (reaction.rs:141-145); 0 = no term.
                double c = 0.;
                if (e[k] != 1.) {
                    double em1 = e[k] - 1.;
                    c = em1 == 1. ? 1. : fold_mul(em1);
                }
                eff_rows.push_back(c);
            }
        }
        if (x.model == CB_TROE) {
            if (!d->troe || !d->k0) { err = "Troe reactions need k0 and troe arrays"; return CB_ERR_INVALID; }
            Falloff f;
            std::memset(&f, 0, sizeof f);
            const double* k0 = &m.k0[r * 3];
            const double* t = &m.troe[r * 4];
            f.k0 = make_arrhenius(k0[0] / rc[0], k0[1], k0[2]);  // A0 / A_inf (reaction.rs:163-170)
            if (rc[1] == 0. && rc[2] == 0.) f.flags |= kKinfConst;
            else x.k = make_arrhenius(1.0, rc[1], rc[2]);
            f.ainf = fold_mul(rc[0]);
            double At = t[0], T3 = t[1], T1 = t[2], T2 = t[3];
            f.c1mA = fold_mul(1. - At);
            f.c3 = fold_mul(1. / (-T3));
            if (f.c1mA != 0.) f.flags |= kTermT3;
            if (T1 < 1e30) {
                f.cA = fold_mul(At);
                f.c1 = fold_mul(1. / (-T1));
                if (f.cA != 0.) f.flags |= kTermT1;
            } else {
                f.cA = fold_add(At);
                if (f.cA != 0.) f.flags |= kTermAConst;
            }
            if (std::isfinite(T2)) { f.cmT2 = fold_mul(-T2); f.flags |= kTermT2; }
            if (!(f.flags & (kTermT3 | kTermT1 | kTermT2))) { f.flags |= kFcentConst; f.ln_fcent = std::log(f.cA); }
            x.falloff = (int32_t)falloff.size();
            falloff.push_back(f);
        } else if (x.model == CB_LINDEMANN) {
            if (!d->k0) { err = "falloff reactions need the k0 array"; return CB_ERR_INVALID; }
            Falloff f;
            std::memset(&f, 0, sizeof f);
            f.k0 = make_arrhenius(m.k0[r * 3], m.k0[r * 3 + 1], m.k0[r * 3 + 2]);
            x.k = make_arrhenius(rc[0], rc[1], rc[2]);
            x.falloff = (int32_t)falloff.size();
            falloff.push_back(f);
        } else if (x.model == CB_SRI) {
            // The reference leaves SRI unimplemented (reaction.rs:194-203); this follows its commented
            // formula: Pr = M k0 / (k_inf + f32::MIN_POSITIVE) with unscaled k0 and k_inf,
            // F = D (A exp(-B/T) + exp(-T/C))^(1/(1 + ln(Pr + f32::MIN_POSITIVE)^2)) T^E.
            if (!d->k0 || !d->sri) { err = "SRI reactions need k0 and sri arrays"; return CB_ERR_INVALID; }
            const double* s = &m.sri[r * 5];
            if (!(s[2] != 0.) || !(s[3] > 0.)) { err = "SRI needs C != 0 and D > 0"; return CB_ERR_MECHANISM; }
            Falloff f;
            std::memset(&f, 0, sizeof f);
            f.k0 = make_arrhenius(m.k0[r * 3], m.k0[r * 3 + 1], m.k0[r * 3 + 2]);
            x.k = make_arrhenius(rc[0], rc[1], rc[2]);
            f.sA = fold_mul(s[0]);
            f.smB = fold_mul(-s[1]);
            f.smrC = fold_mul(-1. / s[2]);
            f.sD = fold_mul(s[3]);
            f.sE = fold_mul(s[4]);
            if (f.sA != 0.) f.sri_flags |= kSriA;
            if (f.sD != 1.) f.sri_flags |= kSriD;
            if (f.sE != 0.) f.sri_flags |= kSriE;
            x.falloff = (int32_t)falloff.size();
            falloff.push_back(f);
        } else {
            x.k = make_arrhenius(rc[0], rc[1], rc[2]);
        }
    }

    RatesHeader h;
    std::memset(&h, 0, sizeof h);
    h.K = K; h.A = A; h.R = R; h.n_eff = (int32_t)(eff_rows.size() / K); h.n_falloff = (int32_t)falloff.size();
    m.n_eff = h.n_eff;
    // Efficiency rows padded with zero rows to a multiple of 4: the kernel sums four rows per pass.
    while ((eff_rows.size() / K) % 4) eff_rows.resize(eff_rows.size() + K, 0.0);
    {
        float mx = std::cbrt(FLT_MAX);  // largest f32 whose cube stays finite (reaction.rs:244-251)
        mx = cbrtf(FLT_MAX);
        while (mx * mx * mx > FLT_MAX) mx = std::nextafter(mx, -INFINITY);
        h.M3 = (double)mx;
        h.cbrt_max = (double)cbrtf(FLT_MAX);
    }
    const double P0 = 101325. / Rgas;  // NASA7::reference_pressure (lib.rs:14)
    h.C0 = fold_mul(P0);
    h.rcp_C0 = fold_mul(1. / P0);
    h.ln10_04 = 0.4 * std::log(10.);
    h.ln10_075 = 0.75 * std::log(10.);
    // Reactions grouped by model (stable): the kernels run one specialised loop per model, with no
    // per-reaction model branches (which the compiler would predicate, costing FP64 pipe slots).
    std::vector<int> order(R);
    for (int r = 0; r < R; r++) order[r] = r;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return reactions[a].model < reactions[b].model; });
    // Efficiency rows renumbered in group order: the reactions with a third body (models 2-5) are
    // consecutive in the grouped tables, so grouped reaction group_end[1] + e uses row e, and the kernels
    // compute the sums of four consecutive rows in one pass over the concentrations as they reach them.
    {
        std::vector<double> rows(eff_rows.size(), 0.0);
        int e = 0;
        for (int i = 0; i < R; i++) {
            Reaction& x = reactions[order[i]];
            if (x.eff_row < 0) continue;
            std::copy_n(&eff_rows[(size_t)x.eff_row * K], K, &rows[(size_t)e * K]);
            x.eff_row = e++;
        }
        eff_rows.swap(rows);
    }
    std::vector<Reaction> grouped(R);
    for (int i = 0; i < R; i++) {
        grouped[i] = reactions[order[i]];
        grouped[i].orig = order[i];
    }
    for (int mdl = 0; mdl < 6; mdl++) {
        int end = 0;
        while (end < R && grouped[end].model <= mdl) end++;
        h.group_end[mdl] = end;
    }
    std::vector<uint8_t>& blob = m.rates_blob;
    begin_blob(blob, h);
    h.off_species = align_blob(blob); append(blob, species.data(), species.size());
    h.off_reactions = align_blob(blob); append(blob, grouped.data(), grouped.size());
    h.off_falloff = align_blob(blob); append(blob, falloff.data(), falloff.size());
    h.off_eff = align_blob(blob); append(blob, eff_rows.data(), eff_rows.size());
    finish_blob(blob, h);

    // ---- mixed-precision tables (tables_mixed.h) -----------------------------------------------
    {
        auto arr_f = [](double A, double b, double Ea) {
            ArrheniusF a{};
            a.b = (float)b; a.mEa = (float)(-Ea); a.lnA = (float)std::log(A);
            a.has_x = (b != 0.0 || Ea != 0.0) ? 1 : 0;
            a.A = A;
            return a;
        };
        std::vector<SpeciesF> sf(K);
        for (int k = 0; k < K; k++) {
            SpeciesF& s = sf[k];
            std::memset(&s, 0, sizeof s);
            s.split = species[k].split;
            for (int p = 0; p < 2; p++) {
                for (int i = 0; i < 7; i++) s.g[p][i] = species[k].g[p][i];
                for (int i = 0; i < 6; i++) s.h[p][i] = (float)species[k].h[p][i];
                for (int i = 0; i < 5; i++) s.cp[p][i] = (float)species[k].cp[p][i];
            }
            s.dtE = species[k].dtE;
            s.need_exp = species[k].need_exp;
            s.need_exp_neg = species[k].need_exp_neg;
        }
        std::vector<ReactionF> rf(R);
        std::vector<FalloffF> ff;
        for (int r = 0; r < R; r++) {
            const Reaction& x = reactions[r];
            ReactionF& y = rf[r];
            std::memset(&y, 0, sizeof y);
            y.model = x.model; y.minus_sigma_net = x.minus_sigma_net; y.eff_row = x.eff_row; y.falloff = x.falloff;
            y.n_r = x.n_r; y.n_p = x.n_p; y.n_net = x.n_net;
            std::memcpy(y.r_k, x.r_k, sizeof y.r_k); std::memcpy(y.p_k, x.p_k, sizeof y.p_k);
            std::memcpy(y.net_k, x.net_k, sizeof y.net_k); std::memcpy(y.r_n, x.r_n, sizeof y.r_n);
            std::memcpy(y.p_n, x.p_n, sizeof y.p_n); std::memcpy(y.net_n, x.net_n, sizeof y.net_n);
            const double* rc = &m.rate[r * 3];
            if (x.model == CB_TROE) {
                const double* k0 = &m.k0[r * 3];
                y.k = arr_f(1.0, rc[1], rc[2]);
                FalloffF f{};
                const Falloff& g = falloff[x.falloff];
                f.k0 = arr_f(k0[0] / rc[0], k0[1], k0[2]);
                f.ainf = g.ainf;
                f.c1mA = (float)g.c1mA; f.cA = (float)g.cA; f.c3 = (float)g.c3; f.c1 = (float)g.c1;
                f.cmT2 = (float)g.cmT2; f.ln_fcent = (float)g.ln_fcent; f.flags = g.flags;
                y.falloff = (int32_t)ff.size();
                ff.push_back(f);
            } else if (x.model == CB_LINDEMANN || x.model == CB_SRI) {
                y.k = arr_f(rc[0], rc[1], rc[2]);
                FalloffF f{};
                f.k0 = arr_f(m.k0[r * 3], m.k0[r * 3 + 1], m.k0[r * 3 + 2]);
                if (x.model == CB_SRI) {
                    const Falloff& g = falloff[x.falloff];
                    f.sA = (float)g.sA; f.smB = (float)g.smB; f.smrC = (float)g.smrC; f.sD = (float)g.sD;
                    f.sE = (float)g.sE; f.sri_flags = g.sri_flags;
                }
                y.falloff = (int32_t)ff.size();
                ff.push_back(f);
            } else {
                y.k = arr_f(rc[0], rc[1], rc[2]);
            }
        }
        std::vector<float> efff(eff_rows.begin(), eff_rows.end());
        RatesMixedHeader hm;
        std::memset(&hm, 0, sizeof hm);
        hm.K = K; hm.A = A; hm.R = R; hm.n_eff = h.n_eff; hm.n_falloff = (int32_t)ff.size();
        hm.M3 = h.M3; hm.cbrt_max = h.cbrt_max; hm.C0 = h.C0; hm.rcp_C0 = h.rcp_C0;
        hm.ln10_04 = (float)h.ln10_04; hm.ln10_075 = (float)h.ln10_075;
        std::vector<ReactionF> rfg(R);
        for (int i = 0; i < R; i++) {
            rfg[i] = rf[order[i]];
            rfg[i].orig = order[i];
        }
        for (int mdl = 0; mdl < 6; mdl++) hm.group_end[mdl] = h.group_end[mdl];
        std::vector<uint8_t>& b = m.rates_mixed_blob;
        begin_blob(b, hm);
        hm.off_species = align_blob(b); append(b, sf.data(), sf.size());
        hm.off_reactions = align_blob(b); append(b, rfg.data(), rfg.size());
        hm.off_falloff = align_blob(b); append(b, ff.data(), ff.size());
        hm.off_eff = align_blob(b); append(b, efff.data(), efff.size());
        finish_blob(b, hm);
    }

    // ---- algorithmic work of reaction.rs:356-391 per cell (the reference's operations) ----------
    Work& w = m.rates_work;
    w = Work{};
    add_work(w, 6 + 2.0 * (K - 1) + (K - 1), 0, 1, 2);  // prologue: powers, concentrations, bulk
    for (int k = 0; k < A; k++) {
        if (species[k].need_exp || species[k].need_exp_neg) add_work(w, 12);          // Gibbs polynomial
        if (species[k].need_exp) add_work(w, 1, 1);                                       // min(exp)
        if (species[k].need_exp_neg) add_work(w, 2, 1);                                   // min(exp(-x))
    }
    auto arrh_work = [&](const Arrhenius& a) {
        double f = 1;  // min
        if (a.has_x) {
            f += a.has_beta_rem + (a.mEa != 0) + (a.has_beta_rem && a.mEa != 0) + (a.lnA != 0);
            add_work(w, 0, 1);
        }
        if (a.factor != kNone) f += 1;
        add_work(w, f);
    };
    for (int r = 0; r < R; r++) {
        const Reaction& x = reactions[r];
        int mult_r = 0, mult_p = 0, mult_net = 0;
        for (int i = 0; i < x.n_r; i++) mult_r += x.r_n[i];
        for (int i = 0; i < x.n_p; i++) mult_p += x.p_n[i];
        for (int i = 0; i < x.n_net; i++) mult_net += std::abs((int)x.net_n[i]);
        if (x.eff_row >= 0) {
            int n = 0;
            for (int k = 0; k < K; k++) n += eff_rows[(size_t)x.eff_row * K + k] != 0.;
            add_work(w, 2.0 * n);
        }
        if (x.model == CB_TROE) {
            const Falloff& f = falloff[x.falloff];
            arrh_work(f.k0);
            if (!(f.flags & kKinfConst)) { arrh_work(x.k); add_work(w, 3, 0, 0, 1); } else add_work(w, 1);
            add_work(w, 2.0 * !!(f.flags & kTermT3) + 2.0 * !!(f.flags & kTermT1) + 1.0 * !!(f.flags & kTermT2) + 2,
                     !!(f.flags & kTermT3) + !!(f.flags & kTermT1) + !!(f.flags & kTermT2), 1);
            add_work(w, 12, 1, 1, 3);  // C, N, lnPr+C, f1, F, numerator, denominator
        } else if (x.model == CB_LINDEMANN) {
            arrh_work(falloff[x.falloff].k0); arrh_work(x.k); add_work(w, 5, 0, 0, 1);
        } else if (x.model == CB_SRI) {
            const Falloff& f = falloff[x.falloff];
            arrh_work(f.k0); arrh_work(x.k);
            // Pr, ln(Pr + eps), the base's terms, its log, the power, T^E, F, numerator, denominator
            add_work(w, 2 + 2 + 3.0 * !!(f.sri_flags & kSriA) + 2 + 3 + 1.0 * !!(f.sri_flags & kSriD) + 2.0 * !!(f.sri_flags & kSriE) + 4,
                     1 + !!(f.sri_flags & kSriA) + 1 + !!(f.sri_flags & kSriE), 2, 2);
        } else {
            arrh_work(x.k);
            if (x.model == CB_THREE_BODY) add_work(w, 1);
        }
        add_work(w, mult_r - 1);
        if (x.model != CB_IRREVERSIBLE) add_work(w, (mult_net - 1) + (x.minus_sigma_net != 0) + (x.minus_sigma_net == -2) + (mult_p - 1) + 2);
        add_work(w, 1);  // cR
        for (int i = 0; i < x.n_net; i++) add_work(w, std::abs((int)x.net_n[i]) == 1 ? 1 : 2);
    }
    add_work(w, 11.0 * A + 9.0 * K + 2.0 * A + 2.0 * K + 2.0 * A + 6, 0, 0, 1);  // h, cp, dot products, dT, dV
    w.bytes_in = 8.0 * (K + 3);
    w.bytes_out = 8.0 * (A + 2);
    return CB_OK;
}

int build_transport(HostMechanism& m, double T0, double mu0, double lambda0, std::string& err) {
    const int K = m.K;
    if (!(T0 > 0.) || !(mu0 > 0.) || !(lambda0 > 0.)) { err = "transport normalisation must be positive"; return CB_ERR_INVALID; }
    // 50 temperatures over [300, 3000] K (transport.rs:127-129); fits in x = ln(T/T0) with 1/y^2 weights.
    const int N = 50;
    double Ts[N], xs[N];
    for (int n = 0; n < N; n++) {
        Ts[n] = 300. + (double)n / (double)(N - 1) * (3000. - 300.);
        xs[n] = std::log(Ts[n] / T0);
    }
    auto fit = [&](const double* y, double* P) -> bool {
        std::vector<long double> A(N * 5), b(N);
        for (int n = 0; n < N; n++) {
            if (!std::isfinite(y[n]) || y[n] == 0.) return false;
            long double w = 1.0L / ((long double)y[n] * y[n]);
            long double p = 1;
            for (int k = 0; k < 5; k++) { A[n * 5 + k] = w * p; p *= xs[n]; }
            b[n] = w * y[n];
        }
        auto x = least_squares(N, 5, A, b);
        for (int k = 0; k < 5; k++) P[k] = x[k];
        return true;
    };
    m.fit_cond.assign((size_t)K * 5, 0.); m.fit_visc.assign((size_t)K * 5, 0.); m.fit_diff.assign((size_t)K * K * 5, 0.);
    std::vector<double> y(N);
    for (int k = 0; k < K; k++) {
        for (int n = 0; n < N; n++) y[n] = species_conductivity(m, k, Ts[n]) / std::sqrt(Ts[n]);
        if (!fit(y.data(), &m.fit_cond[k * 5])) { err = "conductivity fit failed (collision integral outside its table?)"; return CB_ERR_MECHANISM; }
        for (int n = 0; n < N; n++) y[n] = std::sqrt(species_viscosity(m, k, Ts[n]) / std::sqrt(Ts[n]));
        if (!fit(y.data(), &m.fit_visc[k * 5])) { err = "viscosity fit failed (collision integral outside its table?)"; return CB_ERR_MECHANISM; }
    }
    for (int k = 0; k < K; k++)
        for (int j = 0; j < K; j++) {
            for (int n = 0; n < N; n++) y[n] = pair_diffusivity(m, k, j, Ts[n]) / (Ts[n] * std::sqrt(Ts[n]));
            if (!fit(y.data(), &m.fit_diff[((size_t)k * K + j) * 5])) { err = "diffusivity fit failed"; return CB_ERR_MECHANISM; }
        }
    m.T0 = T0; m.mu0 = mu0; m.lambda0 = lambda0;

    // Scaled, canonical tables (transport.rs:180-182) and the Wilke matrices.
    const double sv = std::sqrt(std::sqrt(T0)) / std::sqrt(mu0), sc = std::sqrt(T0) / (2. * lambda0),
                 sd = std::sqrt(T0) / (Rgas * mu0);
    auto scaled = [](const double* P, double s, double* out) {
        out[0] = fold_add(s * P[0]);
        for (int i = 1; i < 5; i++) out[i] = fold_mul(s * P[i]);
    };
    std::vector<double> cond((size_t)K * 5), visc((size_t)K * 5), Wc(K);
    for (int k = 0; k < K; k++) {
        scaled(&m.fit_cond[k * 5], sc, &cond[k * 5]);
        scaled(&m.fit_visc[k * 5], sv, &visc[k * 5]);
        Wc[k] = fold_mul(m.W[k]);
    }
    const int n_pairs = K * (K - 1) / 2;
    std::vector<double> diff((size_t)n_pairs * 5);
    for (int k = 0, p = 0; k < K; k++)
        for (int j = 0; j < k; j++, p++) scaled(&m.fit_diff[((size_t)k * K + j) * 5], sd, &diff[(size_t)p * 5]);
    // Wilke: phi_kj = (a_kj + b_kj v_k / v_j)^2 = a^2 + 2ab (v_k/v_j) + b^2 (v_k/v_j)^2 (transport.rs:152-157)
    // Rows padded with zeros to a multiple of 4: the kernel evaluates four rows per pass over j.
    const int K4 = (K + 3) / 4 * 4;
    std::vector<double> A2((size_t)K4 * K, 0.), AB((size_t)K4 * K, 0.), B2((size_t)K4 * K, 0.);
    for (int k = 0; k < K; k++)
        for (int j = 0; j < K; j++) {
            double Va = std::sqrt(1. / std::sqrt(8.) * 1. / std::sqrt(1. + m.W[k] / m.W[j]));
            double a = fold_add(Va), b = fold_mul(Va * std::sqrt(std::sqrt(m.W[j] / m.W[k])));
            A2[(size_t)k * K + j] = a * a;
            AB[(size_t)k * K + j] = 2. * a * b;
            B2[(size_t)k * K + j] = b * b;
        }
    TransportHeader h;
    std::memset(&h, 0, sizeof h);
    h.K = K; h.n_pairs = n_pairs; h.T0 = T0;
    std::vector<uint8_t>& blob = m.transport_blob;
    begin_blob(blob, h);
    h.off_cond = align_blob(blob); append(blob, cond.data(), cond.size());
    h.off_visc = align_blob(blob); append(blob, visc.data(), visc.size());
    h.off_W = align_blob(blob); append(blob, Wc.data(), Wc.size());
    h.off_diff = align_blob(blob); append(blob, diff.data(), diff.size());
    h.off_A2 = align_blob(blob); append(blob, A2.data(), A2.size());
    h.off_AB = align_blob(blob); append(blob, AB.data(), AB.size());
    h.off_B2 = align_blob(blob); append(blob, B2.data(), B2.size());
    finish_blob(blob, h);

    // ---- mixed-precision (all FP32) transport tables ----------------------------------------------
    {
        auto f32 = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
        TransportMixedHeader hm;
        std::memset(&hm, 0, sizeof hm);
        hm.K = K; hm.n_pairs = n_pairs; hm.T0 = T0;
        std::vector<uint8_t>& b = m.transport_mixed_blob;
        begin_blob(b, hm);
        auto put = [&](const std::vector<double>& v) {
            int32_t off = align_blob(b);
            std::vector<float> f = f32(v);
            append(b, f.data(), f.size());
            return off;
        };
        hm.off_cond = put(cond); hm.off_visc = put(visc); hm.off_W = put(Wc);
        std::vector<double> diff8((size_t)n_pairs * 8, 0.);  // 16-byte loads in the kernel
        for (size_t p = 0; p < (size_t)n_pairs; p++)
            for (int c = 0; c < 5; c++) diff8[p * 8 + c] = diff[p * 5 + c];
        hm.off_diff = put(diff8);
        std::vector<double> wil((size_t)K4 * K * 4, 0.);
        for (size_t e = 0; e < (size_t)K4 * K; e++) {
            wil[e * 4] = A2[e];
            wil[e * 4 + 1] = AB[e];
            wil[e * 4 + 2] = B2[e];
        }
        hm.off_wilke = put(wil);
        finish_blob(b, hm);
    }

    // ---- algorithmic work of transport.rs:179-210 per cell ---------------------------------------
    Work& w = m.transport_work;
    w = Work{};
    add_work(w, 3 + (K - 1) + 2.0 * K + 1, 0, 1, 0, 1);          // lnT powers, bulk, mean molar mass
    add_work(w, K * (8.0 + 3) + 3, 0, 0, K + 2.0);                 // conductivity
    add_work(w, K * 8.0 + 6.0 * K * K + 4.0 * K + 1, 0, 0, 2.0 * K);  // viscosity (Wilke)
    add_work(w, n_pairs * (8.0 + 4) + 3.0 * K, 0, 0, n_pairs + (double)K);  // diffusion
    w.bytes_in = 8.0 * (K + 1);
    w.bytes_out = 8.0 * (K + 2);
    m.transport_ready = true;
    return CB_OK;
}

}  // namespace cbg
