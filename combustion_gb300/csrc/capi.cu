// extern "C" entry points declared in include/combustion_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/combustion_gb300.h"
#include "capi_internal.h"
#include "kernels.h"
#include "mechanism.hpp"
#include "tables.h"

struct cb_mech {
    cbg::HostMechanism host;
    int device = 0;
    int kmax = 0;
    uint8_t* d_rates = nullptr;      // rates table blob
    uint8_t* d_transport = nullptr;  // transport table blob
    uint8_t* d_rates_mixed = nullptr;      // tables of the mixed-precision form
    uint8_t* d_transport_mixed = nullptr;
    int* d_status = nullptr;         // kernel status bits
    unsigned long long* d_count = nullptr;  // cb_count_nonfinite's device counter
    // Device staging for CB_HOST_MEMORY calls: two slots, each holding one chunk of inputs and outputs;
    // streams for host->device copies, kernels and device->host copies, and per-slot events.
    double* d_stage = nullptr;
    size_t stage_doubles = 0;
    cudaStream_t copy_stream[3] = {nullptr, nullptr, nullptr};  // h2d, compute, d2h
    cudaEvent_t slot_event[2][3] = {};                          // per slot: inputs in, kernels done, outputs out
};

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg) {
    g_error = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char* what) {
    return fail(CB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CB_CUDA(call)                                  \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

int check_status(cb_mech* m) {
    int st = 0;
    CB_CUDA(cudaMemcpy(&st, m->d_status, sizeof st, cudaMemcpyDeviceToHost));
    if (st) {
        cudaMemset(m->d_status, 0, sizeof(int));
        return fail(CB_ERR_DEVICE, "a kernel reported status " + std::to_string(st) + " (table staging wait ran out)");
    }
    return CB_OK;
}

enum class Path { Rates, ReactionRates, Transport, Fused, RatesMixed, TransportMixed, FusedMixed };

template <template <int> class Args, int KM>
int fill_and_launch(cb_mech* m, size_t n, const double* const* in, int ni, double* const* out, int no,
                    uint32_t flags, cudaStream_t st,
                    cudaError_t (*launch)(int, const uint8_t*, uint32_t, const void*, size_t, cudaStream_t, int*),
                    const uint8_t* tab, size_t tab_bytes, const char* what) {
    Args<KM> a;
    std::memset(&a, 0, sizeof a);
    for (int q = 0; q < ni; q++) a.in[q] = in[q];
    for (int q = 0; q < no; q++) a.out[q] = out[q];
    a.flags = flags;
    cudaError_t e = launch(KM, tab, (uint32_t)tab_bytes, &a, n, st, m->d_status);
    return e == cudaSuccess ? CB_OK : cuda_fail(e, what);
}

template <template <int> class Args>
int dispatch(cb_mech* m, size_t n, const double* const* in, int ni, double* const* out, int no, uint32_t flags,
             cudaStream_t st,
             cudaError_t (*launch)(int, const uint8_t*, uint32_t, const void*, size_t, cudaStream_t, int*),
             const uint8_t* tab, size_t tab_bytes, const char* what) {
    switch (m->kmax) {
    case 16: return fill_and_launch<Args, 16>(m, n, in, ni, out, no, flags, st, launch, tab, tab_bytes, what);
    case 64: return fill_and_launch<Args, 64>(m, n, in, ni, out, no, flags, st, launch, tab, tab_bytes, what);
    case 256: return fill_and_launch<Args, 256>(m, n, in, ni, out, no, flags, st, launch, tab, tab_bytes, what);
    default: return fail(CB_ERR_UNSUPPORTED, "species count outside the compiled capacities");
    }
}

// One call on device pointers (pointer arrays already resolved).
int launch_path(cb_mech* m, Path path, size_t n, const double* const* in, double* const* out, uint32_t flags,
                cudaStream_t st) {
    const int K = m->host.K, A = m->host.A, R = m->host.R;
    if (n == 0) return CB_OK;
    const size_t rb = m->host.rates_blob.size(), tb = m->host.transport_blob.size();
    switch (path) {
    case Path::Rates:
        return dispatch<cbg::RatesArgs>(m, n, in, K + 3, out, A + 2, flags, st, cbg::launch_rates, m->d_rates, rb,
                                        "rates kernel");
    case Path::ReactionRates:
        if (R > cbg::kMaxReactions) return fail(CB_ERR_UNSUPPORTED, "more reactions than per-reaction outputs support");
        return dispatch<cbg::ReactionRatesArgs>(m, n, in, K + 2, out, R, flags, st, cbg::launch_reaction_rates,
                                                m->d_rates, rb, "reaction rates kernel");
    case Path::Transport:
        return dispatch<cbg::TransportArgs>(m, n, in, K + 1, out, K + 2, flags, st, cbg::launch_transport,
                                            m->d_transport, tb, "transport kernel");
    case Path::Fused: {
        int rc = dispatch<cbg::RatesArgs>(m, n, in, K + 3, out, A + 2, flags, st, cbg::launch_rates, m->d_rates, rb,
                                          "rates kernel");
        if (rc) return rc;
        return dispatch<cbg::TransportArgs>(m, n, in, K + 3, out + (A + 2), K + 2, flags | cbg::kFromRates, st,
                                            cbg::launch_transport, m->d_transport, tb, "transport kernel");
    }
    case Path::RatesMixed:
        return dispatch<cbg::RatesArgs>(m, n, in, K + 3, out, A + 2, flags, st, cbg::launch_rates_mixed,
                                        m->d_rates_mixed, m->host.rates_mixed_blob.size(), "mixed rates kernel");
    case Path::TransportMixed:
        return dispatch<cbg::TransportArgs>(m, n, in, K + 1, out, K + 2, flags, st, cbg::launch_transport_mixed,
                                            m->d_transport_mixed, m->host.transport_mixed_blob.size(),
                                            "mixed transport kernel");
    case Path::FusedMixed: {
        int rc = dispatch<cbg::RatesArgs>(m, n, in, K + 3, out, A + 2, flags, st, cbg::launch_rates_mixed,
                                          m->d_rates_mixed, m->host.rates_mixed_blob.size(), "mixed rates kernel");
        if (rc) return rc;
        return dispatch<cbg::TransportArgs>(m, n, in, K + 3, out + (A + 2), K + 2, flags | cbg::kFromRates, st,
                                            cbg::launch_transport_mixed, m->d_transport_mixed,
                                            m->host.transport_mixed_blob.size(), "mixed transport kernel");
    }
    }
    return fail(CB_ERR_INVALID, "unknown path");
}

int n_inputs(const cb_mech* m, Path p) {
    switch (p) {
    case Path::Rates: case Path::Fused: case Path::RatesMixed: case Path::FusedMixed: return m->host.K + 3;
    case Path::ReactionRates: return m->host.K + 2;
    default: return m->host.K + 1;
    }
}
int n_outputs(const cb_mech* m, Path p) {
    switch (p) {
    case Path::Rates: case Path::RatesMixed: return m->host.A + 2;
    case Path::ReactionRates: return m->host.R;
    case Path::Fused: case Path::FusedMixed: return m->host.A + 2 + m->host.K + 2;
    default: return m->host.K + 2;
    }
}
bool rates_layout(Path p) {
    return p == Path::Rates || p == Path::Fused || p == Path::RatesMixed || p == Path::FusedMixed;
}
bool needs_transport(Path p) {
    return p == Path::Transport || p == Path::Fused || p == Path::TransportMixed || p == Path::FusedMixed;
}

// Cells of one wave of every kernel on the path (the least common multiple of their waves, or the
// largest wave when that multiple would exceed a chunk): a chunk of whole waves gives every thread of
// each persistent grid the same number of cells, so no SM idles through a chunk's last partial wave.
size_t path_wave(const cb_mech* m, Path path) {
    const uint32_t rb = (uint32_t)m->host.rates_blob.size(), tb = (uint32_t)m->host.transport_blob.size();
    const uint32_t rmb = (uint32_t)m->host.rates_mixed_blob.size();
    const uint32_t tmb = (uint32_t)m->host.transport_mixed_blob.size();
    size_t w[2] = {0, 0};
    switch (path) {
    case Path::Rates: w[0] = cbg::wave_rates(m->kmax, rb); break;
    case Path::ReactionRates: w[0] = cbg::wave_reaction_rates(m->kmax, rb); break;
    case Path::Transport: w[0] = cbg::wave_transport(m->kmax, tb); break;
    case Path::Fused: w[0] = cbg::wave_rates(m->kmax, rb); w[1] = cbg::wave_transport(m->kmax, tb); break;
    case Path::RatesMixed: w[0] = cbg::wave_rates_mixed(m->kmax, rmb); break;
    case Path::TransportMixed: w[0] = cbg::wave_transport_mixed(m->kmax, tmb); break;
    case Path::FusedMixed:
        w[0] = cbg::wave_rates_mixed(m->kmax, rmb);
        w[1] = cbg::wave_transport_mixed(m->kmax, tmb);
        break;
    }
    if (!w[0] || !w[1]) return w[0] ? w[0] : w[1];
    size_t a = w[0], b = w[1];
    while (b) { const size_t t = a % b; a = b; b = t; }
    const size_t lcm = w[0] / a * w[1];
    return lcm <= ((size_t)1 << 20) ? lcm : std::max(w[0], w[1]);
}

// Rows [q0, q1) of one chunk between a staging slot (row q at stage + q * chunk) and the caller's host
// arrays (row q at rows[q] + lo): one strided 2-D copy per run of equally spaced, non-overlapping host
// rows (the rows of one 2-D array), single copies otherwise.
cudaError_t copy_rows(double* stage, size_t chunk, const double* const* rows, int q0, int q1, size_t lo, size_t len,
                      bool to_device, cudaStream_t st) {
    for (int a = q0; a < q1;) {
        int b = a + 1;  // run [a, b)
        const ptrdiff_t step = b < q1 ? rows[b] - rows[a] : 0;
        if (step >= (ptrdiff_t)len)
            while (b < q1 && rows[b] - rows[b - 1] == step) b++;
        double* dev = stage + (size_t)a * chunk;
        double* host = const_cast<double*>(rows[a]) + lo;
        cudaError_t e;
        if (b - a >= 2) {
            const size_t hp = (size_t)step * sizeof(double), dp = chunk * sizeof(double), w = len * sizeof(double);
            e = to_device ? cudaMemcpy2DAsync(dev, dp, host, hp, w, (size_t)(b - a), cudaMemcpyHostToDevice, st)
                          : cudaMemcpy2DAsync(host, hp, dev, dp, w, (size_t)(b - a), cudaMemcpyDeviceToHost, st);
        } else {
            e = to_device ? cudaMemcpyAsync(dev, host, len * sizeof(double), cudaMemcpyHostToDevice, st)
                          : cudaMemcpyAsync(host, dev, len * sizeof(double), cudaMemcpyDeviceToHost, st);
        }
        if (e != cudaSuccess) return e;
        a = b;
    }
    return cudaSuccess;
}

// Host arrays: chunks through two device staging slots. Copies run on their own streams and kernels on
// one compute stream (one chunk's kernels at a time: the kernels use persistent grids), so that the
// copies of neighbouring chunks overlap the kernels: H2D(c+1) and D2H(c-1) run while chunk c computes.
// Only the first chunk's upload and the last chunk's download are exposed, so those two chunks are one
// wave of the path's kernels; the others are the standard chunk, one of them taking the remainder.
// One cudaMemcpyAsync per array per chunk (one 2-D copy per run of equally spaced host rows).
int call_host(cb_mech* m, Path path, size_t n, const double* const* in, double* const* out, uint32_t flags) {
    const int ni = n_inputs(m, path), no = n_outputs(m, path);
    const bool uniform = rates_layout(path) && (flags & CB_UNIFORM_PRESSURE);
    // chunks small enough that the first upload and the last download are short, large enough to fill
    // the GPU: about n / 16 cells, between 2^17 and 2^20, rounded to whole waves of the path's kernels
    size_t chunk = n / 16;
    if (chunk < ((size_t)1 << 17)) chunk = (size_t)1 << 17;
    if (chunk > ((size_t)1 << 20)) chunk = (size_t)1 << 20;
    const size_t wave = path_wave(m, path);
    if (wave) chunk = std::max<size_t>(1, (chunk + wave / 2) / wave) * wave;
    if (chunk > n) chunk = n;
    const size_t per_slot = (size_t)(ni + no) * chunk + 2;
    if (m->stage_doubles < 2 * per_slot) {
        if (m->d_stage) {
            CB_CUDA(cudaDeviceSynchronize());
            cudaFree(m->d_stage);
        }
        m->d_stage = nullptr;
        m->stage_doubles = 0;
        CB_CUDA(cudaMalloc(&m->d_stage, 2 * per_slot * sizeof(double)));
        m->stage_doubles = 2 * per_slot;
    }
    for (int s = 0; s < 3; s++)
        if (!m->copy_stream[s]) CB_CUDA(cudaStreamCreateWithFlags(&m->copy_stream[s], cudaStreamNonBlocking));
    for (int s = 0; s < 2; s++)
        for (int e = 0; e < 3; e++)
            if (!m->slot_event[s][e]) CB_CUDA(cudaEventCreateWithFlags(&m->slot_event[s][e], cudaEventDisableTiming));
    cudaStream_t h2d = m->copy_stream[0], comp = m->copy_stream[1], d2h = m->copy_stream[2];
    std::vector<const double*> din(ni);
    std::vector<double*> dout(no);
    std::vector<size_t> sizes;  // chunk lengths, in order
    const size_t edge = wave && wave < chunk ? wave : chunk;
    if (n <= 2 * edge) {
        for (size_t lo = 0; lo < n; lo += chunk) sizes.push_back(std::min(chunk, n - lo));
    } else {
        sizes.push_back(edge);
        size_t mid = n - 2 * edge;
        for (; mid >= chunk; mid -= chunk) sizes.push_back(chunk);
        if (mid) sizes.push_back(mid);
        sizes.push_back(edge);
    }
    size_t lo = 0;
    for (size_t c = 0; c < sizes.size(); lo += sizes[c], c++) {
        const size_t len = sizes[c];
        const int s = (int)(c & 1);
        cudaEvent_t* ev = m->slot_event[s];
        double* base = m->d_stage + s * per_slot;
        if (c >= 2) CB_CUDA(cudaStreamWaitEvent(h2d, ev[1], 0));  // the slot's previous kernels read their inputs
        const int q_arrays = uniform ? 2 : 0;  // uniform pressure: the two constants, one value each
        for (int q = 0; q < q_arrays; q++)
            CB_CUDA(cudaMemcpyAsync(base + (size_t)q * chunk, in[q], sizeof(double), cudaMemcpyHostToDevice, h2d));
        CB_CUDA(copy_rows(base, chunk, in, q_arrays, ni, lo, len, true, h2d));
        for (int q = 0; q < ni; q++) din[q] = base + (size_t)q * chunk;
        CB_CUDA(cudaEventRecord(ev[0], h2d));
        for (int q = 0; q < no; q++) dout[q] = base + (size_t)(ni + q) * chunk;
        CB_CUDA(cudaStreamWaitEvent(comp, ev[0], 0));
        if (c >= 2) CB_CUDA(cudaStreamWaitEvent(comp, ev[2], 0));  // the slot's previous outputs are copied out
        int rc = launch_path(m, path, len, din.data(), dout.data(), flags & ~CB_HOST_MEMORY, comp);
        if (rc) return rc;
        CB_CUDA(cudaEventRecord(ev[1], comp));
        CB_CUDA(cudaStreamWaitEvent(d2h, ev[1], 0));
        CB_CUDA(copy_rows(base + (size_t)ni * chunk, chunk, out, 0, no, lo, len, false, d2h));
        CB_CUDA(cudaEventRecord(ev[2], d2h));
    }
    CB_CUDA(cudaStreamSynchronize(d2h));
    return check_status(m);
}

int call(cb_mech* m, Path path, size_t n, const double* const* inputs, double* const* outputs, uint32_t flags,
         void* stream) {
    if (!m || !inputs || !outputs) return fail(CB_ERR_INVALID, "null argument");
    if (flags & ~(CB_HOST_MEMORY | CB_UNIFORM_PRESSURE)) return fail(CB_ERR_INVALID, "unknown flag");
    if ((flags & CB_UNIFORM_PRESSURE) && !rates_layout(path))
        return fail(CB_ERR_INVALID, "CB_UNIFORM_PRESSURE applies to the rates inputs only");
    if (needs_transport(path) && !m->host.transport_ready)
        return fail(CB_ERR_NOT_READY, "cb_transport_setup has not run");
    const int ni = n_inputs(m, path), no = n_outputs(m, path);
    if (n == 0) return CB_OK;
    for (int q = 0; q < ni; q++) if (!inputs[q]) return fail(CB_ERR_INVALID, "null input array");
    for (int q = 0; q < no; q++) if (!outputs[q]) return fail(CB_ERR_INVALID, "null output array");
    CB_CUDA(cudaSetDevice(m->device));
    if (flags & CB_HOST_MEMORY) return call_host(m, path, n, inputs, outputs, flags);
    return launch_path(m, path, n, inputs, outputs, flags, static_cast<cudaStream_t>(stream));
}

void to_work(const cbg::Work& w, cb_work* o) {
    o->flops = w.flops; o->exps = w.exps; o->logs = w.logs; o->divs = w.divs; o->sqrts = w.sqrts;
    o->bytes_in = w.bytes_in; o->bytes_out = w.bytes_out;
}

template <int KM>
int gather_launch(cb_mech* m, size_t n, const double* const* in, double* const* out, const uint32_t* index,
                  const uint32_t* count, bool compact, uint32_t flags, cudaStream_t st) {
    cbg::TransportArgs<KM> a;
    std::memset(&a, 0, sizeof a);
    for (int q = 0; q < m->host.K + 3; q++) a.in[q] = in[q];
    for (int q = 0; q < m->host.K + 2; q++) a.out[q] = out[q];
    a.flags = (flags & CB_UNIFORM_PRESSURE) | cbg::kFromRates | (compact ? cbg::kCompactOut : 0u);
    a.index = index;
    a.count = count;
    cudaError_t e = cbg::launch_transport(KM, m->d_transport, (uint32_t)m->host.transport_blob.size(), &a, n, st,
                                          m->d_status);
    return e == cudaSuccess ? CB_OK : cuda_fail(e, "transport kernel (gathered cells)");
}

template <int KM>
int gather_launch_mixed(cb_mech* m, size_t n, const double* const* in, double* const* out, const uint32_t* index,
                        const uint32_t* count, bool compact, uint32_t flags, cudaStream_t st) {
    cbg::TransportArgs<KM> a;
    std::memset(&a, 0, sizeof a);
    for (int q = 0; q < m->host.K + 3; q++) a.in[q] = in[q];
    for (int q = 0; q < m->host.K + 2; q++) a.out[q] = out[q];
    a.flags = (flags & CB_UNIFORM_PRESSURE) | cbg::kFromRates | (compact ? cbg::kCompactOut : 0u);
    a.index = index;
    a.count = count;
    cudaError_t e = cbg::launch_transport_mixed(KM, m->d_transport_mixed, (uint32_t)m->host.transport_mixed_blob.size(),
                                                &a, n, st, m->d_status);
    return e == cudaSuccess ? CB_OK : cuda_fail(e, "mixed transport kernel (gathered cells)");
}

}  // namespace

namespace cbi {
int fail(int code, const std::string& msg) { return ::fail(code, msg); }
int cuda_fail(cudaError_t e, const char* what) { return ::cuda_fail(e, what); }
MechView view(const cb_mech* m) {
    return MechView{m->host.K, m->host.A, m->device, m->host.transport_ready ? 1 : 0, m->host.T0, &m->host.rates_blob,
                    &m->host.rates_mixed_blob};
}
int transport_gather(cb_mech* m, size_t n, const double* const* in, double* const* out, const uint32_t* index,
                     const uint32_t* count, bool compact, uint32_t flags, cudaStream_t st) {
    if (!m->host.transport_ready) return ::fail(CB_ERR_NOT_READY, "cb_transport_setup has not run");
    if (n == 0) return CB_OK;
    switch (m->kmax) {
    case 16: return gather_launch<16>(m, n, in, out, index, count, compact, flags, st);
    case 64: return gather_launch<64>(m, n, in, out, index, count, compact, flags, st);
    case 256: return gather_launch<256>(m, n, in, out, index, count, compact, flags, st);
    default: return ::fail(CB_ERR_UNSUPPORTED, "species count outside the compiled capacities");
    }
}
int transport_gather_mixed(cb_mech* m, size_t n, const double* const* in, double* const* out, const uint32_t* index,
                           const uint32_t* count, bool compact, uint32_t flags, cudaStream_t st) {
    if (!m->host.transport_ready) return ::fail(CB_ERR_NOT_READY, "cb_transport_setup has not run");
    if (n == 0) return CB_OK;
    switch (m->kmax) {
    case 16: return gather_launch_mixed<16>(m, n, in, out, index, count, compact, flags, st);
    case 64: return gather_launch_mixed<64>(m, n, in, out, index, count, compact, flags, st);
    case 256: return gather_launch_mixed<256>(m, n, in, out, index, count, compact, flags, st);
    default: return ::fail(CB_ERR_UNSUPPORTED, "species count outside the compiled capacities");
    }
}
int check_status(cb_mech* m) { return ::check_status(m); }
}  // namespace cbi

extern "C" {

const char* cb_last_error(void) { return g_error.c_str(); }
const char* cb_version(void) { return "combustion_gb300 0.1 (sm_103a)"; }

int cb_mech_create(const cb_mech_desc* desc, cb_mech** out) {
    if (!out) return fail(CB_ERR_INVALID, "null output handle");
    *out = nullptr;
    cb_mech* m = new cb_mech();
    std::string err;
    int rc = cbg::build_mechanism(desc, m->host, err);
    if (rc) { delete m; return fail(rc, err); }
    m->kmax = cbg::kmax_for(m->host.K, m->host.n_eff);
    if (!m->kmax) { delete m; return fail(CB_ERR_UNSUPPORTED, "more than 256 species or 1024 third-body reactions"); }
    cudaError_t e = cudaGetDevice(&m->device);
    if (e == cudaSuccess) e = cudaMalloc(&m->d_rates, m->host.rates_blob.size());
    if (e == cudaSuccess) e = cudaMemcpy(m->d_rates, m->host.rates_blob.data(), m->host.rates_blob.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&m->d_rates_mixed, m->host.rates_mixed_blob.size());
    if (e == cudaSuccess)
        e = cudaMemcpy(m->d_rates_mixed, m->host.rates_mixed_blob.data(), m->host.rates_mixed_blob.size(),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&m->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&m->d_count, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(m->d_status, 0, sizeof(int));
    if (e != cudaSuccess) { cb_mech_destroy(m); return cuda_fail(e, "mechanism upload"); }
    *out = m;
    return CB_OK;
}

int cb_mech_validate(const cb_mech_desc* desc, cb_mech_info* info) {
    cbg::HostMechanism h;
    std::string err;
    int rc = cbg::build_mechanism(desc, h, err);
    if (rc) return fail(rc, err);
    if (!cbg::kmax_for(h.K, h.n_eff)) return fail(CB_ERR_UNSUPPORTED, "more than 256 species or 1024 third-body reactions");
    if (info) {
        std::memset(info, 0, sizeof *info);
        info->n_species = h.K; info->n_active = h.A; info->n_reactions = h.R;
        info->rates_inputs = h.K + 3; info->rates_outputs = h.A + 2;
        info->transport_inputs = h.K + 1; info->transport_outputs = h.K + 2;
        info->device_table_bytes = h.rates_blob.size();
    }
    return CB_OK;
}

int cb_transport_fit(const cb_mech_desc* desc, double T0, double* cond, double* visc, double* diff) {
    cbg::HostMechanism h;
    std::string err;
    int rc = cbg::build_mechanism(desc, h, err);
    if (rc) return fail(rc, err);
    rc = cbg::build_transport(h, T0, 1.0, 1.0, err);
    if (rc) return fail(rc, err);
    if (cond) std::memcpy(cond, h.fit_cond.data(), h.fit_cond.size() * sizeof(double));
    if (visc) std::memcpy(visc, h.fit_visc.data(), h.fit_visc.size() * sizeof(double));
    if (diff) std::memcpy(diff, h.fit_diff.data(), h.fit_diff.size() * sizeof(double));
    return CB_OK;
}

int cb_count_nonfinite(cb_mech* m, size_t n, int32_t n_arrays, const double* const* arrays, uint64_t* count,
                       uint32_t flags, void* stream) {
    if (!m || !arrays || !count || n_arrays < 0) return fail(CB_ERR_INVALID, "bad argument");
    if (flags & ~CB_HOST_MEMORY) return fail(CB_ERR_INVALID, "unknown flag");
    for (int q = 0; q < n_arrays; q++) if (!arrays[q]) return fail(CB_ERR_INVALID, "null array");
    if (flags & CB_HOST_MEMORY) {
        uint64_t c = 0;
        for (int q = 0; q < n_arrays; q++)
            for (size_t i = 0; i < n; i++) c += !std::isfinite(arrays[q][i]);
        *count = c;
        return CB_OK;
    }
    CB_CUDA(cudaSetDevice(m->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CB_CUDA(cudaMemsetAsync(m->d_count, 0, sizeof(unsigned long long), st));
    for (int q0 = 0; q0 < n_arrays; q0 += cbg::kCountArrays) {
        cbg::CountArgs a;
        a.m = std::min(cbg::kCountArrays, n_arrays - q0);
        for (int q = 0; q < a.m; q++) a.a[q] = arrays[q0 + q];
        CB_CUDA(cbg::launch_count_nonfinite(a, n, m->d_count, st));
    }
    unsigned long long c = 0;
    CB_CUDA(cudaMemcpyAsync(&c, m->d_count, sizeof c, cudaMemcpyDeviceToHost, st));
    CB_CUDA(cudaStreamSynchronize(st));
    *count = c;
    return CB_OK;
}

int cb_mech_destroy(cb_mech* m) {
    if (!m) return CB_OK;
    cudaSetDevice(m->device);
    for (int s = 0; s < 3; s++) {
        if (m->copy_stream[s]) { cudaStreamSynchronize(m->copy_stream[s]); cudaStreamDestroy(m->copy_stream[s]); }
    }
    for (int s = 0; s < 2; s++)
        for (int e = 0; e < 3; e++)
            if (m->slot_event[s][e]) cudaEventDestroy(m->slot_event[s][e]);
    cudaFree(m->d_rates);
    cudaFree(m->d_transport);
    cudaFree(m->d_rates_mixed);
    cudaFree(m->d_transport_mixed);
    cudaFree(m->d_status);
    cudaFree(m->d_count);
    cudaFree(m->d_stage);
    delete m;
    return CB_OK;
}

int cb_mech_query(const cb_mech* m, cb_mech_info* info) {
    if (!m || !info) return fail(CB_ERR_INVALID, "null argument");
    std::memset(info, 0, sizeof *info);
    info->n_species = m->host.K;
    info->n_active = m->host.A;
    info->n_reactions = m->host.R;
    info->transport_ready = m->host.transport_ready;
    info->T0 = m->host.T0;
    info->viscosity0 = m->host.mu0;
    info->conductivity0 = m->host.lambda0;
    info->rates_inputs = m->host.K + 3;
    info->rates_outputs = m->host.A + 2;
    info->transport_inputs = m->host.K + 1;
    info->transport_outputs = m->host.K + 2;
    info->device_table_bytes = m->host.rates_blob.size() + m->host.transport_blob.size();
    return CB_OK;
}

int cb_transport_setup(cb_mech* m, double T0, double viscosity0, double conductivity0) {
    if (!m) return fail(CB_ERR_INVALID, "null mechanism");
    std::string err;
    int rc = cbg::build_transport(m->host, T0, viscosity0, conductivity0, err);
    if (rc) return fail(rc, err);
    CB_CUDA(cudaSetDevice(m->device));
    if (m->d_transport || m->d_transport_mixed) {
        CB_CUDA(cudaDeviceSynchronize());
        cudaFree(m->d_transport);
        cudaFree(m->d_transport_mixed);
        m->d_transport = m->d_transport_mixed = nullptr;
    }
    CB_CUDA(cudaMalloc(&m->d_transport, m->host.transport_blob.size()));
    CB_CUDA(cudaMemcpy(m->d_transport, m->host.transport_blob.data(), m->host.transport_blob.size(), cudaMemcpyHostToDevice));
    CB_CUDA(cudaMalloc(&m->d_transport_mixed, m->host.transport_mixed_blob.size()));
    CB_CUDA(cudaMemcpy(m->d_transport_mixed, m->host.transport_mixed_blob.data(), m->host.transport_mixed_blob.size(),
                       cudaMemcpyHostToDevice));
    return CB_OK;
}

int cb_transport_coefficients(const cb_mech* m, double* cond, double* visc, double* diff) {
    if (!m) return fail(CB_ERR_INVALID, "null mechanism");
    if (!m->host.transport_ready) return fail(CB_ERR_NOT_READY, "cb_transport_setup has not run");
    if (cond) std::memcpy(cond, m->host.fit_cond.data(), m->host.fit_cond.size() * sizeof(double));
    if (visc) std::memcpy(visc, m->host.fit_visc.data(), m->host.fit_visc.size() * sizeof(double));
    if (diff) std::memcpy(diff, m->host.fit_diff.data(), m->host.fit_diff.size() * sizeof(double));
    return CB_OK;
}

int cb_rates_f64(cb_mech* m, size_t n, const double* const* inputs, double* const* outputs, uint32_t flags,
                 void* stream) {
    return call(m, Path::Rates, n, inputs, outputs, flags, stream);
}

int cb_reaction_rates_f64(cb_mech* m, size_t n, const double* const* inputs, double* const* outputs, uint32_t flags,
                          void* stream) {
    return call(m, Path::ReactionRates, n, inputs, outputs, flags, stream);
}

int cb_transport_f64(cb_mech* m, size_t n, const double* const* inputs, double* const* outputs, uint32_t flags,
                     void* stream) {
    return call(m, Path::Transport, n, inputs, outputs, flags, stream);
}

int cb_rates_mixed(cb_mech* m, size_t n, const double* const* inputs, double* const* outputs, uint32_t flags,
                   void* stream) {
    return call(m, Path::RatesMixed, n, inputs, outputs, flags, stream);
}

int cb_transport_mixed(cb_mech* m, size_t n, const double* const* inputs, double* const* outputs, uint32_t flags,
                       void* stream) {
    return call(m, Path::TransportMixed, n, inputs, outputs, flags, stream);
}

int cb_rates_transport_mixed(cb_mech* m, size_t n, const double* const* inputs, double* const* rates_out,
                             double* const* transport_out, uint32_t flags, void* stream) {
    if (!m || !rates_out || !transport_out) return fail(CB_ERR_INVALID, "null argument");
    std::vector<double*> outs(rates_out, rates_out + m->host.A + 2);
    outs.insert(outs.end(), transport_out, transport_out + m->host.K + 2);
    return call(m, Path::FusedMixed, n, inputs, outs.data(), flags, stream);
}

int cb_rates_transport_f64(cb_mech* m, size_t n, const double* const* inputs, double* const* rates_out,
                           double* const* transport_out, uint32_t flags, void* stream) {
    if (!m || !rates_out || !transport_out) return fail(CB_ERR_INVALID, "null argument");
    std::vector<double*> outs(rates_out, rates_out + m->host.A + 2);
    outs.insert(outs.end(), transport_out, transport_out + m->host.K + 2);
    return call(m, Path::Fused, n, inputs, outs.data(), flags, stream);
}

int cb_work_model(const cb_mech* m, cb_work* rates, cb_work* transport) {
    if (!m) return fail(CB_ERR_INVALID, "null mechanism");
    if (rates) to_work(m->host.rates_work, rates);
    if (transport) to_work(m->host.transport_work, transport);
    return CB_OK;
}

int cb_fp64_math(int which, const double* x, double* y, size_t n, void* stream) {
    if (which < 0 || which > 2 || (n && (!x || !y))) return fail(CB_ERR_INVALID, "bad arguments");
    cbg::MathTables t = cbg::make_math_tables();
    uint8_t* d = nullptr;
    CB_CUDA(cudaMalloc(&d, sizeof t));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(d, &t, sizeof t, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cbg::launch_math_check(d, which, x, y, n, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d);
    return e == cudaSuccess ? CB_OK : cuda_fail(e, "math check");
}

int cb_debug_stage_wait_polls(int64_t polls) {
    CB_CUDA(cbg::set_stage_wait_polls((long long)polls));
    return CB_OK;
}

int cb_synchronize(cb_mech* m, void* stream) {
    if (!m) return fail(CB_ERR_INVALID, "null mechanism");
    CB_CUDA(cudaSetDevice(m->device));
    CB_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    return check_status(m);
}

}  // extern "C"
