// Kernel arguments and launchers shared by the C ABI (capi.cu) and the kernels (kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cbg {

// Threads per block. Each block stages its own copy of the tables in shared memory, which shares the
// SM's 256 KB with the L1 cache that holds the thread-local arrays (concentrations, Gibbs exponentials,
// accumulators); 768-thread blocks keep one or two copies per SM instead of two or three and leave L1
// that room: measured at K = 53, 2^22 cells, the mixed rates kernel 54.2 -> 38.1 ms (256-thread blocks
// before; 1024-thread blocks 45.5 ms), the plain rates kernel 119.6 -> 117.0 ms, mixed transport
// 1 ms faster. Plain transport (tables of 135 KB, one block per SM) keeps 256 threads: 768 ran no
// faster (the FP64 pipe is 97 % busy either way) and its per-thread arrays then spilled past L1 into
// DRAM (24 KB per cell instead of 2 KB).
constexpr int kBlock = 768;
constexpr int kTransportBlock = 256;
constexpr int kTransportMixedBlock = 768;

// One pointer per input / output array (struct of arrays), passed by value as a kernel parameter.
template <int KMAX>
struct RatesArgs {
    const double* in[KMAX + 3];  // P/R, R/P, T, V, n_0 .. n_{K-2}
    double* out[KMAX + 2];       // dT/dt, dV/dt, wdot_0 .. wdot_{A-1}
    uint32_t flags;              // bit 1: P/R and R/P are single values
};

// Per-reaction rates of progress: inputs P/R, T, V, n_0 .. n_{K-2}; one output per reaction.
constexpr int kMaxReactions = 2048;
template <int KMAX>
struct ReactionRatesArgs {
    const double* in[KMAX + 2];
    double* out[kMaxReactions];
    uint32_t flags;
};

// Transport input layouts: the reference's (sum n, T/T0, n...) or, with kFromRates, the rates inputs
// (P/R, R/P, T, V, n...) from which sum n = (P/R * V) / T and T/T0 are derived per cell.
constexpr uint32_t kUniformPressure = 2u;
constexpr uint32_t kFromRates = 4u;
// Gathered cells (the transport surrogate's fallback and audit): cell j of the launch is input cell
// index[j] & kIndexMask, its outputs go to that cell too or, with kCompactOut, to position j.
constexpr uint32_t kCompactOut = 8u;
constexpr uint32_t kIndexMask = 0x7fffffffu;

template <int KMAX>
struct TransportArgs {
    const double* in[KMAX + 3];  // sum n, T/T0, n_0 .. n_{K-2} (or the rates inputs with kFromRates)
    double* out[KMAX + 2];       // lambda/lambda0, mu/mu0, rhoD_k/mu0
    uint32_t flags;
    const uint32_t* index;       // gathered cells (null: cell j is input j)
    const uint32_t* count;       // number of gathered cells, read on the device (null: n)
};

// Smallest compiled capacity holding K species (0 if none).
// (The per-cell efficiency sums of up to 4 * KMAX third-body / falloff reactions are kept per thread.)
inline int kmax_for(int K, int n_eff) {
    for (int km : {16, 64, 256})
        if (K <= km && n_eff <= 4 * km) return km;
    return 0;
}

int max_table_smem();
cudaError_t set_stage_wait_polls(long long polls);

// Non-finite values (NaN, infinity) in up to kCountArrays arrays of n doubles, added to *count.
constexpr int kCountArrays = 512;
struct CountArgs {
    const double* a[kCountArrays];
    int m;
};
cudaError_t launch_count_nonfinite(const CountArgs& args, size_t n, unsigned long long* count, cudaStream_t st);

// Blocks of a persistent table kernel resident per SM, the tables in shared memory (smem: the variant
// ksmem, whose dynamic shared memory limit is raised first) or read from global memory (kglobal, only
// the math tables in shared memory).
template <class KS, class KG>
cudaError_t table_kernel_occupancy(KS ksmem, KG kglobal, int block, uint32_t tab_bytes, uint32_t math_bytes,
                                   bool smem, int* per_sm) {
    *per_sm = 1;
    if (smem) {
        cudaError_t e = cudaFuncSetAttribute(ksmem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tab_bytes);
        if (e != cudaSuccess) return e;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, ksmem, block, tab_bytes);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, kglobal, block, math_bytes);
    }
    if (*per_sm < 1) *per_sm = 1;
    return cudaSuccess;
}

// Cells one wave of a kernel's persistent grid covers (its threads resident on the whole GPU): every
// thread of a launch over a multiple of it gets the same number of cells. Host arrays go through the
// GPU in chunks of whole waves.
size_t wave_rates(int kmax, uint32_t tab_bytes);
size_t wave_reaction_rates(int kmax, uint32_t tab_bytes);
size_t wave_transport(int kmax, uint32_t tab_bytes);
size_t wave_rates_mixed(int kmax, uint32_t tab_bytes);
size_t wave_transport_mixed(int kmax, uint32_t tab_bytes);
cudaError_t launch_math_check(const uint8_t* math, int which, const double* x, double* y, size_t n,
                              cudaStream_t st);
cudaError_t launch_rates(int kmax, const uint8_t* tab, uint32_t tab_bytes, const void* args, size_t n,
                         cudaStream_t st, int* status);
cudaError_t launch_reaction_rates(int kmax, const uint8_t* tab, uint32_t tab_bytes, const void* args, size_t n,
                                  cudaStream_t st, int* status);
cudaError_t launch_rates_mixed(int kmax, const uint8_t* tab, uint32_t tab_bytes, const void* args, size_t n,
                               cudaStream_t st, int* status);
cudaError_t launch_transport_mixed(int kmax, const uint8_t* tab, uint32_t tab_bytes, const void* args, size_t n,
                                   cudaStream_t st, int* status);
cudaError_t launch_transport(int kmax, const uint8_t* tab, uint32_t tab_bytes, const void* args, size_t n,
                             cudaStream_t st, int* status);

}  // namespace cbg
