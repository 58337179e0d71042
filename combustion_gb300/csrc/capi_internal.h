// Internal interface between the C ABI translation unit (capi.cu) and the transport surrogate
// (surrogate.cu): error reporting and the plain and mixed transport kernels on gathered cells.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/combustion_gb300.h"

namespace cbi {

int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

struct MechView {
    int K, A, device;
    int transport_ready;
    double T0;
    const std::vector<uint8_t>* rates_blob;        // host copy of the rates tables
    const std::vector<uint8_t>* rates_mixed_blob;  // host copy of the mixed-precision rates tables
};
MechView view(const cb_mech* m);

// Plain FP64 transport on rates-layout inputs (K + 3 device arrays) for up to n cells. With `index`,
// launch cell j is input cell index[j] (masked with kIndexMask) and `count` (device) bounds j; outputs go
// to the same cell or, with `compact`, to position j of the output arrays.
int transport_gather(cb_mech* m, size_t n, const double* const* in, double* const* out, const uint32_t* index,
                     const uint32_t* count, bool compact, uint32_t flags, cudaStream_t st);

// The same with the mixed-precision transport kernel (FP32 fits and mixing).
int transport_gather_mixed(cb_mech* m, size_t n, const double* const* in, double* const* out,
                           const uint32_t* index, const uint32_t* count, bool compact, uint32_t flags,
                           cudaStream_t st);

int check_status(cb_mech* m);

}  // namespace cbi
