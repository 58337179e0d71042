// Device diagnostics used for roofline reporting: the FP64 FMA issue rate of the current GPU.
#include <cuda_runtime.h>

#include "../../include/combustion_gb300.h"

namespace {
// Eight independent FMA chains per thread; the result is stored so that nothing is optimised away.
__global__ void fma_chains(double* out, int iters, double a, double b) {
    double x[8];
    for (int c = 0; c < 8; c++) x[c] = threadIdx.x * 1e-3 + c;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < 8; c++) x[c] = fma(x[c], a, b);
    }
    double s = 0;
    for (int c = 0; c < 8; c++) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" int cb_device_fp64_peak(double* fma_per_second) {
    if (!fma_per_second) return CB_ERR_INVALID;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CB_ERR_CUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 256, blocks = sms * 8, iters = 4000;
    double* buf = nullptr;
    if (cudaMalloc(&buf, sizeof(double) * threads * blocks) != cudaSuccess) return CB_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains<<<blocks, threads>>>(buf, iters / 10, 1.0000001, 1e-9);
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(e0);
        fma_chains<<<blocks, threads>>>(buf, iters, 1.0000001, 1e-9);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (e != cudaSuccess) return CB_ERR_CUDA;
    *fma_per_second = 8.0 * iters * threads * (double)blocks / (best * 1e-3);
    return CB_OK;
}
