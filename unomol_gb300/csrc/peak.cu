// FMA throughput microbenchmark: the FP64 and FP32 pipe peaks the Fock kernels are measured against
// (the HBM and BF16 peaks of the machine do not bound a scalar FP64 kernel).
#include <cuda_runtime.h>

#include "../../include/unomol_gb300.h"

namespace {

template <typename R, int CHAINS>
__global__ void fma_chains(R* out, int iters, R a, R b) {
    R v[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) v[c] = R(threadIdx.x + c) * R(1e-3);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) v[c] = fma(v[c], a, b);
    }
    R s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += v[c];
    if (s == R(-12345.678)) out[blockIdx.x] = s;  // keeps the chains live; never true for these inputs
}

template <typename R>
int run(double* tflops) {
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return UNOMOL_ENODEV;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return UNOMOL_ECUDA;
    R* out = nullptr;
    if (cudaMalloc(&out, sizeof(R) * 65536) != cudaSuccess) return UNOMOL_ENOMEM;
    constexpr int CH = 8;
    const int threads = 256, blocks = nsm * 8;
    const int iters = sizeof(R) == 8 ? 2048 : 65536;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains<R, CH><<<blocks, threads>>>(out, iters / 8, R(0.999999), R(1e-7));  // warm-up
    cudaEventRecord(e0);
    fma_chains<R, CH><<<blocks, threads>>>(out, iters, R(0.999999), R(1e-7));
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return UNOMOL_ECUDA;
    const double flops = 2.0 * CH * (double)iters * threads * (double)blocks;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return UNOMOL_OK;
}

}  // namespace

extern "C" int unomol_gpu_fma_peak(int fp64, double* tflops) {
    if (!tflops) return UNOMOL_EINVAL;
    return fp64 ? run<double>(tflops) : run<float>(tflops);
}
