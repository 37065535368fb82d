// Microbenchmarks of the peaks the Fock build is measured against: FP64 and FP32 FMA throughput (the
// ERI kernels are bound by these pipes, not by HBM or tensor cores), and the L2 figures of the J/K
// scatter (L2 read bandwidth and FP64 atomic-add throughput on an accumulator of the build's size).
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

// L2 read bandwidth: a 32 MiB buffer (L2 resident after a warm-up pass) read as 16-byte vectors
__global__ void l2_read(const float4* __restrict__ buf, long long n, int passes, float* out) {
    float acc = 0.f;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (int p = 0; p < passes; ++p)
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const float4 v = __ldcg(buf + i);
            acc += v.x + v.y + v.z + v.w;
        }
    if (acc == -12345.678f) out[blockIdx.x] = acc;  // keeps the loads live; the buffer is zero
}

// FP64 atomic adds into a 1.4 MB array (the size of the 416-function accumulator of the Fock build),
// addresses scattered by a multiplicative hash
__global__ void atomics_f64(double* __restrict__ acc, unsigned n, int iters) {
    unsigned h = (blockIdx.x * blockDim.x + threadIdx.x) * 2654435761u;
    for (int i = 0; i < iters; ++i) {
        h = h * 1664525u + 1013904223u;
        atomicAdd(acc + (h >> 8) % n, 1.0);
    }
}

template <typename F>
int time_kernel(F launch, float* ms) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    launch();  // warm-up
    cudaEventRecord(e0);
    launch();
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return err == cudaSuccess ? UNOMOL_OK : UNOMOL_ECUDA;
}

}  // namespace

extern "C" int unomol_gpu_l2_peak(double* read_gbs, double* atomic_gops) {
    if (!read_gbs || !atomic_gops) return UNOMOL_EINVAL;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return UNOMOL_ENODEV;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return UNOMOL_ECUDA;
    const long long bytes = 32ll << 20;
    const long long n = bytes / 16;
    void* buf = nullptr;
    float* out = nullptr;
    if (cudaMalloc(&buf, bytes) != cudaSuccess) return UNOMOL_ENOMEM;
    if (cudaMalloc(&out, sizeof(float) * nsm * 8) != cudaSuccess) {
        cudaFree(buf);
        return UNOMOL_ENOMEM;
    }
    cudaMemset(buf, 0, bytes);
    const int passes = 20;
    float ms = 0.f;
    int rc = time_kernel([&] { l2_read<<<nsm * 8, 256>>>((const float4*)buf, n, passes, out); }, &ms);
    if (!rc) *read_gbs = (double)bytes * passes / (ms * 1e-3) / 1e9;
    const unsigned na = 416u * 416u;
    const int iters = 256;
    if (!rc) {
        cudaMemset(buf, 0, na * sizeof(double));
        rc = time_kernel([&] { atomics_f64<<<nsm * 8, 256>>>((double*)buf, na, iters); }, &ms);
        if (!rc) *atomic_gops = (double)nsm * 8 * 256 * iters / (ms * 1e-3) / 1e9;
    }
    cudaFree(buf);
    cudaFree(out);
    return rc;
}

extern "C" int unomol_gpu_fma_peak(int fp64, double* tflops) {
    if (!tflops) return UNOMOL_EINVAL;
    return fp64 ? run<double>(tflops) : run<float>(tflops);
}
