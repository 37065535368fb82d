// BF16 GEMM on the 5th-generation tensor cores (tcgen05), FP32 accumulation in tensor memory.
//
//   C[M x N] = A[M x K] . B[N x K]^T
//
// Each operand is either K-contiguous in global memory (element (r, k) at [r * ld + k]) or
// row-contiguous ("transposed": element (r, k) at [k * ld + r]); the transpose happens while staging,
// so the weight-gradient products dW = dZ^T . H read the activations as they were written.
//
// One CTA (128 threads) computes a 128 x BN tile over a range of K chunks (split-K: blockIdx.z picks
// the range, partial tiles are added with atomics).  Per K chunk of 64 the 128 threads stage A and B
// into shared memory in the no-swizzle K-major canonical layout (8-row x 16-byte core matrices; LBO =
// 128 B between core matrices along K, SBO = 1024 B between 8-row groups), make the writes visible to
// the async proxy, and one elected thread issues four tcgen05.mma (K = 16 each) into the TMEM
// accumulator and commits them to an mbarrier that every thread waits on (bounded).  The epilogue
// reads the accumulator with tcgen05.ld (warp w owns rows 32w..32w+31), applies the fused epilogue and
// stores.  A wait that gives up sets an error flag and skips the stores; the TMEM allocation is always
// released.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace ugb {

constexpr int TC_BM = 128;   // MMA M
constexpr int TC_BK = 64;    // K per shared-memory stage (4 MMAs of K = 16)
constexpr int TC_THREADS = 128;
constexpr int TC_WAIT_POLLS = 1 << 22;

enum TcEpilogue : int {
    TC_EPI_F32 = 0,         // Cf = acc
    TC_EPI_BIAS_SILU = 1,   // Z = acc + bias; Cb = silu(Z)
    TC_EPI_BIAS_F32 = 2,    // Cf = acc + bias
    TC_EPI_DSILU = 3,       // Cb = acc * silu'(Z), and Cf = the same in fp32 when Cf is set
    TC_EPI_F32_ADD = 4,     // Cf += acc (atomic; split-K partial tiles)
};

struct TcGemmArgs {
    const __nv_bfloat16* A;
    const __nv_bfloat16* B;
    int M, N, K, lda, ldb;
    int a_trans, b_trans;    // 1: element (r, k) at [k * ld + r]
    int vec_a, vec_b;        // 16-byte loads allowed (ld % 8 == 0 and a 16-byte aligned base)
    int epi;
    const float* bias;       // [N]
    float* Cf;               // fp32 output [M][ldc]
    __nv_bfloat16* Cb;       // bf16 output [M][ldc]
    float* Z;                // fp32 pre-activation out (BIAS_SILU) / in (DSILU), [M][ldc]
    int ldc;
    int chunks_per_split;    // K chunks of one blockIdx.z
    int* status;             // set to 1 when a wait gave up
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor (no swizzle, K-major): start >> 4, LBO >> 4, SBO >> 4, version 1
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of tcgen05
    return d;                // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor, kind::f16: BF16 A and B, FP32 D, both K-major, M x N
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
    return (1u << 4)                          // D format: F32
           | (1u << 7)                        // A format: BF16
           | (1u << 10)                       // B format: BF16
           | ((uint32_t)(N >> 3) << 17)       // N / 8
           | ((uint32_t)(M >> 4) << 24);      // M / 16
}

// byte offset of element (row, k) in a [rows x 64] K-major no-swizzle tile
__device__ __forceinline__ int tc_off(int row, int k) {
    return (k >> 3) * 128 + (row >> 3) * 1024 + (row & 7) * 16 + (k & 7) * 2;
}

// Stage rows [r0, r0 + ROWS) x k [k0, k0 + 64) of an operand into the canonical tile, zero outside
// rows < rlim and k < klim.
template <int ROWS>
__device__ __forceinline__ void tc_stage(unsigned char* s, const __nv_bfloat16* src, int ld, int trans, int vec, int r0,
                                         int rlim, int k0, int klim) {
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    if (!trans) {
        // one thread: 8 consecutive k of one row (one 16-byte row of a core matrix)
        for (int e = threadIdx.x; e < ROWS * (TC_BK / 8); e += TC_THREADS) {
            const int r = e >> 3, kq = (e & 7) * 8;
            const int gr = r0 + r, gk = k0 + kq;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (gr < rlim) {
                const __nv_bfloat16* p = src + (long long)gr * ld + gk;
                if (vec && gk + 8 <= klim) {
                    v = *reinterpret_cast<const uint4*>(p);
                } else {
                    __nv_bfloat16 t[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) t[q] = gk + q < klim ? p[q] : zero;
                    v = *reinterpret_cast<uint4*>(t);
                }
            }
            *reinterpret_cast<uint4*>(s + tc_off(r, kq)) = v;
        }
    } else {
        // one thread: 8 consecutive rows at one k (a contiguous 16 bytes of the source)
        for (int e = threadIdx.x; e < (ROWS / 8) * TC_BK; e += TC_THREADS) {
            const int rq = (e % (ROWS / 8)) * 8, k = e / (ROWS / 8);
            const int gk = k0 + k, gr = r0 + rq;
            __align__(16) __nv_bfloat16 t[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) t[q] = zero;
            if (gk < klim) {
                const __nv_bfloat16* p = src + (long long)gk * ld + gr;
                if (vec && gr + 8 <= rlim) {
                    *reinterpret_cast<uint4*>(t) = *reinterpret_cast<const uint4*>(p);
                } else {
#pragma unroll
                    for (int q = 0; q < 8; ++q) t[q] = gr + q < rlim ? p[q] : zero;
                }
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) *reinterpret_cast<__nv_bfloat16*>(s + tc_off(rq + q, k)) = t[q];
        }
    }
}

template <int BN>
__global__ void __launch_bounds__(TC_THREADS) tc_gemm_kernel(const TcGemmArgs g) {
    __shared__ __align__(1024) unsigned char sA[TC_BM * TC_BK * 2];
    __shared__ __align__(1024) unsigned char sB[BN * TC_BK * 2];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int failed;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * TC_BM, n0 = blockIdx.y * BN;
    const int nk_all = (g.K + TC_BK - 1) / TC_BK;
    const int kc_begin = blockIdx.z * g.chunks_per_split;
    const int kc_end = min(nk_all, kc_begin + g.chunks_per_split);
    if (kc_begin >= kc_end) return;  // uniform over the CTA, before any allocation
    constexpr uint32_t NCOL = BN < 32 ? 32 : BN;  // TMEM columns: power of two >= 32
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)), "r"(NCOL));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        failed = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = tc_idesc(TC_BM, BN);
    uint32_t phase = 0;
    for (int kc = kc_begin; kc < kc_end; ++kc) {
        const int k0 = kc * TC_BK;
        tc_stage<TC_BM>(sA, g.A, g.lda, g.a_trans, g.vec_a, m0, g.M, k0, g.K);
        tc_stage<BN>(sB, g.B, g.ldb, g.b_trans, g.vec_b, n0, g.N, k0, g.K);
        asm volatile("fence.proxy.async.shared::cta;");  // generic-proxy stores -> tensor-core reads
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
            for (int s = 0; s < TC_BK / 16; ++s) {
                const uint64_t ad = tc_desc(smem_u32(sA) + s * 256, 128, 1024);
                const uint64_t bd = tc_desc(smem_u32(sB) + s * 256, 128, 1024);
                const uint32_t acc = (kc > kc_begin || s > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&mbar)));
        }
        // bounded wait for the MMAs of this chunk (their completion also frees the staging tiles)
        uint32_t done = 0;
        for (int it = 0; it < TC_WAIT_POLLS && !done; ++it) {
            asm volatile(
                "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
                : "=r"(done)
                : "r"(smem_u32(&mbar)), "r"(phase));
        }
        if (!done) failed = 1;
        phase ^= 1;
        __syncthreads();
        if (failed) break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (!failed) {
        // epilogue: warp w reads accumulator rows (lanes) 32w..32w+31, 16 columns per load
        const int row = m0 + warp * 32 + lane;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            if (row < g.M) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int col = n0 + c0 + j;
                    if (col >= g.N) continue;
                    const float acc = __uint_as_float(r[j]);
                    const long long o = (long long)row * g.ldc + col;
                    if (g.epi == TC_EPI_F32) {
                        g.Cf[o] = acc;
                    } else if (g.epi == TC_EPI_F32_ADD) {
                        atomicAdd(g.Cf + o, acc);
                    } else if (g.epi == TC_EPI_BIAS_F32) {
                        g.Cf[o] = acc + g.bias[col];
                    } else if (g.epi == TC_EPI_BIAS_SILU) {
                        const float z = acc + g.bias[col];
                        g.Z[o] = z;
                        g.Cb[o] = __float2bfloat16(z / (1.f + __expf(-z)));
                    } else {  // TC_EPI_DSILU
                        const float z = g.Z[o];
                        const float s = 1.f / (1.f + __expf(-z));
                        const float d = acc * s * (1.f + z * (1.f - s));
                        g.Cb[o] = __float2bfloat16(d);
                        if (g.Cf) g.Cf[o] = d;
                    }
                }
            }
        }
    } else if (tid == 0 && g.status) {
        atomicExch(g.status, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOL));
}

// Launch C = A . B^T with split-K when the output has too few tiles for the GPU.  Split-K needs an
// additive epilogue (TC_EPI_F32_ADD on a zeroed or accumulating Cf); other epilogues run unsplit.
inline cudaError_t tc_gemm_launch(TcGemmArgs g, cudaStream_t s, int num_sms) {
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) return cudaSuccess;
    const int bn = g.N <= 32 ? 32 : g.N <= 64 ? 64 : 128;
    const int tiles_m = (g.M + TC_BM - 1) / TC_BM, tiles_n = (g.N + bn - 1) / bn;
    const int nk = (g.K + TC_BK - 1) / TC_BK;
    int splits = 1;
    if (g.epi == TC_EPI_F32_ADD) {
        const int want = (2 * num_sms + tiles_m * tiles_n - 1) / (tiles_m * tiles_n);
        splits = want < nk ? want : nk;
        if (splits < 1) splits = 1;
    }
    g.chunks_per_split = (nk + splits - 1) / splits;
    splits = (nk + g.chunks_per_split - 1) / g.chunks_per_split;  // every split has >= 1 chunk
    dim3 grid(tiles_m, tiles_n, splits);
    // Unused dynamic shared memory caps the CTAs per SM so that their TMEM columns fit the SM's 512
    // (BN = 128: 4 CTAs of 46 KB; BN = 64: 8 CTAs of 26 KB) and no tcgen05.alloc has to wait.
    if (bn == 32) tc_gemm_kernel<32><<<grid, TC_THREADS, 0, s>>>(g);
    else if (bn == 64) tc_gemm_kernel<64><<<grid, TC_THREADS, 2 * 1024, s>>>(g);
    else tc_gemm_kernel<128><<<grid, TC_THREADS, 14 * 1024, s>>>(g);
    return cudaGetLastError();
}

}  // namespace ugb
