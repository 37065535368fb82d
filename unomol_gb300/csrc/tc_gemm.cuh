// BF16 GEMM on the 5th-generation tensor cores, TMA-fed, FP32 accumulation in tensor memory.
//
//   C[M x N] = A[M x K] . B[N x K]^T      (A and B row major with K contiguous: both K-major)
//
// One CTA (4 warps) computes a 128 x BN tile over a range of K chunks of 64 (split-K: blockIdx.z
// picks the range and partial tiles are added with atomics).  Data movement and MMA are decoupled by
// a ring of TC_STAGES shared-memory stages:
//   * warp 0 / lane 0 (producer): for every chunk, waits until the stage is free, arms its "full"
//     mbarrier with the stage's byte count and issues two TMA tile loads (cp.async.bulk.tensor.2d,
//     128-byte swizzle; rows or K beyond the matrix are zero-filled by the TMA unit);
//   * warp 1 / lane 0 (MMA issuer): waits for the stage's "full" barrier, issues four
//     tcgen05.mma.cta_group::1.kind::f16 (K = 16 each; shared-memory descriptors in the 128-byte-swizzle
//     K-major layout: 8-row atoms of 1024 bytes, the start address advanced by 32 bytes per K step),
//     and commits them to the stage's "empty" barrier, which hands the stage back to the producer;
//     after the last chunk it commits to the "done" barrier;
//   * all four warps: wait for "done", read the accumulator with tcgen05.ld (warp w owns rows
//     32w..32w+31), apply the fused epilogue and store.
// Every wait is bounded: a wait that gives up sets the CTA's error flag and the kernel's status word;
// before returning, the CTA waits (bounded) for the TMA loads it issued and the MMAs it committed, and
// always releases its tensor memory.  The pipeline waits (producer on "empty", MMA issuer on "full")
// poll TcGemmArgs::pipeline_polls times (0: TC_WAIT_POLLS; negative: not at all, so that the first
// of them gives up -- the host-side test of this failure path); the drain waits for work already
// issued ("done", the outstanding "full" phases) always poll TC_WAIT_POLLS times, so nothing issued is
// still in flight when the CTA releases its tensor memory and exits.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cstdint>

namespace ugb {

constexpr int TC_BM = 128;   // MMA M
constexpr int TC_BK = 64;    // K per stage: one 128-byte swizzle row of BF16
constexpr int TC_THREADS = 128;
constexpr int TC_STAGES = 4;
constexpr int TC_WAIT_POLLS = 1 << 22;

enum TcEpilogue : int {
    TC_EPI_F32 = 0,         // Cf = acc
    TC_EPI_BIAS_SILU = 1,   // Z = acc + bias; Cb = silu(Z)
    TC_EPI_BIAS_F32 = 2,    // Cf = acc + bias
    TC_EPI_DSILU = 3,       // Cb = acc * silu'(Z), and Cf = the same in fp32 when Cf is set
    TC_EPI_F32_ADD = 4,     // Cf += acc (atomic; split-K partial tiles)
};

struct TcGemmArgs {
    const __nv_bfloat16* A;  // [M][lda], K contiguous
    const __nv_bfloat16* B;  // [N][ldb], K contiguous
    int M, N, K, lda, ldb;
    int epi;
    const float* bias;       // [N]
    float* Cf;               // fp32 output [M][ldc]
    __nv_bfloat16* Cb;       // bf16 output [M][ldc]
    float* Z;                // fp32 pre-activation out (BIAS_SILU) / in (DSILU), [M][ldc]
    int ldc;
    int chunks_per_split;    // K chunks of one blockIdx.z
    int* status;             // set to 1 when a wait gave up
    int pipeline_polls;      // polls of the pipeline waits: 0 = TC_WAIT_POLLS, < 0 = none (give up at once)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor, K-major with 128-byte swizzle: start >> 4, LBO = 16 bytes (unused
// for swizzled K-major), SBO = 1024 bytes (one 8-row atom), descriptor version 1, layout 2 = SWIZZLE_128B
__device__ __forceinline__ uint64_t tc_desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// instruction descriptor, kind::f16: BF16 A and B, FP32 D, both K-major, M x N
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
    return (1u << 4)                          // D format: F32
           | (1u << 7)                        // A format: BF16
           | (1u << 10)                       // B format: BF16
           | ((uint32_t)(N >> 3) << 17)       // N / 8
           | ((uint32_t)(M >> 4) << 24);      // M / 16
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int polls = TC_WAIT_POLLS) {
    uint32_t done = 0;
    for (int it = 0; it < polls && !done; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
    }
    return done != 0;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

template <int BN>
struct TcSmem {
    static constexpr int A_BYTES = TC_BM * TC_BK * 2;  // 16 KB
    static constexpr int B_BYTES = BN * TC_BK * 2;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr int DYN = TC_STAGES * STAGE + 1024;  // + alignment slack (1024-byte aligned stages)
};

template <int BN>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_tma(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const TcGemmArgs g) {
    extern __shared__ unsigned char dsm[];
    __shared__ __align__(8) uint64_t full[TC_STAGES], empty[TC_STAGES], done;
    __shared__ uint32_t tmem_base;
    __shared__ int failed, issued, consumed;
    using SM = TcSmem<BN>;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * TC_BM, n0 = blockIdx.y * BN;
    const int nk_all = (g.K + TC_BK - 1) / TC_BK;
    const int kc_begin = blockIdx.z * g.chunks_per_split;
    const int kc_end = min(nk_all, kc_begin + g.chunks_per_split);
    const int nk = kc_end - kc_begin;
    if (nk <= 0) return;  // uniform over the CTA, before any allocation
    const uint32_t base = (smem_u32(dsm) + 1023u) & ~1023u;
    constexpr uint32_t NCOL = BN;  // 64, 128 or 256 TMEM columns
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)), "r"(NCOL));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 32) {
        failed = 0;
        issued = 0;
        consumed = 0;
        for (int s = 0; s < TC_STAGES; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    const int polls = g.pipeline_polls == 0 ? TC_WAIT_POLLS : max(g.pipeline_polls, 0);
    if (warp == 0 && lane == 0) {
        // producer: TMA loads into the ring
        for (int i = 0; i < nk; ++i) {
            const int s = i % TC_STAGES;
            if (i >= TC_STAGES && !mbar_wait(smem_u32(&empty[s]), (uint32_t)((i / TC_STAGES - 1) & 1), polls)) {
                atomicExch(&failed, 1);
                break;
            }
            if (*(volatile int*)&failed) break;
            const uint32_t sa = base + s * SM::STAGE;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&full[s])), "r"(SM::STAGE)
                         : "memory");
            const int kx = (kc_begin + i) * TC_BK;
            tma_load_2d(sa, &tmA, kx, m0, smem_u32(&full[s]));
            tma_load_2d(sa + SM::A_BYTES, &tmB, kx, n0, smem_u32(&full[s]));
            issued = i + 1;
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = tc_idesc(TC_BM, BN);
        int i = 0;
        for (; i < nk; ++i) {
            const int s = i % TC_STAGES;
            if (!mbar_wait(smem_u32(&full[s]), (uint32_t)((i / TC_STAGES) & 1), polls)) {
                atomicExch(&failed, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t sa = base + s * SM::STAGE;
#pragma unroll
            for (int k = 0; k < TC_BK / 16; ++k) {
                const uint64_t ad = tc_desc_sw128(sa + k * 32);
                const uint64_t bd = tc_desc_sw128(sa + SM::A_BYTES + k * 32);
                const uint32_t acc = (i > 0 || k > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&empty[s]))
                         : "memory");
        }
        consumed = i;
        // completion of everything issued so far (also after a failure, so that nothing is in flight)
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&done))
                     : "memory");
    }
    __syncwarp();
    const bool ok = mbar_wait(smem_u32(&done), 0);
    if (!ok) atomicExch(&failed, 1);
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
    if (!failed) {
        const int row = m0 + warp * 32 + lane;
        const bool vec4 = (g.ldc & 3) == 0;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            if (n0 + c0 >= g.N) break;  // uniform
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            if (row >= g.M) continue;
            const int col0 = n0 + c0;
            const long long o0 = (long long)row * g.ldc + col0;
            float v[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
            const bool full16 = col0 + 16 <= g.N;
            if (g.epi == TC_EPI_F32 || g.epi == TC_EPI_BIAS_F32) {
                if (g.epi == TC_EPI_BIAS_F32)
#pragma unroll
                    for (int j = 0; j < 16; ++j) v[j] += col0 + j < g.N ? g.bias[col0 + j] : 0.f;
                if (full16 && vec4) {
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        *reinterpret_cast<float4*>(g.Cf + o0 + 4 * q) = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                } else {
                    for (int j = 0; j < 16 && col0 + j < g.N; ++j) g.Cf[o0 + j] = v[j];
                }
            } else if (g.epi == TC_EPI_F32_ADD) {
                for (int j = 0; j < 16 && col0 + j < g.N; ++j) atomicAdd(g.Cf + o0 + j, v[j]);
            } else if (g.epi == TC_EPI_BIAS_SILU) {
                __align__(16) __nv_bfloat16 h[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const float z = v[j] + (col0 + j < g.N ? g.bias[col0 + j] : 0.f);
                    v[j] = z;
                    h[j] = __float2bfloat16(z / (1.f + __expf(-z)));
                }
                if (full16 && (g.ldc & 7) == 0) {
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        *reinterpret_cast<float4*>(g.Z + o0 + 4 * q) = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                    *reinterpret_cast<uint4*>(g.Cb + o0) = *reinterpret_cast<const uint4*>(h);
                    *reinterpret_cast<uint4*>(g.Cb + o0 + 8) = *reinterpret_cast<const uint4*>(h + 8);
                } else {
                    for (int j = 0; j < 16 && col0 + j < g.N; ++j) {
                        g.Z[o0 + j] = v[j];
                        g.Cb[o0 + j] = h[j];
                    }
                }
            } else {  // TC_EPI_DSILU
                __align__(16) __nv_bfloat16 h[16];
                for (int j = 0; j < 16; ++j) {
                    const float z = col0 + j < g.N ? g.Z[o0 + j] : 0.f;
                    const float s = 1.f / (1.f + __expf(-z));
                    v[j] = v[j] * s * (1.f + z * (1.f - s));
                    h[j] = __float2bfloat16(v[j]);
                }
                if (full16 && (g.ldc & 7) == 0) {
                    *reinterpret_cast<uint4*>(g.Cb + o0) = *reinterpret_cast<const uint4*>(h);
                    *reinterpret_cast<uint4*>(g.Cb + o0 + 8) = *reinterpret_cast<const uint4*>(h + 8);
                    if (g.Cf)
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            *reinterpret_cast<float4*>(g.Cf + o0 + 4 * q) = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                } else {
                    for (int j = 0; j < 16 && col0 + j < g.N; ++j) {
                        g.Cb[o0 + j] = h[j];
                        if (g.Cf) g.Cf[o0 + j] = v[j];
                    }
                }
            }
        }
    } else if (tid == 0) {
        if (g.status) atomicExch(g.status, 1);
        // TMA loads issued but not consumed still land in this CTA's shared memory: wait for them
        for (int j = consumed; j < issued; ++j) mbar_wait(smem_u32(&full[j % TC_STAGES]), (uint32_t)((j / TC_STAGES) & 1));
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOL));
}

}  // namespace ugb
