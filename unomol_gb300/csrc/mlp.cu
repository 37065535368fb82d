// The learned-guess network on the tensor cores: forward and backward passes built from the tcgen05
// BF16 GEMM of tc_gemm.cuh with fused epilogues (bias + SiLU forward, SiLU derivative backward, split-K
// atomic accumulation of the weight gradients), plus small FP32 kernels for the bias gradients, the
// BF16 conversions and Adam.  Master weights are FP32; the GEMM operands are BF16 copies.
#include <atomic>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/unomol_gb300.h"
#include "mlp.h"
#include "tc_gemm.cuh"

namespace ugb {

namespace {

unsigned nblk(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// ---- tensor maps and the GEMM launch ----

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                                  const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// row-major BF16 [rows x K] (row stride ld elements) read in boxes of box_rows x 64, 128-byte swizzle
cudaError_t make_map(CUtensorMap* m, const void* ptr, int rows, int K, int ld, int box_rows) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return cudaErrorNotSupported;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows};
    const cuuint32_t es[2] = {1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int BN>
cudaError_t launch_bn(const CUtensorMap& ma, const CUtensorMap& mb, const TcGemmArgs& g, dim3 grid, cudaStream_t s) {
    static const cudaError_t attr =
        cudaFuncSetAttribute(tc_gemm_tma<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcSmem<BN>::DYN);
    if (attr != cudaSuccess) return attr;
    tc_gemm_tma<BN><<<grid, TC_THREADS, TcSmem<BN>::DYN, s>>>(ma, mb, g);
    return cudaGetLastError();
}

// C = A . B^T; operands K-major, row strides multiples of 8 elements, 16-byte aligned.  Split-K (an
// additive epilogue) when the output has fewer tiles than the GPU has SMs.
// Poll limit of the GEMMs' pipeline waits for the whole process (unomol_tc_set_wait_polls).
std::atomic<int> g_tc_pipeline_polls{0};

cudaError_t tc_gemm_launch(TcGemmArgs g, cudaStream_t s, int num_sms) {
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) return cudaSuccess;
    g.pipeline_polls = g_tc_pipeline_polls.load();
    if ((g.lda & 7) || (g.ldb & 7) || (reinterpret_cast<uintptr_t>(g.A) & 15) || (reinterpret_cast<uintptr_t>(g.B) & 15))
        return cudaErrorInvalidValue;
    const int bn = g.N <= 64 ? 64 : g.N <= 128 ? 128 : 256;
    const int tiles_m = (g.M + TC_BM - 1) / TC_BM, tiles_n = (g.N + bn - 1) / bn;
    const int nk = (g.K + TC_BK - 1) / TC_BK;
    int splits = 1;
    if (g.epi == TC_EPI_F32_ADD) {
        splits = std::min(num_sms / (tiles_m * tiles_n), nk / 4);
        splits = std::max(1, std::min(splits, nk));
    }
    g.chunks_per_split = (nk + splits - 1) / splits;
    splits = (nk + g.chunks_per_split - 1) / g.chunks_per_split;  // every split has >= 1 chunk
    CUtensorMap ma, mb;
    cudaError_t e = make_map(&ma, g.A, g.M, g.K, g.lda, TC_BM);
    if (e == cudaSuccess) e = make_map(&mb, g.B, g.N, g.K, g.ldb, bn);
    if (e != cudaSuccess) return e;
    const dim3 grid(tiles_m, tiles_n, splits);
    if (bn == 64) return launch_bn<64>(ma, mb, g, grid, s);
    if (bn == 128) return launch_bn<128>(ma, mb, g, grid, s);
    return launch_bn<256>(ma, mb, g, grid, s);
}

// dst[c][r] = src[r][c] (BF16), 32 x 32 tiles through shared memory
__global__ void k_transpose_bf16(const __nv_bfloat16* __restrict__ src, int rows, int cols, int lds,
                                 __nv_bfloat16* __restrict__ dst, int ldd) {
    __shared__ __nv_bfloat16 t[32][34];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) t[i][threadIdx.x] = src[(long long)r * lds + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (r < rows && c < cols) dst[(long long)c * ldd + r] = t[threadIdx.x][i];
    }
}

cudaError_t transpose(const __nv_bfloat16* src, int rows, int cols, int lds, __nv_bfloat16* dst, int ldd, cudaStream_t s) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    k_transpose_bf16<<<dim3((cols + 31) / 32, (rows + 31) / 32), dim3(32, 8), 0, s>>>(src, rows, cols, lds, dst, ldd);
    return cudaGetLastError();
}

// fp32 [rows x ldx] (first n_in columns) -> bf16 [rows x n_pad], zero padding
__global__ void k_to_bf16_pad(const float* __restrict__ x, int ldx, int rows, int n_in, int n_pad,
                              __nv_bfloat16* __restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)rows * n_pad) return;
    const int r = (int)(t / n_pad), c = (int)(t % n_pad);
    out[t] = __float2bfloat16(c < n_in ? x[(long long)r * ldx + c] : 0.f);
}

// out[c] += sum_r a[r][c]: one block per 256 rows, one thread per column
__global__ void k_colsum(const float* __restrict__ a, int rows, int cols, int lda, float* __restrict__ out) {
    const int c = blockIdx.y * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    const int r0 = blockIdx.x * 256, r1 = min(rows, r0 + 256);
    float s = 0.f;
    for (int r = r0; r < r1; ++r) s += a[(long long)r * lda + c];
    atomicAdd(out + c, s);
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float wd, float c1, float c2) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float gi = g[t];
    const float mi = b1 * m[t] + (1.f - b1) * gi;
    const float vi = b2 * v[t] + (1.f - b2) * gi * gi;
    m[t] = mi;
    v[t] = vi;
    p[t] -= lr * ((mi / c1) / (sqrtf(vi / c2) + eps) + wd * p[t]);
}

// W (fp32 [dout x din_pad]) -> Wb (bf16, same) and Wt (bf16 [din_pad x dout])
__global__ void k_refresh(const float* __restrict__ w, int dout, int din_pad, __nv_bfloat16* __restrict__ wb,
                          __nv_bfloat16* __restrict__ wt) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)dout * din_pad) return;
    const int o = (int)(t / din_pad), i = (int)(t % din_pad);
    const __nv_bfloat16 v = __float2bfloat16(w[t]);
    wb[t] = v;
    wt[(long long)i * dout + o] = v;
}

__global__ void k_f32_to_bf16(const float* __restrict__ a, long long n, __nv_bfloat16* __restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = __float2bfloat16(a[t]);
}

// splitmix64: the initialisation stream (identical on every host)
uint64_t mix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

#define MLP_CK(call)                                                              \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);             \
            return e_ == cudaErrorMemoryAllocation ? UNOMOL_ENOMEM : UNOMOL_ECUDA; \
        }                                                                         \
    } while (0)

Mlp::~Mlp() {
    for (void* p : std::vector<void*>{P, G, Am, Av, Wb, Wt, X, Y, dYb, dZb[0], dZb[1], dZf, Ta, Tb, status})
        if (p) cudaFree(p);
    for (float* p : Z)
        if (p) cudaFree(p);
    for (__nv_bfloat16* p : H)
        if (p) cudaFree(p);
}

int Mlp::init(int n_in_, int hidden_, int layers_, int n_out_, unsigned long long seed) {
    if (n_in_ <= 0 || hidden_ <= 0 || layers_ <= 0 || n_out_ <= 0 || hidden_ % 8 || n_out_ % 8) {
        err = "mlp: sizes must be positive, hidden and n_out multiples of 8";
        return UNOMOL_EINVAL;
    }
    n_in = n_in_;
    n_in_pad = (n_in + 7) / 8 * 8;
    hidden = hidden_;
    layers = layers_;
    n_out = n_out_;
    const int nm = layers + 1;
    din.resize(nm);
    din_pad.resize(nm);
    dout.resize(nm);
    w_off.resize(nm);
    b_off.resize(nm);
    wt_off.resize(nm);
    long long off = 0, offt = 0;
    np = 0;
    for (int l = 0; l < nm; ++l) {
        din[l] = l == 0 ? n_in : hidden;
        din_pad[l] = l == 0 ? n_in_pad : hidden;
        dout[l] = l == layers ? n_out : hidden;
        w_off[l] = off;
        wt_off[l] = offt;
        off += (long long)dout[l] * din_pad[l];
        offt += (long long)dout[l] * din_pad[l];
        b_off[l] = off;
        off += dout[l];
        np += (long long)dout[l] * din[l] + dout[l];
    }
    np_pad = off;
    int dev = 0;
    MLP_CK(cudaGetDevice(&dev));
    MLP_CK(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
    for (float** p : {&P, &G, &Am, &Av}) MLP_CK(cudaMalloc(p, np_pad * sizeof(float)));
    MLP_CK(cudaMalloc(&Wb, offt * sizeof(__nv_bfloat16)));
    MLP_CK(cudaMalloc(&Wt, offt * sizeof(__nv_bfloat16)));
    MLP_CK(cudaMalloc(&status, sizeof(int)));
    MLP_CK(cudaMemset(status, 0, sizeof(int)));
    MLP_CK(cudaMemset(G, 0, np_pad * sizeof(float)));
    MLP_CK(cudaMemset(Am, 0, np_pad * sizeof(float)));
    MLP_CK(cudaMemset(Av, 0, np_pad * sizeof(float)));
    // uniform(-a, a), a = sqrt(3 / din) (unit-variance pre-activations for unit-variance inputs);
    // the output map starts 10x smaller; biases zero
    uint64_t st = seed * 0x2545F4914F6CDD1Dull + 1;
    std::vector<float> h((size_t)np);
    size_t k = 0;
    for (int l = 0; l < nm; ++l) {
        const double a = std::sqrt(3.0 / din[l]) * (l == layers ? 0.1 : 1.0);
        for (long long i = 0; i < (long long)dout[l] * din[l]; ++i) {
            const double u = (double)(mix64(st) >> 11) * (1.0 / 9007199254740992.0);
            h[k++] = (float)((2.0 * u - 1.0) * a);
        }
        for (int i = 0; i < dout[l]; ++i) h[k++] = 0.f;
    }
    return set(h.data());
}

int Mlp::reserve(int r) {
    if (r <= cap) return UNOMOL_OK;
    const int c = std::max(r, cap + cap / 2);
    auto rel = [](void* p) {
        if (p) cudaFree(p);
    };
    rel(X), rel(Y), rel(dYb), rel(dZb[0]), rel(dZb[1]), rel(dZf), rel(Ta), rel(Tb);
    Ta = Tb = nullptr;
    for (float* p : Z) rel(p);
    for (__nv_bfloat16* p : H) rel(p);
    X = nullptr, Y = nullptr, dYb = nullptr, dZb[0] = dZb[1] = nullptr, dZf = nullptr;
    Z.assign(layers, nullptr);
    H.assign(layers, nullptr);
    cap = 0;
    const size_t R = (size_t)c;
    MLP_CK(cudaMalloc(&X, R * n_in_pad * sizeof(__nv_bfloat16)));
    MLP_CK(cudaMalloc(&Y, R * n_out * sizeof(float)));
    MLP_CK(cudaMalloc(&dYb, R * n_out * sizeof(__nv_bfloat16)));
    MLP_CK(cudaMalloc(&dZb[0], R * hidden * sizeof(__nv_bfloat16)));
    MLP_CK(cudaMalloc(&dZb[1], R * hidden * sizeof(__nv_bfloat16)));
    MLP_CK(cudaMalloc(&dZf, R * hidden * sizeof(float)));
    const size_t Rp = (R + 7) / 8 * 8;  // transposed operands: row stride a multiple of 8 elements
    MLP_CK(cudaMalloc(&Ta, Rp * std::max(hidden, n_out) * sizeof(__nv_bfloat16)));
    MLP_CK(cudaMalloc(&Tb, Rp * std::max(hidden, n_in_pad) * sizeof(__nv_bfloat16)));
    for (int l = 0; l < layers; ++l) {
        MLP_CK(cudaMalloc(&Z[l], R * hidden * sizeof(float)));
        MLP_CK(cudaMalloc(&H[l], R * hidden * sizeof(__nv_bfloat16)));
    }
    cap = c;
    return UNOMOL_OK;
}

int Mlp::forward(const float* x, int ldx, int r, cudaStream_t s) {
    if (!x || ldx < n_in || r < 0) {
        err = "mlp forward: bad input";
        return UNOMOL_EINVAL;
    }
    int rc = reserve(r);
    if (rc) return rc;
    if (r > 0) k_to_bf16_pad<<<nblk((long long)r * n_in_pad), 256, 0, s>>>(x, ldx, r, n_in, n_in_pad, X);
    MLP_CK(cudaGetLastError());
    return forward_x(r, s);
}

int Mlp::forward_x(int r, cudaStream_t s) {
    if (r > cap) {
        err = "mlp forward: more rows than reserved";
        return UNOMOL_EINVAL;
    }
    rows = r;
    if (r == 0) return UNOMOL_OK;
    for (int l = 0; l <= layers; ++l) {
        TcGemmArgs g{};
        g.A = l == 0 ? X : H[l - 1];
        g.lda = din_pad[l];
        g.B = Wb + wt_off[l];
        g.ldb = din_pad[l];
        g.M = r;
        g.N = dout[l];
        g.K = din_pad[l];
        g.bias = P + b_off[l];
        g.status = status;
        if (l < layers) {
            g.epi = TC_EPI_BIAS_SILU;
            g.Z = Z[l];
            g.Cb = H[l];
            g.ldc = hidden;
        } else {
            g.epi = TC_EPI_BIAS_F32;
            g.Cf = Y;
            g.ldc = n_out;
        }
        MLP_CK(tc_gemm_launch(g, s, num_sms));
    }
    return UNOMOL_OK;
}

int Mlp::backward(const float* dy, bool accumulate, cudaStream_t s) {
    if (!dy) {
        err = "mlp backward: null gradient";
        return UNOMOL_EINVAL;
    }
    if (!accumulate) MLP_CK(cudaMemsetAsync(G, 0, np_pad * sizeof(float), s));
    const int r = rows;
    if (r == 0) return UNOMOL_OK;
    const int L = layers;
    k_f32_to_bf16<<<nblk((long long)r * n_out), 256, 0, s>>>(dy, (long long)r * n_out, dYb);
    {
        dim3 grid(nblk(r), nblk(n_out, 64));
        k_colsum<<<grid, 64, 0, s>>>(dy, r, n_out, n_out, G + b_off[L]);
    }
    MLP_CK(cudaGetLastError());
    const int rp = (r + 7) / 8 * 8;
    // dW_L = dY^T . h_L  (operands transposed to K-major: K = rows)
    {
        MLP_CK(transpose(dYb, r, n_out, n_out, Ta, rp, s));
        MLP_CK(transpose(H[L - 1], r, hidden, hidden, Tb, rp, s));
        TcGemmArgs g{};
        g.A = Ta, g.lda = rp;
        g.B = Tb, g.ldb = rp;
        g.M = n_out, g.N = hidden, g.K = r;
        g.epi = TC_EPI_F32_ADD, g.Cf = G + w_off[L], g.ldc = din_pad[L];
        g.status = status;
        MLP_CK(tc_gemm_launch(g, s, num_sms));
    }
    const __nv_bfloat16* dg = dYb;
    int dg_ld = n_out;
    int cur = 0;
    for (int l = L - 1; l >= 0; --l) {
        // dz_l = (dg . W_{l+1}) * silu'(z_l)
        {
            TcGemmArgs g{};
            g.A = dg, g.lda = dg_ld;
            g.B = Wt + wt_off[l + 1], g.ldb = dout[l + 1];
            g.M = r, g.N = hidden, g.K = dout[l + 1];
            g.epi = TC_EPI_DSILU, g.Z = Z[l], g.Cb = dZb[cur], g.Cf = dZf, g.ldc = hidden;
            g.status = status;
            MLP_CK(tc_gemm_launch(g, s, num_sms));
        }
        {
            dim3 grid(nblk(r), nblk(hidden, 256));
            k_colsum<<<grid, 256, 0, s>>>(dZf, r, hidden, hidden, G + b_off[l]);
            MLP_CK(cudaGetLastError());
        }
        // dW_l = dz_l^T . h_l  (h_0 = x; operands transposed to K-major)
        {
            MLP_CK(transpose(dZb[cur], r, hidden, hidden, Ta, rp, s));
            MLP_CK(transpose(l == 0 ? X : H[l - 1], r, din_pad[l], din_pad[l], Tb, rp, s));
            TcGemmArgs g{};
            g.A = Ta, g.lda = rp;
            g.B = Tb, g.ldb = rp;
            g.M = hidden, g.N = din_pad[l], g.K = r;
            g.epi = TC_EPI_F32_ADD, g.Cf = G + w_off[l], g.ldc = din_pad[l];
            g.status = status;
            MLP_CK(tc_gemm_launch(g, s, num_sms));
        }
        dg = dZb[cur];
        dg_ld = hidden;
        cur ^= 1;
    }
    return UNOMOL_OK;
}

int Mlp::adam(float lr, float b1, float b2, float eps, float wd, cudaStream_t s) {
    ++step;
    const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
    k_adam<<<nblk(np_pad), 256, 0, s>>>(P, G, Am, Av, np_pad, lr, b1, b2, eps, wd, c1, c2);
    MLP_CK(cudaGetLastError());
    return refresh_bf16(s);
}

int Mlp::refresh_bf16(cudaStream_t s) {
    for (int l = 0; l <= layers; ++l)
        k_refresh<<<nblk((long long)dout[l] * din_pad[l]), 256, 0, s>>>(P + w_off[l], dout[l], din_pad[l], Wb + wt_off[l],
                                                                        Wt + wt_off[l]);
    MLP_CK(cudaGetLastError());
    return UNOMOL_OK;
}

int Mlp::get(const float* dev, float* host) const {
    std::vector<float> pad((size_t)np_pad);
    if (cudaMemcpy(pad.data(), dev, np_pad * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) return UNOMOL_ECUDA;
    size_t k = 0;
    for (int l = 0; l <= layers; ++l) {
        for (int o = 0; o < dout[l]; ++o)
            for (int i = 0; i < din[l]; ++i) host[k++] = pad[(size_t)w_off[l] + (size_t)o * din_pad[l] + i];
        for (int o = 0; o < dout[l]; ++o) host[k++] = pad[(size_t)b_off[l] + o];
    }
    return UNOMOL_OK;
}

int Mlp::set(const float* host) {
    std::vector<float> pad((size_t)np_pad, 0.f);
    size_t k = 0;
    for (int l = 0; l <= layers; ++l) {
        for (int o = 0; o < dout[l]; ++o)
            for (int i = 0; i < din[l]; ++i) pad[(size_t)w_off[l] + (size_t)o * din_pad[l] + i] = host[k++];
        for (int o = 0; o < dout[l]; ++o) pad[(size_t)b_off[l] + o] = host[k++];
    }
    MLP_CK(cudaMemcpy(P, pad.data(), np_pad * sizeof(float), cudaMemcpyHostToDevice));
    int rc = refresh_bf16(nullptr);
    if (rc) return rc;
    MLP_CK(cudaDeviceSynchronize());
    return UNOMOL_OK;
}

int Mlp::check_status(cudaStream_t s) {
    int h = 0;
    MLP_CK(cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, s));
    MLP_CK(cudaStreamSynchronize(s));
    if (h) {
        err = "tensor-core GEMM: a bounded wait gave up";
        MLP_CK(cudaMemsetAsync(status, 0, sizeof(int), s));  // reported once; later calls start clean
        MLP_CK(cudaStreamSynchronize(s));
        return UNOMOL_ETIMEOUT;
    }
    return UNOMOL_OK;
}

}  // namespace ugb

using namespace ugb;

struct UnomolMlp : Mlp {};

namespace {
thread_local std::string g_mlp_err;
}

extern "C" {

int unomol_tc_set_wait_polls(int polls) {
    g_tc_pipeline_polls.store(polls);
    return UNOMOL_OK;
}

int unomol_tc_gemm_bf16(const void* A, const void* B, int M, int N, int K, float* C, int* status, void* stream) {
    if (!A || !B || !C || M < 0 || N < 0 || K < 0) return UNOMOL_EINVAL;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t s = (cudaStream_t)stream;
    // the TMA unit wants 16-byte row strides and bases: copy ragged operands into padded rows
    const int kp = (K + 7) / 8 * 8;
    const bool pad = kp != K || (reinterpret_cast<uintptr_t>(A) & 15) || (reinterpret_cast<uintptr_t>(B) & 15);
    __nv_bfloat16 *pa = nullptr, *pb = nullptr;
    cudaError_t e = cudaSuccess;
    if (pad && M > 0 && N > 0 && K > 0) {
        e = cudaMalloc(&pa, (size_t)M * kp * 2);
        if (e == cudaSuccess) e = cudaMalloc(&pb, (size_t)N * kp * 2);
        if (e == cudaSuccess) e = cudaMemsetAsync(pa, 0, (size_t)M * kp * 2, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(pb, 0, (size_t)N * kp * 2, s);
        if (e == cudaSuccess) e = cudaMemcpy2DAsync(pa, kp * 2, A, (size_t)K * 2, (size_t)K * 2, M, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpy2DAsync(pb, kp * 2, B, (size_t)K * 2, (size_t)K * 2, N, cudaMemcpyDeviceToDevice, s);
    }
    if (e == cudaSuccess) {
        TcGemmArgs g{};
        g.A = pad ? pa : static_cast<const __nv_bfloat16*>(A);
        g.B = pad ? pb : static_cast<const __nv_bfloat16*>(B);
        g.M = M, g.N = N, g.K = K, g.lda = pad ? kp : K, g.ldb = pad ? kp : K;
        g.epi = TC_EPI_F32;
        g.Cf = C;
        g.ldc = N;
        g.status = status;
        e = tc_gemm_launch(g, s, sms);
    }
    if (pad) {
        cudaStreamSynchronize(s);
        if (pa) cudaFree(pa);
        if (pb) cudaFree(pb);
    }
    if (e != cudaSuccess) {
        g_mlp_err = cudaGetErrorString(e);
        return UNOMOL_ECUDA;
    }
    return UNOMOL_OK;
}

int unomol_mlp_create(int n_in, int hidden, int layers, int n_out, unsigned long long seed, UnomolMlp** out) {
    if (!out) return UNOMOL_EINVAL;
    *out = nullptr;
    auto* m = new UnomolMlp();
    int rc = m->init(n_in, hidden, layers, n_out, seed);
    if (rc) {
        g_mlp_err = m->err;
        delete m;
        return rc;
    }
    *out = m;
    return UNOMOL_OK;
}

long long unomol_mlp_num_params(const UnomolMlp* m) { return m ? m->np : -1; }

int unomol_mlp_get_params(UnomolMlp* m, float* out) {
    if (!m || !out) return UNOMOL_EINVAL;
    return m->get(m->P, out);
}

int unomol_mlp_set_params(UnomolMlp* m, const float* in) {
    if (!m || !in) return UNOMOL_EINVAL;
    return m->set(in);
}

int unomol_mlp_get_grads(UnomolMlp* m, float* out) {
    if (!m || !out) return UNOMOL_EINVAL;
    return m->get(m->G, out);
}

int unomol_mlp_forward(UnomolMlp* m, const float* x, int rows, float* y, void* stream) {
    if (!m || !x || !y || rows < 0) return UNOMOL_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = m->forward(x, m->n_in, rows, s);
    if (!rc && rows > 0 && cudaMemcpyAsync(y, m->Y, (size_t)rows * m->n_out * sizeof(float), cudaMemcpyDeviceToDevice, s))
        rc = UNOMOL_ECUDA;
    if (!rc) rc = m->check_status(s);
    return rc;
}

int unomol_mlp_backward(UnomolMlp* m, const float* dy, void* stream) {
    if (!m || !dy) return UNOMOL_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = m->backward(dy, false, s);
    if (!rc) rc = m->check_status(s);
    return rc;
}

int unomol_mlp_adam(UnomolMlp* m, float lr, float beta1, float beta2, float eps, float weight_decay, void* stream) {
    if (!m) return UNOMOL_EINVAL;
    return m->adam(lr, beta1, beta2, eps, weight_decay, (cudaStream_t)stream);
}

void unomol_mlp_destroy(UnomolMlp* m) { delete m; }

const char* unomol_mlp_last_error(const UnomolMlp* m) { return m ? m->err.c_str() : g_mlp_err.c_str(); }

}  // extern "C"
