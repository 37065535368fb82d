// The learned-guess network on the tensor cores: forward and backward passes built from the tcgen05
// BF16 GEMM of tc_gemm.cuh with fused epilogues (bias + SiLU forward, SiLU derivative backward, split-K
// atomic accumulation of the weight gradients), plus small FP32 kernels for the bias gradients, the
// BF16 conversions and Adam.  Master weights are FP32; the GEMM operands are BF16 copies.
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

bool vec_ok(const void* p, int ld) { return ld % 8 == 0 && (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

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
    for (void* p : std::vector<void*>{P, G, Am, Av, Wb, Wt, X, Y, dYb, dZb[0], dZb[1], dZf, status})
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
    rel(X), rel(Y), rel(dYb), rel(dZb[0]), rel(dZb[1]), rel(dZf);
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
        g.vec_a = vec_ok(g.A, g.lda);
        g.vec_b = vec_ok(g.B, g.ldb);
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
    // dW_L = dY^T . h_L
    {
        TcGemmArgs g{};
        g.A = dYb, g.lda = n_out, g.a_trans = 1;
        g.B = H[L - 1], g.ldb = hidden, g.b_trans = 1;
        g.M = n_out, g.N = hidden, g.K = r;
        g.vec_a = vec_ok(g.A, g.lda), g.vec_b = vec_ok(g.B, g.ldb);
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
            g.vec_a = vec_ok(g.A, g.lda), g.vec_b = vec_ok(g.B, g.ldb);
            g.epi = TC_EPI_DSILU, g.Z = Z[l], g.Cb = dZb[cur], g.Cf = dZf, g.ldc = hidden;
            g.status = status;
            MLP_CK(tc_gemm_launch(g, s, num_sms));
        }
        {
            dim3 grid(nblk(r), nblk(hidden, 256));
            k_colsum<<<grid, 256, 0, s>>>(dZf, r, hidden, hidden, G + b_off[l]);
            MLP_CK(cudaGetLastError());
        }
        // dW_l = dz_l^T . h_l  (h_0 = x)
        {
            TcGemmArgs g{};
            g.A = dZb[cur], g.lda = hidden, g.a_trans = 1;
            g.B = l == 0 ? X : H[l - 1], g.ldb = din_pad[l], g.b_trans = 1;
            g.M = hidden, g.N = din_pad[l], g.K = r;
            g.vec_a = vec_ok(g.A, g.lda), g.vec_b = vec_ok(g.B, g.ldb);
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

int unomol_tc_gemm_bf16(const void* A, const void* B, int M, int N, int K, float* C, int* status, void* stream) {
    if (!A || !B || !C || M < 0 || N < 0 || K < 0) return UNOMOL_EINVAL;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    TcGemmArgs g{};
    g.A = static_cast<const __nv_bfloat16*>(A);
    g.B = static_cast<const __nv_bfloat16*>(B);
    g.M = M, g.N = N, g.K = K, g.lda = K, g.ldb = K;
    g.vec_a = vec_ok(A, K), g.vec_b = vec_ok(B, K);
    g.epi = TC_EPI_F32;
    g.Cf = C;
    g.ldc = N;
    g.status = status;
    cudaError_t e = tc_gemm_launch(g, (cudaStream_t)stream, sms);
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
