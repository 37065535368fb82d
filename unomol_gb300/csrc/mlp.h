// The multilayer perceptron of the learned density guess, on the tensor cores.
//
//   h_0 = x;  z_l = h_l W_l^T + b_l,  h_{l+1} = silu(z_l)  (l < layers);  y = h_layers W_L^T + b_L
//
// Master weights, gradients and Adam moments are FP32; every GEMM runs on BF16 copies of the
// weights (W_l and W_l^T, refreshed after each update) and BF16 activations with FP32 accumulation
// (tc_gemm.cuh).  Pre-activations z_l are kept in FP32 for the SiLU derivative of the backward pass.
// Parameter layout (host side, unpadded): for every linear map l, W_l [dout x din] row major, then
// b_l [dout].  On the device the first map's rows are padded to a multiple of 8 inputs.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace ugb {

struct Mlp {
    int n_in = 0, n_in_pad = 0, hidden = 0, layers = 0, n_out = 0;
    std::vector<int> din, din_pad, dout;       // per linear map (layers + 1 maps)
    std::vector<long long> w_off, b_off;       // into P / G / Am / Av (padded layout)
    std::vector<long long> wt_off;             // into Wb and Wt
    long long np_pad = 0, np = 0;              // padded / unpadded parameter counts
    float *P = nullptr, *G = nullptr, *Am = nullptr, *Av = nullptr;
    __nv_bfloat16 *Wb = nullptr, *Wt = nullptr;  // W_l [dout x din_pad] and W_l^T [din_pad x dout], both at wt_off
    long long step = 0;
    int num_sms = 0;
    int cap = 0, rows = 0;                     // activation capacity / rows of the last forward
    __nv_bfloat16* X = nullptr;                // [cap x n_in_pad]
    std::vector<float*> Z;                     // [layers][cap x hidden]
    std::vector<__nv_bfloat16*> H;             // [layers][cap x hidden]
    float* Y = nullptr;                        // [cap x n_out]
    __nv_bfloat16* dYb = nullptr;              // [cap x n_out]
    __nv_bfloat16* dZb[2] = {nullptr, nullptr};  // [cap x hidden]
    float* dZf = nullptr;                      // [cap x hidden]
    __nv_bfloat16 *Ta = nullptr, *Tb = nullptr;  // transposed operands of the weight gradients
    int* status = nullptr;                     // device flag: a GEMM wait gave up
    std::string err;

    ~Mlp();
    int init(int n_in, int hidden, int layers, int n_out, unsigned long long seed);
    int reserve(int rows);
    // y = f(x) for rows already written to X (bf16, [rows x n_in_pad], padding zero)
    int forward_x(int rows, cudaStream_t s);
    // x from fp32 [rows x ldx], then forward
    int forward(const float* x, int ldx, int rows, cudaStream_t s);
    // G (+)= d loss / d params for the rows of the last forward, dy fp32 [rows x n_out]
    int backward(const float* dy, bool accumulate, cudaStream_t s);
    int adam(float lr, float beta1, float beta2, float eps, float weight_decay, cudaStream_t s);
    int refresh_bf16(cudaStream_t s);
    int get(const float* dev_padded, float* host) const;   // padded device -> unpadded host
    int set(const float* host);                            // unpadded host -> P (+ bf16 copies)
    int check_status(cudaStream_t s);
};

}  // namespace ugb
