// DPM polarisation-potential integrals on the GPU: the one-electron term that GDPMInts adds to the
// core Hamiltonian of the positron-augmented basis (GDPMInts.cpp:5-143),
//
//   H[mu nu] -= sum_k c_k (mu nu | g_k),   g_k(r) = exp(-a_k |r - q|^2),
//
// the six-Gaussian charge of a positron at q (the fitted a_k, c_k of GDPMInts.cpp:13-18, kept as the
// reference writes them: they define the model).  (mu nu | g_k) is a two-electron integral whose ket
// "pair" is the single Gaussian g_k, so it is evaluated by the Rys kernel of the Fock build
// (shell_quartet_eri) on the quartet class (la lb | s s) with a synthetic ket: six primitive pairs with
// exponent a_k, centre q, Q - C = 0, prefactor 1 / a_k (K_cd = 1) and coefficient c_k.  As in the
// reference there is no prefactor screen, and the Rys roots follow the context's Rys mode (the
// reference evaluates them with its own Rys::Recur, two-root regime included).  One thread per shell
// pair; every packed element belongs to exactly one pair, so the results are stored, not accumulated.
#include <algorithm>
#include <string>
#include <vector>

#include "../../include/unomol_gb300.h"
#include "ctx_view.h"
#include "fock_dispatch.cuh"

namespace ugb {
namespace {

constexpr int GDPM_N = 6;
constexpr double GDPM_ALF[GDPM_N] = {6.8505018000, 4.0491646000, 3.5941062989, 1.2478274000, 0.7927690989, 0.3377107978};
constexpr double GDPM_COF[GDPM_N] = {0.0766926784, 0.1483475912, 0.0462334641, 0.0717376427, 0.0447149792, 0.0069678529};

template <int LA, int LB>
__global__ void __launch_bounds__(128) gdpm_kernel(const ShellPair* __restrict__ pairs, int begin, int count,
                                                   const PrimPair* __restrict__ prims, int gbegin, const NormTable nt,
                                                   const double* __restrict__ rys, int compat, double* __restrict__ out) {
    using Q = QClass<LA, LB, 0, 0>;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const ShellPair bra = pairs[begin + t];
    ShellPair ket{};
    ket.prim_begin = gbegin;
    ket.nprim = GDPM_N;
    ket.prim_stride = 1;
    double acc[Q::NF];
    shell_quartet_eri<LA, LB, 0, 0, double, PrimPair>(bra, ket, prims, rys, 0.0, 0.f, compat != 0, acc);
#pragma unroll
    for (int ia = 0; ia < Q::NA; ++ia)
#pragma unroll
        for (int ib = 0; ib < Q::NB; ++ib) {
            const int i = bra.a_off + ia, j = bra.b_off + ib;
            if (bra.same && j > i) continue;
            const int hi = i > j ? i : j, lo = i > j ? j : i;
            out[(long long)hi * (hi + 1) / 2 + lo] = acc[ia * Q::NB + ib] * nt.v[LA][ia] * nt.v[LB][ib];
        }
}

template <int LA, int LB>
cudaError_t launch(const ShellPair* pairs, int begin, int count, const PrimPair* prims, int gbegin, const CtxView& v,
                   double* out, cudaStream_t s) {
    gdpm_kernel<LA, LB><<<(count + 127) / 128, 128, 0, s>>>(pairs, begin, count, prims, gbegin, v.nt, v.d_rys,
                                                          v.rys_compat, out);
    return cudaGetLastError();
}

thread_local std::string g_dpm_err;

}  // namespace
}  // namespace ugb

using namespace ugb;

extern "C" int unomol_gpu_gdpm(UnomolCtx* ctx, const double* q, double* H) {
    if (!ctx || !q || !H) return UNOMOL_EINVAL;
    const CtxView v = ctx_view(ctx);
    for (int cls : *v.block_class)
        if (pc_la(cls) > 2) {
            g_dpm_err = "DPM integrals: shells above d are not supported";
            return UNOMOL_EINVAL;
        }
    // the context's primitive pairs (on the device) followed by the six of the positron charge
    std::vector<PrimPair> gp(GDPM_N);
    for (int k = 0; k < GDPM_N; ++k) {
        PrimPair g{};
        g.p = GDPM_ALF[k];
        g.rp = 1.0 / GDPM_ALF[k];
        for (int x = 0; x < 3; ++x) g.P[x] = q[x], g.PA[x] = 0.0;
        g.E = 1.0 / GDPM_ALF[k];  // exp(0) / a_k: the Gaussian is its own product, K_cd = 1
        g.cc = GDPM_COF[k];
        g.Ecc = SQRT_SRTERM * g.E * g.cc;
        g.pf = (float)g.p;
        g.Ef = (float)g.E;
        gp[k] = g;
    }
    const int gbegin = (int)v.nprims;
    const long long no2 = (long long)v.nbf * (v.nbf + 1) / 2;
    PrimPair* d_prims = nullptr;
    double* d_out = nullptr;
    cudaStream_t s = v.stream;
    cudaError_t e = cudaMalloc(&d_prims, sizeof(PrimPair) * (v.nprims + GDPM_N));
    if (e == cudaSuccess) e = cudaMalloc(&d_out, sizeof(double) * std::max<long long>(1, no2));
    if (e == cudaSuccess && v.nprims > 0)
        e = cudaMemcpyAsync(d_prims, v.d_prims, sizeof(PrimPair) * v.nprims, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_prims + gbegin, gp.data(), sizeof(PrimPair) * GDPM_N, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_out, 0, sizeof(double) * std::max<long long>(1, no2), s);
    // one launch per run of blocks of one class (pairs are sorted by class)
    const std::vector<int>& bb = *v.block_begin;
    const std::vector<int>& bn = *v.block_count;
    const std::vector<int>& bc = *v.block_class;
    for (size_t k = 0; e == cudaSuccess && k < bc.size();) {
        size_t k2 = k;
        while (k2 < bc.size() && bc[k2] == bc[k]) ++k2;
        const int begin = bb[k], cnt = bb[k2 - 1] + bn[k2 - 1] - begin;
        const int la = pc_la(bc[k]), lb = pc_lb(bc[k]);
        if (la == 0) e = launch<0, 0>(v.d_pairs, begin, cnt, d_prims, gbegin, v, d_out, s);
        else if (la == 1 && lb == 0) e = launch<1, 0>(v.d_pairs, begin, cnt, d_prims, gbegin, v, d_out, s);
        else if (la == 1) e = launch<1, 1>(v.d_pairs, begin, cnt, d_prims, gbegin, v, d_out, s);
        else if (lb == 0) e = launch<2, 0>(v.d_pairs, begin, cnt, d_prims, gbegin, v, d_out, s);
        else if (lb == 1) e = launch<2, 1>(v.d_pairs, begin, cnt, d_prims, gbegin, v, d_out, s);
        else e = launch<2, 2>(v.d_pairs, begin, cnt, d_prims, gbegin, v, d_out, s);
        k = k2;
    }
    std::vector<double> out((size_t)std::max<long long>(1, no2));
    if (e == cudaSuccess) e = cudaMemcpyAsync(out.data(), d_out, sizeof(double) * no2, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_prims);
    cudaFree(d_out);
    if (e != cudaSuccess) {
        g_dpm_err = std::string("DPM integrals: ") + cudaGetErrorString(e);
        return UNOMOL_ECUDA;
    }
    for (long long k = 0; k < no2; ++k) H[k] -= out[k];
    return UNOMOL_OK;
}

extern "C" const char* unomol_gpu_gdpm_last_error(void) { return ugb::g_dpm_err.c_str(); }
