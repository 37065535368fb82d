// SCF driver on the GPU: the loop of RestrictedHartreeFock / UnRestrictedHartreeFock::findEnergy
// (RHF.hpp:114-176, UHF.hpp:137-177) with every Fock build on the GPU and the linear algebra in FP64
// on the GPU (cuSOLVER syevd for S^{-1/2} and the Fock eigenproblem, cuBLAS for X^T F X, C and P).
//
// Parity mode (accel 0/1) follows the reference step by step: update() (RHF.hpp:87-112), the damping
// of scf_converger() (RHF.hpp:536-569; the "Anderson" branch is dead in the serial reference because
// `extrap` stays 0, so only the averaging runs), is_converged() on the signed ediff and/or pdiff
// (RHF.hpp:390-402), canonical X = U s^{-1/2} (RHF.hpp:214-233) and the core-Hamiltonian guess
// (RHF.hpp:205-211).  DIIS (accel 2) is new: Pulay extrapolation of F on the orthonormal-basis error
// X^T (F P S - S P F) X, for systems on which the damped loop oscillates.  Two new ways to the density
// of F beside the eigen-solve: second-order spectral projection (SP2) and pseudo-diagonalisation steps
// on the last orbitals (both fall back to the eigen-solve where their conditions fail).
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/unomol_gb300.h"

namespace {

struct Dev {
    int n = 0;
    cudaStream_t s = nullptr;
    cublasHandle_t cb = nullptr;
    cusolverDnHandle_t cs = nullptr;
    double *X = nullptr, *F = nullptr, *W = nullptr, *C = nullptr, *T1 = nullptr, *ev = nullptr, *work = nullptr;
    int* info = nullptr;
    int lwork = 0;
    std::string err;
    ~Dev() {
        for (double* p : {X, F, W, C, T1, ev, work})
            if (p) cudaFree(p);
        if (info) cudaFree(info);
        if (cb) cublasDestroy(cb);
        if (cs) cusolverDnDestroy(cs);
    }
};

#define CK(call, code)                                                         \
    do {                                                                       \
        if ((call) != 0) {                                                     \
            d.err = std::string(#call) + " failed";                            \
            return code;                                                       \
        }                                                                      \
    } while (0)

int dev_init(Dev& d, int n, cudaStream_t s) {
    d.n = n;
    d.s = s;
    const size_t n2 = (size_t)n * n * sizeof(double);
    CK(cublasCreate(&d.cb), UNOMOL_ECUDA);
    CK(cublasSetStream(d.cb, s), UNOMOL_ECUDA);
    CK(cusolverDnCreate(&d.cs), UNOMOL_ECUDA);
    CK(cusolverDnSetStream(d.cs, s), UNOMOL_ECUDA);
    for (double** p : {&d.X, &d.F, &d.W, &d.C, &d.T1}) CK(cudaMalloc(p, n2), UNOMOL_ENOMEM);
    CK(cudaMalloc(&d.ev, n * sizeof(double)), UNOMOL_ENOMEM);
    CK(cudaMalloc(&d.info, sizeof(int)), UNOMOL_ENOMEM);
    CK(cusolverDnDsyevd_bufferSize(d.cs, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, d.F, n, d.ev, &d.lwork), UNOMOL_ECUDA);
    CK(cudaMalloc(&d.work, (size_t)d.lwork * sizeof(double)), UNOMOL_ENOMEM);
    return UNOMOL_OK;
}

// symmetric eigen-decomposition of A (n x n, in place -> eigenvectors in columns), eigenvalues in ev
int syevd(Dev& d, double* A) {
    CK(cusolverDnDsyevd(d.cs, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, d.n, A, d.n, d.ev, d.work, d.lwork, d.info),
       UNOMOL_ECUDA);
    int info = 0;
    CK(cudaMemcpyAsync(&info, d.info, sizeof(int), cudaMemcpyDeviceToHost, d.s), UNOMOL_ECUDA);
    CK(cudaStreamSynchronize(d.s), UNOMOL_ECUDA);
    if (info != 0) {
        d.err = "syevd did not converge (info " + std::to_string(info) + ")";
        return UNOMOL_ESCF;
    }
    return UNOMOL_OK;
}

__global__ void k_unpack(const double* __restrict__ pk, double* __restrict__ full, int n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * n) return;
    const int i = (int)(t / n), j = (int)(t % n);
    const int hi = i > j ? i : j, lo = i > j ? j : i;
    full[t] = pk[(long long)hi * (hi + 1) / 2 + lo];
}
__global__ void k_pack(const double* __restrict__ full, double* __restrict__ pk, int n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long np = (long long)n * (n + 1) / 2;
    if (t >= np) return;
    int i = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((long long)i * (i + 1) / 2 > t) --i;
    while ((long long)(i + 1) * (i + 2) / 2 <= t) ++i;
    const int j = (int)(t - (long long)i * (i + 1) / 2);
    pk[t] = full[(long long)j * n + i];  // column-major (symmetric: either)
}
// X[:, j] = U[:, j] * sv[j]  (column-major)
__global__ void k_scale_cols(const double* __restrict__ U, const double* __restrict__ sv, double* __restrict__ X, int n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * n) return;
    X[t] = U[t] * sv[t / n];
}

unsigned blocks(long long n) { return (unsigned)((n + 255) / 256); }

// packed trace of SymmPack::TraceSymmPackProduct (SymmPack.cpp:7-18): sum_{i>j} 2 a b + sum_i a b
double trace_packed(const std::vector<double>& a, const std::vector<double>& b, int n) {
    double sum = 0.0;
    size_t ij = 0;
    for (int i = 0; i < n; ++ij, ++i) {
        for (int j = 0; j < i; ++ij, ++j) sum += a[ij] * b[ij];
        sum += 0.5 * a[ij] * b[ij];
    }
    return sum + sum;
}
// SymmPack::SymmPackDiffNorm (SymmPack.cpp:20-36)
double diffnorm_packed(const std::vector<double>& a, const std::vector<double>& b, int n) {
    double sum = 0.0;
    size_t ij = 0;
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < i; ++ij, ++j) {
            double t = a[ij] - b[ij];
            sum += t * t;
        }
        double t = a[ij] - b[ij];
        sum += 0.5 * t * t;
        ++ij;
    }
    sum += sum;
    return std::sqrt(sum) / n;
}

// X = U s^{-1/2} from the overlap (RHF.hpp:214-233)
int form_x(Dev& d, const std::vector<double>& S, double* d_pk) {
    const int n = d.n;
    CK(cudaMemcpyAsync(d_pk, S.data(), S.size() * sizeof(double), cudaMemcpyHostToDevice, d.s), UNOMOL_ECUDA);
    k_unpack<<<blocks((long long)n * n), 256, 0, d.s>>>(d_pk, d.F, n);
    int rc = syevd(d, d.F);
    if (rc) return rc;
    std::vector<double> ev(n);
    CK(cudaMemcpy(ev.data(), d.ev, n * sizeof(double), cudaMemcpyDeviceToHost), UNOMOL_ECUDA);
    for (int i = 0; i < n; ++i) {
        double f = ev[i];
        if (std::fabs(f) < 1.e-7 && f < 0.0) f = -f;
        if (f == 0.0) { d.err = "Zero Eigenvalue in Overlap Matrix"; return UNOMOL_ESCF; }
        if (f < 0.0) { d.err = "Negative Eigenvalue in Overlap Matrix"; return UNOMOL_ESCF; }
        ev[i] = 1.0 / std::sqrt(f);
    }
    CK(cudaMemcpy(d.ev, ev.data(), n * sizeof(double), cudaMemcpyHostToDevice), UNOMOL_ECUDA);
    k_scale_cols<<<blocks((long long)n * n), 256, 0, d.s>>>(d.F, d.ev, d.X, n);
    return UNOMOL_OK;
}

// F (packed, host) -> eigenvalues and C = X W on the device, then P = C_occ C_occ^T packed (host)
int diag_density(Dev& d, const std::vector<double>& Fpk, double* d_pk, int nocc, std::vector<double>& P,
                 std::vector<double>& evals, std::vector<double>* Cout) {
    const int n = d.n;
    const double one = 1.0, zero = 0.0;
    CK(cudaMemcpyAsync(d_pk, Fpk.data(), Fpk.size() * sizeof(double), cudaMemcpyHostToDevice, d.s), UNOMOL_ECUDA);
    k_unpack<<<blocks((long long)n * n), 256, 0, d.s>>>(d_pk, d.F, n);
    // T1 = F X ; W = X^T T1
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, d.F, n, d.X, n, &zero, d.T1, n), UNOMOL_ECUDA);
    CK(cublasDgemm(d.cb, CUBLAS_OP_T, CUBLAS_OP_N, n, n, n, &one, d.X, n, d.T1, n, &zero, d.W, n), UNOMOL_ECUDA);
    int rc = syevd(d, d.W);
    if (rc) return rc;
    evals.resize(n);
    CK(cudaMemcpyAsync(evals.data(), d.ev, n * sizeof(double), cudaMemcpyDeviceToHost, d.s), UNOMOL_ECUDA);
    // C = X W
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, d.X, n, d.W, n, &zero, d.C, n), UNOMOL_ECUDA);
    // P = C_occ C_occ^T
    if (nocc > 0)
        CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_T, n, n, nocc, &one, d.C, n, d.C, n, &zero, d.T1, n), UNOMOL_ECUDA);
    else
        CK(cudaMemsetAsync(d.T1, 0, (size_t)n * n * sizeof(double), d.s), UNOMOL_ECUDA);
    k_pack<<<blocks((long long)n * (n + 1) / 2), 256, 0, d.s>>>(d.T1, d_pk, n);
    P.resize((size_t)n * (n + 1) / 2);
    CK(cudaMemcpyAsync(P.data(), d_pk, P.size() * sizeof(double), cudaMemcpyDeviceToHost, d.s), UNOMOL_ECUDA);
    if (Cout) {
        Cout->resize((size_t)n * n);
        CK(cudaMemcpyAsync(Cout->data(), d.C, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost, d.s), UNOMOL_ECUDA);
    }
    CK(cudaStreamSynchronize(d.s), UNOMOL_ECUDA);
    return UNOMOL_OK;
}

// ---- Density by second-order spectral projection (SP2; A. M. N. Niklasson, Phys. Rev. B 66, 155115
// (2002)), in place of the eigen-solve ----
// With F' = X^T F X scaled so that its spectrum lies in [0, 1] with the occupied (lowest) states near 1,
// X_{k+1} = X_k^2 or 2 X_k - X_k^2, whichever brings tr X_{k+1} closer to nocc, converges to the
// projector onto the nocc lowest eigenvectors of F' when a gap separates them from the rest; then
// P = X P' X^T, the same density as C_occ C_occ^T.  Each step is one symmetric rank-n update (DSYRK, half
// a DGEMM) at N = 416 instead of a cuSOLVER syevd.

// Gershgorin bounds of a symmetric matrix (one block): out[0] = min_i (A_ii - r_i), out[1] = max_i (A_ii + r_i)
__global__ void k_gershgorin(const double* __restrict__ A, int n, double* __restrict__ out) {
    __shared__ double lo_s[256], hi_s[256];
    double lo = 1e300, hi = -1e300;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double r = 0.0;
        for (int j = 0; j < n; ++j)
            if (j != i) r += fabs(A[(size_t)j * n + i]);
        const double c = A[(size_t)i * n + i];
        lo = fmin(lo, c - r);
        hi = fmax(hi, c + r);
    }
    lo_s[threadIdx.x] = lo;
    hi_s[threadIdx.x] = hi;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            lo_s[threadIdx.x] = fmin(lo_s[threadIdx.x], lo_s[threadIdx.x + o]);
            hi_s[threadIdx.x] = fmax(hi_s[threadIdx.x], hi_s[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = lo_s[0];
        out[1] = hi_s[0];
    }
}

// X = (hi I - A) / (hi - lo), in place
__global__ void k_sp2_start(double* __restrict__ A, int n, const double* __restrict__ bounds) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * n) return;
    const int i = (int)(t % n), j = (int)(t / n);
    const double lo = bounds[0], hi = bounds[1];
    A[t] = ((i == j ? hi : 0.0) - A[t]) / (hi - lo);
}

// One SP2 step's decision on the device (one block), so that steps follow each other without a host
// round trip.  X2 = lower triangle of X^2 (DSYRK output).  st: [0] tr X, [1] square? (1/0), [2] and [3]
// the idempotency errors tr X - tr X^2 of the last two steps, [4] converged (1/0), [5] steps taken,
// [6] nocc.  Converged: the error is at rounding level (< 1e-9 n) and no longer falls (Niklasson's
// stopping rule); from then on the steps change nothing.
__global__ void k_sp2_decide(const double* __restrict__ X2, int n, double* __restrict__ st) {
    __shared__ double s_[256];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += X2[(size_t)i * n + i];
    s_[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s_[threadIdx.x] += s_[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x != 0 || st[4] != 0.0) return;
    const double tr = st[0], tr2 = s_[0], nocc = st[6];
    const double e = tr - tr2;
    if (st[5] >= 2.0 && e < 1e-9 * n && e >= st[3]) {
        st[4] = 1.0;
        st[1] = -1.0;  // no update
        return;
    }
    const bool square = fabs(tr2 - nocc) < fabs(2.0 * tr - tr2 - nocc);
    st[1] = square ? 1.0 : 0.0;
    st[0] = square ? tr2 : 2.0 * tr - tr2;
    st[3] = st[2];
    st[2] = e;
    st[5] += 1.0;
}

// X = X2 (square) or 2 X - X2 as st[1] says (nothing once converged), X2 the lower triangle of X^2
__global__ void k_sp2_step(double* __restrict__ X, const double* __restrict__ X2, int n, const double* __restrict__ st) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * n) return;
    const double mode = st[1];
    if (mode < 0.0) return;
    const int r = (int)(t % n), c = (int)(t / n);
    const double x2 = r >= c ? X2[(size_t)c * n + r] : X2[(size_t)r * n + c];
    X[t] = mode > 0.5 ? x2 : 2.0 * X[t] - x2;
}

// tr X into st[0] (one block)
__global__ void k_sp2_trace0(const double* __restrict__ X, int n, double* __restrict__ st, double nocc) {
    __shared__ double s_[256];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += X[(size_t)i * n + i];
    s_[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s_[threadIdx.x] += s_[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        st[0] = s_[0];
        st[1] = 0.0;
        st[2] = st[3] = 1e300;
        st[4] = 0.0;
        st[5] = 0.0;
        st[6] = nocc;
    }
}

// F (packed, host) -> P packed (host) by SP2; ok = false (and P untouched) when it does not reach an
// idempotent projector of trace nocc (no gap at the Fermi level): the caller then diagonalises.  The
// steps run in chunks of SP2_CHUNK on the device; the host reads the state once per chunk.
constexpr int SP2_CHUNK = 8;
constexpr int SP2_MAX_STEPS = 120;

int sp2_density(Dev& d, const std::vector<double>& Fpk, double* d_pk, int nocc, std::vector<double>& P, bool& ok,
                int& steps) {
    const int n = d.n;
    const double one = 1.0, zero = 0.0;
    ok = false;
    steps = 0;
    if (nocc <= 0 || nocc >= n) return UNOMOL_OK;
    double* h = d.work;  // [0..1] spectral bounds, [8..14] the SP2 state (the eigen-solver workspace is free here)
    if (d.lwork < 16) return UNOMOL_OK;
    double* stt = h + 8;
    CK(cudaMemcpyAsync(d_pk, Fpk.data(), Fpk.size() * sizeof(double), cudaMemcpyHostToDevice, d.s), UNOMOL_ECUDA);
    k_unpack<<<blocks((long long)n * n), 256, 0, d.s>>>(d_pk, d.F, n);
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, d.F, n, d.X, n, &zero, d.T1, n), UNOMOL_ECUDA);
    CK(cublasDgemm(d.cb, CUBLAS_OP_T, CUBLAS_OP_N, n, n, n, &one, d.X, n, d.T1, n, &zero, d.W, n), UNOMOL_ECUDA);
    k_gershgorin<<<1, 256, 0, d.s>>>(d.W, n, h);
    k_sp2_start<<<blocks((long long)n * n), 256, 0, d.s>>>(d.W, n, h);
    k_sp2_trace0<<<1, 256, 0, d.s>>>(d.W, n, stt, (double)nocc);
    double state[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int done = 0; done < SP2_MAX_STEPS; done += SP2_CHUNK) {
        for (int k = 0; k < SP2_CHUNK; ++k) {
            CK(cublasDsyrk(d.cb, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, n, n, &one, d.W, n, &zero, d.T1, n), UNOMOL_ECUDA);
            k_sp2_decide<<<1, 256, 0, d.s>>>(d.T1, n, stt);
            k_sp2_step<<<blocks((long long)n * n), 256, 0, d.s>>>(d.W, d.T1, n, stt);
        }
        CK(cudaMemcpyAsync(state, stt, sizeof(state), cudaMemcpyDeviceToHost, d.s), UNOMOL_ECUDA);
        CK(cudaStreamSynchronize(d.s), UNOMOL_ECUDA);
        if (state[4] != 0.0) break;
    }
    steps = (int)state[5];
    if (!(state[4] != 0.0 && std::fabs(state[0] - nocc) < 1e-8)) return UNOMOL_OK;  // no projector: diagonalise
    // P = X P' X^T
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, d.X, n, d.W, n, &zero, d.T1, n), UNOMOL_ECUDA);
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_T, n, n, n, &one, d.T1, n, d.X, n, &zero, d.C, n), UNOMOL_ECUDA);
    k_pack<<<blocks((long long)n * (n + 1) / 2), 256, 0, d.s>>>(d.C, d_pk, n);
    P.resize((size_t)n * (n + 1) / 2);
    CK(cudaMemcpyAsync(P.data(), d_pk, P.size() * sizeof(double), cudaMemcpyDeviceToHost, d.s), UNOMOL_ECUDA);
    CK(cudaStreamSynchronize(d.s), UNOMOL_ECUDA);
    ok = true;
    return UNOMOL_OK;
}

// ---- Density by pseudo-diagonalisation (J. J. P. Stewart, P. Csaszar, P. Pulay, J. Comput. Chem. 3,
// 227 (1982)), in place of the eigen-solve once the orbitals change little ----
// C holds the orbitals of the last step (AO coefficients, columns, C^T S C = I; the nocc occupied first).
// In those orbitals F_mo = C^T F C is nearly diagonal; its occupied-virtual block is rotated away to
// first order, theta_ai = F_ai / (e_i - e_a) with e the diagonal of F_mo, by the rotation exp(A) of the
// antisymmetric generator A = [[0, -theta^T], [theta, 0]] taken to second order block by block,
//   C_o <- C_o + C_v theta - C_o (theta^T theta) / 2,   C_v <- C_v - C_o theta^T - C_v (theta theta^T) / 2,
// then re-orthonormalised in the S metric by Newton-Schulz, C <- C (3 I - C^T S C) / 2.  At
// self-consistency F_ai -> 0, so the density converges to the projector of F; a step whose rotation is
// large or whose occupied and virtual levels come close takes the eigen-solve.
constexpr double PSEUDO_MAX_THETA = 0.2;  // largest |theta| of a step (else the eigen-solve)
constexpr double PSEUDO_MIN_GAP = 1e-3;   // smallest e_a - e_i (Eh) of a step (else the eigen-solve)

// e[j] = sum_k A[k, j] B[k, j] (column-major n x n; one block per column)
__global__ void k_coldot(const double* __restrict__ A, const double* __restrict__ B, int n, double* __restrict__ e) {
    __shared__ double s_[128];
    const size_t c = (size_t)blockIdx.x * n;
    double v = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) v = fma(A[c + k], B[c + k], v);
    s_[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s_[threadIdx.x] += s_[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) e[blockIdx.x] = s_[0];
}

// theta (nv x nocc, column-major, in place over F_vo) = F_ai / (e_i - e_a); st[0] = max |theta|,
// st[1] = min e_virtual - max e_occupied (one block)
__global__ void k_pseudo_theta(double* __restrict__ th, const double* __restrict__ e, int nocc, int nv, double* __restrict__ st) {
    __shared__ double s_th[256], s_eo[256], s_ev[256];
    double t = 0.0, eo = -1e300, ev = 1e300;
    for (long long q = threadIdx.x; q < (long long)nv * nocc; q += blockDim.x) {
        const int a = (int)(q % nv), i = (int)(q / nv);
        const double v = th[q] / (e[i] - e[nocc + a]);
        th[q] = v;
        t = fmax(t, fabs(v));
    }
    for (int k = threadIdx.x; k < nocc + nv; k += blockDim.x) {
        if (k < nocc) eo = fmax(eo, e[k]);
        else ev = fmin(ev, e[k]);
    }
    s_th[threadIdx.x] = t;
    s_eo[threadIdx.x] = eo;
    s_ev[threadIdx.x] = ev;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s_th[threadIdx.x] = fmax(s_th[threadIdx.x], s_th[threadIdx.x + o]);
            s_eo[threadIdx.x] = fmax(s_eo[threadIdx.x], s_eo[threadIdx.x + o]);
            s_ev[threadIdx.x] = fmin(s_ev[threadIdx.x], s_ev[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        st[0] = s_th[0];
        st[1] = s_ev[0] - s_eo[0];
    }
}

// M = a I + c M, in place (column-major n x n)
__global__ void k_scale_ident(double* __restrict__ M, int n, double a, double c) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * n) return;
    M[t] = ((t % n) == (t / n) ? a : 0.0) + c * M[t];
}

// F (packed, host) -> P packed (host) by one pseudo-diagonalisation step on the orbitals Cs (updated in
// place); ok = false (P and Cs untouched) when the step is too large or the gap too small: the caller
// then takes the eigen-solve.
int pseudo_density(Dev& d, double* Cs, const double* d_S, const std::vector<double>& Fpk, double* d_pk, int nocc,
                   std::vector<double>& P, bool& ok) {
    const int n = d.n, nv = n - nocc;
    const double one = 1.0, zero = 0.0, mone = -1.0, mhalf = -0.5;
    ok = false;
    if (nocc <= 0 || nv <= 0 || d.lwork < 48) return UNOMOL_OK;
    double* st = d.work + 32;  // the eigen-solver workspace is free here
    const unsigned nb = blocks((long long)n * n);
    double *FC = d.T1, *th = d.C, *Goo = d.F, *Gvv = d.F + (size_t)nocc * nocc, *Cn = d.W;
    CK(cudaMemcpyAsync(d_pk, Fpk.data(), Fpk.size() * sizeof(double), cudaMemcpyHostToDevice, d.s), UNOMOL_ECUDA);
    k_unpack<<<nb, 256, 0, d.s>>>(d_pk, d.F, n);
    // FC = F Cs; e = diag(Cs^T F Cs); F_vo = Cs_v^T FC_o -> theta
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, d.F, n, Cs, n, &zero, FC, n), UNOMOL_ECUDA);
    k_coldot<<<n, 128, 0, d.s>>>(Cs, FC, n, d.ev);
    CK(cublasDgemm(d.cb, CUBLAS_OP_T, CUBLAS_OP_N, nv, nocc, n, &one, Cs + (size_t)nocc * n, n, FC, n, &zero, th, nv),
       UNOMOL_ECUDA);
    k_pseudo_theta<<<1, 256, 0, d.s>>>(th, d.ev, nocc, nv, st);
    double h[2] = {0.0, 0.0};
    CK(cudaMemcpyAsync(h, st, sizeof(h), cudaMemcpyDeviceToHost, d.s), UNOMOL_ECUDA);
    CK(cudaStreamSynchronize(d.s), UNOMOL_ECUDA);
    if (!(h[0] <= PSEUDO_MAX_THETA && h[1] >= PSEUDO_MIN_GAP)) return UNOMOL_OK;
    // the rotation, block by block, into Cn (second-order terms only where they reach 1e-6)
    const bool second = h[0] > 1e-3;
    double* Co = Cs;
    double* Cv = Cs + (size_t)nocc * n;
    CK(cudaMemcpyAsync(Cn, Cs, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToDevice, d.s), UNOMOL_ECUDA);
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, nocc, nv, &one, Cv, n, th, nv, &one, Cn, n), UNOMOL_ECUDA);
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_T, n, nv, nocc, &mone, Co, n, th, nv, &one, Cn + (size_t)nocc * n, n),
       UNOMOL_ECUDA);
    if (second) {
        CK(cublasDgemm(d.cb, CUBLAS_OP_T, CUBLAS_OP_N, nocc, nocc, nv, &one, th, nv, th, nv, &zero, Goo, nocc), UNOMOL_ECUDA);
        CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_T, nv, nv, nocc, &one, th, nv, th, nv, &zero, Gvv, nv), UNOMOL_ECUDA);
        CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, nocc, nocc, &mhalf, Co, n, Goo, nocc, &one, Cn, n), UNOMOL_ECUDA);
        CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, nv, nv, &mhalf, Cv, n, Gvv, nv, &one, Cn + (size_t)nocc * n, n),
           UNOMOL_ECUDA);
    }
    // Newton-Schulz in the S metric: C <- C (3 I - C^T S C) / 2, twice for the larger steps; the result in Cs
    const int ns = h[0] > 1e-2 ? 2 : 1;
    for (int k = 0; k < ns; ++k) {
        double* src = k == 0 ? Cn : Cs;
        double* dst = k == 0 ? Cs : Cn;
        CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, d_S, n, src, n, &zero, FC, n), UNOMOL_ECUDA);
        CK(cublasDgemm(d.cb, CUBLAS_OP_T, CUBLAS_OP_N, n, n, n, &one, src, n, FC, n, &zero, d.C, n), UNOMOL_ECUDA);
        k_scale_ident<<<nb, 256, 0, d.s>>>(d.C, n, 1.5, -0.5);
        CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, src, n, d.C, n, &zero, dst, n), UNOMOL_ECUDA);
    }
    if (ns == 2) CK(cudaMemcpyAsync(Cs, Cn, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToDevice, d.s), UNOMOL_ECUDA);
    // P = C_occ C_occ^T
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_T, n, n, nocc, &one, Cs, n, Cs, n, &zero, FC, n), UNOMOL_ECUDA);
    k_pack<<<blocks((long long)n * (n + 1) / 2), 256, 0, d.s>>>(FC, d_pk, n);
    P.resize((size_t)n * (n + 1) / 2);
    CK(cudaMemcpyAsync(P.data(), d_pk, P.size() * sizeof(double), cudaMemcpyDeviceToHost, d.s), UNOMOL_ECUDA);
    CK(cudaStreamSynchronize(d.s), UNOMOL_ECUDA);
    ok = true;
    return UNOMOL_OK;
}

// ---- DIIS (Pulay) on the packed Fock matrices ----
struct Diis {
    int maxv = 8;
    std::vector<std::vector<double>> F, E;
    std::vector<std::vector<double>> gram;  // gram[i][j] = E_i . E_j (j <= i), one new row per push
    void push(const std::vector<double>& f, const std::vector<double>& e) {
        if ((int)F.size() == maxv) {
            F.erase(F.begin());
            E.erase(E.begin());
            gram.erase(gram.begin());
            for (auto& row : gram) row.erase(row.begin());
        }
        F.push_back(f);
        E.push_back(e);
        std::vector<double> row(E.size());
        for (size_t j = 0; j < E.size(); ++j) {
            double s = 0.0;
            for (size_t k = 0; k < e.size(); ++k) s += e[k] * E[j][k];
            row[j] = s;
        }
        gram.push_back(std::move(row));
    }
    bool extrapolate(std::vector<double>& out) {
        const int m = (int)F.size();
        if (m < 2) return false;
        std::vector<double> B((m + 1) * (m + 1), 0.0), rhs(m + 1, 0.0);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j <= i; ++j) B[i * (m + 1) + j] = B[j * (m + 1) + i] = gram[i][j];
        for (int i = 0; i < m; ++i) B[i * (m + 1) + m] = B[m * (m + 1) + i] = -1.0;
        rhs[m] = -1.0;
        // Gaussian elimination with partial pivoting
        const int N = m + 1;
        std::vector<int> piv(N);
        for (int c = 0; c < N; ++c) {
            int p = c;
            for (int r = c + 1; r < N; ++r)
                if (std::fabs(B[r * N + c]) > std::fabs(B[p * N + c])) p = r;
            if (std::fabs(B[p * N + c]) < 1e-300) return false;
            if (p != c) {
                for (int k = 0; k < N; ++k) std::swap(B[c * N + k], B[p * N + k]);
                std::swap(rhs[c], rhs[p]);
            }
            for (int r = c + 1; r < N; ++r) {
                const double f = B[r * N + c] / B[c * N + c];
                for (int k = c; k < N; ++k) B[r * N + k] -= f * B[c * N + k];
                rhs[r] -= f * rhs[c];
            }
        }
        std::vector<double> x(N);
        for (int r = N - 1; r >= 0; --r) {
            double s = rhs[r];
            for (int k = r + 1; k < N; ++k) s -= B[r * N + k] * x[k];
            x[r] = s / B[r * N + r];
        }
        out.assign(F[0].size(), 0.0);
        for (int i = 0; i < m; ++i)
            for (size_t k = 0; k < out.size(); ++k) out[k] += x[i] * F[i][k];
        return true;
    }
};

// Error vector X^T (F P S - S P F) X, packed (antisymmetric: strict lower triangle is enough)
int diis_error(Dev& d, const std::vector<double>& Fpk, const std::vector<double>& Ppk, const double* d_S,
               double* d_pk, std::vector<double>& err) {
    const int n = d.n;
    const double one = 1.0, zero = 0.0, mone = -1.0;
    double *dF = d.F, *dP = d.W, *t = d.T1, *u = d.C;  // W and C are free between diagonalisations
    CK(cudaMemcpyAsync(d_pk, Fpk.data(), Fpk.size() * sizeof(double), cudaMemcpyHostToDevice, d.s), UNOMOL_ECUDA);
    k_unpack<<<blocks((long long)n * n), 256, 0, d.s>>>(d_pk, dF, n);
    CK(cudaMemcpyAsync(d_pk, Ppk.data(), Ppk.size() * sizeof(double), cudaMemcpyHostToDevice, d.s), UNOMOL_ECUDA);
    k_unpack<<<blocks((long long)n * n), 256, 0, d.s>>>(d_pk, dP, n);
    // t = F P ; u = t S = F P S ; u -= (F P S)^T  (S P F = (F P S)^T)
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, dF, n, dP, n, &zero, t, n), UNOMOL_ECUDA);
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, t, n, d_S, n, &zero, u, n), UNOMOL_ECUDA);
    CK(cublasDgeam(d.cb, CUBLAS_OP_N, CUBLAS_OP_T, n, n, &one, u, n, &mone, u, n, t, n), UNOMOL_ECUDA);
    // u = X^T t X
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, t, n, d.X, n, &zero, dP, n), UNOMOL_ECUDA);
    CK(cublasDgemm(d.cb, CUBLAS_OP_T, CUBLAS_OP_N, n, n, n, &one, d.X, n, dP, n, &zero, u, n), UNOMOL_ECUDA);
    std::vector<double> full((size_t)n * n);
    CK(cudaMemcpyAsync(full.data(), u, full.size() * sizeof(double), cudaMemcpyDeviceToHost, d.s), UNOMOL_ECUDA);
    CK(cudaStreamSynchronize(d.s), UNOMOL_ECUDA);
    err.resize((size_t)n * (n - 1) / 2);
    size_t k = 0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) err[k++] = full[(size_t)j * n + i];
    return UNOMOL_OK;
}

double maxabs(const std::vector<double>& v) {
    double m = 0.0;
    for (double x : v) m = std::max(m, std::fabs(x));
    return m;
}

// Level shift sigma (S - S P S), packed: raises the virtual orbital energies by sigma and leaves the
// occupied ones (P = C_occ C_occ^T, C^T S C = 1), damping the occupied/virtual rotations of early
// iterations.
int level_shift(Dev& d, const std::vector<double>& Ppk, const double* d_S, double* d_pk, double sigma,
                std::vector<double>& shift) {
    const int n = d.n;
    const double one = 1.0, zero = 0.0, ms = -sigma;
    double *dP = d.W, *t = d.T1, *u = d.C;
    CK(cudaMemcpyAsync(d_pk, Ppk.data(), Ppk.size() * sizeof(double), cudaMemcpyHostToDevice, d.s), UNOMOL_ECUDA);
    k_unpack<<<blocks((long long)n * n), 256, 0, d.s>>>(d_pk, dP, n);
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, d_S, n, dP, n, &zero, t, n), UNOMOL_ECUDA);
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, t, n, d_S, n, &zero, u, n), UNOMOL_ECUDA);
    // t = sigma S - sigma S P S
    CK(cublasDgeam(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, &sigma, d_S, n, &ms, u, n, t, n), UNOMOL_ECUDA);
    k_pack<<<blocks((long long)n * (n + 1) / 2), 256, 0, d.s>>>(t, d_pk, n);
    shift.resize(Ppk.size());
    CK(cudaMemcpyAsync(shift.data(), d_pk, shift.size() * sizeof(double), cudaMemcpyDeviceToHost, d.s), UNOMOL_ECUDA);
    CK(cudaStreamSynchronize(d.s), UNOMOL_ECUDA);
    return UNOMOL_OK;
}

// McWeeny purification of a guess density (new; for the learned guess).  In the orthonormal basis of X
// (X^T S X = 1, so X^{-1} = X^T S) the density is Q = X^T S P S X; Q <- 3 Q^2 - 2 Q^3 drives every
// eigenvalue of Q in (-1/2, 1/2) to 0 and in (1/2, 3/2) to 1.  Accepted when ||Q^2 - Q||_F falls
// below 1e-10 within 60 steps and tr Q = nocc within 1e-6; then P = X Q X^T.  Otherwise (diverging
// or non-finite values, wrong electron count) ok = false and P is left unchanged.
int purify(Dev& d, const double* d_S, double* d_pk, std::vector<double>& P, int nocc, int& iters, double& err,
           double& trace, bool& ok) {
    const int n = d.n;
    const double one = 1.0, zero = 0.0, mone = -1.0, three = 3.0, mtwo = -2.0;
    double *Q = d.W, *t = d.T1, *u = d.C, *v = d.F;
    ok = false;
    iters = 0;
    err = 0.0;
    trace = 0.0;
    CK(cudaMemcpyAsync(d_pk, P.data(), P.size() * sizeof(double), cudaMemcpyHostToDevice, d.s), UNOMOL_ECUDA);
    k_unpack<<<blocks((long long)n * n), 256, 0, d.s>>>(d_pk, v, n);
    // Q = X^T (S P S) X
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, d_S, n, v, n, &zero, t, n), UNOMOL_ECUDA);
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, t, n, d_S, n, &zero, u, n), UNOMOL_ECUDA);
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, u, n, d.X, n, &zero, t, n), UNOMOL_ECUDA);
    CK(cublasDgemm(d.cb, CUBLAS_OP_T, CUBLAS_OP_N, n, n, n, &one, d.X, n, t, n, &zero, Q, n), UNOMOL_ECUDA);
    bool conv = false;
    for (int it = 0; it < 60; ++it) {
        CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, Q, n, Q, n, &zero, t, n), UNOMOL_ECUDA);  // Q^2
        CK(cublasDgeam(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, &one, t, n, &mone, Q, n, u, n), UNOMOL_ECUDA);
        double e = 0.0;
        CK(cublasDnrm2(d.cb, n * n, u, 1, &e), UNOMOL_ECUDA);  // host pointer mode: synchronous
        err = e;
        iters = it;
        if (!(e < 1e6)) return UNOMOL_OK;  // diverging or not finite
        if (e < 1e-10) {
            conv = true;
            break;
        }
        CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, t, n, Q, n, &zero, u, n), UNOMOL_ECUDA);  // Q^3
        CK(cublasDgeam(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, &three, t, n, &mtwo, u, n, Q, n), UNOMOL_ECUDA);
        iters = it + 1;
    }
    if (!conv) return UNOMOL_OK;
    std::vector<double> diag(n);
    CK(cublasGetVectorAsync(n, sizeof(double), Q, n + 1, diag.data(), 1, d.s), UNOMOL_ECUDA);
    CK(cudaStreamSynchronize(d.s), UNOMOL_ECUDA);
    for (double x : diag) trace += x;
    if (!(std::fabs(trace - nocc) < 1e-6)) return UNOMOL_OK;
    // P = X Q X^T
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, d.X, n, Q, n, &zero, t, n), UNOMOL_ECUDA);
    CK(cublasDgemm(d.cb, CUBLAS_OP_N, CUBLAS_OP_T, n, n, n, &one, t, n, d.X, n, &zero, u, n), UNOMOL_ECUDA);
    k_pack<<<blocks((long long)n * (n + 1) / 2), 256, 0, d.s>>>(u, d_pk, n);
    CK(cudaMemcpyAsync(P.data(), d_pk, P.size() * sizeof(double), cudaMemcpyDeviceToHost, d.s), UNOMOL_ECUDA);
    CK(cudaStreamSynchronize(d.s), UNOMOL_ECUDA);
    ok = true;
    return UNOMOL_OK;
}

}  // namespace

extern "C" int unomol_scf(UnomolCtx* ctx, const UnomolScfInput* in, const UnomolScfOptions* opt, UnomolScfResult* res,
                          double* P_io, double* orbital_energies) {
    if (!ctx || !in || !opt || !res || !P_io || !in->S || !in->H) return UNOMOL_EINVAL;
    const int n = in->norb;
    const size_t no2 = (size_t)n * (n + 1) / 2;
    const bool uhf = in->nelec % 2 != 0;
    const int noccA = uhf ? in->nelec - in->nelec / 2 : in->nelec / 2;
    const int noccB = in->nelec / 2;
    auto t0 = std::chrono::steady_clock::now();
    Dev d;
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return UNOMOL_ECUDA;
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamSynchronize(s); cudaStreamDestroy(s); }
    } sg{s};
    int rc = dev_init(d, n, s);
    double *d_pk = nullptr, *d_P = nullptr, *d_G = nullptr, *d_Pb = nullptr, *d_Gb = nullptr, *d_S = nullptr;
    double* d_Ws[2] = {nullptr, nullptr};  // pseudo-diagonalisation: the orbitals of each spin (AO coefficients)
    struct Bufs {
        double** p[8];
        ~Bufs() { for (auto q : p) if (*q) cudaFree(*q); }
    } bufs{{&d_pk, &d_P, &d_G, &d_Pb, &d_Gb, &d_S, &d_Ws[0], &d_Ws[1]}};
    auto fail = [&](int code) {
        res->status = code;
        std::snprintf(res->message, sizeof(res->message), "%s", d.err.c_str());
        return code;
    };
    if (rc) return fail(rc);
    if (cudaMalloc(&d_pk, no2 * sizeof(double)) || cudaMalloc(&d_P, no2 * sizeof(double)) ||
        cudaMalloc(&d_G, no2 * sizeof(double)) || cudaMalloc(&d_Pb, no2 * sizeof(double)) ||
        cudaMalloc(&d_Gb, no2 * sizeof(double)) || cudaMalloc(&d_S, (size_t)n * n * sizeof(double))) {
        d.err = "device allocation failed";
        return fail(UNOMOL_ENOMEM);
    }
    const bool pseudo = opt->density == UNOMOL_DENSITY_PSEUDO;
    if (pseudo && (cudaMalloc(&d_Ws[0], (size_t)n * n * sizeof(double)) ||
                   (uhf && cudaMalloc(&d_Ws[1], (size_t)n * n * sizeof(double))))) {
        d.err = "device allocation failed";
        return fail(UNOMOL_ENOMEM);
    }
    bool have_orbitals[2] = {false, false};
    int pseudo_steps = 0;
    std::vector<double> S(in->S, in->S + no2), H(in->H, in->H + no2);
    rc = form_x(d, S, d_pk);
    if (rc) return fail(rc);
    cudaMemcpyAsync(d_pk, S.data(), no2 * sizeof(double), cudaMemcpyHostToDevice, s);
    k_unpack<<<blocks((long long)n * n), 256, 0, s>>>(d_pk, d_S, n);
    std::vector<double> Pa(no2), Pb(no2), Ga(no2), Gb(no2), Fa(no2), Fb(no2), PoldA(no2), PoldB(no2), PoldA2(no2),
        PoldB2(no2), evA, evB, tmp;
    // guess: caller's P (RHF.hpp:120-123), the caller's P purified (new), or core Hamiltonian
    // (RHF.hpp:205-211; UHF.hpp:487-496)
    int guess_used = UNOMOL_GUESS_USED_CORE, pur_it = 0;
    double pur_err = 0.0, pur_tr = 0.0;
    if (opt->guess == UNOMOL_GUESS_GIVEN || opt->guess == UNOMOL_GUESS_PURIFY) {
        std::memcpy(Pa.data(), P_io, no2 * sizeof(double));
        if (uhf) std::memcpy(Pb.data(), P_io + no2, no2 * sizeof(double));
        guess_used = UNOMOL_GUESS_USED_GIVEN;
    }
    if (opt->guess == UNOMOL_GUESS_PURIFY) {
        bool okA = false, okB = true;
        int itB = 0;
        double eB = 0.0, trB = 0.0;
        rc = purify(d, d_S, d_pk, Pa, noccA, pur_it, pur_err, pur_tr, okA);
        if (!rc && okA && uhf) rc = purify(d, d_S, d_pk, Pb, noccB, itB, eB, trB, okB);
        if (rc) return fail(rc);
        pur_it = std::max(pur_it, itB);
        pur_err = std::max(pur_err, eB);
        guess_used = okA && okB ? UNOMOL_GUESS_USED_PURIFIED : UNOMOL_GUESS_USED_FALLBACK;
    }
    if (guess_used == UNOMOL_GUESS_USED_CORE || guess_used == UNOMOL_GUESS_USED_FALLBACK) {
        rc = diag_density(d, H, d_pk, noccA, Pa, evA, nullptr);
        if (rc) return fail(rc);
        if (uhf) {
            rc = diag_density(d, H, d_pk, noccB, Pb, evB, nullptr);
            if (rc) return fail(rc);
        }
    }
    using clk = std::chrono::steady_clock;
    auto since = [](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
    double t_fock = 0.0, t_diis = 0.0, t_diag = 0.0;
    int sp2_steps = 0, sp2_fallbacks = 0;
    const double t_setup = since(t0);
    const int maxits = opt->maxits > 0 ? opt->maxits : 300;
    const double eps = opt->eps;
    const int cflag = opt->conv_type;
    double eold = 0.0, energy = 0.0, ediff = 10.0, pdiff = 10.0, init_energy = 0.0;
    int iteration = 0, builds = 0;
    Diis diisA;
    diisA.maxv = opt->diis_size > 1 ? opt->diis_size : 8;
    const double diis_start = opt->diis_start > 0.0 ? opt->diis_start : 1e30;
    double diis_err = 0.0;
    // update(): RHF.hpp:87-112 / UHF.hpp:101-134
    // incremental builds: d_G / d_Gb keep G(P_prev); a build adds G(P - P_prev) (G is linear in P)
    const int rebuild_every = opt->rebuild_every > 0 ? opt->rebuild_every : 8;
    double fock_ms = 0.0;
    int since_full = 1 << 30;
    std::vector<double> PprevA, PprevB, dPa(no2), dPb(no2);
    auto update = [&]() -> int {
        std::fill(Ga.begin(), Ga.end(), 0.0);
        const bool full = !opt->incremental || since_full >= rebuild_every;
        const double* srcA = Pa.data();
        const double* srcB = Pb.data();
        if (!full) {
            for (size_t k = 0; k < no2; ++k) dPa[k] = Pa[k] - PprevA[k];
            srcA = dPa.data();
            if (uhf) {
                for (size_t k = 0; k < no2; ++k) dPb[k] = Pb[k] - PprevB[k];
                srcB = dPb.data();
            }
            ++since_full;
        } else {
            since_full = 1;
            cudaMemsetAsync(d_G, 0, no2 * sizeof(double), s);
            if (uhf) cudaMemsetAsync(d_Gb, 0, no2 * sizeof(double), s);
        }
        if (res->densities && builds < res->densities_cap) {
            double* dst = res->densities + (size_t)builds * no2 * (uhf ? 2 : 1);
            std::memcpy(dst, Pa.data(), no2 * sizeof(double));
            if (uhf) std::memcpy(dst + no2, Pb.data(), no2 * sizeof(double));
        }
        PprevA = Pa;
        if (uhf) PprevB = Pb;
        const auto tf = clk::now();
        cudaMemcpyAsync(d_P, srcA, no2 * sizeof(double), cudaMemcpyHostToDevice, s);
        int r;
        if (!uhf) {
            r = unomol_gpu_fock_rhf_device(ctx, d_P, d_G, s);
        } else {
            cudaMemcpyAsync(d_Pb, srcB, no2 * sizeof(double), cudaMemcpyHostToDevice, s);
            r = unomol_gpu_fock_uhf_device(ctx, d_P, d_Pb, d_G, d_Gb, s);
        }
        if (r) {
            d.err = unomol_gpu_last_error(ctx);
            return r;
        }
        ++builds;
        {
            double me = 0.0, mt = 0.0;
            if (unomol_gpu_last_build_ms(ctx, &me, &mt) == UNOMOL_OK) fock_ms += mt;
        }
        cudaMemcpyAsync(Ga.data(), d_G, no2 * sizeof(double), cudaMemcpyDeviceToHost, s);
        if (uhf) cudaMemcpyAsync(Gb.data(), d_Gb, no2 * sizeof(double), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) {
            d.err = "Fock build failed on the device";
            return UNOMOL_ECUDA;
        }
        t_fock += since(tf);
        if (!uhf) {
            energy = 2.0 * trace_packed(Pa, H, n) + trace_packed(Pa, Ga, n);
        } else {
            energy = trace_packed(Pa, H, n) + trace_packed(Pb, H, n) + 0.5 * (trace_packed(Pa, Ga, n) + trace_packed(Pb, Gb, n));
        }
        ediff = energy - eold;
        eold = energy;
        for (size_t k = 0; k < no2; ++k) Fa[k] = H[k] + Ga[k];
        if (uhf)
            for (size_t k = 0; k < no2; ++k) Fb[k] = H[k] + Gb[k];
        const auto td = clk::now();
        if (opt->accel == 2) {
            // DIIS on F; for UHF one set of coefficients for both spins (errors and Fock matrices of
            // the two spins concatenated), extrapolation only once the error is below diis_start
            std::vector<double> e, eb;
            r = diis_error(d, Fa, Pa, d_S, d_pk, e);
            if (r) return r;
            diis_err = maxabs(e);
            std::vector<double> fcat = Fa;
            if (uhf) {
                r = diis_error(d, Fb, Pb, d_S, d_pk, eb);
                if (r) return r;
                diis_err = std::max(diis_err, maxabs(eb));
                e.insert(e.end(), eb.begin(), eb.end());
                fcat.insert(fcat.end(), Fb.begin(), Fb.end());
            }
            diisA.push(fcat, e);
            if (diis_err < diis_start && diisA.extrapolate(fcat)) {
                std::copy(fcat.begin(), fcat.begin() + no2, Fa.begin());
                if (uhf) std::copy(fcat.begin() + no2, fcat.end(), Fb.begin());
            }
            if (opt->level_shift > 0.0 && diis_err > opt->level_shift_until) {
                std::vector<double> sh;
                r = level_shift(d, Pa, d_S, d_pk, opt->level_shift, sh);
                if (r) return r;
                for (size_t k = 0; k < no2; ++k) Fa[k] += sh[k];
                if (uhf) {
                    r = level_shift(d, Pb, d_S, d_pk, opt->level_shift, sh);
                    if (r) return r;
                    for (size_t k = 0; k < no2; ++k) Fb[k] += sh[k];
                }
            }
        }
        t_diis += since(td);
        const auto tg = clk::now();
        PoldA2 = PoldA;
        PoldA = Pa;
        // the density of F: SP2 or a pseudo-diagonalisation step when asked for (each falls back to the
        // eigen-solve: no gap, a large rotation, no orbitals yet), else syevd
        auto density_of = [&](int spin, const std::vector<double>& F, int nocc, std::vector<double>& P,
                              std::vector<double>& ev) -> int {
            if (opt->density == UNOMOL_DENSITY_SP2) {
                bool ok = false;
                int st = 0;
                const int rr = sp2_density(d, F, d_pk, nocc, P, ok, st);
                if (rr) return rr;
                sp2_steps += st;
                if (ok) return UNOMOL_OK;
                ++sp2_fallbacks;
            }
            if (pseudo && have_orbitals[spin]) {
                bool ok = false;
                const int rr = pseudo_density(d, d_Ws[spin], d_S, F, d_pk, nocc, P, ok);
                if (rr) return rr;
                if (ok) {
                    ++pseudo_steps;
                    return UNOMOL_OK;
                }
            }
            const int rr = diag_density(d, F, d_pk, nocc, P, ev, nullptr);
            if (!rr && pseudo) {  // the orbitals C = X W start the next pseudo step
                if (cudaMemcpyAsync(d_Ws[spin], d.C, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
                    d.err = "orbital copy failed";
                    return UNOMOL_ECUDA;
                }
                have_orbitals[spin] = true;
            }
            return rr;
        };
        r = density_of(0, Fa, noccA, Pa, evA);
        if (r) return r;
        pdiff = diffnorm_packed(Pa, PoldA, n);
        if (uhf) {
            PoldB2 = PoldB;
            PoldB = Pb;
            r = density_of(1, Fb, noccB, Pb, evB);
            if (r) return r;
            pdiff += diffnorm_packed(Pb, PoldB, n);
        }
        t_diag += since(tg);
        if (res->energies && iteration < res->energies_cap) res->energies[iteration] = energy + in->nucrep;
        ++iteration;
        return UNOMOL_OK;
    };
    // scf_converger(): RHF.hpp:536-569 (averaging; skipped when the energy went down)
    auto converger = [&]() {
        if (opt->accel == 2) return;
        if (ediff < 0.0) return;
        for (size_t k = 0; k < no2; ++k) Pa[k] = (Pa[k] + PoldA[k]) * 0.5;
        if (uhf)
            for (size_t k = 0; k < no2; ++k) Pb[k] = (Pb[k] + PoldB[k]) * 0.5;
    };
    // is_converged(): RHF.hpp:390-402 (signed ediff); DIIS: |ediff| < eps and max|error| < diis_tol
    auto converged = [&]() {
        if (opt->accel == 2) return std::fabs(ediff) < eps && diis_err < opt->diis_tol;
        switch (cflag) {
            case 0: return ediff < eps;
            case 1: return pdiff < eps;
            default: return pdiff < eps && ediff < eps;
        }
    };
    eold = 0.0;
    if ((rc = update())) return fail(rc);
    init_energy = energy + in->nucrep;
    if (opt->loop != UNOMOL_SCF_LOOP_DPM) {
        iteration = 1;
        if (uhf) eold = 0.0;  // UHF.hpp:158-160 resets eold before the second update, RHF does not
        if ((rc = update())) return fail(rc);
        iteration = 2;
    }
    bool conv = false;
    while (iteration < maxits) {
        converger();
        if ((rc = update())) return fail(rc);
        if (converged()) {
            conv = true;
            break;
        }
    }
    std::memcpy(P_io, Pa.data(), no2 * sizeof(double));
    if (uhf) std::memcpy(P_io + no2, Pb.data(), no2 * sizeof(double));
    if (orbital_energies) {
        if (opt->density == UNOMOL_DENSITY_SP2 || pseudo) {  // no eigenvalues from those steps: one eigen-solve
            const auto tg = std::chrono::steady_clock::now();
            if ((rc = diag_density(d, Fa, d_pk, noccA, tmp, evA, nullptr))) return fail(rc);
            if (uhf && (rc = diag_density(d, Fb, d_pk, noccB, tmp, evB, nullptr))) return fail(rc);
            t_diag += std::chrono::duration<double>(std::chrono::steady_clock::now() - tg).count();
        }
        std::memcpy(orbital_energies, evA.data(), n * sizeof(double));
        if (uhf) std::memcpy(orbital_energies + n, evB.data(), n * sizeof(double));
    }
    res->status = UNOMOL_OK;
    res->message[0] = 0;
    res->energy = energy + in->nucrep;
    res->e_electronic = energy;
    res->init_energy = init_energy;
    res->ediff = ediff;
    res->pdiff = pdiff;
    res->iterations = iteration;
    res->converged = conv ? 1 : 0;
    res->fock_builds = builds;
    res->fock_ms = fock_ms;
    res->diis_error = diis_err;
    res->guess_used = guess_used;
    res->purify_iterations = pur_it;
    res->purify_error = pur_err;
    res->guess_trace = pur_tr;
    res->seconds_setup = t_setup;
    res->seconds_fock = t_fock;
    res->seconds_diis = t_diis;
    res->seconds_diag = t_diag;
    res->sp2_steps = sp2_steps;
    res->sp2_fallbacks = sp2_fallbacks;
    res->pseudo_steps = pseudo_steps;
    res->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return UNOMOL_OK;
}
