// RHF SCF of every molecule of a batch at once (no reference counterpart: the reference runs one
// molecule per process).  Each iteration is the loop body of RestrictedHartreeFock::findEnergy
// (RHF.hpp:114-176) for all molecules in lockstep, with the same DIIS update as the single-molecule
// driver (scf.cu): one batched Fock build (fock_batch.cu: persistent kernels over the merged work
// lists), F = H + G and the energy 2 tr(PH) + tr(PG) per molecule, the DIIS error X^T (FPS - SPF) X,
// Pulay extrapolation over the last diis_size Fock matrices, F' = X^T F X, the eigenvectors of F'
// (cuSOLVER batched syev, FP64), C = X W and P = C_occ C_occ^T -- or, with the reference's
// accelerator, its damping (RHF.hpp:536-569) and convergence tests.  With `graph` set the whole iteration is
// captured once as a CUDA graph and replayed; the host reads only the per-molecule convergence flags
// after each replay.  A molecule that has converged is frozen (its P and energy stop changing) while
// the others go on.  With UNOMOL_DENSITY_PSEUDO (DIIS loop) the iterations after the second replace the
// batched eigen-solve by a pseudo-diagonalisation step (grouped matrix products) whenever every active
// molecule passes its step check; the host reads the check between the iteration's head and its tail.
//
// Layout: molecules are grouped by (nbf, nocc); full N x N matrices (column major, symmetric) of a
// group are contiguous with stride N^2 so that each group is one batched eigen-solve and one entry of
// every grouped GEMM.  Packed P and G live in the batch's own buffers (fock_batch.cu order).
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/unomol_gb300.h"

namespace {

constexpr int MAXV = 8;  // DIIS vectors

struct MolDev {  // per-molecule device view (group order)
    int n, nocc, bidx;     // size, occupied orbitals, index in the batch (packed-buffer order)
    long long o2, o1;      // offsets of its N x N block and its N-vector
    long long po;          // packed offset in the batch buffers
};

struct BState {
    int nmol = 0, maxv = MAXV;
    std::vector<MolDev> mols;            // group order
    std::vector<int> gstart, gn, gocc;   // groups: first molecule, size, nocc
    long long tot2 = 0, tot1 = 0;
    MolDev* d_mols = nullptr;
    double *S = nullptr, *X = nullptr, *H = nullptr, *F = nullptr, *Fo = nullptr, *T1 = nullptr, *T2 = nullptr,
           *Pf = nullptr, *Ecur = nullptr, *W = nullptr, *Hpk = nullptr;
    double *Fh = nullptr, *Eh = nullptr;  // [maxv][tot2]
    double *B = nullptr, *coef = nullptr;  // [nmol][maxv][maxv], [nmol][maxv]
    double *Enew = nullptr, *Eold = nullptr, *err = nullptr, *dE = nullptr, *pdiff = nullptr, *Einit = nullptr;  // [nmol]
    double* Pold = nullptr;               // packed, batch order: the density before the last update's diagonalisation
    double* Wp = nullptr;                 // pseudo-diagonalisation: every molecule's orbitals (orthonormal basis)
    int* pbad = nullptr;                  // pseudo-diagonalisation: per molecule (batch order), 1 = step refused
    // incremental builds: the density of the last build, the G kept, the build count (device)
    double *Pprev = nullptr, *Gacc = nullptr;
    int* step = nullptr;
    long long ptot = 0;
    cudaEvent_t eb[2] = {nullptr, nullptr};  // around every iteration's Fock build
    double fock_ms = 0.0;
    int builds = 0;
    int pseudo_steps = 0, pseudo_refused = 0;  // iterations by the pseudo-diagonalisation tail / the eigen-solve tail
    int *nupd = nullptr, *conv = nullptr, *its = nullptr, *info = nullptr, *bad = nullptr;
    // grouped-GEMM pointer arrays (device) per product
    static constexpr int NPROD = 16;
    const double** pa[NPROD] = {};
    const double** pb[NPROD] = {};
    double** pc[NPROD] = {};
    cublasHandle_t cb = nullptr;
    cusolverDnHandle_t cs = nullptr;
    cusolverDnParams_t prm = nullptr;
    void* dwork = nullptr;
    void* cublas_ws = nullptr;
    size_t dwork_size = 0;
    std::vector<char> hwork;
    std::vector<char> loop_group;  // 1: per-matrix syevd for this group
    int loop_groups = 0;
    std::string err_msg, capture_error;
    ~BState() {
        for (void* p : std::vector<void*>{d_mols, S, X, H, F, Fo, T1, T2, Pf, Ecur, W, Hpk, Fh, Eh, B, coef, Enew, Eold,
                                          err, dE, pdiff, Einit, Pold, nupd, conv, its, info, bad, dwork, cublas_ws,
                                          Pprev, Gacc, step, Wp, pbad})
            if (p) cudaFree(p);
        for (cudaEvent_t e : eb)
            if (e) cudaEventDestroy(e);
        for (int k = 0; k < NPROD; ++k) {
            if (pa[k]) cudaFree(pa[k]);
            if (pb[k]) cudaFree(pb[k]);
            if (pc[k]) cudaFree(pc[k]);
        }
        if (prm) cusolverDnDestroyParams(prm);
        if (cs) cusolverDnDestroy(cs);
        if (cb) cublasDestroy(cb);
    }
};

#define BK(call, code)                                     \
    do {                                                   \
        if ((call) != 0) {                                 \
            st.err_msg = std::string(#call) + " failed";   \
            return code;                                   \
        }                                                  \
    } while (0)

// ---- per-molecule kernels: one CTA per molecule (blockIdx.x = group-order index) ----

__device__ __forceinline__ long long pk_index(int i, int j) {
    const int hi = i > j ? i : j, lo = i > j ? j : i;
    return (long long)hi * (hi + 1) / 2 + lo;
}

__device__ double block_sum(double v) {
    __shared__ double ws[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;  // valid in thread 0
}

__device__ double block_max(double v) {
    __shared__ double ws[32];
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
    }
    __syncthreads();
    return t;
}

// the same for values of any sign (block_max's idle lanes hold 0, which suits magnitudes only)
__device__ double block_max_signed(double v) {
    __shared__ double ws[32];
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = -1e300;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : -1e300;
        for (int o = 16; o > 0; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
    }
    __syncthreads();
    return t;  // valid in thread 0
}

// packed (batch order) -> full (group order)
__global__ void k_unpack(const MolDev* __restrict__ M, const double* __restrict__ pk, double* __restrict__ full) {
    const MolDev m = M[blockIdx.x];
    for (int e = threadIdx.x; e < m.n * m.n; e += blockDim.x) {
        const int i = e % m.n, j = e / m.n;
        full[m.o2 + e] = pk[m.po + pk_index(i, j)];
    }
}

// F = H + G (full), E = sum_{i>=j} w (2H + G) P (packed; w = 2 off the diagonal): 2 tr(PH) + tr(PG)
__global__ void k_fock(const MolDev* __restrict__ M, const double* __restrict__ Hpk, const double* __restrict__ G,
                       const double* __restrict__ P, double* __restrict__ F, double* __restrict__ Enew) {
    const MolDev m = M[blockIdx.x];
    double e = 0.0;
    for (int t = threadIdx.x; t < m.n * m.n; t += blockDim.x) {
        const int i = t % m.n, j = t / m.n;
        const long long k = pk_index(i, j);
        const double h = Hpk[m.po + k], g = G[m.po + k];
        F[m.o2 + t] = h + g;
        if (i >= j) e += (i == j ? 1.0 : 2.0) * (2.0 * h + g) * P[m.po + k];
    }
    e = block_sum(e);
    if (threadIdx.x == 0) Enew[m.bidx] = e;
}

// E = T - T^T (the antisymmetric FPS - SPF)
__global__ void k_antisym(const MolDev* __restrict__ M, const double* __restrict__ T, double* __restrict__ E) {
    const MolDev m = M[blockIdx.x];
    for (int t = threadIdx.x; t < m.n * m.n; t += blockDim.x) {
        const int i = t % m.n, j = t / m.n;
        E[m.o2 + t] = T[m.o2 + t] - T[m.o2 + (long long)i * m.n + j];
    }
}

// DIIS: store F and the error in the ring slot of this update, max |error|, the new row of B
__global__ void k_diis_push(const MolDev* __restrict__ M, const int* __restrict__ conv, const int* __restrict__ nupd,
                            int maxv, long long tot2, const double* __restrict__ F, const double* __restrict__ E,
                            double* __restrict__ Fh, double* __restrict__ Eh, double* __restrict__ err) {
    const MolDev m = M[blockIdx.x];
    if (conv[m.bidx]) return;
    const int slot = nupd[m.bidx] % maxv;
    double mx = 0.0;
    for (int t = threadIdx.x; t < m.n * m.n; t += blockDim.x) {
        Fh[slot * tot2 + m.o2 + t] = F[m.o2 + t];
        const double v = E[m.o2 + t];
        Eh[slot * tot2 + m.o2 + t] = v;
        mx = fmax(mx, fabs(v));
    }
    mx = block_max(mx);
    if (threadIdx.x == 0) err[m.bidx] = mx;
}

// B[slot][j] = <E_slot, E_j> over the stored vectors; grid (molecules, maxv)
__global__ void k_diis_dots(const MolDev* __restrict__ M, const int* __restrict__ conv, const int* __restrict__ nupd,
                            int maxv, long long tot2, const double* __restrict__ Eh, double* __restrict__ B) {
    const MolDev m = M[blockIdx.x];
    const int j = blockIdx.y;
    if (conv[m.bidx]) return;
    const int cnt = min(nupd[m.bidx] + 1, maxv), slot = nupd[m.bidx] % maxv;
    if (j >= cnt) return;
    double s = 0.0;
    for (int t = threadIdx.x; t < m.n * m.n; t += blockDim.x) s += Eh[slot * tot2 + m.o2 + t] * Eh[j * tot2 + m.o2 + t];
    s = block_sum(s);
    if (threadIdx.x == 0) {
        double* Bm = B + (long long)m.bidx * maxv * maxv;
        Bm[slot * maxv + j] = s;
        Bm[j * maxv + slot] = s;
    }
}

// Pulay coefficients: [B -1; -1 0] [c; l] = [0; -1] by Gaussian elimination with partial pivoting;
// coef[0] = NaN when there is nothing to extrapolate (fewer than 2 vectors or a singular system)
__global__ void k_diis_solve(int nmol, const int* __restrict__ conv, const int* __restrict__ nupd, int maxv,
                             const double* __restrict__ B, double* __restrict__ coef) {
    const int mol = blockIdx.x * blockDim.x + threadIdx.x;
    if (mol >= nmol || conv[mol]) return;
    const int cnt = min(nupd[mol] + 1, maxv);
    double* c = coef + (long long)mol * maxv;
    if (cnt < 2) {
        c[0] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    const int N = cnt + 1;
    double A[(MAXV + 1) * (MAXV + 1)], r[MAXV + 1], x[MAXV + 1];
    const double* Bm = B + (long long)mol * maxv * maxv;
    for (int i = 0; i < N; ++i) {
        for (int j = 0; j < N; ++j)
            A[i * N + j] = (i < cnt && j < cnt) ? Bm[i * maxv + j] : (i == cnt && j == cnt) ? 0.0 : -1.0;
        r[i] = i < cnt ? 0.0 : -1.0;
    }
    for (int col = 0; col < N; ++col) {
        int p = col;
        for (int i = col + 1; i < N; ++i)
            if (fabs(A[i * N + col]) > fabs(A[p * N + col])) p = i;
        if (fabs(A[p * N + col]) < 1e-300) {
            c[0] = __longlong_as_double(0x7ff8000000000000ll);
            return;
        }
        if (p != col) {
            for (int k = 0; k < N; ++k) {
                const double t = A[col * N + k];
                A[col * N + k] = A[p * N + k];
                A[p * N + k] = t;
            }
            const double t = r[col];
            r[col] = r[p];
            r[p] = t;
        }
        for (int i = col + 1; i < N; ++i) {
            const double f = A[i * N + col] / A[col * N + col];
            for (int k = col; k < N; ++k) A[i * N + k] -= f * A[col * N + k];
            r[i] -= f * r[col];
        }
    }
    for (int i = N - 1; i >= 0; --i) {
        double s = r[i];
        for (int k = i + 1; k < N; ++k) s -= A[i * N + k] * x[k];
        x[i] = s / A[i * N + i];
    }
    for (int i = 0; i < cnt; ++i) c[i] = x[i];
}

__global__ void k_diis_extrap(const MolDev* __restrict__ M, const int* __restrict__ conv, const int* __restrict__ nupd,
                              int maxv, long long tot2, const double* __restrict__ coef, const double* __restrict__ Fh,
                              double* __restrict__ F) {
    const MolDev m = M[blockIdx.x];
    if (conv[m.bidx]) return;
    const double* c = coef + (long long)m.bidx * maxv;
    if (isnan(c[0])) return;
    const int cnt = min(nupd[m.bidx] + 1, maxv);
    for (int t = threadIdx.x; t < m.n * m.n; t += blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < cnt; ++j) s += c[j] * Fh[j * tot2 + m.o2 + t];
        F[m.o2 + t] = s;
    }
}

// full P -> the batch's packed P (frozen molecules keep theirs)
__global__ void k_pack(const MolDev* __restrict__ M, const int* __restrict__ conv, const double* __restrict__ Pf,
                       double* __restrict__ P) {
    const MolDev m = M[blockIdx.x];
    if (conv[m.bidx]) return;
    for (int t = threadIdx.x; t < m.n * (m.n + 1) / 2; t += blockDim.x) {
        int i = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
        while ((long long)i * (i + 1) / 2 > t) --i;
        while ((long long)(i + 1) * (i + 2) / 2 <= t) ++i;
        const int j = t - i * (i + 1) / 2;
        P[m.po + t] = Pf[m.o2 + (long long)j * m.n + i];
    }
}

// X = U s^{-1/2} (RHF.hpp:214-233); bad[mol] = 1 on a non-positive overlap eigenvalue
__global__ void k_form_x(const MolDev* __restrict__ M, const double* __restrict__ W, double* __restrict__ U,
                         int* __restrict__ bad) {
    const MolDev m = M[blockIdx.x];
    for (int t = threadIdx.x; t < m.n * m.n; t += blockDim.x) {
        double f = W[m.o1 + t / m.n];
        if (fabs(f) < 1.e-7 && f < 0.0) f = -f;
        if (f <= 0.0) {
            bad[m.bidx] = 1;
            f = 1.0;
        }
        U[m.o2 + t] *= 1.0 / sqrt(f);
    }
}

// The reference's scf_converger (RHF.hpp:536-569): before an update from the damp_from-th on, a
// molecule whose energy went up in the last update averages its density with the one before it.
__global__ void k_damp(const MolDev* __restrict__ M, const int* __restrict__ conv, const int* __restrict__ nupd,
                       const double* __restrict__ dE, int damp_from, const double* __restrict__ Pold, double* __restrict__ P) {
    const MolDev m = M[blockIdx.x];
    if (conv[m.bidx] || nupd[m.bidx] < damp_from || dE[m.bidx] < 0.0) return;
    for (int t = threadIdx.x; t < m.n * (m.n + 1) / 2; t += blockDim.x) P[m.po + t] = 0.5 * (P[m.po + t] + Pold[m.po + t]);
}

// Pold = P (packed) of the active molecules, before the update replaces P (RHF.hpp:108)
__global__ void k_save_old(const MolDev* __restrict__ M, const int* __restrict__ conv, const double* __restrict__ P,
                           double* __restrict__ Pold) {
    const MolDev m = M[blockIdx.x];
    if (conv[m.bidx]) return;
    for (int t = threadIdx.x; t < m.n * (m.n + 1) / 2; t += blockDim.x) Pold[m.po + t] = P[m.po + t];
}

// SymmPack::SymmPackDiffNorm (SymmPack.cpp:20-36): sqrt(2 (sum_{i>j} d^2 + sum_i d^2 / 2)) / N
__global__ void k_pdiff(const MolDev* __restrict__ M, const int* __restrict__ conv, const double* __restrict__ P,
                        const double* __restrict__ Pold, double* __restrict__ pdiff) {
    const MolDev m = M[blockIdx.x];
    if (conv[m.bidx]) return;
    double sum = 0.0;
    for (int t = threadIdx.x; t < m.n * (m.n + 1) / 2; t += blockDim.x) {
        int i = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
        while ((long long)i * (i + 1) / 2 > t) --i;
        while ((long long)(i + 1) * (i + 2) / 2 <= t) ++i;
        const double d = P[m.po + t] - Pold[m.po + t];
        sum += (t - (long long)i * (i + 1) / 2 == i ? 0.5 : 1.0) * d * d;
    }
    sum = block_sum(sum);
    if (threadIdx.x == 0) pdiff[m.bidx] = sqrt(2.0 * sum) / m.n;
}

// per-update bookkeeping: energies, the update counter and the convergence test from the
// first_check-th update on.  DIIS (accel 2): |dE| < eps and max |error| < tol (the single-molecule
// driver's test); otherwise is_converged (RHF.hpp:390-402) on the signed dE and/or pdiff (cflag).
__global__ void k_converge(int nmol, const double* __restrict__ Enew, double* __restrict__ Eold, double* __restrict__ dE,
                           double* __restrict__ Einit, int* __restrict__ nupd, int* __restrict__ conv, int* __restrict__ its,
                           const double* __restrict__ err, const double* __restrict__ pdiff, int accel, int cflag,
                           int first_check, double eps, double tol) {
    const int mol = blockIdx.x * blockDim.x + threadIdx.x;
    if (mol >= nmol || conv[mol]) return;
    const double de = Enew[mol] - Eold[mol];
    Eold[mol] = Enew[mol];
    dE[mol] = de;
    const int u = ++nupd[mol];
    its[mol] = u;
    if (u == 1) Einit[mol] = Enew[mol];
    if (u < first_check) return;
    bool ok;
    if (accel == 2) ok = fabs(de) < eps && err[mol] < tol;
    else if (cflag == 0) ok = de < eps;
    else if (cflag == 1) ok = pdiff[mol] < eps;
    else ok = pdiff[mol] < eps && de < eps;
    if (ok) conv[mol] = 1;
}

unsigned blocks(long long n) { return (unsigned)((n + 255) / 256); }

// Incremental builds (UnomolScfOptions.incremental), as the single-molecule SCF does them: G is linear in
// P, so a build of P - P_prev added to the G kept gives G(P); every rebuild-th build is a full one.
// The build count lives on the device, so that one captured iteration serves every build.
// Before the build: the batch's density buffer takes the change (a full build keeps P); P_prev takes P.
__global__ void k_inc_pre(long long n, double* __restrict__ P, double* __restrict__ Pprev, const int* __restrict__ step,
                          int rebuild) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double p = P[i];
    if (*step % rebuild != 0) P[i] = p - Pprev[i];
    Pprev[i] = p;
}

// After the build: G kept plus this build's G (a full build replaces it), the density restored.
__global__ void k_inc_post(long long n, double* __restrict__ P, const double* __restrict__ Pprev, double* __restrict__ G,
                           double* __restrict__ Gacc, const int* __restrict__ step, int rebuild) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double g = *step % rebuild == 0 ? G[i] : Gacc[i] + G[i];
    Gacc[i] = g;
    G[i] = g;
    P[i] = Pprev[i];
}

__global__ void k_inc_step(int* step) { ++*step; }

// Pseudo-diagonalisation (J. J. P. Stewart, P. Csaszar, P. Pulay, J. Comput. Chem. 3, 227 (1982)), as
// the single-molecule driver's: in the last orbitals W, F_mo = W^T F' W; A = the antisymmetric generator
// of the occupied-virtual rotation theta_ai = F_ai / (e_i - e_a) (e the diagonal of F_mo).  bad[m] = 1
// when an active molecule's step is large (max |theta| > thmax) or its occupied and virtual levels are
// not separated by gap_min (the occupation of the last orbitals is then no longer the lowest one): the
// iteration then takes the eigen-solve for every molecule.
__global__ void k_pseudo_gen(const MolDev* __restrict__ M, const int* __restrict__ conv, const double* __restrict__ Fmo,
                             double* __restrict__ A, int* __restrict__ bad, double thmax, double gap_min) {
    const MolDev m = M[blockIdx.x];
    const int n = m.n, no = m.nocc;
    const double* F = Fmo + m.o2;
    double* Am = A + m.o2;
    double th = 0.0, eo = -1e300, ev = 1e300;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int r = t % n, c = t / n;
        double v = 0.0;
        if (r >= no && c < no) {  // theta_rc: r virtual, c occupied
            v = F[t] / (F[(long long)c * n + c] - F[(long long)r * n + r]);
            th = fmax(th, fabs(v));
        } else if (r < no && c >= no) {  // -theta_cr
            v = -F[(long long)r * n + c] / (F[(long long)r * n + r] - F[(long long)c * n + c]);
        }
        Am[t] = v;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double e = F[(long long)i * n + i];
        if (i < no) eo = fmax(eo, e);
        else ev = fmin(ev, e);
    }
    th = block_max(th);
    eo = block_max_signed(eo);
    ev = -block_max_signed(-ev);
    if (threadIdx.x == 0) {
        const bool ok = no <= 0 || no >= n || (th <= thmax && ev - eo >= gap_min);  // NaN: not ok
        bad[m.bidx] = conv[m.bidx] || ok ? 0 : 1;
    }
}

// per molecule: Mt = a I + b A + c Mt (A may be null)
__global__ void k_mident(const MolDev* __restrict__ M, double* __restrict__ Mt, const double* __restrict__ A, double a, double b,
                         double c) {
    const MolDev m = M[blockIdx.x];
    for (int t = threadIdx.x; t < m.n * m.n; t += blockDim.x) {
        const bool diag = (t % m.n) == (t / m.n);
        Mt[m.o2 + t] = (diag ? a : 0.0) + (A ? b * A[m.o2 + t] : 0.0) + c * Mt[m.o2 + t];
    }
}

// grouped GEMM C = op(A) op(B) for every molecule; pointer arrays were filled once for product `id`
int gemm(BState& st, int id, cublasOperation_t ta, cublasOperation_t tb, bool k_occ) {
    const int ng = (int)st.gn.size();
    std::vector<cublasOperation_t> TA(ng, ta), TB(ng, tb);
    std::vector<int> m(ng), n(ng), k(ng), ld(ng), gs(ng);
    std::vector<double> al(ng, 1.0), be(ng, 0.0);
    for (int g = 0; g < ng; ++g) {
        m[g] = n[g] = ld[g] = st.gn[g];
        k[g] = k_occ ? st.gocc[g] : st.gn[g];
        gs[g] = (g + 1 < ng ? st.gstart[g + 1] : st.nmol) - st.gstart[g];
    }
    BK(cublasDgemmGroupedBatched(st.cb, TA.data(), TB.data(), m.data(), n.data(), k.data(), al.data(), st.pa[id],
                                 ld.data(), st.pb[id], ld.data(), be.data(), st.pc[id], ld.data(), ng, gs.data()),
       UNOMOL_ECUDA);
    return UNOMOL_OK;
}

int set_ptrs(BState& st, int id, const double* A, const double* B, double* C) {
    std::vector<const double*> a(st.nmol), b(st.nmol);
    std::vector<double*> c(st.nmol);
    for (int i = 0; i < st.nmol; ++i) {
        a[i] = A + st.mols[i].o2;
        b[i] = B + st.mols[i].o2;
        c[i] = C + st.mols[i].o2;
    }
    BK(cudaMalloc(&st.pa[id], st.nmol * sizeof(void*)), UNOMOL_ENOMEM);
    BK(cudaMalloc(&st.pb[id], st.nmol * sizeof(void*)), UNOMOL_ENOMEM);
    BK(cudaMalloc(&st.pc[id], st.nmol * sizeof(void*)), UNOMOL_ENOMEM);
    BK(cudaMemcpy(st.pa[id], a.data(), st.nmol * sizeof(void*), cudaMemcpyHostToDevice), UNOMOL_ECUDA);
    BK(cudaMemcpy(st.pb[id], b.data(), st.nmol * sizeof(void*), cudaMemcpyHostToDevice), UNOMOL_ECUDA);
    BK(cudaMemcpy(st.pc[id], c.data(), st.nmol * sizeof(void*), cudaMemcpyHostToDevice), UNOMOL_ECUDA);
    return UNOMOL_OK;
}

// eigenvectors (in place) and eigenvalues of every group's matrices in A (W: eigenvalues): one batched
// cuSOLVER call per group, or one syevd per matrix for a group the batched solver does not take
int eig(BState& st, double* A) {
    for (size_t g = 0; g < st.gn.size(); ++g) {
        const int n = st.gn[g];
        const int first = st.gstart[g], cnt = (g + 1 < st.gn.size() ? st.gstart[g + 1] : st.nmol) - first;
        const MolDev& m0 = st.mols[first];
        if (st.loop_group[g]) {
            for (int i = 0; i < cnt; ++i) {
                const MolDev& m = st.mols[first + i];
                BK(cusolverDnDsyevd(st.cs, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, A + m.o2, n, st.W + m.o1,
                                    (double*)st.dwork, (int)(st.dwork_size / sizeof(double)), st.info + first + i),
                   UNOMOL_ECUDA);
            }
            continue;
        }
        size_t dsz = 0, hsz = 0;
        BK(cusolverDnXsyevBatched_bufferSize(st.cs, st.prm, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                                             CUDA_R_64F, A + m0.o2, n, CUDA_R_64F, st.W + m0.o1, CUDA_R_64F, &dsz, &hsz,
                                             cnt),
           UNOMOL_ECUDA);
        if (dsz > st.dwork_size) {
            st.err_msg = "batched eigen-solver workspace larger than reserved";
            return UNOMOL_ENOMEM;
        }
        if (hsz > st.hwork.size()) st.hwork.resize(hsz);
        BK(cusolverDnXsyevBatched(st.cs, st.prm, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_R_64F,
                                  A + m0.o2, n, CUDA_R_64F, st.W + m0.o1, CUDA_R_64F, st.dwork, st.dwork_size,
                                  hsz ? st.hwork.data() : nullptr, hsz, st.info + first, cnt),
           UNOMOL_ECUDA);
    }
    return UNOMOL_OK;
}

// Fo = F' -> P: the eigenvectors of F' (in place), C = X Fo, P = C_occ C_occ^T, packed into the batch
// buffer (and the eigenvectors kept for the pseudo-diagonalisation steps)
int density_eig_tail(BState& st, double* dP, cudaStream_t s) {
    int rc;
    if ((rc = eig(st, st.Fo))) return rc;
    if (st.Wp) BK(cudaMemcpyAsync(st.Wp, st.Fo, st.tot2 * sizeof(double), cudaMemcpyDeviceToDevice, s), UNOMOL_ECUDA);
    if ((rc = gemm(st, 6, CUBLAS_OP_N, CUBLAS_OP_N, false))) return rc;  // T2 = C = X Fo
    if ((rc = gemm(st, 7, CUBLAS_OP_N, CUBLAS_OP_T, true))) return rc;   // Pf = C_occ C_occ^T
    k_pack<<<st.nmol, 256, 0, s>>>(st.d_mols, st.conv, st.Pf, dP);
    BK(cudaGetLastError(), UNOMOL_ECUDA);
    return UNOMOL_OK;
}

// F (full) -> P: F' = X^T F X, then the eigen-solve tail
int density_from_F(BState& st, double* dP, cudaStream_t s) {
    int rc;
    if ((rc = gemm(st, 4, CUBLAS_OP_N, CUBLAS_OP_N, false))) return rc;  // T1 = F X
    if ((rc = gemm(st, 5, CUBLAS_OP_T, CUBLAS_OP_N, false))) return rc;  // Fo = X^T T1
    return density_eig_tail(st, dP, s);
}

// Pseudo-diagonalisation, first part: F' = X^T F X (Fo), F_mo = Wp^T F' Wp (T2), the rotation generator
// (T1) and the per-molecule check (st.pbad)
int pseudo_head(BState& st, cudaStream_t s) {
    int rc;
    if ((rc = gemm(st, 4, CUBLAS_OP_N, CUBLAS_OP_N, false))) return rc;  // T1 = F X
    if ((rc = gemm(st, 5, CUBLAS_OP_T, CUBLAS_OP_N, false))) return rc;  // Fo = X^T T1
    if ((rc = gemm(st, 8, CUBLAS_OP_N, CUBLAS_OP_N, false))) return rc;  // T1 = Fo Wp
    if ((rc = gemm(st, 9, CUBLAS_OP_T, CUBLAS_OP_N, false))) return rc;  // T2 = Wp^T T1 = F_mo
    k_pseudo_gen<<<st.nmol, 256, 0, s>>>(st.d_mols, st.conv, st.T2, st.T1, st.pbad, 0.2, 1e-3);  // T1 = A
    BK(cudaGetLastError(), UNOMOL_ECUDA);
    return UNOMOL_OK;
}

// Pseudo-diagonalisation, second part: Wp <- Wp (I + A + A^2 / 2), two Newton-Schulz steps
// W <- W (3 I - W^T W) / 2, then C = X Wp and P = C_occ C_occ^T as the eigen-solve tail
int pseudo_tail(BState& st, double* dP, cudaStream_t s) {
    int rc;
    const unsigned nm = (unsigned)st.nmol;
    if ((rc = gemm(st, 10, CUBLAS_OP_N, CUBLAS_OP_N, false))) return rc;  // T2 = A A
    k_mident<<<nm, 256, 0, s>>>(st.d_mols, st.T2, st.T1, 1.0, 1.0, 0.5);   // T2 = I + A + A^2 / 2
    if ((rc = gemm(st, 11, CUBLAS_OP_N, CUBLAS_OP_N, false))) return rc;  // Fo = Wp T2
    if ((rc = gemm(st, 12, CUBLAS_OP_T, CUBLAS_OP_N, false))) return rc;  // T1 = Fo^T Fo
    k_mident<<<nm, 256, 0, s>>>(st.d_mols, st.T1, nullptr, 1.5, 0.0, -0.5);
    if ((rc = gemm(st, 13, CUBLAS_OP_N, CUBLAS_OP_N, false))) return rc;  // Wp = Fo T1
    if ((rc = gemm(st, 14, CUBLAS_OP_T, CUBLAS_OP_N, false))) return rc;  // T1 = Wp^T Wp
    k_mident<<<nm, 256, 0, s>>>(st.d_mols, st.T1, nullptr, 1.5, 0.0, -0.5);
    if ((rc = gemm(st, 15, CUBLAS_OP_N, CUBLAS_OP_N, false))) return rc;  // Fo = Wp T1
    BK(cudaMemcpyAsync(st.Wp, st.Fo, st.tot2 * sizeof(double), cudaMemcpyDeviceToDevice, s), UNOMOL_ECUDA);
    if ((rc = gemm(st, 6, CUBLAS_OP_N, CUBLAS_OP_N, false))) return rc;   // T2 = C = X Fo
    if ((rc = gemm(st, 7, CUBLAS_OP_N, CUBLAS_OP_T, true))) return rc;    // Pf = C_occ C_occ^T
    k_pack<<<nm, 256, 0, s>>>(st.d_mols, st.conv, st.Pf, dP);
    BK(cudaGetLastError(), UNOMOL_ECUDA);
    return UNOMOL_OK;
}

struct BOpts {
    int accel, cflag, first_check;
    double eps, tol;
    int incremental, rebuild;
};

// Parts of one DIIS-loop iteration with pseudo-diagonalisation: the whole iteration with the eigen-solve
// (ITER_FULL), or its head up to the pseudo-diagonalisation check (ITER_HEAD) followed, after the host
// has read the check, by the pseudo-diagonalisation tail (ITER_PSEUDO) or the eigen-solve tail (ITER_EIG).
enum IterPart { ITER_FULL = 0, ITER_HEAD = 1, ITER_PSEUDO = 2, ITER_EIG = 3 };

// one SCF update of every active molecule (the part that is captured as a graph)
int iteration(BState& st, UnomolBatch* batch, double* dP, double* dG, const BOpts& o, cudaStream_t s,
              int part = ITER_FULL) {
    int rc;
    if (part == ITER_PSEUDO || part == ITER_EIG) {  // the tails of a pseudo-diagonalisation iteration (DIIS loop)
        if ((rc = part == ITER_PSEUDO ? pseudo_tail(st, dP, s) : density_eig_tail(st, dP, s))) return rc;
        k_converge<<<blocks(st.nmol), 256, 0, s>>>(st.nmol, st.Enew, st.Eold, st.dE, st.Einit, st.nupd, st.conv, st.its, st.err,
                                                   st.pdiff, o.accel, o.cflag, o.first_check, o.eps, o.tol);
        BK(cudaGetLastError(), UNOMOL_ECUDA);
        return UNOMOL_OK;
    }
    if (o.accel != 2) k_damp<<<st.nmol, 256, 0, s>>>(st.d_mols, st.conv, st.nupd, st.dE, o.first_check - 1, st.Pold, dP);
    if (o.incremental) k_inc_pre<<<blocks(st.ptot), 256, 0, s>>>(st.ptot, dP, st.Pprev, st.step, o.rebuild);
    // in a captured iteration the records are external event nodes, timed after every replay
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    BK(cudaStreamIsCapturing(s, &cap), UNOMOL_ECUDA);
    const unsigned evf = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    BK(cudaEventRecordWithFlags(st.eb[0], s, evf), UNOMOL_ECUDA);
    rc = unomol_gpu_batch_fock(batch, UNOMOL_BATCH_LAUNCHES, s);
    if (rc) {
        st.err_msg = unomol_gpu_batch_last_error(batch);
        return rc;
    }
    BK(cudaEventRecordWithFlags(st.eb[1], s, evf), UNOMOL_ECUDA);
    if (o.incremental) {
        k_inc_post<<<blocks(st.ptot), 256, 0, s>>>(st.ptot, dP, st.Pprev, dG, st.Gacc, st.step, o.rebuild);
        k_inc_step<<<1, 1, 0, s>>>(st.step);
    }
    k_fock<<<st.nmol, 256, 0, s>>>(st.d_mols, st.Hpk, dG, dP, st.F, st.Enew);
    BK(cudaGetLastError(), UNOMOL_ECUDA);
    if (o.accel != 2) {
        k_save_old<<<st.nmol, 256, 0, s>>>(st.d_mols, st.conv, dP, st.Pold);
        if ((rc = density_from_F(st, dP, s))) return rc;
        k_pdiff<<<st.nmol, 256, 0, s>>>(st.d_mols, st.conv, dP, st.Pold, st.pdiff);
        k_converge<<<blocks(st.nmol), 256, 0, s>>>(st.nmol, st.Enew, st.Eold, st.dE, st.Einit, st.nupd, st.conv, st.its, st.err,
                                                   st.pdiff, o.accel, o.cflag, o.first_check, o.eps, o.tol);
        BK(cudaGetLastError(), UNOMOL_ECUDA);
        return UNOMOL_OK;
    }
    k_unpack<<<st.nmol, 256, 0, s>>>(st.d_mols, dP, st.Pf);
    BK(cudaGetLastError(), UNOMOL_ECUDA);
    // DIIS error X^T (F P S - S P F) X
    if ((rc = gemm(st, 0, CUBLAS_OP_N, CUBLAS_OP_N, false))) return rc;  // T1 = F P
    if ((rc = gemm(st, 1, CUBLAS_OP_N, CUBLAS_OP_N, false))) return rc;  // T2 = T1 S
    k_antisym<<<st.nmol, 256, 0, s>>>(st.d_mols, st.T2, st.T1);          // T1 = T2 - T2^T
    if ((rc = gemm(st, 2, CUBLAS_OP_N, CUBLAS_OP_N, false))) return rc;  // T2 = T1 X
    if ((rc = gemm(st, 3, CUBLAS_OP_T, CUBLAS_OP_N, false))) return rc;  // Ecur = X^T T2
    k_diis_push<<<st.nmol, 256, 0, s>>>(st.d_mols, st.conv, st.nupd, st.maxv, st.tot2, st.F, st.Ecur, st.Fh, st.Eh, st.err);
    k_diis_dots<<<dim3(st.nmol, st.maxv), 256, 0, s>>>(st.d_mols, st.conv, st.nupd, st.maxv, st.tot2, st.Eh, st.B);
    k_diis_solve<<<blocks(st.nmol), 256, 0, s>>>(st.nmol, st.conv, st.nupd, st.maxv, st.B, st.coef);
    k_diis_extrap<<<st.nmol, 256, 0, s>>>(st.d_mols, st.conv, st.nupd, st.maxv, st.tot2, st.coef, st.Fh, st.F);
    BK(cudaGetLastError(), UNOMOL_ECUDA);
    if (part == ITER_HEAD) return pseudo_head(st, s);
    if ((rc = density_from_F(st, dP, s))) return rc;
    k_converge<<<blocks(st.nmol), 256, 0, s>>>(st.nmol, st.Enew, st.Eold, st.dE, st.Einit, st.nupd, st.conv, st.its, st.err,
                                               st.pdiff, o.accel, o.cflag, o.first_check, o.eps, o.tol);
    BK(cudaGetLastError(), UNOMOL_ECUDA);
    return UNOMOL_OK;
}

thread_local std::string g_bscf_err;

int batch_scf(BState& st, UnomolBatch* batch, const UnomolScfInput* in, int nmol, const UnomolScfOptions* opt, int graph,
              UnomolBatchScfResult* res, double* P_out, int* graph_used) {
    auto fail = [&](int rc) { return rc; };
    double *dP = nullptr, *dG = nullptr;
    const long long* poff = nullptr;
    int64_t ptot = 0;
    if (unomol_gpu_batch_buffers(batch, &dP, &dG, &poff, &ptot)) {
        st.err_msg = unomol_gpu_batch_last_error(batch);
        return fail(UNOMOL_EINVAL);
    }
    if (opt->guess != UNOMOL_GUESS_CORE && (opt->guess != UNOMOL_GUESS_GIVEN || !P_out)) {
        st.err_msg = "batched SCF: the guess is the core Hamiltonian or the densities passed in P_io";
        return UNOMOL_EINVAL;
    }
    if (unomol_gpu_batch_size(batch) != nmol) {
        st.err_msg = "batched SCF: " + std::to_string(nmol) + " inputs for a batch of " +
                     std::to_string(unomol_gpu_batch_size(batch)) + " molecules";
        return UNOMOL_EINVAL;
    }
    st.nmol = nmol;
    st.maxv = std::min(MAXV, std::max(2, opt->diis_size > 1 ? opt->diis_size : MAXV));
    // groups by (nbf, nocc)
    std::map<std::pair<int, int>, std::vector<int>> groups;
    for (int m = 0; m < nmol; ++m) {
        if (in[m].nelec % 2 != 0 || in[m].norb <= 0 || !in[m].S || !in[m].H) {
            st.err_msg = "batched SCF: molecule " + std::to_string(m) + " is not a closed-shell RHF input";
            return fail(UNOMOL_EINVAL);
        }
        if ((m + 1 < nmol ? poff[m + 1] : ptot) - poff[m] != (long long)in[m].norb * (in[m].norb + 1) / 2) {
            st.err_msg = "batched SCF: molecule " + std::to_string(m) + " does not match the batch's basis";
            return fail(UNOMOL_EINVAL);
        }
        groups[{in[m].norb, in[m].nelec / 2}].push_back(m);
    }
    for (auto& kv : groups) {
        st.gstart.push_back((int)st.mols.size());
        st.gn.push_back(kv.first.first);
        st.gocc.push_back(kv.first.second);
        for (int m : kv.second) {
            MolDev d{};
            d.n = kv.first.first, d.nocc = kv.first.second, d.bidx = m, d.o2 = st.tot2, d.o1 = st.tot1, d.po = poff[m];
            st.tot2 += (long long)d.n * d.n;
            st.tot1 += d.n;
            st.mols.push_back(d);
        }
    }
    const size_t b2 = st.tot2 * sizeof(double);
    BK(cudaMalloc(&st.d_mols, nmol * sizeof(MolDev)), UNOMOL_ENOMEM);
    for (double** p : {&st.S, &st.X, &st.H, &st.F, &st.Fo, &st.T1, &st.T2, &st.Pf, &st.Ecur}) BK(cudaMalloc(p, b2), UNOMOL_ENOMEM);
    BK(cudaMalloc(&st.W, st.tot1 * sizeof(double)), UNOMOL_ENOMEM);
    BK(cudaMalloc(&st.Hpk, ptot * sizeof(double)), UNOMOL_ENOMEM);
    BK(cudaMalloc(&st.Fh, b2 * st.maxv), UNOMOL_ENOMEM);
    BK(cudaMalloc(&st.Eh, b2 * st.maxv), UNOMOL_ENOMEM);
    BK(cudaMalloc(&st.B, sizeof(double) * nmol * st.maxv * st.maxv), UNOMOL_ENOMEM);
    BK(cudaMalloc(&st.coef, sizeof(double) * nmol * st.maxv), UNOMOL_ENOMEM);
    for (double** p : {&st.Enew, &st.Eold, &st.err, &st.dE, &st.pdiff, &st.Einit}) BK(cudaMalloc(p, sizeof(double) * nmol), UNOMOL_ENOMEM);
    BK(cudaMalloc(&st.Pold, sizeof(double) * ptot), UNOMOL_ENOMEM);
    // pseudo-diagonalisation (DIIS loop only; the damped loop keeps the reference's eigen-solve)
    const bool pseudo = opt->density == UNOMOL_DENSITY_PSEUDO && opt->accel == UNOMOL_SCF_DIIS;
    if (pseudo) {
        BK(cudaMalloc(&st.Wp, b2), UNOMOL_ENOMEM);
        BK(cudaMalloc(&st.pbad, sizeof(int) * nmol), UNOMOL_ENOMEM);
    }
    st.ptot = ptot;
    if (opt->incremental) {
        BK(cudaMalloc(&st.Pprev, sizeof(double) * ptot), UNOMOL_ENOMEM);
        BK(cudaMalloc(&st.Gacc, sizeof(double) * ptot), UNOMOL_ENOMEM);
        BK(cudaMalloc(&st.step, sizeof(int)), UNOMOL_ENOMEM);
        BK(cudaMemset(st.step, 0, sizeof(int)), UNOMOL_ECUDA);
    }
    for (cudaEvent_t& e : st.eb) BK(cudaEventCreate(&e), UNOMOL_ECUDA);
    BK(cudaMemset(st.dE, 0, sizeof(double) * nmol), UNOMOL_ECUDA);
    BK(cudaMemset(st.pdiff, 0, sizeof(double) * nmol), UNOMOL_ECUDA);
    for (int** p : {&st.nupd, &st.conv, &st.its, &st.info, &st.bad}) BK(cudaMalloc(p, sizeof(int) * nmol), UNOMOL_ENOMEM);
    for (int** p : {&st.nupd, &st.conv, &st.its, &st.info, &st.bad}) BK(cudaMemset(*p, 0, sizeof(int) * nmol), UNOMOL_ECUDA);
    BK(cudaMemset(st.Eold, 0, sizeof(double) * nmol), UNOMOL_ECUDA);
    BK(cudaMemset(st.B, 0, sizeof(double) * nmol * st.maxv * st.maxv), UNOMOL_ECUDA);
    BK(cudaMemcpy(st.d_mols, st.mols.data(), nmol * sizeof(MolDev), cudaMemcpyHostToDevice), UNOMOL_ECUDA);
    // S, H: host packed -> batch-order packed scratch -> full, group order
    {
        std::vector<double> pk((size_t)ptot);
        auto len = [&](int m) { return (size_t)((long long)in[m].norb * (in[m].norb + 1) / 2); };
        for (int m = 0; m < nmol; ++m) std::memcpy(pk.data() + poff[m], in[m].S, sizeof(double) * len(m));
        BK(cudaMemcpy(st.Hpk, pk.data(), ptot * sizeof(double), cudaMemcpyHostToDevice), UNOMOL_ECUDA);
        k_unpack<<<nmol, 256>>>(st.d_mols, st.Hpk, st.S);
        for (int m = 0; m < nmol; ++m) std::memcpy(pk.data() + poff[m], in[m].H, sizeof(double) * len(m));
        BK(cudaMemcpy(st.Hpk, pk.data(), ptot * sizeof(double), cudaMemcpyHostToDevice), UNOMOL_ECUDA);
        k_unpack<<<nmol, 256>>>(st.d_mols, st.Hpk, st.H);
        BK(cudaDeviceSynchronize(), UNOMOL_ECUDA);
    }
    cudaStream_t s = nullptr;
    BK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), UNOMOL_ECUDA);
    struct SG {
        cudaStream_t s;
        ~SG() { cudaStreamSynchronize(s), cudaStreamDestroy(s); }
    } sg{s};
    BK(cublasCreate(&st.cb), UNOMOL_ECUDA);
    BK(cublasSetStream(st.cb, s), UNOMOL_ECUDA);
    BK(cusolverDnCreate(&st.cs), UNOMOL_ECUDA);
    BK(cusolverDnSetStream(st.cs, s), UNOMOL_ECUDA);
    BK(cusolverDnCreateParams(&st.prm), UNOMOL_ECUDA);
    BK(cudaMalloc(&st.cublas_ws, 32u << 20), UNOMOL_ENOMEM);  // explicit workspace: nothing allocated in capture
    BK(cublasSetWorkspace(st.cb, st.cublas_ws, 32u << 20), UNOMOL_ECUDA);
    // eigen-solver workspace: the largest group (batched solver, or per-matrix syevd where the batched
    // solver declines the size)
    st.loop_group.assign(st.gn.size(), 0);
    for (size_t g = 0; g < st.gn.size(); ++g) {
        const int first = st.gstart[g], cnt = (g + 1 < st.gn.size() ? st.gstart[g + 1] : nmol) - first;
        size_t dsz = 0, hsz = 0;
        if (cusolverDnXsyevBatched_bufferSize(st.cs, st.prm, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, st.gn[g],
                                              CUDA_R_64F, st.Fo + st.mols[first].o2, st.gn[g], CUDA_R_64F,
                                              st.W + st.mols[first].o1, CUDA_R_64F, &dsz, &hsz, cnt) != CUSOLVER_STATUS_SUCCESS) {
            st.loop_group[g] = 1;
            int lw = 0;
            BK(cusolverDnDsyevd_bufferSize(st.cs, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, st.gn[g],
                                           st.Fo + st.mols[first].o2, st.gn[g], st.W + st.mols[first].o1, &lw),
               UNOMOL_ECUDA);
            dsz = (size_t)lw * sizeof(double);
            hsz = 0;
        }
        st.dwork_size = std::max(st.dwork_size, dsz);
        st.hwork.resize(std::max(st.hwork.size(), hsz));
    }
    st.loop_groups = (int)std::count(st.loop_group.begin(), st.loop_group.end(), 1);
    BK(cudaMalloc(&st.dwork, std::max<size_t>(st.dwork_size, 16)), UNOMOL_ENOMEM);
    // pointer arrays of the products
    int rc = 0;
    if ((rc = set_ptrs(st, 0, st.F, st.Pf, st.T1)) || (rc = set_ptrs(st, 1, st.T1, st.S, st.T2)) ||
        (rc = set_ptrs(st, 2, st.T1, st.X, st.T2)) || (rc = set_ptrs(st, 3, st.X, st.T2, st.Ecur)) ||
        (rc = set_ptrs(st, 4, st.F, st.X, st.T1)) || (rc = set_ptrs(st, 5, st.X, st.T1, st.Fo)) ||
        (rc = set_ptrs(st, 6, st.X, st.Fo, st.T2)) || (rc = set_ptrs(st, 7, st.T2, st.T2, st.Pf)))
        return fail(rc);
    if (pseudo && ((rc = set_ptrs(st, 8, st.Fo, st.Wp, st.T1)) || (rc = set_ptrs(st, 9, st.Wp, st.T1, st.T2)) ||
                   (rc = set_ptrs(st, 10, st.T1, st.T1, st.T2)) || (rc = set_ptrs(st, 11, st.Wp, st.T2, st.Fo)) ||
                   (rc = set_ptrs(st, 12, st.Fo, st.Fo, st.T1)) || (rc = set_ptrs(st, 13, st.Fo, st.T1, st.Wp)) ||
                   (rc = set_ptrs(st, 14, st.Wp, st.Wp, st.T1)) || (rc = set_ptrs(st, 15, st.Wp, st.T1, st.Fo))))
        return fail(rc);
    // X from S (canonical, RHF.hpp:214-233)
    BK(cudaMemcpyAsync(st.X, st.S, b2, cudaMemcpyDeviceToDevice, s), UNOMOL_ECUDA);
    if ((rc = eig(st, st.X))) return fail(rc);
    k_form_x<<<nmol, 256, 0, s>>>(st.d_mols, st.W, st.X, st.bad);
    if (opt->guess == UNOMOL_GUESS_GIVEN) {
        // the caller's densities (PMATRIX.DAT form, batch order; RHF.hpp:120-123, 318)
        BK(cudaMemcpyAsync(dP, P_out, sizeof(double) * ptot, cudaMemcpyHostToDevice, s), UNOMOL_ECUDA);
    } else {
        // core-Hamiltonian guess (RHF.hpp:205-211): F = H
        BK(cudaMemcpyAsync(st.F, st.H, b2, cudaMemcpyDeviceToDevice, s), UNOMOL_ECUDA);
        if ((rc = density_from_F(st, dP, s))) return fail(rc);
    }
    BK(cudaStreamSynchronize(s), UNOMOL_ECUDA);
    {
        std::vector<int> bad(nmol), info(nmol);
        BK(cudaMemcpy(bad.data(), st.bad, sizeof(int) * nmol, cudaMemcpyDeviceToHost), UNOMOL_ECUDA);
        BK(cudaMemcpy(info.data(), st.info, sizeof(int) * nmol, cudaMemcpyDeviceToHost), UNOMOL_ECUDA);
        for (int m = 0; m < nmol; ++m) {
            if (bad[m]) {
                st.err_msg = "molecule " + std::to_string(m) + ": non-positive eigenvalue in the overlap matrix";
                return fail(UNOMOL_ESCF);
            }
            if (info[m]) {
                st.err_msg = "molecule " + std::to_string(m) + ": eigen-solver failed";
                return fail(UNOMOL_ESCF);
            }
        }
    }
    const int maxits = opt->maxits > 0 ? opt->maxits : 300;
    const BOpts o{opt->accel == UNOMOL_SCF_DIIS ? 2 : 0, opt->conv_type, opt->loop == UNOMOL_SCF_LOOP_DPM ? 2 : 3, opt->eps,
                  opt->diis_tol, opt->incremental ? 1 : 0, opt->rebuild_every > 0 ? opt->rebuild_every : 8};
    // the eigen-solve for the first PSEUDO_AFTER iterations, then pseudo-diagonalisation steps where every
    // active molecule passes the check, the eigen-solve tail where one does not
    constexpr int PSEUDO_AFTER = 2;
    const int nparts = pseudo ? 4 : 1;
    cudaGraphExec_t exec[4] = {nullptr, nullptr, nullptr, nullptr};
    struct ExecGuard {
        cudaGraphExec_t* e;
        ~ExecGuard() { for (int k = 0; k < 4; ++k) if (e[k]) cudaGraphExecDestroy(e[k]); }
    } eg{exec};
    int used_graph = 0;
    if (graph) {
        // capture one iteration (and its parts with pseudo-diagonalisation); a library call that cannot be
        // captured leaves plain launches
        used_graph = 1;
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < nparts && used_graph; ++k) {
            cudaGraph_t gr = nullptr;
            BK(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed), UNOMOL_ECUDA);
            rc = iteration(st, batch, dP, dG, o, s, k);
            e = cudaStreamEndCapture(s, &gr);
            if (rc || e != cudaSuccess || !gr || cudaGraphInstantiate(&exec[k], gr, 0) != cudaSuccess) used_graph = 0;
            if (gr) cudaGraphDestroy(gr);
            cudaGetLastError();
        }
        if (!used_graph) {
            for (int k = 0; k < 4; ++k)
                if (exec[k]) cudaGraphExecDestroy(exec[k]), exec[k] = nullptr;
            st.capture_error = st.err_msg.empty() ? std::string(cudaGetErrorString(e)) : st.err_msg;
            st.err_msg.clear();
            BK(cudaStreamSynchronize(s), UNOMOL_ECUDA);
        }
    }
    if (graph_used) *graph_used = used_graph;
    auto run = [&](int part) -> int {
        if (used_graph) BK(cudaGraphLaunch(exec[part], s), UNOMOL_ECUDA);
        else return iteration(st, batch, dP, dG, o, s, part);
        return UNOMOL_OK;
    };
    std::vector<int> conv(nmol), pbad(pseudo ? nmol : 0);
    for (int it = 0; it < maxits; ++it) {
        if (!pseudo || it < PSEUDO_AFTER) {
            if ((rc = run(ITER_FULL))) return fail(rc);
        } else {
            if ((rc = run(ITER_HEAD))) return fail(rc);
            BK(cudaMemcpyAsync(pbad.data(), st.pbad, sizeof(int) * nmol, cudaMemcpyDeviceToHost, s), UNOMOL_ECUDA);
            BK(cudaStreamSynchronize(s), UNOMOL_ECUDA);
            const bool refuse = std::any_of(pbad.begin(), pbad.end(), [](int b) { return b != 0; });
            if ((rc = run(refuse ? ITER_EIG : ITER_PSEUDO))) return fail(rc);
            if (refuse) ++st.pseudo_refused;
            else ++st.pseudo_steps;
        }
        BK(cudaMemcpyAsync(conv.data(), st.conv, sizeof(int) * nmol, cudaMemcpyDeviceToHost, s), UNOMOL_ECUDA);
        BK(cudaStreamSynchronize(s), UNOMOL_ECUDA);
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, st.eb[0], st.eb[1]) == cudaSuccess) st.fock_ms += ms;
        ++st.builds;
        if (std::all_of(conv.begin(), conv.end(), [](int c) { return c != 0; })) break;
    }
    std::vector<double> E(nmol), err(nmol), E1(nmol), pd(nmol), de(nmol);
    BK(cudaMemcpy(E1.data(), st.Einit, sizeof(double) * nmol, cudaMemcpyDeviceToHost), UNOMOL_ECUDA);
    BK(cudaMemcpy(pd.data(), st.pdiff, sizeof(double) * nmol, cudaMemcpyDeviceToHost), UNOMOL_ECUDA);
    BK(cudaMemcpy(de.data(), st.dE, sizeof(double) * nmol, cudaMemcpyDeviceToHost), UNOMOL_ECUDA);
    std::vector<int> its(nmol), info(nmol);
    BK(cudaMemcpy(E.data(), st.Eold, sizeof(double) * nmol, cudaMemcpyDeviceToHost), UNOMOL_ECUDA);
    BK(cudaMemcpy(err.data(), st.err, sizeof(double) * nmol, cudaMemcpyDeviceToHost), UNOMOL_ECUDA);
    BK(cudaMemcpy(its.data(), st.its, sizeof(int) * nmol, cudaMemcpyDeviceToHost), UNOMOL_ECUDA);
    BK(cudaMemcpy(info.data(), st.info, sizeof(int) * nmol, cudaMemcpyDeviceToHost), UNOMOL_ECUDA);
    for (int m = 0; m < nmol; ++m) {
        if (info[m]) {
            st.err_msg = "batched SCF: the eigen-solver failed on a matrix";
            return fail(UNOMOL_ESCF);
        }
    }
    for (int m = 0; m < nmol; ++m) {
        res[m].energy = E[m] + in[m].nucrep;
        res[m].e_electronic = E[m];
        res[m].iterations = its[m];
        res[m].converged = conv[m];
        res[m].diis_error = err[m];
        res[m].init_energy = E1[m] + in[m].nucrep;
        res[m].ediff = de[m];
        res[m].pdiff = pd[m];
    }
    if (P_out) BK(cudaMemcpy(P_out, dP, sizeof(double) * ptot, cudaMemcpyDeviceToHost), UNOMOL_ECUDA);
    return UNOMOL_OK;
}

}  // namespace

thread_local double g_bscf_fock_ms = 0.0;
thread_local int g_bscf_builds = 0;
thread_local int g_bscf_pseudo[2] = {0, 0};

extern "C" int unomol_gpu_batch_scf(UnomolBatch* batch, const UnomolScfInput* in, int nmol, const UnomolScfOptions* opt,
                                    int graph, UnomolBatchScfResult* res, double* P_out, double* seconds, int* graph_used) {
    if (!batch || !in || !opt || !res || nmol <= 0) return UNOMOL_EINVAL;
    const auto t0 = std::chrono::steady_clock::now();
    int rc;
    std::string capture_error;
    {
        BState st;
        rc = batch_scf(st, batch, in, nmol, opt, graph, res, P_out, graph_used);
        g_bscf_err = rc ? st.err_msg : st.capture_error;
        g_bscf_fock_ms = st.fock_ms;
        g_bscf_builds = st.builds;
        g_bscf_pseudo[0] = st.pseudo_steps;
        g_bscf_pseudo[1] = st.pseudo_refused;
    }
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

extern "C" const char* unomol_gpu_batch_scf_last_error(void) { return g_bscf_err.c_str(); }

extern "C" int unomol_gpu_batch_scf_last_builds(double* fock_ms, int* builds) {
    if (!fock_ms || !builds) return UNOMOL_EINVAL;
    *fock_ms = g_bscf_fock_ms;
    *builds = g_bscf_builds;
    return UNOMOL_OK;
}

extern "C" int unomol_gpu_batch_scf_last_pseudo(int* steps, int* refused) {
    if (!steps || !refused) return UNOMOL_EINVAL;
    *steps = g_bscf_pseudo[0];
    *refused = g_bscf_pseudo[1];
    return UNOMOL_OK;
}
