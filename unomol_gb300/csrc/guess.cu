// Learned initial density: a per-atom-pair MLP (mlp.h, tensor-core GEMMs) predicts the blocks of the
// RHF density matrix P (the half density C_occ C_occ^T of PMATRIX.DAT, RHF.hpp:120-123,172-174) from
// the two elements and their distance; the SCF purifies and trace-checks it (scf.cu).  There is no
// reference counterpart: the reference starts from the core Hamiltonian (RHF.hpp:205-211) or reads
// PMATRIX.DAT.
//
// Rotation covariance.  The network sees only invariants (element one-hots, radial basis functions of
// the distance r_ij); its outputs are Slater-Koster-like coefficients in the bond frame of the ordered
// pair (i, j), e = (R_j - R_i) / r_ij, for shells of s and p type:
//   off-diagonal block P_ij:  s-s: t;  s-p_k: t e_k;  p_k-s: t e_k;  p_k-p_l: t_sigma e_k e_l + t_pi (d_kl - e_k e_l)
//   on-site block P_ii (contribution of neighbour j): the same forms over the shell pairs a <= b of atom i
//   self row (i, i), r = 0: isotropic s-s and p-p (d_kl) terms only.
// P_ij = (B_ij + B_ji^T) / 2 and P_ii = B_self(i) + sum_j B_onsite(i; j), every output scaled by the
// smooth cutoff f_c(r) = (cos(pi r / r_cut) + 1) / 2; pairs with r >= r_cut are left out.  The map
// outputs -> P is linear, so the loss gradient is its exact transpose (k_assemble_grad).
//
// Loss of a set of molecules: mean over molecules of sum_{mu nu} (P_pred - P_target)^2 over the full
// symmetric matrix.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/unomol_gb300.h"
#include "mlp.h"

namespace {

using ugb::Mlp;

enum : unsigned char { T_OFF = 0, T_MIRROR = 1, T_DIAG = 2 };

// one term of the linear map: P[target] += w * f_c * theta_p * (c0 + c1 * e_a * e_b), e_3 = 1
struct GTerm {
    short r, c;           // function offsets within the atom blocks (row atom i, column atom j or i)
    signed char a, b;     // direction components (3: the constant 1)
    unsigned char kind;   // T_OFF: (bi+r, bj+c) and mirror, 1/2 each; T_MIRROR: (bi+r, bi+c) and mirror; T_DIAG: (bi+r, bi+r)
    unsigned char pad;
    float c0, c1;
};
static_assert(sizeof(GTerm) == 16, "GTerm layout");

struct GRow {
    int mol;              // molecule index (into the matrix offset / size tables)
    short type;           // self type = element index; pair type = E + ei * E + ej
    signed char ei, ej;   // element indices
    int bi, bj;           // first basis function of atoms i and j
    float e[3];           // unit vector i -> j (zero for self rows)
    float r;              // distance (bohr), 0 for self rows
};
static_assert(sizeof(GRow) == 32, "GRow layout");

struct Elem {
    int Z;
    std::vector<int> l, off;  // shells of one atom: angular momentum and first function (relative)
    int nbf;
};

unsigned nblk(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

__device__ __forceinline__ float comp(const float e0, const float e1, const float e2, int a) {
    return a == 0 ? e0 : a == 1 ? e1 : a == 2 ? e2 : 1.f;
}

__device__ __forceinline__ float cutoff_fc(float r, float r_cut) {
    return r <= 0.f ? 1.f : 0.5f * (cospif(r / r_cut) + 1.f);
}

// features: [onehot(ei) | onehot(ej) | exp(-((r - k delta) / delta)^2), k < n_rbf | zero padding]
__global__ void k_features(const GRow* __restrict__ rows, int n, int E, int n_rbf, float delta, int kpad,
                           __nv_bfloat16* __restrict__ X) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * kpad) return;
    const int r = (int)(t / kpad), c = (int)(t % kpad);
    const GRow& w = rows[r];
    float v = 0.f;
    if (c < E) {
        v = c == w.ei ? 1.f : 0.f;
    } else if (c < 2 * E) {
        v = c - E == w.ej ? 1.f : 0.f;
    } else if (c < 2 * E + n_rbf) {
        const float d = (w.r - (float)(c - 2 * E) * delta) / delta;
        v = expf(-d * d);
    }
    X[t] = __float2bfloat16(v);
}

// P += A(theta): one warp per row, lanes over outputs
__global__ void k_assemble(const GRow* __restrict__ rows, int n, const float* __restrict__ theta, int n_out,
                           const GTerm* __restrict__ terms, const int* __restrict__ tstart,
                           const long long* __restrict__ moff, const int* __restrict__ mnbf, long long off_base,
                           float r_cut, float* __restrict__ P) {
    const int row = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (row >= n) return;
    const GRow w = rows[row];
    const int nbf = mnbf[w.mol];
    float* Pm = P + (moff[w.mol] - off_base);
    const float fc = cutoff_fc(w.r, r_cut);
    const int* ts = tstart + (long long)w.type * (n_out + 1);
    for (int p = lane; p < n_out; p += 32) {
        const int t0 = ts[p], t1 = ts[p + 1];
        if (t0 == t1) continue;
        const float th = theta[(long long)row * n_out + p] * fc;
        for (int k = t0; k < t1; ++k) {
            const GTerm T = terms[k];
            const float v = th * (T.c0 + T.c1 * comp(w.e[0], w.e[1], w.e[2], T.a) * comp(w.e[0], w.e[1], w.e[2], T.b));
            if (T.kind == T_OFF) {
                const int rr = w.bi + T.r, cc = w.bj + T.c;
                atomicAdd(Pm + (long long)rr * nbf + cc, 0.5f * v);
                atomicAdd(Pm + (long long)cc * nbf + rr, 0.5f * v);
            } else {
                const int rr = w.bi + T.r, cc = w.bi + T.c;
                atomicAdd(Pm + (long long)rr * nbf + cc, v);
                if (T.kind == T_MIRROR) atomicAdd(Pm + (long long)cc * nbf + rr, v);
            }
        }
    }
}

// dy = scale * A^T(D): the exact transpose of k_assemble (deterministic gather)
__global__ void k_assemble_grad(const GRow* __restrict__ rows, int n, const float* __restrict__ D, int n_out,
                                const GTerm* __restrict__ terms, const int* __restrict__ tstart,
                                const long long* __restrict__ moff, const int* __restrict__ mnbf, long long off_base,
                                float r_cut, float scale, float* __restrict__ dy) {
    const int row = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (row >= n) return;
    const GRow w = rows[row];
    const int nbf = mnbf[w.mol];
    const float* Dm = D + (moff[w.mol] - off_base);
    const float fc = cutoff_fc(w.r, r_cut);
    const int* ts = tstart + (long long)w.type * (n_out + 1);
    for (int p = lane; p < n_out; p += 32) {
        const int t0 = ts[p], t1 = ts[p + 1];
        float acc = 0.f;
        for (int k = t0; k < t1; ++k) {
            const GTerm T = terms[k];
            const float coef = T.c0 + T.c1 * comp(w.e[0], w.e[1], w.e[2], T.a) * comp(w.e[0], w.e[1], w.e[2], T.b);
            float g;
            if (T.kind == T_OFF) {
                const int rr = w.bi + T.r, cc = w.bj + T.c;
                g = 0.5f * (Dm[(long long)rr * nbf + cc] + Dm[(long long)cc * nbf + rr]);
            } else {
                const int rr = w.bi + T.r, cc = w.bi + T.c;
                g = Dm[(long long)rr * nbf + cc];
                if (T.kind == T_MIRROR) g += Dm[(long long)cc * nbf + rr];
            }
            acc += coef * g;
        }
        dy[(long long)row * n_out + p] = scale * fc * acc;
    }
}

// D = pred - target (in place), loss += sum D^2
__global__ void k_diff_loss(float* __restrict__ pred, const float* __restrict__ tgt, long long n, double* __restrict__ loss) {
    double s = 0.0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const float d = pred[t] - tgt[t];
        pred[t] = d;
        s += (double)d * d;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += ws[i];
        atomicAdd(loss, t);
    }
}

// full fp32 [n x n] -> packed double (row i, columns j <= i)
__global__ void k_pack_f64(const float* __restrict__ full, int n, double* __restrict__ pk) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * n) return;
    const int i = (int)(t / n), j = (int)(t % n);
    if (j > i) return;
    pk[(long long)i * (i + 1) / 2 + j] = 0.5 * ((double)full[t] + (double)full[(long long)j * n + i]);
}

uint64_t mix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    bool reserve(size_t n) {
        if (n <= cap) return true;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return false;
        cap = n;
        return true;
    }
};

}  // namespace

struct UnomolGuess {
    UnomolGuessConfig cfg{};
    std::vector<Elem> elems;
    std::map<int, int> zmap;            // nuclear charge -> element index
    int E = 0, n_types = 0, n_in = 0, n_out = 0;
    std::vector<int> nparam;            // outputs used by each row type
    std::vector<GTerm> terms;
    std::vector<int> tstart;            // [n_types][n_out + 1]
    float delta = 1.f;
    Mlp mlp;
    cudaStream_t s = nullptr;
    // data set
    std::vector<GRow> rows;
    std::vector<float> targets;
    std::vector<long long> moff, mrow0;
    std::vector<int> mnbf, mnrows;
    bool dirty = true;
    DevBuf<GTerm> d_terms;
    DevBuf<int> d_tstart, d_mnbf;
    DevBuf<GRow> d_rows;
    DevBuf<float> d_tgt, d_pred, d_dy;
    DevBuf<long long> d_moff;
    DevBuf<double> d_loss;
    // one-molecule scratch of predict()
    DevBuf<GRow> p_rows;
    DevBuf<long long> p_moff;
    DevBuf<int> p_mnbf;
    DevBuf<double> p_pk;
    std::string err;
    ~UnomolGuess() {
        if (s) cudaStreamDestroy(s);
    }
};

namespace {

thread_local std::string g_guess_err;

#define GK(call)                                                                    \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            g->err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
            return e_ == cudaErrorMemoryAllocation ? UNOMOL_ENOMEM : UNOMOL_ECUDA;  \
        }                                                                           \
    } while (0)

// shells of every centre, checked against the element's shell list
int atom_blocks(UnomolGuess* g, const UnomolBasisDesc* b, const int* charges, std::vector<int>& first,
                std::vector<int>& elem, bool learn) {
    const int nc = b->ncen;
    std::vector<std::vector<int>> sh(nc);
    for (int s = 0; s < b->nshell; ++s) {
        const int c = b->shell_center[s];
        if (c < 0 || c >= nc) {
            g->err = "learned guess: shell centre out of range";
            return UNOMOL_EINVAL;
        }
        sh[c].push_back(s);
    }
    first.assign(nc, 0);
    elem.assign(nc, -1);
    for (int c = 0; c < nc; ++c) {
        if (sh[c].empty()) {
            g->err = "learned guess: a centre without shells";
            return UNOMOL_EINVAL;
        }
        Elem e;
        e.Z = charges[c];
        int f0 = b->shell_offset[sh[c][0]], nb = 0;
        for (int s : sh[c]) {
            const int l = b->shell_l[s];
            if (l > 1) {
                g->err = "learned guess: only s and p shells are supported";
                return UNOMOL_EINVAL;
            }
            if (b->shell_offset[s] != f0 + nb) {
                g->err = "learned guess: the functions of a centre must be contiguous";
                return UNOMOL_EINVAL;
            }
            e.l.push_back(l);
            e.off.push_back(nb);
            nb += (l + 1) * (l + 2) / 2;
        }
        e.nbf = nb;
        auto it = g->zmap.find(e.Z);
        if (it == g->zmap.end()) {
            if (!learn) {
                g->err = "learned guess: element " + std::to_string(e.Z) + " was not in the model's basis";
                return UNOMOL_EINVAL;
            }
            g->zmap[e.Z] = -1;
            g->elems.push_back(e);
        } else if (it->second < 0) {  // seen earlier in the example molecule
            for (const Elem& x : g->elems)
                if (x.Z == e.Z && x.l != e.l) {
                    g->err = "learned guess: element " + std::to_string(e.Z) + " has two shell lists";
                    return UNOMOL_EINVAL;
                }
        } else if (g->elems[it->second].l != e.l) {
            g->err = "learned guess: element " + std::to_string(e.Z) + " has a different shell list";
            return UNOMOL_EINVAL;
        }
        first[c] = f0;
    }
    if (learn) {
        std::sort(g->elems.begin(), g->elems.end(), [](const Elem& x, const Elem& y) { return x.Z < y.Z; });
        // one entry per element (a repeated element was appended only once through zmap)
        for (size_t i = 0; i < g->elems.size(); ++i) g->zmap[g->elems[i].Z] = (int)i;
    }
    for (int c = 0; c < nc; ++c) elem[c] = g->zmap[charges[c]];
    return UNOMOL_OK;
}

struct TermBuilder {
    std::vector<std::vector<GTerm>> per_param;
    int p = 0;
    void next() {
        per_param.emplace_back();
        p = (int)per_param.size() - 1;
    }
    void add(int r, int c, int a, int b, unsigned char kind, float c0, float c1) {
        GTerm t{};
        t.r = (short)r, t.c = (short)c, t.a = (signed char)a, t.b = (signed char)b, t.kind = kind, t.c0 = c0, t.c1 = c1;
        per_param[p].push_back(t);
    }
};

// self row (i, i): isotropic s-s and p-p terms over the shell pairs a <= b
void self_terms(const Elem& A, TermBuilder& tb) {
    const int ns = (int)A.l.size();
    for (int a = 0; a < ns; ++a)
        for (int b = a; b < ns; ++b) {
            const unsigned char kind = a == b ? T_DIAG : T_MIRROR;
            if (A.l[a] == 0 && A.l[b] == 0) {
                tb.next();
                tb.add(A.off[a], A.off[b], 3, 3, kind, 1.f, 0.f);
            } else if (A.l[a] == 1 && A.l[b] == 1) {
                tb.next();
                for (int k = 0; k < 3; ++k) tb.add(A.off[a] + k, A.off[b] + k, 3, 3, kind, 1.f, 0.f);
            }
        }
}

// ordered pair (i, j): off-diagonal block terms, then the on-site terms of atom i
void pair_terms(const Elem& A, const Elem& B, TermBuilder& tb) {
    for (size_t a = 0; a < A.l.size(); ++a)
        for (size_t b = 0; b < B.l.size(); ++b) {
            const int la = A.l[a], lb = B.l[b], oa = A.off[a], ob = B.off[b];
            if (la == 0 && lb == 0) {
                tb.next();
                tb.add(oa, ob, 3, 3, T_OFF, 1.f, 0.f);
            } else if (la == 0 && lb == 1) {
                tb.next();
                for (int k = 0; k < 3; ++k) tb.add(oa, ob + k, k, 3, T_OFF, 0.f, 1.f);
            } else if (la == 1 && lb == 0) {
                tb.next();
                for (int k = 0; k < 3; ++k) tb.add(oa + k, ob, k, 3, T_OFF, 0.f, 1.f);
            } else {
                tb.next();  // sigma
                for (int k = 0; k < 3; ++k)
                    for (int l = 0; l < 3; ++l) tb.add(oa + k, ob + l, k, l, T_OFF, 0.f, 1.f);
                tb.next();  // pi
                for (int k = 0; k < 3; ++k)
                    for (int l = 0; l < 3; ++l) tb.add(oa + k, ob + l, k, l, T_OFF, k == l ? 1.f : 0.f, -1.f);
            }
        }
    const int ns = (int)A.l.size();
    for (int a = 0; a < ns; ++a)
        for (int b = a; b < ns; ++b) {
            const int la = A.l[a], lb = A.l[b], oa = A.off[a], ob = A.off[b];
            if (la == 0 && lb == 0) {
                tb.next();
                tb.add(oa, ob, 3, 3, a == b ? T_DIAG : T_MIRROR, 1.f, 0.f);
            } else if (la != lb) {
                const int os = la == 0 ? oa : ob, op = la == 0 ? ob : oa;
                tb.next();
                for (int k = 0; k < 3; ++k) tb.add(os, op + k, k, 3, T_MIRROR, 0.f, 1.f);
            } else {
                for (int form = 0; form < 2; ++form) {  // sigma, pi
                    tb.next();
                    for (int k = 0; k < 3; ++k)
                        for (int l = 0; l < 3; ++l) {
                            if (a == b && l < k) continue;
                            const unsigned char kind = a == b && k == l ? T_DIAG : T_MIRROR;
                            if (form == 0) tb.add(oa + k, ob + l, k, l, kind, 0.f, 1.f);
                            else tb.add(oa + k, ob + l, k, l, kind, k == l ? 1.f : 0.f, -1.f);
                        }
                }
            }
        }
}

int build_rows(UnomolGuess* g, const UnomolBasisDesc* b, const int* charges, int mol, std::vector<GRow>& out) {
    std::vector<int> first, elem;
    int rc = atom_blocks(g, b, charges, first, elem, false);
    if (rc) return rc;
    const int nc = b->ncen;
    const double rcut = g->cfg.r_cut;
    for (int i = 0; i < nc; ++i) {
        GRow w{};
        w.mol = mol, w.type = (short)elem[i], w.ei = (signed char)elem[i], w.ej = (signed char)elem[i];
        w.bi = w.bj = first[i];
        out.push_back(w);
    }
    for (int i = 0; i < nc; ++i)
        for (int j = 0; j < nc; ++j) {
            if (i == j) continue;
            const double dx = b->centers[3 * j] - b->centers[3 * i], dy = b->centers[3 * j + 1] - b->centers[3 * i + 1],
                         dz = b->centers[3 * j + 2] - b->centers[3 * i + 2];
            const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
            if (r >= rcut || r <= 0.0) continue;
            GRow w{};
            w.mol = mol;
            w.type = (short)(g->E + elem[i] * g->E + elem[j]);
            w.ei = (signed char)elem[i], w.ej = (signed char)elem[j];
            w.bi = first[i], w.bj = first[j];
            w.e[0] = (float)(dx / r), w.e[1] = (float)(dy / r), w.e[2] = (float)(dz / r);
            w.r = (float)r;
            out.push_back(w);
        }
    return UNOMOL_OK;
}

int upload(UnomolGuess* g) {
    if (!g->dirty) return UNOMOL_OK;
    const size_t nm = g->mnbf.size();
    if (!g->d_rows.reserve(g->rows.size()) || !g->d_tgt.reserve(g->targets.size()) || !g->d_moff.reserve(nm) ||
        !g->d_mnbf.reserve(nm)) {
        g->err = "learned guess: device allocation failed";
        return UNOMOL_ENOMEM;
    }
    GK(cudaMemcpy(g->d_rows.p, g->rows.data(), g->rows.size() * sizeof(GRow), cudaMemcpyHostToDevice));
    GK(cudaMemcpy(g->d_tgt.p, g->targets.data(), g->targets.size() * sizeof(float), cudaMemcpyHostToDevice));
    GK(cudaMemcpy(g->d_moff.p, g->moff.data(), nm * sizeof(long long), cudaMemcpyHostToDevice));
    GK(cudaMemcpy(g->d_mnbf.p, g->mnbf.data(), nm * sizeof(int), cudaMemcpyHostToDevice));
    g->dirty = false;
    return UNOMOL_OK;
}

// forward + loss + gradient of the outputs for molecules [m0, m1); adds sum D^2 to d_loss, leaves the
// output gradient (scaled by grad_scale) in d_dy and the MLP activations of these rows in place
int batch_pass(UnomolGuess* g, int m0, int m1, float grad_scale) {
    const long long r0 = g->mrow0[m0], r1 = g->mrow0[m1 - 1] + g->mnrows[m1 - 1];
    const int nr = (int)(r1 - r0);
    const long long o0 = g->moff[m0], o1 = g->moff[m1 - 1] + (long long)g->mnbf[m1 - 1] * g->mnbf[m1 - 1];
    int rc = g->mlp.reserve(nr);
    if (rc) {
        g->err = g->mlp.err;
        return rc;
    }
    if (!g->d_pred.reserve((size_t)(o1 - o0)) || !g->d_dy.reserve((size_t)nr * g->n_out)) {
        g->err = "learned guess: device allocation failed";
        return UNOMOL_ENOMEM;
    }
    const GRow* rows = g->d_rows.p + r0;
    k_features<<<nblk((long long)nr * g->mlp.n_in_pad), 256, 0, g->s>>>(rows, nr, g->E, g->cfg.n_rbf, g->delta,
                                                                          g->mlp.n_in_pad, g->mlp.X);
    GK(cudaGetLastError());
    rc = g->mlp.forward_x(nr, g->s);
    if (rc) {
        g->err = g->mlp.err;
        return rc;
    }
    GK(cudaMemsetAsync(g->d_pred.p, 0, (size_t)(o1 - o0) * sizeof(float), g->s));
    const float rcut = (float)g->cfg.r_cut;
    k_assemble<<<nblk((long long)nr * 32), 256, 0, g->s>>>(rows, nr, g->mlp.Y, g->n_out, g->d_terms.p, g->d_tstart.p,
                                                            g->d_moff.p, g->d_mnbf.p, o0, rcut, g->d_pred.p);
    k_diff_loss<<<(unsigned)std::min<long long>(1024, nblk(o1 - o0)), 256, 0, g->s>>>(g->d_pred.p, g->d_tgt.p + o0, o1 - o0,
                                                                             g->d_loss.p);
    k_assemble_grad<<<nblk((long long)nr * 32), 256, 0, g->s>>>(rows, nr, g->d_pred.p, g->n_out, g->d_terms.p,
                                                                 g->d_tstart.p, g->d_moff.p, g->d_mnbf.p, o0, rcut,
                                                                 grad_scale, g->d_dy.p);
    GK(cudaGetLastError());
    return UNOMOL_OK;
}

int status_check(UnomolGuess* g) {
    int rc = g->mlp.check_status(g->s);
    if (rc) g->err = g->mlp.err;
    return rc;
}

}  // namespace

extern "C" {

int unomol_guess_create(const UnomolGuessConfig* cfg, const UnomolBasisDesc* basis, const int* charges,
                        UnomolGuess** out) {
    if (!cfg || !basis || !charges || !out) return UNOMOL_EINVAL;
    *out = nullptr;
    auto* g = new UnomolGuess();
    g->cfg = *cfg;
    if (g->cfg.hidden <= 0) g->cfg.hidden = 256;
    if (g->cfg.layers <= 0) g->cfg.layers = 3;
    if (g->cfg.n_rbf <= 1) g->cfg.n_rbf = 16;
    if (g->cfg.r_cut <= 0.0) g->cfg.r_cut = 15.0;
    g->delta = (float)(g->cfg.r_cut / (g->cfg.n_rbf - 1));
    std::vector<int> first, elem;
    int rc = atom_blocks(g, basis, charges, first, elem, true);
    if (rc) {
        g_guess_err = g->err;
        delete g;
        return rc;
    }
    g->E = (int)g->elems.size();
    g->n_types = g->E + g->E * g->E;
    std::vector<TermBuilder> tbs(g->n_types);
    for (int e = 0; e < g->E; ++e) self_terms(g->elems[e], tbs[e]);
    for (int i = 0; i < g->E; ++i)
        for (int j = 0; j < g->E; ++j) pair_terms(g->elems[i], g->elems[j], tbs[g->E + i * g->E + j]);
    int maxp = 1;
    for (auto& tb : tbs) maxp = std::max(maxp, (int)tb.per_param.size());
    g->n_out = (maxp + 15) / 16 * 16;
    g->n_in = 2 * g->E + g->cfg.n_rbf;
    g->tstart.assign((size_t)g->n_types * (g->n_out + 1), 0);
    g->nparam.assign(g->n_types, 0);
    for (int t = 0; t < g->n_types; ++t) {
        g->nparam[t] = (int)tbs[t].per_param.size();
        for (int p = 0; p < g->n_out; ++p) {
            g->tstart[(size_t)t * (g->n_out + 1) + p] = (int)g->terms.size();
            if (p < g->nparam[t]) g->terms.insert(g->terms.end(), tbs[t].per_param[p].begin(), tbs[t].per_param[p].end());
        }
        g->tstart[(size_t)t * (g->n_out + 1) + g->n_out] = (int)g->terms.size();
    }
    if (cudaStreamCreateWithFlags(&g->s, cudaStreamNonBlocking) != cudaSuccess) {
        g_guess_err = "learned guess: cannot create a stream";
        delete g;
        return UNOMOL_ECUDA;
    }
    rc = g->mlp.init(g->n_in, g->cfg.hidden, g->cfg.layers, g->n_out, g->cfg.seed);
    if (!rc && (!g->d_terms.reserve(g->terms.size()) || !g->d_tstart.reserve(g->tstart.size()) || !g->d_loss.reserve(1)))
        rc = UNOMOL_ENOMEM, g->mlp.err = "learned guess: device allocation failed";
    if (!rc && (cudaMemcpy(g->d_terms.p, g->terms.data(), g->terms.size() * sizeof(GTerm), cudaMemcpyHostToDevice) ||
                cudaMemcpy(g->d_tstart.p, g->tstart.data(), g->tstart.size() * sizeof(int), cudaMemcpyHostToDevice)))
        rc = UNOMOL_ECUDA, g->mlp.err = "learned guess: upload of the term tables failed";
    if (rc) {
        g_guess_err = g->mlp.err;
        delete g;
        return rc;
    }
    *out = g;
    return UNOMOL_OK;
}

int unomol_guess_info(const UnomolGuess* g, int* n_in, int* n_out, long long* n_params, int* n_elements) {
    if (!g) return UNOMOL_EINVAL;
    if (n_in) *n_in = g->n_in;
    if (n_out) *n_out = g->n_out;
    if (n_params) *n_params = g->mlp.np;
    if (n_elements) *n_elements = g->E;
    return UNOMOL_OK;
}

int unomol_guess_add_molecule(UnomolGuess* g, const UnomolBasisDesc* basis, const int* charges, const double* P) {
    if (!g || !basis || !charges || !P) return UNOMOL_EINVAL;
    const int mol = (int)g->mnbf.size();
    std::vector<GRow> rr;
    int rc = build_rows(g, basis, charges, mol, rr);
    if (rc) return rc;
    const int n = basis->norb;
    g->mrow0.push_back((long long)g->rows.size());
    g->mnrows.push_back((int)rr.size());
    g->rows.insert(g->rows.end(), rr.begin(), rr.end());
    g->moff.push_back((long long)g->targets.size());
    g->mnbf.push_back(n);
    const size_t base = g->targets.size();
    g->targets.resize(base + (size_t)n * n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j) {
            const float v = (float)P[(size_t)i * (i + 1) / 2 + j];
            g->targets[base + (size_t)i * n + j] = v;
            g->targets[base + (size_t)j * n + i] = v;
        }
    g->dirty = true;
    return UNOMOL_OK;
}

int unomol_guess_num_molecules(const UnomolGuess* g) { return g ? (int)g->mnbf.size() : -1; }

int unomol_guess_train(UnomolGuess* g, const UnomolGuessTrainOptions* opt, double* loss_history) {
    if (!g || !opt) return UNOMOL_EINVAL;
    const int nmol = (int)g->mnbf.size();
    if (opt->first < 0 || opt->count <= 0 || opt->first + opt->count > nmol || opt->epochs <= 0) {
        g->err = "learned guess: bad training range";
        return UNOMOL_EINVAL;
    }
    int rc = upload(g);
    if (rc) return rc;
    const int B = opt->batch_molecules > 0 ? opt->batch_molecules : 16;
    const int nb = (opt->count + B - 1) / B;
    const long long total = (long long)opt->epochs * nb;
    const float lr0 = opt->lr > 0.f ? opt->lr : 1e-3f, lr1 = opt->lr_final > 0.f ? opt->lr_final : lr0 * 0.01f;
    uint64_t st = opt->seed * 0x9E3779B97F4A7C15ull + 7;
    std::vector<int> order(nb);
    long long step = 0;
    for (int ep = 0; ep < opt->epochs; ++ep) {
        for (int i = 0; i < nb; ++i) order[i] = i;
        for (int i = nb - 1; i > 0; --i) std::swap(order[i], order[(int)(mix64(st) % (uint64_t)(i + 1))]);
        GK(cudaMemsetAsync(g->d_loss.p, 0, sizeof(double), g->s));
        for (int bi = 0; bi < nb; ++bi) {
            const int m0 = opt->first + order[bi] * B, m1 = std::min(opt->first + opt->count, m0 + B);
            rc = batch_pass(g, m0, m1, 2.f / (float)(m1 - m0));
            if (rc) return rc;
            rc = g->mlp.backward(g->d_dy.p, false, g->s);
            if (!rc) {
                const double f = (double)step / (double)std::max<long long>(1, total - 1);
                const float lr = (float)(lr1 + 0.5 * (lr0 - lr1) * (1.0 + std::cos(3.14159265358979323846 * f)));
                rc = g->mlp.adam(lr, 0.9f, 0.999f, 1e-8f, opt->weight_decay, g->s);
            }
            if (rc) {
                g->err = g->mlp.err;
                return rc;
            }
            ++step;
        }
        if (loss_history) {
            double l = 0.0;
            GK(cudaMemcpyAsync(&l, g->d_loss.p, sizeof(double), cudaMemcpyDeviceToHost, g->s));
            GK(cudaStreamSynchronize(g->s));
            loss_history[ep] = l / opt->count;
        }
    }
    GK(cudaStreamSynchronize(g->s));
    return status_check(g);
}

int unomol_guess_loss(UnomolGuess* g, int first, int count, int batch_molecules, double* loss, float* grads) {
    if (!g || !loss || first < 0 || count <= 0 || first + count > (int)g->mnbf.size()) return UNOMOL_EINVAL;
    int rc = upload(g);
    if (rc) return rc;
    const int B = batch_molecules > 0 ? batch_molecules : 16;
    GK(cudaMemsetAsync(g->d_loss.p, 0, sizeof(double), g->s));
    GK(cudaMemsetAsync(g->mlp.G, 0, g->mlp.np_pad * sizeof(float), g->s));
    for (int m0 = first; m0 < first + count; m0 += B) {
        const int m1 = std::min(first + count, m0 + B);
        rc = batch_pass(g, m0, m1, 2.f / (float)count);
        if (rc) return rc;
        if (grads) {
            rc = g->mlp.backward(g->d_dy.p, true, g->s);
            if (rc) {
                g->err = g->mlp.err;
                return rc;
            }
        }
    }
    double l = 0.0;
    GK(cudaMemcpyAsync(&l, g->d_loss.p, sizeof(double), cudaMemcpyDeviceToHost, g->s));
    GK(cudaStreamSynchronize(g->s));
    rc = status_check(g);
    if (rc) return rc;
    *loss = l / count;
    if (grads) {
        rc = g->mlp.get(g->mlp.G, grads);
        if (rc) g->err = "learned guess: gradient copy failed";
    }
    return rc;
}

int unomol_guess_predict(UnomolGuess* g, const UnomolBasisDesc* basis, const int* charges, double* P) {
    if (!g || !basis || !charges || !P) return UNOMOL_EINVAL;
    std::vector<GRow> rr;
    int rc = build_rows(g, basis, charges, 0, rr);
    if (rc) return rc;
    const int n = basis->norb, nr = (int)rr.size();
    const long long off0 = 0;
    const size_t no2 = (size_t)n * (n + 1) / 2;
    rc = g->mlp.reserve(nr);
    if (rc) {
        g->err = g->mlp.err;
        return rc;
    }
    if (!g->p_rows.reserve(rr.size()) || !g->p_moff.reserve(1) || !g->p_mnbf.reserve(1) ||
        !g->d_pred.reserve((size_t)n * n) || !g->p_pk.reserve(no2)) {
        g->err = "learned guess: device allocation failed";
        return UNOMOL_ENOMEM;
    }
    GK(cudaMemcpyAsync(g->p_rows.p, rr.data(), rr.size() * sizeof(GRow), cudaMemcpyHostToDevice, g->s));
    GK(cudaMemcpyAsync(g->p_moff.p, &off0, sizeof(long long), cudaMemcpyHostToDevice, g->s));
    GK(cudaMemcpyAsync(g->p_mnbf.p, &n, sizeof(int), cudaMemcpyHostToDevice, g->s));
    k_features<<<nblk((long long)nr * g->mlp.n_in_pad), 256, 0, g->s>>>(g->p_rows.p, nr, g->E, g->cfg.n_rbf, g->delta,
                                                                          g->mlp.n_in_pad, g->mlp.X);
    GK(cudaGetLastError());
    rc = g->mlp.forward_x(nr, g->s);
    if (rc) {
        g->err = g->mlp.err;
        return rc;
    }
    GK(cudaMemsetAsync(g->d_pred.p, 0, (size_t)n * n * sizeof(float), g->s));
    k_assemble<<<nblk((long long)nr * 32), 256, 0, g->s>>>(g->p_rows.p, nr, g->mlp.Y, g->n_out, g->d_terms.p,
                                                            g->d_tstart.p, g->p_moff.p, g->p_mnbf.p, 0,
                                                            (float)g->cfg.r_cut, g->d_pred.p);
    k_pack_f64<<<nblk((long long)n * n), 256, 0, g->s>>>(g->d_pred.p, n, g->p_pk.p);
    GK(cudaGetLastError());
    GK(cudaMemcpyAsync(P, g->p_pk.p, no2 * sizeof(double), cudaMemcpyDeviceToHost, g->s));
    GK(cudaStreamSynchronize(g->s));
    return status_check(g);
}

int unomol_guess_get_params(UnomolGuess* g, float* out) {
    if (!g || !out) return UNOMOL_EINVAL;
    return g->mlp.get(g->mlp.P, out);
}

int unomol_guess_set_params(UnomolGuess* g, const float* in) {
    if (!g || !in) return UNOMOL_EINVAL;
    int rc = g->mlp.set(in);
    if (rc) g->err = g->mlp.err;
    return rc;
}

void unomol_guess_destroy(UnomolGuess* g) { delete g; }

const char* unomol_guess_last_error(const UnomolGuess* g) { return g ? g->err.c_str() : g_guess_err.c_str(); }

}  // extern "C"
