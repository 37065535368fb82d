// Device-side set-up of the direct Fock build: the shell-pair enumeration, primitive-pair data and
// sorting of TwoElectronInts::calculate's quartet loops (TwoElectronInts.cpp:511-697, with the
// primitive loops of :439-460), rebuilt as data-parallel passes: one thread per canonical shell pair
// builds its records, CUB radix sorts order them into blocks and, after the Schwarz diagonal, by
// descending bound inside every block; one CTA per block pair binary-searches the Schwarz staircase of
// its bra rows and a device scan turns the row counts into the prefix sums that the Fock kernels decode.
#include <cub/cub.cuh>

#include "setup.h"

namespace ugb {
namespace {

// canonical pair id c = i(i+1)/2 + j (i >= j) -> (i, j)
__device__ __forceinline__ void canon_ij(int c, int& i, int& j) {
    long long r = (long long)((sqrt(8.0 * (double)c + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > c) --r;
    while ((r + 1) * (r + 2) / 2 <= c) ++r;
    i = (int)r;
    j = (int)(c - r * (r + 1) / 2);
}

__global__ void k_pair_keys(const ShellsDev sh, int npairs, unsigned* __restrict__ key, int* __restrict__ nprim,
                            int* __restrict__ iota) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= npairs) return;
    int i, j;
    canon_ij(c, i, j);
    const int li = sh.sl[i], lj = sh.sl[j];
    const int la = li > lj ? li : lj, lb = li > lj ? lj : li;
    const int n = i == j ? sh.snp[i] * (sh.snp[i] + 1) / 2 : sh.snp[i] * sh.snp[j];
    key[c] = ((unsigned)pair_class(la, lb) << 17) | ((unsigned)(i >= sh.start_shell) << 16) | (unsigned)n;
    nprim[c] = n;
    iota[c] = c;
}

// One canonical shell pair (ish >= jsh) after the L swap (a = larger L, TwoElectronInts.cpp:563-579) and
// its primitive pairs in the loop order of TwoElectronInts.cpp:439-460: a same-shell pair keeps j <= i
// with the factor 2 for j < i.  Products and sums are rounded one at a time (no contraction into FMA),
// in the order the expressions are written.
__global__ void k_build_pairs(const ShellsDev sh, int npairs, const int* __restrict__ poff, ShellPair* __restrict__ out,
                              PrimPair* __restrict__ prims, PrimPair32* __restrict__ prims32) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= npairs) return;
    int ish, jsh;
    canon_ij(c, ish, jsh);
    int a = ish, b = jsh;
    if (sh.sl[a] < sh.sl[b]) {
        a = jsh;
        b = ish;
    }
    ShellPair sp{};
    sp.ish = ish;
    sp.jsh = jsh;
    sp.maxsh = ish;
    sp.prim_stride = 1;  // canonical layout until the pairs are interleaved by block
    sp.same = ish == jsh;
    sp.la = sh.sl[a];
    sp.lb = sh.sl[b];
    sp.a_off = sh.soff[a];
    sp.b_off = sh.soff[b];
    const double* A = sh.centers + 3 * sh.scen[a];
    const double* B = sh.centers + 3 * sh.scen[b];
    for (int k = 0; k < 3; ++k) {
        sp.AB[k] = __dsub_rn(A[k], B[k]);
        sp.ABf[k] = (float)sp.AB[k];
    }
    const double ab2 = __dadd_rn(__dadd_rn(__dmul_rn(sp.AB[0], sp.AB[0]), __dmul_rn(sp.AB[1], sp.AB[1])),
                                 __dmul_rn(sp.AB[2], sp.AB[2]));
    const int p0 = poff[c];
    sp.prim_begin = p0;
    const int na = sh.snp[a], nb = sh.snp[b];
    int m = p0;
    for (int i = 0; i < na; ++i) {
        const double ai = sh.alpha[sh.sprim[a] + i], ci = sh.coef[sh.sprim[a] + i];
        const int jend = sp.same ? i + 1 : nb;
        for (int j = 0; j < jend; ++j, ++m) {
            const double bj = sh.alpha[sh.sprim[b] + j], cj = sh.coef[sh.sprim[b] + j];
            const double f = (sp.same && i != j) ? 2.0 : 1.0;
            PrimPair pp;
            pp.p = __dadd_rn(ai, bj);
            pp.rp = 1.0 / pp.p;
            for (int k = 0; k < 3; ++k) {
                pp.P[k] = __dmul_rn(__dadd_rn(__dmul_rn(ai, A[k]), __dmul_rn(bj, B[k])), pp.rp);
                pp.PA[k] = __dsub_rn(pp.P[k], A[k]);
            }
            pp.E = __dmul_rn(exp(__dmul_rn(__dmul_rn(__dmul_rn(-ai, bj), ab2), pp.rp)), pp.rp);
            pp.cc = __dmul_rn(__dmul_rn(ci, cj), f);
            pp.Ecc = SQRT_SRTERM * pp.E * pp.cc;
            pp.pf = (float)pp.p;
            pp.Ef = (float)pp.E;
            prims[m] = pp;
            PrimPair32 q;
            q.p = (float)pp.p;
            q.rp = (float)pp.rp;
            for (int k = 0; k < 3; ++k) {
                q.P[k] = (float)pp.P[k];
                q.PA[k] = (float)pp.PA[k];
            }
            q.E = (float)pp.E;
            q.cc = (float)pp.cc;
            q.Ecc = (float)pp.Ecc;
            q.pad_ = 0.f;
            prims32[m] = q;
        }
    }
    sp.nprim = m - p0;
    sp.q = 0.0;
    sp.qf = 0.f;
    out[c] = sp;
}

__global__ void k_gather_pairs(const ShellPair* __restrict__ src, const int* __restrict__ perm, const double* __restrict__ q,
                               int n, ShellPair* __restrict__ dst) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    ShellPair sp = src[perm[t]];
    if (q) {
        sp.q = q[t];
        sp.qf = (float)sp.q;
    }
    dst[t] = sp;
}

// One CTA per block pair: for every bra pair i the number of ket pairs j (q descending within the block)
// with q_i q_j >= cut, capped at i + 1 on a triangle (TwoElectronInts.cpp:517-541 with the Schwarz test).
__global__ void k_staircase(const BlockPair* __restrict__ bps, const ShellPair* __restrict__ pairs, double cut,
                            long long* __restrict__ x) {
    const BlockPair bp = bps[blockIdx.x];
    if (threadIdx.x == 0) x[bp.prefix_off] = 0;
    const ShellPair* kp = pairs + bp.ket_begin;
    for (int i = threadIdx.x; i < bp.bra_count; i += blockDim.x) {
        const double qi = pairs[bp.bra_begin + i].q;
        int lo = 0, hi = bp.ket_count;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (qi * kp[mid].q >= cut) lo = mid + 1;
            else hi = mid;
        }
        const int full = bp.triangle ? i + 1 : bp.ket_count;
        x[bp.prefix_off + 1 + i] = lo < full ? lo : full;
    }
}

__global__ void k_prefix_fix(const BlockPair* __restrict__ bps, const long long* __restrict__ S, long long* __restrict__ prefix,
                             long long* __restrict__ totals) {
    const BlockPair bp = bps[blockIdx.x];
    const long long base = S[bp.prefix_off];
    for (int i = threadIdx.x; i <= bp.bra_count; i += blockDim.x) prefix[bp.prefix_off + i] = S[bp.prefix_off + i] - base;
    if (threadIdx.x == 0) totals[blockIdx.x] = S[bp.prefix_off + bp.bra_count] - base;
}

__global__ void k_row_bp(const BlockPair* __restrict__ bps, int* __restrict__ row_bp) {
    const BlockPair bp = bps[blockIdx.x];
    for (int i = threadIdx.x; i < bp.bra_count; i += blockDim.x) row_bp[bp.prefix_off + i] = (int)blockIdx.x;
}

// Final layout of the primitive pairs: block b (pairs bbegin[b] .. + bcount[b], all with the same
// primitive-pair count) owns records bprim[b] .. + bcount[b] * nprim, and primitive ik of its j-th pair
// sits at bprim[b] + ik * bcount[b] + j, so that the lanes of a warp, which hold consecutive pairs of a
// block, read adjacent records.  One thread per pair; src is the canonical layout.
__global__ void k_interleave_prims(ShellPair* __restrict__ pairs, int n, const int* __restrict__ bbegin,
                                   const int* __restrict__ bcount, const long long* __restrict__ bprim, int nb,
                                   const PrimPair* __restrict__ src, const PrimPair32* __restrict__ src32,
                                   PrimPair* __restrict__ dst, PrimPair32* __restrict__ dst32) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int lo = 0, hi = nb - 1;  // the block: last with bbegin <= k
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (bbegin[mid] <= k) lo = mid; else hi = mid - 1;
    }
    const int j = k - bbegin[lo], cnt = bcount[lo];
    ShellPair sp = pairs[k];
    const long long first = bprim[lo] + j;
    for (int ik = 0; ik < sp.nprim; ++ik) {
        dst[first + (long long)ik * cnt] = src[sp.prim_begin + ik];
        dst32[first + (long long)ik * cnt] = src32[sp.prim_begin + ik];
    }
    sp.prim_begin = (int)first;
    sp.prim_stride = cnt;
    pairs[k] = sp;
}

__global__ void k_offset_pairs(ShellPair* __restrict__ pairs, int n, int prim0, int mol) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    pairs[t].prim_begin += prim0;
    pairs[t].pad = mol;
}

unsigned blocks_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

cudaError_t setup_pair_keys(const ShellsDev& sh, int npairs, unsigned* key, int* nprim, int* iota, cudaStream_t s) {
    if (npairs <= 0) return cudaSuccess;
    k_pair_keys<<<blocks_for(npairs, 256), 256, 0, s>>>(sh, npairs, key, nprim, iota);
    return cudaGetLastError();
}

cudaError_t setup_build_pairs(const ShellsDev& sh, int npairs, const int* poff, ShellPair* pairs, PrimPair* prims,
                              PrimPair32* prims32, cudaStream_t s) {
    if (npairs <= 0) return cudaSuccess;
    k_build_pairs<<<blocks_for(npairs, 128), 128, 0, s>>>(sh, npairs, poff, pairs, prims, prims32);
    return cudaGetLastError();
}

cudaError_t setup_gather_pairs(const ShellPair* src, const int* perm, const double* q, int n, ShellPair* dst, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_gather_pairs<<<blocks_for(n, 256), 256, 0, s>>>(src, perm, q, n, dst);
    return cudaGetLastError();
}

cudaError_t setup_staircase(const BlockPair* bps, int nbp, const ShellPair* pairs, double cut, long long* x, cudaStream_t s) {
    if (nbp <= 0) return cudaSuccess;
    k_staircase<<<(unsigned)nbp, 128, 0, s>>>(bps, pairs, cut, x);
    return cudaGetLastError();
}

cudaError_t setup_prefix_fix(const BlockPair* bps, int nbp, const long long* S, long long* prefix, long long* totals,
                             cudaStream_t s) {
    if (nbp <= 0) return cudaSuccess;
    k_prefix_fix<<<(unsigned)nbp, 128, 0, s>>>(bps, S, prefix, totals);
    return cudaGetLastError();
}

cudaError_t setup_row_bp(const BlockPair* bps, int nbp, int* row_bp, cudaStream_t s) {
    if (nbp <= 0) return cudaSuccess;
    k_row_bp<<<(unsigned)nbp, 128, 0, s>>>(bps, row_bp);
    return cudaGetLastError();
}

cudaError_t setup_interleave_prims(ShellPair* pairs, int n, const int* bbegin, const int* bcount, const long long* bprim,
                                   int nb, const PrimPair* src, const PrimPair32* src32, PrimPair* dst, PrimPair32* dst32,
                                   cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_interleave_prims<<<blocks_for(n, 128), 128, 0, s>>>(pairs, n, bbegin, bcount, bprim, nb, src, src32, dst, dst32);
    return cudaGetLastError();
}

cudaError_t setup_offset_pairs(ShellPair* pairs, int n, int prim0, int mol, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_offset_pairs<<<blocks_for(n, 256), 256, 0, s>>>(pairs, n, prim0, mol);
    return cudaGetLastError();
}

cudaError_t setup_exclusive_sum(void* tmp, size_t& tmp_bytes, const int* in, int* out, int n, cudaStream_t s) {
    return cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, in, out, n, s);
}

cudaError_t setup_inclusive_sum(void* tmp, size_t& tmp_bytes, const long long* in, long long* out, int n, cudaStream_t s) {
    return cub::DeviceScan::InclusiveSum(tmp, tmp_bytes, in, out, n, s);
}

cudaError_t setup_sort_keys(void* tmp, size_t& tmp_bytes, const unsigned* k_in, unsigned* k_out, const int* v_in, int* v_out,
                            int n, cudaStream_t s) {
    return cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k_in, k_out, v_in, v_out, n, 0, PAIR_KEY_BITS, s);
}

cudaError_t setup_run_length(void* tmp, size_t& tmp_bytes, const unsigned* k_in, unsigned* uniq, int* counts, int* nruns,
                             int n, cudaStream_t s) {
    return cub::DeviceRunLengthEncode::Encode(tmp, tmp_bytes, k_in, uniq, counts, nruns, n, s);
}

cudaError_t setup_sort_desc_segments(void* tmp, size_t& tmp_bytes, const double* k_in, double* k_out, const int* v_in,
                                     int* v_out, int n, int nseg, const int* seg_begin, const int* seg_end, cudaStream_t s) {
    return cub::DeviceSegmentedRadixSort::SortPairsDescending(tmp, tmp_bytes, k_in, k_out, v_in, v_out, n, nseg, seg_begin,
                                                              seg_end, 0, (int)sizeof(double) * 8, s);
}

}  // namespace ugb
