// Device-side set-up of the direct Fock build (setup.cu): shell pairs and their primitive pairs built
// from the basis on the GPU, sorted on the GPU into blocks of equal (pair class, new/old for
// start_shell, primitive-pair count) and within a block by descending Schwarz bound, and the Schwarz
// staircase of every block pair (bra pair i keeps the first n_i ket pairs of the ket block).  The host
// keeps only the block boundaries and the block-pair list, both of a size set by the number of blocks.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

#include "eri_common.cuh"

namespace ugb {

// The basis on the device (shell arrays as in UnomolBasisDesc, primitive offsets per shell).
struct ShellsDev {
    int nshell = 0, start_shell = 0;
    const int *sl = nullptr, *snp = nullptr, *scen = nullptr, *soff = nullptr, *sprim = nullptr;
    const double *alpha = nullptr, *coef = nullptr, *centers = nullptr;
};

// Sort key of a shell pair: class (bits 17-20), new/old for start_shell (bit 16), primitive pairs (0-15).
constexpr int PAIR_KEY_BITS = 21;
constexpr unsigned pair_key_class(unsigned k) { return k >> 17; }
constexpr unsigned pair_key_new(unsigned k) { return (k >> 16) & 1u; }
constexpr unsigned pair_key_nprim(unsigned k) { return k & 0xffffu; }

// key, primitive-pair count and identity permutation of every canonical shell pair c = i(i+1)/2 + j
cudaError_t setup_pair_keys(const ShellsDev& sh, int npairs, unsigned* key, int* nprim, int* iota, cudaStream_t s);
// ShellPair (q = 0) and PrimPair / PrimPair32 records of every canonical pair, primitives at poff[c]
cudaError_t setup_build_pairs(const ShellsDev& sh, int npairs, const int* poff, ShellPair* pairs, PrimPair* prims,
                              PrimPair32* prims32, cudaStream_t s);
// dst[k] = src[perm[k]], with dst[k].q = q[k] when q is given
cudaError_t setup_gather_pairs(const ShellPair* src, const int* perm, const double* q, int n, ShellPair* dst,
                               cudaStream_t s);
// staircase row counts of every block pair: x[prefix_off] = 0, x[prefix_off + 1 + i] = n_i
cudaError_t setup_staircase(const BlockPair* bps, int nbp, const ShellPair* pairs, double cut, long long* x,
                            cudaStream_t s);
// prefix[prefix_off + i] = S[prefix_off + i] - S[prefix_off] (S = inclusive scan of x), totals per block pair
cudaError_t setup_prefix_fix(const BlockPair* bps, int nbp, const long long* S, long long* prefix, long long* totals,
                             cudaStream_t s);
// row_bp[prefix_off + i] = k for the bra rows of block pair k (other entries untouched)
cudaError_t setup_row_bp(const BlockPair* bps, int nbp, int* row_bp, cudaStream_t s);
// primitive pairs of the sorted pairs moved from the canonical layout (src) into the block-interleaved
// one (dst): block b's pairs bbegin[b] .. + bcount[b] own records bprim[b] .., primitive ik of its j-th
// pair at bprim[b] + ik * bcount[b] + j; prim_begin / prim_stride of the pairs updated
cudaError_t setup_interleave_prims(ShellPair* pairs, int n, const int* bbegin, const int* bcount, const long long* bprim,
                                   int nb, const PrimPair* src, const PrimPair32* src32, PrimPair* dst, PrimPair32* dst32,
                                   cudaStream_t s);
// ShellPair::prim_begin += prim0 and ShellPair::pad = mol for n pairs (merging molecules into a batch)
cudaError_t setup_offset_pairs(ShellPair* pairs, int n, int prim0, int mol, cudaStream_t s);

// Library primitives (CUB) on device arrays; with tmp == nullptr they only set tmp_bytes.
cudaError_t setup_exclusive_sum(void* tmp, size_t& tmp_bytes, const int* in, int* out, int n, cudaStream_t s);
cudaError_t setup_inclusive_sum(void* tmp, size_t& tmp_bytes, const long long* in, long long* out, int n,
                                cudaStream_t s);
cudaError_t setup_sort_keys(void* tmp, size_t& tmp_bytes, const unsigned* k_in, unsigned* k_out, const int* v_in,
                            int* v_out, int n, cudaStream_t s);
cudaError_t setup_run_length(void* tmp, size_t& tmp_bytes, const unsigned* k_in, unsigned* uniq, int* counts,
                             int* nruns, int n, cudaStream_t s);
cudaError_t setup_sort_desc_segments(void* tmp, size_t& tmp_bytes, const double* k_in, double* k_out, const int* v_in,
                                     int* v_out, int n, int nseg, const int* seg_begin, const int* seg_end,
                                     cudaStream_t s);

}  // namespace ugb
