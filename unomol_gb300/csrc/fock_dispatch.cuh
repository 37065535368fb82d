// Launch table of the class-templated Fock kernels.  Pair class c = la(la+1)/2 + lb (la >= lb);
// quartet classes are (bra class >= ket class).  One translation unit per arithmetic type
// instantiates all of them (fock_fp64.cu, fock_fp32.cu).
#pragma once
#include "eri_common.cuh"

namespace ugb {

struct NormTable;

__host__ __device__ constexpr int pc_la(int c) { return (c >= 1) + (c >= 3) + (c >= 6) + (c >= 10); }
__host__ __device__ constexpr int pc_lb(int c) { return c - pc_la(c) * (pc_la(c) + 1) / 2; }

// Launches the Fock kernel of quartet class (bc | kc) over `A.nwork` work items on `stream`.
// Returns cudaSuccess or the launch error.
cudaError_t launch_fock_fp64(int bc, int kc, bool uhf, const FockArgs& A, const NormTable& nt,
                             const double* rys, cudaStream_t stream);
cudaError_t launch_fock_fp32(int bc, int kc, bool uhf, const FockArgs& A, const NormTable& nt,
                             const float* rys, cudaStream_t stream);
// Both parts of a mixed build of one class in one launch (their CTAs alternate); only for the classes
// that fock_mixed_fused accepts (templated, at most 81 function quartets).
bool fock_mixed_fused(int bc, int kc);
cudaError_t launch_fock_mixed(int bc, int kc, bool uhf, const FockArgs& A64, const FockArgs& A32, const NormTable& nt,
                              const double* rys64, const float* rys32, cudaStream_t stream);
// The FP64 part of a mixed build of one class alone (classes that fock_mixed_fused accepts), on a grid of
// at most `grid` CTAs whose warps step over the part's quartets (NP lanes per quartet).
cudaError_t launch_fock_fp64_part(int bc, int kc, bool uhf, const FockArgs& A64, const FockArgs& A32, const NormTable& nt,
                                  const double* rys64, const float* rys32, int grid, cudaStream_t stream);
cudaError_t launch_schwarz(int pc, const ShellPair* pairs, const PrimPair* prims, int begin, int count,
                           const NormTable& nt, const double* rys, double* q_out, cudaStream_t stream);

// Runtime-L Rys kernel (classes with f or g shells and la+lb+lc+ld <= 8), FP64 or FP32.
cudaError_t launch_fock_generic(int la, int lb, int lc, int ld, bool uhf, bool fp32, const FockArgs& A,
                                const NormTable& nt, const double* rys, const float* rys32, cudaStream_t stream);
// McMurchie-Davidson kernel (la+lb+lc+ld > 8, or every class in the MD mode), FP64.
cudaError_t launch_fock_md(int la, int lb, int lc, int ld, bool uhf, const FockArgs& A, const NormTable& nt,
                           cudaStream_t stream);
// Schwarz diagonal for pairs with la+lb > 2: Rys (la+lb <= 4) into q_out, MD (la+lb > 4) via qbits.
cudaError_t launch_schwarz_high(int la, int lb, const ShellPair* pairs, const PrimPair* prims, int begin, int count,
                                const NormTable& nt, const double* rys, double* q_out, unsigned long long* qbits,
                                cudaStream_t stream);

constexpr int FOCK_THREADS = 128;

}  // namespace ugb
