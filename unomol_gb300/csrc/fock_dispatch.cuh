// Launch table of the class-templated Fock kernels.  Pair class c = la(la+1)/2 + lb (la >= lb);
// quartet classes are (bra class >= ket class).  One translation unit per arithmetic type
// instantiates all of them (fock_fp64.cu, fock_fp32.cu).
#pragma once
#include "eri_common.cuh"

namespace ugb {

struct NormTable;

__host__ __device__ constexpr int pc_la(int c) { return c == 0 ? 0 : c <= 2 ? 1 : c <= 5 ? 2 : 3; }
__host__ __device__ constexpr int pc_lb(int c) { return c - pc_la(c) * (pc_la(c) + 1) / 2; }

// Launches the Fock kernel of quartet class (bc | kc) over `A.nwork` work items on `stream`.
// Returns cudaSuccess or the launch error.
cudaError_t launch_fock_fp64(int bc, int kc, bool uhf, const FockArgs& A, const NormTable& nt,
                             const double* rys, cudaStream_t stream);
cudaError_t launch_fock_fp32(int bc, int kc, bool uhf, const FockArgs& A, const NormTable& nt,
                             const float* rys, cudaStream_t stream);
cudaError_t launch_schwarz(int pc, const ShellPair* pairs, const PrimPair* prims, int begin, int count,
                           const NormTable& nt, const double* rys, double* q_out, cudaStream_t stream);

constexpr int FOCK_THREADS = 128;

}  // namespace ugb
