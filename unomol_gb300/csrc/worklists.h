// Per-build work lists of the density-screened and mixed-precision Fock builds (worklists.cu): the
// FP32 copy of the dense density, max |P| per shell-pair block, the split of every staircase row into
// its FP64 / FP32 / skipped segments and their scans per block pair.  All on the device, no host sync.
#pragma once
#include <cuda_runtime.h>

#include "eri_common.cuh"

namespace ugb {

cudaError_t wl_to_float(const double* full, float* f32, long long n, cudaStream_t s);
// max |P| (of Pa and, when given, Pb) per shell-pair block of one molecule, and over all blocks into dmax[0]
cudaError_t wl_shell_pmax(const double* Pa, const double* Pb, const int* soff, const int* sl, int nshell, int nbf,
                          float* pmax, float* dmax, cudaStream_t s);
// the same for every molecule of a batch: molecule m's blocks at pmax + pmax_off[m] (nshell[m]^2 floats,
// shells shell0[m] .. of the concatenated soff / sl), its dense P at P + doff[m], its maximum in dmax[m];
// total = sum of nshell[m]^2
cudaError_t wl_shell_pmax_batch(const double* P, const long long* doff, const int* nbf, const int* shell0,
                                const int* nshell, const long long* pmax_off, const int* soff, const int* sl, int nmol,
                                long long total, float* pmax, float* dmax, cudaStream_t s);
cudaError_t wl_split_rows(const ShellPair* pairs, const BlockPair* bps, const int* row_bp, const long long* prefix,
                          long long nrows, const float* dmax, double cut64, double skip, long long* c64, long long* c32,
                          int* mseg, cudaStream_t s);
cudaError_t wl_scan_rows(const BlockPair* bps, int nbp, const long long* c64, const long long* c32, long long* p64,
                         long long* p32, long long* n64, long long* n32, cudaStream_t s);
// compact numbering of both parts per class launch (launch l: block pairs launch_bp[2l] ..
// + launch_bp[2l+1]): first item of every block pair and the launch's total, counts rounded up to 32
cudaError_t wl_scan_launches(const int* launch_bp, int nlaunch, const long long* n64, const long long* n32,
                             long long* begin64, long long* begin32, long long* total64, long long* total32,
                             cudaStream_t s);

}  // namespace ugb
