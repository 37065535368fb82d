// Emission of canonical integral records (the reference's TwoInts, TwoElectronInts.hpp:20-23) from the
// integral kernels of the conventional build: which element of a shell quartet's function rectangle
// carries a canonical label, and a warp-aggregated append into a device record array.
#pragma once
#include "../../include/unomol_gb300.h"
#include "eri_common.cuh"

namespace ugb {

struct RecSink {
    UnomolRecord* rec;          // cap records
    unsigned long long* count;  // records appended so far (may pass cap: then overflow is set)
    unsigned long long cap;
    int* overflow;
};

// Function quartet (a b | c d) of a shell quartet's rectangle (a, b from the bra shell pair, c, d from the
// ket pair) -> its canonical label (i >= j, k >= l, (i, j) >= (k, l) in that order: the labels of
// TwoElectronInts.cpp:622-653).  A rectangle holds a label twice when the bra (or ket) pair is one shell
// twice, or when bra and ket are the same pair; only one of those elements returns true.
__device__ __forceinline__ bool canonical_label(int a, int b, int c, int d, bool bra_same, bool ket_same, bool same_pair,
                                                int& i, int& j, int& k, int& l) {
    if (bra_same && a < b) return false;
    if (ket_same && c < d) return false;
    i = max(a, b), j = min(a, b), k = max(c, d), l = min(c, d);
    const long long ij = (long long)i * (i + 1) / 2 + j, kl = (long long)k * (k + 1) / 2 + l;
    if (same_pair && ij < kl) return false;
    if (ij < kl) {
        int t = i;
        i = k;
        k = t;
        t = j;
        j = l;
        l = t;
    }
    return true;
}

// Reserves n consecutive slots of the array counted by *counter for each lane of a warp with one atomic
// per warp; every lane of the warp must call it.  Returns the lane's first slot.
__device__ __forceinline__ unsigned long long warp_reserve(unsigned long long* counter, unsigned n) {
    const int lane = threadIdx.x & 31;
    unsigned incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    const unsigned total = __shfl_sync(0xffffffffu, incl, 31);
    unsigned long long base = 0;
    if (lane == 31 && total) base = atomicAdd(counter, (unsigned long long)total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + incl - n;
}

__device__ __forceinline__ unsigned long long reserve_records(const RecSink& S, unsigned n) { return warp_reserve(S.count, n); }

__device__ __forceinline__ void put_record(const RecSink& S, unsigned long long slot, double v, int i, int j, int k, int l) {
    if (slot >= S.cap) {
        atomicExch(S.overflow, 1);
        return;
    }
    UnomolRecord* r = S.rec + slot;
    r->val = v;
    r->i = i;
    r->j = j;
    r->k = k;
    r->l = l;
}

struct NormTable;
// Record passes of one class for the classes the templated kernels do not cover (fock_md.cu).
cudaError_t launch_store_generic(int la, int lb, int lc, int ld, const FockArgs& A, const NormTable& nt, const double* rys,
                                 const RecSink& S, cudaStream_t s);
cudaError_t launch_store_md(int la, int lb, int lc, int ld, const FockArgs& A, const NormTable& nt, const RecSink& S,
                            cudaStream_t s);

}  // namespace ugb
