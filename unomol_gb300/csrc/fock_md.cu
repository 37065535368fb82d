// Launchers of the classes with f and g shells: runtime-L Rys (la+lb+lc+ld <= 8, FP64 or FP32),
// McMurchie-Davidson (la+lb+lc+ld > 8, and every class in the MD mode), and their Schwarz diagonals;
// the same two methods as record passes of the conventional build (store.cu).
#include <algorithm>

#include "fock_dispatch.cuh"
#include "md_kernels.cuh"
#include "store_emit.cuh"

namespace ugb {

cudaError_t launch_fock_generic(int la, int lb, int lc, int ld, bool uhf, bool fp32, const FockArgs& A,
                                const NormTable& nt, const double* rys, const float* rys32, cudaStream_t s) {
    if (A.nwork <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((A.nwork + 63) / 64);
    if (fp32) {
        if (uhf)
            fock_jk_generic<true, float, PrimPair32><<<blocks, 64, 0, s>>>(A, nt, rys32, A.prims32, la, lb, lc, ld);
        else
            fock_jk_generic<false, float, PrimPair32><<<blocks, 64, 0, s>>>(A, nt, rys32, A.prims32, la, lb, lc, ld);
    } else {
        if (uhf)
            fock_jk_generic<true, double, PrimPair><<<blocks, 64, 0, s>>>(A, nt, rys, A.prims, la, lb, lc, ld);
        else
            fock_jk_generic<false, double, PrimPair><<<blocks, 64, 0, s>>>(A, nt, rys, A.prims, la, lb, lc, ld);
    }
    return cudaGetLastError();
}

cudaError_t launch_fock_md(int la, int lb, int lc, int ld, bool uhf, const FockArgs& A, const NormTable& nt,
                           cudaStream_t s) {
    if (A.nwork <= 0) return cudaSuccess;
    const long long nf = (long long)ncart(la) * ncart(lb) * ncart(lc) * ncart(ld);
    const long long nthreads = A.nwork * nf;
    const long long want = (nthreads + 127) / 128;
    const unsigned blocks = (unsigned)std::min<long long>(want, 1LL << 20);  // grid-stride beyond
    if (uhf)
        fock_jk_md<true><<<blocks, 128, 0, s>>>(A, nt, la, lb, lc, ld, nthreads);
    else
        fock_jk_md<false><<<blocks, 128, 0, s>>>(A, nt, la, lb, lc, ld, nthreads);
    return cudaGetLastError();
}

static __global__ void qbits_to_q(const unsigned long long* __restrict__ qbits, double* __restrict__ q, int begin, int count) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < count) q[begin + t] = sqrt(__longlong_as_double((long long)qbits[begin + t]));
}

cudaError_t launch_schwarz_high(int la, int lb, const ShellPair* pairs, const PrimPair* prims, int begin, int count,
                                const NormTable& nt, const double* rys, double* q_out, unsigned long long* qbits,
                                cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    if (la + lb <= 4) {  // (ab|ab) within the Rys domain
        schwarz_generic<<<(count + 63) / 64, 64, 0, s>>>(pairs, prims, begin, count, nt, rys, q_out);
        return cudaGetLastError();
    }
    const long long n = (long long)count * ncart(la) * ncart(lb);
    cudaError_t e = cudaMemsetAsync(qbits + begin, 0, sizeof(unsigned long long) * count, s);
    if (e != cudaSuccess) return e;
    schwarz_md<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(pairs, prims, begin, count, nt, qbits);
    qbits_to_q<<<(count + 127) / 128, 128, 0, s>>>(qbits, q_out, begin, count);
    return cudaGetLastError();
}

// Conventional build, record pass of one class by the runtime-L Rys kernel: one thread per shell quartet
// of the class's work list, its integrals in thread-local memory, the canonical elements with
// |v| > 1e-14 appended as records (TwoElectronInts.cpp:622-671).
static __global__ void __launch_bounds__(64) store_records_generic(const FockArgs A, const NormTable nt, const double* __restrict__ rys,
                                                                   const RecSink S, int la, int lb, int lc, int ld) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int bi = 0, ki = 0;
    const bool ok = decode_work_warp<false>(A, g, bi, ki);  // warp-collective
    const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
    double acc[GEN_NF];
    ShellPair bra{}, ket{};
    unsigned n = 0, npass = 0;
    if (ok) {
        bra = A.pairs[bi];
        ket = A.pairs[ki];
        generic_quartet_eri<double, PrimPair>(A, bra, ket, rys, A.prims, la, lb, lc, ld, acc, npass);
    }
    for (int pass = 0; pass < 2; ++pass) {  // count, then write
        unsigned long long slot = 0;
        if (pass == 1) slot = reserve_records(S, n);
        if (!ok) continue;
        int f = 0;
        for (int ia = 0; ia < NA; ++ia)
            for (int ib = 0; ib < NB; ++ib)
                for (int ic = 0; ic < NC; ++ic)
                    for (int id = 0; id < ND; ++id, ++f) {
                        const double v = acc[f] * (nt.v[la][ia] * nt.v[lb][ib] * nt.v[lc][ic] * nt.v[ld][id]);
                        if (!above_cut(v, A.thr_int)) continue;  // TwoElectronInts.cpp:668
                        int i, j, k, l;
                        if (!canonical_label(bra.a_off + ia, bra.b_off + ib, ket.a_off + ic, ket.b_off + id, bra.same, ket.same,
                                             bi == ki, i, j, k, l))
                            continue;
                        if (pass == 0) ++n;
                        else put_record(S, slot++, v, i, j, k, l);
                    }
    }
}

// The same by McMurchie-Davidson: one thread per (shell quartet, function quartet), as fock_jk_md; only
// the canonical elements are evaluated.  The loop steps whole warps, so that every lane reaches the
// warp-collective append.
static __global__ void __launch_bounds__(128) store_records_md(const FockArgs A, const NormTable nt, const RecSink S, int la, int lb,
                                                               int lc, int ld, long long nthreads) {
    const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
    const long long NF = (long long)NA * NB * NC * ND;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long g0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); g0 < nthreads; g0 += stride) {
        const long long g = g0 + (threadIdx.x & 31);
        bool have = false;
        double v = 0.0;
        int i = 0, j = 0, k = 0, l = 0, bi, ki;
        if (g < nthreads && decode_work(A, g / NF, bi, ki)) {
            const int f = (int)(g % NF);
            const ShellPair bra = A.pairs[bi];
            const ShellPair ket = A.pairs[ki];
            const int id = f % ND, ic = (f / ND) % NC, ib = (f / (ND * NC)) % NB, ia = f / (ND * NC * NB);
            if (canonical_label(bra.a_off + ia, bra.b_off + ib, ket.a_off + ic, ket.b_off + id, bra.same, ket.same, bi == ki, i,
                                j, k, l)) {
                v = md_function_quartet(bra, ket, A.prims, la, lb, lc, ld, ia, ib, ic, id);
                v *= nt.v[la][ia] * nt.v[lb][ib] * nt.v[lc][ic] * nt.v[ld][id];
                have = above_cut(v, A.thr_int);  // TwoElectronInts.cpp:668
            }
        }
        const unsigned long long slot = reserve_records(S, have ? 1u : 0u);
        if (have) put_record(S, slot, v, i, j, k, l);
    }
}

cudaError_t launch_store_generic(int la, int lb, int lc, int ld, const FockArgs& A, const NormTable& nt, const double* rys,
                                 const RecSink& S, cudaStream_t s) {
    if (A.nwork <= 0) return cudaSuccess;
    store_records_generic<<<(unsigned)((A.nwork + 63) / 64), 64, 0, s>>>(A, nt, rys, S, la, lb, lc, ld);
    return cudaGetLastError();
}

cudaError_t launch_store_md(int la, int lb, int lc, int ld, const FockArgs& A, const NormTable& nt, const RecSink& S,
                            cudaStream_t s) {
    if (A.nwork <= 0) return cudaSuccess;
    const long long nthreads = A.nwork * ncart(la) * ncart(lb) * ncart(lc) * ncart(ld);
    const unsigned blocks = (unsigned)std::min<long long>((nthreads + 127) / 128, 1LL << 20);  // grid-stride beyond
    store_records_md<<<blocks, 128, 0, s>>>(A, nt, S, la, lb, lc, ld, nthreads);
    return cudaGetLastError();
}

}  // namespace ugb
