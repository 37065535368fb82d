// Launchers of the classes with f and g shells: runtime-L Rys (la+lb+lc+ld <= 8, FP64 or FP32),
// McMurchie-Davidson (la+lb+lc+ld > 8, and every class in the MD mode), and their Schwarz diagonals.
#include <algorithm>

#include "fock_dispatch.cuh"
#include "md_kernels.cuh"

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

}  // namespace ugb
