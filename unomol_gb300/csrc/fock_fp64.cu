// FP64 instances of the class-templated Fock kernels (the plain path) and the Schwarz diagonal.
#include "fock_kernels.cuh"
#include "fock_dispatch.cuh"

namespace ugb {

template <int BC, int KC, bool UHF>
static cudaError_t launch_one(const FockArgs& A, const NormTable& nt, const double* rys, cudaStream_t s) {
    constexpr int LA = pc_la(BC), LB = pc_lb(BC), LC = pc_la(KC), LD = pc_lb(KC);
    if (A.nwork <= 0) return cudaSuccess;
    if constexpr (QClass<LA, LB, LC, LD>::NF <= 81) {
        const long long blocks = (A.nwork + FOCK_THREADS - 1) / FOCK_THREADS;
        fock_jk_kernel<LA, LB, LC, LD, UHF, double><<<(unsigned)blocks, FOCK_THREADS, 0, s>>>(A, nt, rys);
    } else {
        const long long blocks = (A.nwork + 63) / 64;
        fock_jk_generic<UHF, double, PrimPair><<<(unsigned)blocks, 64, 0, s>>>(A, nt, rys, A.prims, LA, LB, LC, LD);
    }
    return cudaGetLastError();
}

#define UGB_CASE(BC, KC)                                                              \
    case (BC) * 8 + (KC):                                                             \
        return uhf ? launch_one<BC, KC, true>(A, nt, rys, stream)                    \
                   : launch_one<BC, KC, false>(A, nt, rys, stream);

cudaError_t launch_fock_fp64(int bc, int kc, bool uhf, const FockArgs& A, const NormTable& nt,
                             const double* rys, cudaStream_t stream) {
    switch (bc * 8 + kc) {
#include "fock_cases.inc"
        default:
            return cudaErrorInvalidValue;
    }
}

template <int PC>
static cudaError_t schwarz_one(const ShellPair* pairs, const PrimPair* prims, int begin, int count,
                               const NormTable& nt, const double* rys, double* q, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    constexpr int NAB = ncart(pc_la(PC)) * ncart(pc_lb(PC));
    if constexpr (NAB * NAB <= 81)
        schwarz_kernel<pc_la(PC), pc_lb(PC)><<<(unsigned)(((long long)count * 32 + 127) / 128), 128, 0, s>>>(pairs, prims, begin, count, nt, rys, q);
    else
        schwarz_generic<<<(count + 63) / 64, 64, 0, s>>>(pairs, prims, begin, count, nt, rys, q);
    return cudaGetLastError();
}

cudaError_t launch_schwarz(int pc, const ShellPair* pairs, const PrimPair* prims, int begin, int count,
                           const NormTable& nt, const double* rys, double* q_out, cudaStream_t stream) {
    switch (pc) {
        case 0: return schwarz_one<0>(pairs, prims, begin, count, nt, rys, q_out, stream);
        case 1: return schwarz_one<1>(pairs, prims, begin, count, nt, rys, q_out, stream);
        case 2: return schwarz_one<2>(pairs, prims, begin, count, nt, rys, q_out, stream);
#if UGB_MAX_PAIRCLASS > 3
        case 3: return schwarz_one<3>(pairs, prims, begin, count, nt, rys, q_out, stream);
        case 4: return schwarz_one<4>(pairs, prims, begin, count, nt, rys, q_out, stream);
        case 5: return schwarz_one<5>(pairs, prims, begin, count, nt, rys, q_out, stream);
#endif
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace ugb
