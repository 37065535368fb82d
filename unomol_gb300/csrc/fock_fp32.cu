// FP32 instances of the class-templated Fock kernels (the small-bound part of the mixed-precision path).
#include "fock_kernels.cuh"
#include "fock_dispatch.cuh"

namespace ugb {

template <int BC, int KC, bool UHF>
static cudaError_t launch_one(const FockArgs& A, const NormTable& nt, const float* rys, cudaStream_t s) {
    constexpr int LA = pc_la(BC), LB = pc_lb(BC), LC = pc_la(KC), LD = pc_lb(KC);
    if (A.nwork <= 0) return cudaSuccess;
    if constexpr (QClass<LA, LB, LC, LD>::NF <= 81) {
        const long long blocks = (A.nwork + FOCK_THREADS - 1) / FOCK_THREADS;
        fock_jk_kernel<LA, LB, LC, LD, UHF, float><<<(unsigned)blocks, FOCK_THREADS, 0, s>>>(A, nt, rys);
    } else {
        const long long blocks = (A.nwork + 63) / 64;
        fock_jk_generic<UHF, float, PrimPair32><<<(unsigned)blocks, 64, 0, s>>>(A, nt, rys, A.prims32, LA, LB, LC, LD);
    }
    return cudaGetLastError();
}

#define UGB_CASE(BC, KC)                                                              \
    case (BC) * 8 + (KC):                                                             \
        return uhf ? launch_one<BC, KC, true>(A, nt, rys, stream)                    \
                   : launch_one<BC, KC, false>(A, nt, rys, stream);

cudaError_t launch_fock_fp32(int bc, int kc, bool uhf, const FockArgs& A, const NormTable& nt,
                             const float* rys, cudaStream_t stream) {
    switch (bc * 8 + kc) {
#include "fock_cases.inc"
        default:
            return cudaErrorInvalidValue;
    }
}

}  // namespace ugb

