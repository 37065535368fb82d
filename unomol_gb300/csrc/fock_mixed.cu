// The class-templated Fock kernels of the mixed build with both parts in one launch (fock_jk_mixed).
#include <algorithm>

#include "fock_kernels.cuh"
#include "fock_dispatch.cuh"

namespace ugb {

template <int BC, int KC, bool UHF>
static cudaError_t launch_one(const FockArgs& A64, const FockArgs& A32, const NormTable& nt, const double* rys64,
                              const float* rys32, cudaStream_t s) {
    constexpr int LA = pc_la(BC), LB = pc_lb(BC), LC = pc_la(KC), LD = pc_lb(KC);
    if (A64.nwork <= 0) return cudaSuccess;
    if constexpr (QClass<LA, LB, LC, LD>::NF <= 81) {
        const long long blocks = (A64.nwork + FOCK_THREADS - 1) / FOCK_THREADS;
        fock_jk_mixed<LA, LB, LC, LD, UHF><<<(unsigned)(2 * blocks), FOCK_THREADS, 0, s>>>(A64, A32, nt, rys64, rys32);
        return cudaGetLastError();
    } else {
        return cudaErrorInvalidValue;  // large classes take the two separate launches
    }
}

template <int BC, int KC, bool UHF>
static cudaError_t launch_fp64_part(const FockArgs& A64, const FockArgs& A32, const NormTable& nt, const double* rys64,
                                    const float* rys32, int grid, cudaStream_t s) {
    constexpr int LA = pc_la(BC), LB = pc_lb(BC), LC = pc_la(KC), LD = pc_lb(KC);
    if (A64.nwork <= 0) return cudaSuccess;
    if constexpr (QClass<LA, LB, LC, LD>::NF <= 81) {
        const long long blocks = std::min<long long>((A64.nwork + FOCK_THREADS - 1) / FOCK_THREADS, grid);
        fock_jk_fp64_part<LA, LB, LC, LD, UHF><<<(unsigned)blocks, FOCK_THREADS, 0, s>>>(A64, A32, nt, rys64, rys32);
        return cudaGetLastError();
    } else {
        return cudaErrorInvalidValue;
    }
}

#define UGB_CASE(BC, KC)                                                                      \
    case (BC) * 8 + (KC):                                                                     \
        return uhf ? launch_one<BC, KC, true>(A64, A32, nt, rys64, rys32, stream)            \
                   : launch_one<BC, KC, false>(A64, A32, nt, rys64, rys32, stream);

bool fock_mixed_fused(int bc, int kc) {
    const int la = pc_la(bc), lb = pc_lb(bc), lc = pc_la(kc), ld = pc_lb(kc);
    return bc < NTMPLCLASS && kc < NTMPLCLASS &&
           ncart(la) * ncart(lb) * ncart(lc) * ncart(ld) <= 81;
}

cudaError_t launch_fock_mixed(int bc, int kc, bool uhf, const FockArgs& A64, const FockArgs& A32, const NormTable& nt,
                              const double* rys64, const float* rys32, cudaStream_t stream) {
    switch (bc * 8 + kc) {
#include "fock_cases.inc"
        default:
            return cudaErrorInvalidValue;
    }
}

#undef UGB_CASE
#define UGB_CASE(BC, KC)                                                                      \
    case (BC) * 8 + (KC):                                                                     \
        return uhf ? launch_fp64_part<BC, KC, true>(A64, A32, nt, rys64, rys32, grid, stream) \
                   : launch_fp64_part<BC, KC, false>(A64, A32, nt, rys64, rys32, grid, stream);

cudaError_t launch_fock_fp64_part(int bc, int kc, bool uhf, const FockArgs& A64, const FockArgs& A32, const NormTable& nt,
                                  const double* rys64, const float* rys32, int grid, cudaStream_t stream) {
    switch (bc * 8 + kc) {
#include "fock_cases.inc"
        default:
            return cudaErrorInvalidValue;
    }
}

}  // namespace ugb
