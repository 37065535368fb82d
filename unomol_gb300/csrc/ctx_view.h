// Internal: read-only view of a context's set-up (device shell pairs, primitive pairs and staircase prefix
// sums; host block pairs, blocks and class launches), used to merge the work of many molecules into one
// batch and by the DPM integrals.
#pragma once
#include <vector>

#include "../../include/unomol_gb300.h"
#include "eri_common.cuh"
#include "fock_kernels.cuh"

namespace ugb {

struct ClassLaunchInfo {
    int bc, kc;          // bra / ket pair classes
    int bp_begin, nbp;   // range in the context's block-pair array
    long long nwork;     // padded work items
    long long quartets;  // unpadded
};

struct CtxView {
    int nbf = 0, nshell = 0, rys_compat = 1, eri_method = 0;
    const ShellPair* d_pairs = nullptr;  // device arrays of the setup
    int npairs = 0;
    const PrimPair* d_prims = nullptr;
    const PrimPair32* d_prims32 = nullptr;
    long long nprims = 0;
    const long long* d_prefix = nullptr;
    const BlockPair* d_bps = nullptr;  // device block pairs (the class launches' ranges index them)
    long long nrows = 0;
    const std::vector<BlockPair>* bps = nullptr;  // host: block pairs, blocks of equal (class, primitive pairs)
    const std::vector<int>* block_begin = nullptr;
    const std::vector<int>* block_count = nullptr;
    const std::vector<int>* block_class = nullptr;
    const std::vector<int>* soff = nullptr;  // host: first AO and L of every shell
    const std::vector<int>* sl = nullptr;
    cudaStream_t stream = nullptr;  // the context's stream (its setup ran there)
    std::vector<ClassLaunchInfo> launches;
    NormTable nt{};
    const double* d_rys = nullptr;
    const float* d_rys32 = nullptr;
};

CtxView ctx_view(const UnomolCtx* ctx);

}  // namespace ugb
