// Internal: read-only view of a context's set-up (shell pairs, primitive pairs, block pairs, staircase
// prefix sums, class launches), used to merge the work of many molecules into one batch.
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
    const std::vector<ShellPair>* pairs = nullptr;
    const std::vector<PrimPair>* prims = nullptr;
    const std::vector<BlockPair>* bps = nullptr;
    const std::vector<long long>* prefix = nullptr;
    std::vector<ClassLaunchInfo> launches;
    NormTable nt{};
    const double* d_rys = nullptr;
};

CtxView ctx_view(const UnomolCtx* ctx);

}  // namespace ugb
