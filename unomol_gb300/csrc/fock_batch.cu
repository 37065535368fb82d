// Batched Fock build over many molecules (the batching form): merged work lists, one persistent kernel
// per quartet class pulling tiles from an atomic counter, the whole build captured as a CUDA graph,
// and an autotuner choosing the CTA size (quartets per tile) and the CTAs per SM of every class.
// RHF, shells up to d (the batch workload is s/p); FP64, or the precision form (per-build FP64 / FP32 /
// skipped parts with each molecule's own density bound), whose two parts of a templated class run as
// one grid launch with alternating CTAs.
#include <algorithm>
#include <climits>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/unomol_gb300.h"
#include "ctx_view.h"
#include "fock_dispatch.cuh"
#include "setup.h"
#include "worklists.h"

using namespace ugb;

#ifndef UGB_BATCH_FUSE_MAXL
#define UGB_BATCH_FUSE_MAXL 1  // classes with la+lb+lc+ld above this launch their two parts separately
#endif

namespace {

template <int BC, int KC, typename R>
cudaError_t persistent_one(const FockArgs& A, const NormTable& nt, const R* rys, int grid, int block, cudaStream_t s) {
    constexpr int LA = pc_la(BC), LB = pc_lb(BC), LC = pc_la(KC), LD = pc_lb(KC);
    if constexpr (QClass<LA, LB, LC, LD>::NF <= 81) {
        fock_jk_persistent<LA, LB, LC, LD, false, R><<<grid, block, 0, s>>>(A, nt, rys);
    } else if constexpr (sizeof(R) == 8) {
        // large classes: one item per thread over the whole launch
        fock_jk_generic<false, double, PrimPair><<<(unsigned)((A.nwork + 63) / 64), 64, 0, s>>>(A, nt, rys, A.prims, LA, LB, LC, LD);
    } else {
        fock_jk_generic<false, float, PrimPair32><<<(unsigned)((A.nwork + 63) / 64), 64, 0, s>>>(A, nt, rys, A.prims32, LA, LB, LC, LD);
    }
    return cudaGetLastError();
}

#define UGB_CASE(BC, KC) \
    case (BC) * 8 + (KC): \
        return persistent_one<BC, KC, R>(A, nt, rys, grid, block, s);

// FP64 (R = double, FP64 tables) or FP32 (R = float, FP32 tables) persistent launch of one class
template <typename R>
cudaError_t launch_persistent(int bc, int kc, const FockArgs& A, const NormTable& nt, const R* rys, int grid,
                              int block, cudaStream_t s) {
    switch (bc * 8 + kc) {
#include "fock_cases.inc"
        default:
            return cudaErrorInvalidValue;
    }
}
#undef UGB_CASE

// dense <- packed for every molecule of the batch
__global__ void batch_expand(const double* __restrict__ pk, const long long* __restrict__ poff, double* __restrict__ full,
                             const long long* __restrict__ doff, const int* __restrict__ nbf, int nmol, long long total) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    int lo = 0, hi = nmol - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (doff[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const int n = nbf[lo];
    const long long r = t - doff[lo];
    const int i = (int)(r / n), j = (int)(r % n);
    const int a = i > j ? i : j, b = i > j ? j : i;
    full[t] = pk[poff[lo] + (long long)a * (a + 1) / 2 + b];
}

// packed G = T + T^T for every molecule
__global__ void batch_fold(const double* __restrict__ T, const long long* __restrict__ doff, double* __restrict__ G,
                           const long long* __restrict__ poff, const int* __restrict__ nbf, int nmol, long long total) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    int lo = 0, hi = nmol - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (poff[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const int n = nbf[lo];
    const long long r = t - poff[lo];
    int i = (int)((sqrt(8.0 * (double)r + 1.0) - 1.0) * 0.5);
    while ((long long)i * (i + 1) / 2 > r) --i;
    while ((long long)(i + 1) * (i + 2) / 2 <= r) ++i;
    const int j = (int)(r - (long long)i * (i + 1) / 2);
    const double* Tm = T + doff[lo];
    G[t] = Tm[(long long)i * n + j] + Tm[(long long)j * n + i];
}

struct BLaunch {
    int bc, kc, bp_begin, nbp;
    long long nwork;
    int block = 128, ctas_per_sm = 4;
};

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

thread_local std::string g_batch_err;

}  // namespace

struct UnomolBatch {
    std::vector<UnomolCtx*> mols;
    std::vector<int> nbf;
    std::vector<long long> doff, poff;  // dense / packed offsets per molecule (+ total at the end)
    long long dense_total = 0, packed_total = 0;
    ShellPair* d_pairs = nullptr;
    PrimPair* d_prims = nullptr;
    BlockPair* d_bps = nullptr;
    long long* d_prefix = nullptr;
    int* d_nbf = nullptr;
    long long *d_doff = nullptr, *d_poff = nullptr;
    double *d_P = nullptr, *d_G = nullptr, *d_Pfull = nullptr, *d_T = nullptr;
    unsigned long long* d_tiles = nullptr;  // two per class launch (FP64 part, FP32 part)
    std::vector<BLaunch> launches;
    NormTable nt{};
    const double* rys = nullptr;
    const float* rys32 = nullptr;
    // precision form (UNOMOL_PREC_MIXED): per-build work lists as for one context, over all molecules
    int prec_mode = UNOMOL_PREC_FP64;
    double fp32_cut = 1e-10, skip_cut = 1e-13;
    long long nrows = 0, pmax_total = 0;
    int nbps = 0;
    PrimPair32* d_prims32 = nullptr;
    float* d_Pfull32 = nullptr;
    float *d_pmax = nullptr, *d_dmax = nullptr;
    int *d_nshell = nullptr, *d_shell0 = nullptr, *d_soff = nullptr, *d_sl = nullptr;
    long long* d_pmax_off = nullptr;
    int *d_rowbp = nullptr, *d_mseg = nullptr;
    long long *d_c64 = nullptr, *d_c32 = nullptr, *d_pre64 = nullptr, *d_pre32 = nullptr;
    long long *d_cnt64 = nullptr, *d_cnt32 = nullptr;
    long long *d_begin64 = nullptr, *d_begin32 = nullptr, *d_total64 = nullptr, *d_total32 = nullptr;
    int* d_launch_bp = nullptr;
    int rys_compat = 1;
    int nsm = 152;
    cudaStream_t stream = nullptr;
    cudaStream_t part_stream[2] = {nullptr, nullptr};  // mixed builds: FP64 / FP32 parts side by side
    cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};
    cudaGraphExec_t graph = nullptr;
    std::string err;
};

namespace {

int bfail(UnomolBatch* b, int code, const std::string& m) {
    if (b) b->err = m;
    g_batch_err = m;
    return code;
}

#define BCU(call)                                                                                 \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return bfail(b, e_ == cudaErrorMemoryAllocation ? UNOMOL_ENOMEM : UNOMOL_ECUDA,       \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                     \
    } while (0)

FockArgs batch_args(UnomolBatch* b, const BLaunch& L, int k) {
    FockArgs A{};
    A.pairs = b->d_pairs;
    A.prims = b->d_prims;
    A.bps = b->d_bps + L.bp_begin;
    A.prefix = b->d_prefix;
    A.nbp = L.nbp;
    A.nwork = L.nwork;
    A.nbf = 0;
    A.Pa = b->d_Pfull;
    A.Ta = b->d_T;
    A.thr_int = STORE_CUT;
    A.prim_cut = PRIM_CUT;
    A.thr_int32 = (float)STORE_CUT;
    A.prim_cut32 = (float)PRIM_CUT;
    A.rys_compat = b->rys_compat;
    A.mol_nbf = b->d_nbf;
    A.mol_base = b->d_doff;
    A.tile_counter = b->d_tiles + 2 * k;
    A.mode = 0;
    A.prims32 = b->d_prims32;
    A.Pa32 = b->d_Pfull32;
    A.pmax = b->d_pmax;
    A.dmax = b->d_dmax;
    A.skip_cut = b->skip_cut;
    A.skip_cut32 = (float)b->skip_cut;
    A.fp32_cut = b->fp32_cut;
    A.fp32_cut32 = b->fp32_cut > b->skip_cut ? (float)b->fp32_cut : 0.f;  // per-quartet FP32 choice of the fused kernel
    A.dyn_mseg = b->d_mseg;
    A.mol_nshell = b->d_nshell;
    A.mol_pmax = b->d_pmax_off;
    return A;
}

// the batched build on stream s (persistent launches); G = G(P) for every molecule
int batch_build(UnomolBatch* b, cudaStream_t s) {
    const int nmol = (int)b->mols.size();
    batch_expand<<<(unsigned)((b->dense_total + 255) / 256), 256, 0, s>>>(b->d_P, b->d_poff, b->d_Pfull, b->d_doff, b->d_nbf,
                                                                          nmol, b->dense_total);
    BCU(cudaGetLastError());
    BCU(cudaMemsetAsync(b->d_T, 0, sizeof(double) * b->dense_total, s));
    BCU(cudaMemsetAsync(b->d_tiles, 0, sizeof(unsigned long long) * 2 * std::max<size_t>(1, b->launches.size()), s));
    const bool mixed = b->prec_mode == UNOMOL_PREC_MIXED;
    if (mixed) {
        // this build's work lists: max|P| per shell-pair block and per molecule, split of every staircase
        // row into FP64 / FP32 / skipped segments, scan per block pair; FP32 copy of the densities
        BCU(cudaMemsetAsync(b->d_dmax, 0, sizeof(float) * nmol, s));
        BCU(wl_shell_pmax_batch(b->d_Pfull, b->d_doff, b->d_nbf, b->d_shell0, b->d_nshell, b->d_pmax_off, b->d_soff, b->d_sl,
                                nmol, b->pmax_total, b->d_pmax, b->d_dmax, s));
        BCU(wl_split_rows(b->d_pairs, b->d_bps, b->d_rowbp, b->d_prefix, b->nrows, b->d_dmax,
                          std::max(b->fp32_cut, b->skip_cut), b->skip_cut, b->d_c64, b->d_c32, b->d_mseg, s));
        BCU(wl_scan_rows(b->d_bps, (int)b->nbps, b->d_c64, b->d_c32, b->d_pre64, b->d_pre32, b->d_cnt64, b->d_cnt32, s));
        BCU(wl_scan_launches(b->d_launch_bp, (int)b->launches.size(), b->d_cnt64, b->d_cnt32, b->d_begin64, b->d_begin32,
                             b->d_total64, b->d_total32, s));
        BCU(wl_to_float(b->d_Pfull, b->d_Pfull32, b->dense_total, s));
    }
    // the FP64 and the FP32 parts on two streams forked from s (joined before the fold): their persistent
    // CTAs share the SMs, one kind on the FP64 pipe, the other on the FP32 pipe and the loads
    const bool split = mixed && b->fp32_cut > b->skip_cut;
    cudaStream_t ls[2] = {s, s};
    if (split) {
        BCU(cudaEventRecord(b->fork, s));
        for (int q = 0; q < 2; ++q) {
            BCU(cudaStreamWaitEvent(b->part_stream[q], b->fork, 0));
            ls[q] = b->part_stream[q];
        }
    }
    for (size_t k = 0; k < b->launches.size(); ++k) {
        const BLaunch& L = b->launches[k];
        FockArgs A = batch_args(b, L, (int)k);
        if (!mixed) {
            BCU(launch_persistent(L.bc, L.kc, A, b->nt, b->rys, b->nsm * L.ctas_per_sm, L.block, s));
            continue;
        }
        A.mode = 1;  // FP64 part
        A.dyn_prefix = b->d_pre64;
        A.dyn_count = b->d_cnt64 + L.bp_begin;
        A.dyn_begin = b->d_begin64 + L.bp_begin;
        A.dyn_total = b->d_total64 + k;
        // both parts of a templated class in one grid launch with alternating CTAs (fock_jk_mixed, as for
        // one molecule; the merged work lists balance the molecules): 14 % faster than the two persistent
        // parts for the 32-water cluster, the same for 256 molecules
        if (split && fock_mixed_fused(L.bc, L.kc)) {
            FockArgs A32 = A;
            A32.mode = 2;
            A32.dyn_prefix = b->d_pre32;
            A32.dyn_count = b->d_cnt32 + L.bp_begin;
            A32.dyn_begin = b->d_begin32 + L.bp_begin;
            A32.dyn_total = b->d_total32 + k;
            if (pc_la(L.bc) + pc_lb(L.bc) + pc_la(L.kc) + pc_lb(L.kc) <= UGB_BATCH_FUSE_MAXL) {
                BCU(launch_fock_mixed(L.bc, L.kc, false, A, A32, b->nt, b->rys, b->rys32, ls[k & 1]));
            } else {
                // as for one molecule: the heavier classes' FP64 part (four lanes per quartet) and FP32 part
                // (persistent) as two kernels on the two streams, each at its own register count
                BCU(launch_fock_fp64_part(L.bc, L.kc, false, A, A32, b->nt, b->rys, b->rys32, b->nsm * 8, ls[k & 1]));
                A32.tile_counter = b->d_tiles + 2 * k + 1;
                BCU(launch_persistent(L.bc, L.kc, A32, b->nt, b->rys32, b->nsm * L.ctas_per_sm, L.block, ls[(k + 1) & 1]));
            }
            continue;
        }
        BCU(launch_persistent(L.bc, L.kc, A, b->nt, b->rys, b->nsm * L.ctas_per_sm, L.block, ls[0]));
        if (b->fp32_cut > b->skip_cut) {
            A.mode = 2;  // FP32 part
            A.dyn_prefix = b->d_pre32;
            A.dyn_count = b->d_cnt32 + L.bp_begin;
            A.dyn_begin = b->d_begin32 + L.bp_begin;
            A.dyn_total = b->d_total32 + k;
            A.tile_counter = b->d_tiles + 2 * k + 1;
            BCU(launch_persistent(L.bc, L.kc, A, b->nt, b->rys32, b->nsm * L.ctas_per_sm, L.block, ls[1]));
        }
    }
    if (split)
        for (int q = 0; q < 2; ++q) {
            BCU(cudaEventRecord(b->join[q], ls[q]));
            BCU(cudaStreamWaitEvent(s, b->join[q], 0));
        }
    batch_fold<<<(unsigned)((b->packed_total + 255) / 256), 256, 0, s>>>(b->d_T, b->d_doff, b->d_G, b->d_poff, b->d_nbf,
                                                                         nmol, b->packed_total);
    BCU(cudaGetLastError());
    return UNOMOL_OK;
}

// Buffers of the precision form, made on first use: the molecules' FP32 primitive pairs side by side,
// the shell arrays of all molecules (for max|P| per shell-pair block), the FP32 dense densities and the
// per-build row lists of the merged staircases.
int ensure_mixed(UnomolBatch* b) {
    if (b->d_prims32) return UNOMOL_OK;
    const int nmol = (int)b->mols.size();
    std::vector<int> nshell(nmol), shell0(nmol), soff, sl;
    std::vector<long long> pmax_off(nmol);
    long long nprim_tot = 0, ptot = 0;
    for (int m = 0; m < nmol; ++m) {
        const CtxView v = ctx_view(b->mols[m]);
        nshell[m] = v.nshell;
        shell0[m] = (int)soff.size();
        soff.insert(soff.end(), v.soff->begin(), v.soff->end());
        sl.insert(sl.end(), v.sl->begin(), v.sl->end());
        pmax_off[m] = ptot;
        ptot += (long long)v.nshell * v.nshell;
        nprim_tot += v.nprims;
    }
    b->pmax_total = ptot;
    const size_t nr = (size_t)std::max<long long>(1, b->nrows), nbp = (size_t)std::max(1, b->nbps);
    BCU(cudaMalloc(&b->d_prims32, sizeof(PrimPair32) * std::max<long long>(1, nprim_tot)));
    BCU(cudaMalloc(&b->d_Pfull32, sizeof(float) * std::max<long long>(1, b->dense_total)));
    BCU(cudaMalloc(&b->d_pmax, sizeof(float) * std::max<long long>(1, ptot)));
    BCU(cudaMalloc(&b->d_dmax, sizeof(float) * nmol));
    BCU(cudaMalloc(&b->d_nshell, sizeof(int) * nmol));
    BCU(cudaMalloc(&b->d_shell0, sizeof(int) * nmol));
    BCU(cudaMalloc(&b->d_pmax_off, sizeof(long long) * nmol));
    BCU(cudaMalloc(&b->d_soff, sizeof(int) * std::max<size_t>(1, soff.size())));
    BCU(cudaMalloc(&b->d_sl, sizeof(int) * std::max<size_t>(1, sl.size())));
    BCU(cudaMalloc(&b->d_rowbp, sizeof(int) * nr));
    BCU(cudaMalloc(&b->d_mseg, sizeof(int) * nr));
    for (long long** p : {&b->d_c64, &b->d_c32, &b->d_pre64, &b->d_pre32}) BCU(cudaMalloc(p, sizeof(long long) * nr));
    BCU(cudaMalloc(&b->d_cnt64, sizeof(long long) * nbp));
    BCU(cudaMalloc(&b->d_cnt32, sizeof(long long) * nbp));
    BCU(cudaMalloc(&b->d_begin64, sizeof(long long) * nbp));
    BCU(cudaMalloc(&b->d_begin32, sizeof(long long) * nbp));
    const size_t nl = std::max<size_t>(1, b->launches.size());
    BCU(cudaMalloc(&b->d_total64, sizeof(long long) * nl));
    BCU(cudaMalloc(&b->d_total32, sizeof(long long) * nl));
    BCU(cudaMalloc(&b->d_launch_bp, sizeof(int) * 2 * nl));
    std::vector<int> launch_bp;
    for (const BLaunch& L : b->launches) {
        launch_bp.push_back(L.bp_begin);
        launch_bp.push_back(L.nbp);
    }
    cudaStream_t s = b->stream;
    if (!launch_bp.empty())
        BCU(cudaMemcpyAsync(b->d_launch_bp, launch_bp.data(), sizeof(int) * launch_bp.size(), cudaMemcpyHostToDevice, s));
    long long p0 = 0;
    for (int m = 0; m < nmol; ++m) {
        const CtxView v = ctx_view(b->mols[m]);
        if (v.nprims > 0)
            BCU(cudaMemcpyAsync(b->d_prims32 + p0, v.d_prims32, sizeof(PrimPair32) * v.nprims, cudaMemcpyDeviceToDevice, s));
        p0 += v.nprims;
    }
    BCU(cudaMemcpyAsync(b->d_nshell, nshell.data(), sizeof(int) * nmol, cudaMemcpyHostToDevice, s));
    BCU(cudaMemcpyAsync(b->d_shell0, shell0.data(), sizeof(int) * nmol, cudaMemcpyHostToDevice, s));
    BCU(cudaMemcpyAsync(b->d_pmax_off, pmax_off.data(), sizeof(long long) * nmol, cudaMemcpyHostToDevice, s));
    if (!soff.empty()) {
        BCU(cudaMemcpyAsync(b->d_soff, soff.data(), sizeof(int) * soff.size(), cudaMemcpyHostToDevice, s));
        BCU(cudaMemcpyAsync(b->d_sl, sl.data(), sizeof(int) * sl.size(), cudaMemcpyHostToDevice, s));
    }
    // row -> block pair of the merged list (-1 on end-of-block-pair entries and rows of empty block pairs)
    BCU(cudaMemsetAsync(b->d_rowbp, 0xff, sizeof(int) * nr, s));
    BCU(setup_row_bp(b->d_bps, b->nbps, b->d_rowbp, s));
    BCU(cudaMemsetAsync(b->d_c64, 0, sizeof(long long) * nr, s));
    BCU(cudaMemsetAsync(b->d_c32, 0, sizeof(long long) * nr, s));
    BCU(cudaMemsetAsync(b->d_mseg, 0, sizeof(int) * nr, s));
    BCU(cudaStreamSynchronize(s));
    return UNOMOL_OK;
}

}  // namespace

extern "C" {

int unomol_gpu_batch_set_precision(UnomolBatch* b, int mode, double fp32_cut, double skip_cut) {
    if (!b) return bfail(b, UNOMOL_EINVAL, "null batch");
    if (mode != UNOMOL_PREC_FP64 && mode != UNOMOL_PREC_MIXED) return bfail(b, UNOMOL_EINVAL, "unknown precision mode");
    if (!(fp32_cut >= 0.0) || !(skip_cut >= 0.0)) return bfail(b, UNOMOL_EINVAL, "bad cutoff");
    if (mode == UNOMOL_PREC_MIXED) {
        const int rc = ensure_mixed(b);
        if (rc) return rc;
    }
    b->prec_mode = mode;
    b->fp32_cut = fp32_cut;
    b->skip_cut = skip_cut;
    if (b->graph) {  // the captured build has the previous form's launches: capture again on next use
        BCU(cudaStreamSynchronize(b->stream));
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return UNOMOL_OK;
}

int unomol_gpu_batch_create(const UnomolBasisDesc* bases, int nmol, UnomolBatch** out) {
    UnomolBatch* b = nullptr;
    if (!bases || nmol <= 0 || !out) return bfail(nullptr, UNOMOL_EINVAL, "bad batch arguments");
    *out = nullptr;
    b = new UnomolBatch();
    auto cleanup = [&](int rc) {
        unomol_gpu_batch_destroy(b);
        return rc;
    };
    std::vector<std::vector<BlockPair>> per_class(NTMPLCLASS * NTMPLCLASS);
    std::vector<int> pair0s, prim0s;
    std::vector<long long> row0s;
    long long npair_tot = 0, nprim_tot = 0, nrow_tot = 0;
    long long dense = 0, packed = 0;
    for (int m = 0; m < nmol; ++m) {
        UnomolCtx* c = nullptr;
        int rc = unomol_gpu_create(&bases[m], 0, &c);
        if (rc) {
            bfail(b, rc, std::string("molecule ") + std::to_string(m) + ": " + unomol_gpu_last_error(nullptr));
            return cleanup(rc);
        }
        b->mols.push_back(c);
        const CtxView v = ctx_view(c);
        if (m == 0) {
            b->nt = v.nt;
            b->rys = v.d_rys;
            b->rys32 = v.d_rys32;
            b->rys_compat = v.rys_compat;
        }
        if (npair_tot + v.npairs >= INT_MAX || nprim_tot + v.nprims >= INT_MAX || nrow_tot + v.nrows >= INT_MAX) {
            bfail(b, UNOMOL_EINVAL, "batched build: too many shell pairs for one batch");
            return cleanup(UNOMOL_EINVAL);
        }
        pair0s.push_back((int)npair_tot);
        prim0s.push_back((int)nprim_tot);
        row0s.push_back(nrow_tot);
        for (const ClassLaunchInfo& L : v.launches) {
            if (L.bc >= NTMPLCLASS || L.kc >= NTMPLCLASS) {
                bfail(b, UNOMOL_EINVAL, "batched build: shells above d are not supported");
                return cleanup(UNOMOL_EINVAL);
            }
            for (int k = 0; k < L.nbp; ++k) {
                BlockPair bp = (*v.bps)[L.bp_begin + k];
                bp.bra_begin += (int)npair_tot;
                bp.ket_begin += (int)npair_tot;
                bp.prefix_off += (int)nrow_tot;
                per_class[L.bc * NTMPLCLASS + L.kc].push_back(bp);
            }
        }
        npair_tot += v.npairs;
        nprim_tot += v.nprims;
        nrow_tot += v.nrows;
        b->nbf.push_back(v.nbf);
        b->doff.push_back(dense);
        b->poff.push_back(packed);
        dense += (long long)v.nbf * v.nbf;
        packed += (long long)v.nbf * (v.nbf + 1) / 2;
    }
    b->dense_total = dense;
    b->packed_total = packed;
    // launches: one per class over all molecules, work ranges 32-aligned (warps never straddle)
    std::vector<BlockPair> bps;
    for (int cls = 0; cls < NTMPLCLASS * NTMPLCLASS; ++cls) {
        auto& v = per_class[cls];
        if (v.empty()) continue;
        // the costliest quartets of all molecules first (as for one context: no long tail of
        // many-primitive quartets at the end of a launch)
        std::stable_sort(v.begin(), v.end(),
                         [](const BlockPair& x, const BlockPair& y) { return x.prim_quartets > y.prim_quartets; });
        BLaunch L;
        L.bc = cls / NTMPLCLASS;
        L.kc = cls % NTMPLCLASS;
        L.bp_begin = (int)bps.size();
        L.nbp = (int)v.size();
        long long w = 0;
        for (auto& bp : v) {
            bp.work_begin = w;
            w += (bp.work_count + 31) / 32 * 32;
            bps.push_back(bp);
        }
        L.nwork = w;
        b->launches.push_back(L);
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev);
    BCU(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    {
        int lo = 0, hi = 0;  // the FP64 part first on the SMs, the FP32 part fills in (as for one context)
        BCU(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        BCU(cudaStreamCreateWithPriority(&b->part_stream[0], cudaStreamNonBlocking, hi));
        BCU(cudaStreamCreateWithPriority(&b->part_stream[1], cudaStreamNonBlocking, lo));
    }
    BCU(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    for (auto& e : b->join) BCU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    BCU(cudaMalloc(&b->d_pairs, sizeof(ShellPair) * std::max<long long>(1, npair_tot)));
    BCU(cudaMalloc(&b->d_prims, sizeof(PrimPair) * std::max<long long>(1, nprim_tot)));
    BCU(cudaMalloc(&b->d_bps, sizeof(BlockPair) * std::max<size_t>(1, bps.size())));
    BCU(cudaMalloc(&b->d_prefix, sizeof(long long) * std::max<long long>(1, nrow_tot)));
    // the molecules' device set-ups side by side: pairs point into the merged primitive array and carry
    // their molecule; prefix sums are relative to their block pair and copy unchanged
    for (int m = 0; m < nmol; ++m) {
        const CtxView v = ctx_view(b->mols[m]);
        if (v.npairs > 0) {
            BCU(cudaMemcpyAsync(b->d_pairs + pair0s[m], v.d_pairs, sizeof(ShellPair) * v.npairs, cudaMemcpyDeviceToDevice, b->stream));
            BCU(setup_offset_pairs(b->d_pairs + pair0s[m], v.npairs, prim0s[m], m, b->stream));
        }
        if (v.nprims > 0)
            BCU(cudaMemcpyAsync(b->d_prims + prim0s[m], v.d_prims, sizeof(PrimPair) * v.nprims, cudaMemcpyDeviceToDevice, b->stream));
        if (v.nrows > 0)
            BCU(cudaMemcpyAsync(b->d_prefix + row0s[m], v.d_prefix, sizeof(long long) * v.nrows, cudaMemcpyDeviceToDevice, b->stream));
    }
    BCU(cudaStreamSynchronize(b->stream));
    BCU(cudaMalloc(&b->d_nbf, sizeof(int) * nmol));
    BCU(cudaMalloc(&b->d_doff, sizeof(long long) * nmol));
    BCU(cudaMalloc(&b->d_poff, sizeof(long long) * nmol));
    BCU(cudaMalloc(&b->d_P, sizeof(double) * packed));
    BCU(cudaMalloc(&b->d_G, sizeof(double) * packed));
    BCU(cudaMalloc(&b->d_Pfull, sizeof(double) * dense));
    BCU(cudaMalloc(&b->d_T, sizeof(double) * dense));
    BCU(cudaMalloc(&b->d_tiles, sizeof(unsigned long long) * 2 * std::max<size_t>(1, b->launches.size())));
    BCU(cudaMemcpy(b->d_bps, bps.data(), sizeof(BlockPair) * bps.size(), cudaMemcpyHostToDevice));
    b->nbps = (int)bps.size();
    b->nrows = nrow_tot;
    BCU(cudaMemcpy(b->d_nbf, b->nbf.data(), sizeof(int) * nmol, cudaMemcpyHostToDevice));
    BCU(cudaMemcpy(b->d_doff, b->doff.data(), sizeof(long long) * nmol, cudaMemcpyHostToDevice));
    BCU(cudaMemcpy(b->d_poff, b->poff.data(), sizeof(long long) * nmol, cudaMemcpyHostToDevice));
    BCU(cudaMemset(b->d_P, 0, sizeof(double) * packed));
    *out = b;
    return UNOMOL_OK;
}

int unomol_gpu_batch_buffers(UnomolBatch* b, double** dP, double** dG, const long long** packed_offsets, int64_t* packed_total) {
    if (!b) return bfail(b, UNOMOL_EINVAL, "null batch");
    if (dP) *dP = b->d_P;
    if (dG) *dG = b->d_G;
    if (packed_offsets) *packed_offsets = b->poff.data();
    if (packed_total) *packed_total = b->packed_total;
    return UNOMOL_OK;
}

int unomol_gpu_batch_size(const UnomolBatch* b) { return b ? (int)b->mols.size() : UNOMOL_EINVAL; }

int unomol_gpu_batch_fock(UnomolBatch* b, int mode, void* stream) {
    if (!b) return bfail(b, UNOMOL_EINVAL, "null batch");
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    if (mode == UNOMOL_BATCH_GRAPH) {
        if (!b->graph) {
            cudaGraph_t g = nullptr;
            BCU(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            int rc = batch_build(b, b->stream);
            cudaError_t e = cudaStreamEndCapture(b->stream, &g);
            if (rc) return rc;
            BCU(e);
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            BCU(e);
        }
        if (s != b->stream) {  // order the graph after the caller's stream and back
            cudaEvent_t ev;
            BCU(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            BCU(cudaEventRecord(ev, s));
            BCU(cudaStreamWaitEvent(b->stream, ev, 0));
            BCU(cudaGraphLaunch(b->graph, b->stream));
            BCU(cudaEventRecord(ev, b->stream));
            BCU(cudaStreamWaitEvent(s, ev, 0));
            cudaEventDestroy(ev);
            return UNOMOL_OK;
        }
        BCU(cudaGraphLaunch(b->graph, b->stream));
        return UNOMOL_OK;
    }
    if (mode == UNOMOL_BATCH_LAUNCHES) return batch_build(b, s);
    if (mode == UNOMOL_BATCH_SEQUENTIAL) {  // one molecule after the other through the single-molecule path
        BCU(cudaMemsetAsync(b->d_G, 0, sizeof(double) * b->packed_total, s));
        for (size_t m = 0; m < b->mols.size(); ++m) {
            int rc = unomol_gpu_fock_rhf_device(b->mols[m], b->d_P + b->poff[m], b->d_G + b->poff[m], s);
            if (rc) return bfail(b, rc, unomol_gpu_last_error(b->mols[m]));
        }
        return UNOMOL_OK;
    }
    return bfail(b, UNOMOL_EINVAL, "unknown batch mode");
}

int unomol_gpu_batch_fock_device(UnomolBatch* b, const double* dP, double* dG, int mode, void* stream) {
    if (!b) return bfail(b, UNOMOL_EINVAL, "null batch");
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    if (dP && dP != b->d_P)
        BCU(cudaMemcpyAsync(b->d_P, dP, sizeof(double) * b->packed_total, cudaMemcpyDeviceToDevice, s));
    const int rc = unomol_gpu_batch_fock(b, mode, stream);
    if (rc) return rc;
    if (dG && dG != b->d_G)
        BCU(cudaMemcpyAsync(dG, b->d_G, sizeof(double) * b->packed_total, cudaMemcpyDeviceToDevice, s));
    return UNOMOL_OK;
}

// Autotuner: for every class launch, time each (CTA size, CTAs per SM) and keep the fastest; the
// CUDA graph is rebuilt on the next graph launch.  Uses the densities currently in the P buffer.
int unomol_gpu_batch_autotune(UnomolBatch* b, int reps, int* chosen) {
    if (!b) return bfail(b, UNOMOL_EINVAL, "null batch");
    if (reps <= 0) reps = 2;
    const int blocks[3] = {64, 128, 256};
    const int ctas[4] = {1, 2, 4, 8};
    cudaStream_t s = b->stream;
    int rc = batch_build(b, s);  // dense P in place
    if (rc) return rc;
    cudaEvent_t e0, e1;
    BCU(cudaEventCreate(&e0));
    BCU(cudaEventCreate(&e1));
    for (size_t k = 0; k < b->launches.size(); ++k) {
        BLaunch& L = b->launches[k];
        float best = 1e30f;
        int bb = L.block, bc = L.ctas_per_sm;
        for (int blk : blocks)
            for (int c : ctas) {
                float tot = 0.f;
                for (int r = 0; r < reps; ++r) {
                    BCU(cudaMemsetAsync(b->d_tiles + 2 * k, 0, sizeof(unsigned long long), s));
                    FockArgs A = batch_args(b, L, (int)k);
                    BCU(cudaEventRecord(e0, s));
                    BCU(launch_persistent(L.bc, L.kc, A, b->nt, b->rys, b->nsm * c, blk, s));
                    BCU(cudaEventRecord(e1, s));
                    BCU(cudaEventSynchronize(e1));
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    tot += ms;
                }
                if (tot < best) {
                    best = tot;
                    bb = blk;
                    bc = c;
                }
            }
        L.block = bb;
        L.ctas_per_sm = bc;
        if (chosen) {
            chosen[3 * k + 0] = L.bc * NTMPLCLASS + L.kc;
            chosen[3 * k + 1] = bb;
            chosen[3 * k + 2] = bc;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    BCU(cudaMemsetAsync(b->d_T, 0, sizeof(double) * b->dense_total, s));  // leave no partial sums
    BCU(cudaStreamSynchronize(s));
    return (int)b->launches.size();
}

int unomol_gpu_batch_set_density(UnomolBatch* b, const double* P) {
    if (!b || !P) return bfail(b, UNOMOL_EINVAL, "null argument");
    BCU(cudaMemcpyAsync(b->d_P, P, sizeof(double) * b->packed_total, cudaMemcpyHostToDevice, b->stream));
    BCU(cudaStreamSynchronize(b->stream));
    return UNOMOL_OK;
}

int unomol_gpu_batch_get_fock(UnomolBatch* b, double* G) {
    if (!b || !G) return bfail(b, UNOMOL_EINVAL, "null argument");
    BCU(cudaDeviceSynchronize());
    BCU(cudaMemcpy(G, b->d_G, sizeof(double) * b->packed_total, cudaMemcpyDeviceToHost));
    return UNOMOL_OK;
}

void unomol_gpu_batch_destroy(UnomolBatch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    dfree(b->d_pairs);
    dfree(b->d_prims);
    dfree(b->d_bps);
    dfree(b->d_prefix);
    dfree(b->d_nbf);
    dfree(b->d_doff);
    dfree(b->d_poff);
    dfree(b->d_P);
    dfree(b->d_G);
    dfree(b->d_Pfull);
    dfree(b->d_T);
    dfree(b->d_prims32);
    dfree(b->d_Pfull32);
    dfree(b->d_pmax);
    dfree(b->d_dmax);
    dfree(b->d_nshell);
    dfree(b->d_shell0);
    dfree(b->d_pmax_off);
    dfree(b->d_soff);
    dfree(b->d_sl);
    dfree(b->d_rowbp);
    dfree(b->d_mseg);
    for (long long** p : {&b->d_c64, &b->d_c32, &b->d_pre64, &b->d_pre32, &b->d_cnt64, &b->d_cnt32, &b->d_begin64,
                          &b->d_begin32, &b->d_total64, &b->d_total32})
        dfree(*p);
    dfree(b->d_launch_bp);
    dfree(b->d_tiles);
    for (UnomolCtx* c : b->mols) unomol_gpu_destroy(c);
    for (cudaEvent_t e : {b->fork, b->join[0], b->join[1]})
        if (e) cudaEventDestroy(e);
    for (cudaStream_t st : b->part_stream)
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

const char* unomol_gpu_batch_last_error(const UnomolBatch* b) {
    if (b && !b->err.empty()) return b->err.c_str();
    return g_batch_err.c_str();
}

}  // extern "C"
