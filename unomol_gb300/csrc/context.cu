// C ABI of the direct Fock build (include/unomol_gb300.h): the GPU counterpart of unomol's
// TwoElectronInts (TwoElectronInts.hpp:79-110).
//
// Setup (create / recalculate), on the device (setup.cu): shell pairs with their primitive-pair data are
// built and sorted into blocks of equal (pair class, primitive-pair count); the Schwarz diagonal
// (ab|ab) is computed; pairs are re-sorted by descending bound within their block; then for every pair
// of blocks the Schwarz "staircase" (bra i keeps the first n_i ket pairs) gives a compact work list per
// quartet class.  The host keeps the block boundaries and the block-pair list.
// Fock build (fock_rhf / fock_uhf): expand packed P to a dense N x N copy, zero the accumulators,
// launch one kernel per quartet class (classes alternating over two streams forked from the build's
// stream; in the mixed-precision build both parts of a class in one launch), fold G += T + T^T into
// packed storage.
#include <algorithm>
#include <climits>
#include <memory>
#include <mutex>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/unomol_gb300.h"
#include "ctx_view.h"
#include "fock_dispatch.cuh"
#include "fock_kernels.cuh"
#include "setup.h"
#include "store.h"
#include "worklists.h"

using namespace ugb;

namespace {

thread_local std::string g_last_error;

struct ClassLaunch {
    int bc, kc;          // bra / ket pair classes
    int bp_begin, nbp;   // range in the block-pair array
    long long nwork;     // padded work items
    long long quartets;  // unpadded
};

}  // namespace

struct UnomolCtx {
    int dev = 0;
    int nsm = 1;  // SMs of the device
    cudaStream_t stream = nullptr;
    int nshell = 0, nbf = 0, ncen = 0, start_shell = 0, maxl = 0;
    std::vector<int> sl, snp, scen, soff, sprim;
    std::vector<double> alpha, coef, centers;
    NormTable nt{};
    // host side of the setup: block boundaries and keys, block pairs, class launches
    int npairs = 0;
    long long nprims = 0, nrows = 0;
    std::vector<int> block_begin, block_count, block_class, block_nprim;
    std::vector<char> block_new;
    std::vector<BlockPair> bps;
    std::vector<ClassLaunch> launches;
    std::vector<int> launch_bp;
    // the basis on the device (centres refreshed by recalculate) and the setup's scratch
    int *d_snp = nullptr, *d_scen = nullptr, *d_sprim = nullptr;
    double *d_alpha = nullptr, *d_coef = nullptr, *d_centers = nullptr;
    char* d_ws = nullptr;
    size_t ws_bytes = 0;
    // device memory in four allocations: the basis (status flag, shell arrays, exponents, coefficients,
    // centres); the pair records (ShellPair, PrimPair, PrimPair32); the work lists (block pairs,
    // staircase prefix sums, per-build row lists); the setup's scratch (d_ws).  The arrays below point
    // into them; the pair and list allocations are kept while the next setup fits.
    char* d_basis = nullptr;
    char* d_setup = nullptr;
    size_t setup_bytes = 0;
    char* d_lists = nullptr;
    size_t lists_bytes = 0;
    // per-build work lists of the density-screened / mixed-precision build
    int *d_rowbp = nullptr, *d_mseg = nullptr;
    long long *d_c64 = nullptr, *d_c32 = nullptr, *d_pre64 = nullptr, *d_pre32 = nullptr;
    long long *d_cnt64 = nullptr, *d_cnt32 = nullptr;
    long long *d_begin64 = nullptr, *d_begin32 = nullptr, *d_total64 = nullptr, *d_total32 = nullptr;
    int* d_launch_bp = nullptr;  // per class launch: first block pair, block pairs
    float* d_dmax = nullptr;
    double skip_cut = 1e-13;
    // device buffers
    ShellPair* d_pairs = nullptr;
    PrimPair* d_prims = nullptr;
    PrimPair32* d_prims32 = nullptr;
    BlockPair* d_bps = nullptr;
    long long* d_prefix = nullptr;
    double* d_rys = nullptr;
    float* d_rys32 = nullptr;
    double *d_Pa = nullptr, *d_Pb = nullptr, *d_Ta = nullptr, *d_Tb = nullptr;
    double *d_Ga = nullptr, *d_Gb = nullptr, *d_pk_a = nullptr, *d_pk_b = nullptr;
    float* d_pmax = nullptr;
    float *d_Pa32 = nullptr, *d_Pb32 = nullptr;
    int *d_soff = nullptr, *d_sl = nullptr;
    int* d_status = nullptr;
    unsigned long long* d_counters = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // mixed builds: the FP64 and the FP32 parts on two side streams forked from and joined back into
    // the build's stream, so that the two kinds of kernels (FP64 pipe / FP32 pipe and loads) share the SMs
    cudaStream_t part_stream[3] = {nullptr, nullptr, nullptr};  // FP64 part, FP32 part, second plain stream
    cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};
    // options
    double schwarz_cut = STORE_CUT;
    int prec_mode = UNOMOL_PREC_FP64;
    int rys_mode = UNOMOL_RYS_REFERENCE;
    int eri_method = UNOMOL_ERI_REFERENCE;
    int counting = 0;
    int reverse_launches = 0;  // class launches in reverse order (unomol_gpu_set_launch_order)
    double fp32_cut = 1e-10;
    // conventional build: the stored integral matrix (store.cu); while set, Fock builds stream it
    ugb::IntStore* store = nullptr;
    UnomolStats stats{};
    std::string err;
};

namespace {

int fail(UnomolCtx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    g_last_error = msg;
    return code;
}

#define CU(call)                                                                                \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? UNOMOL_ENOMEM : UNOMOL_ECUDA,    \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                    \
    } while (0)

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// Component normalisation 1/sqrt(d(lx) d(ly) d(lz)) with the double-factorial table of
// AuxFunctions.hpp:48-63, kept exactly as the reference builds it (d = 1, 1, 3, 45, 4725 for
// l = 0..4; the l >= 3 entries differ from (2l-1)!!, which only matters for f and g shells).
void build_norms(NormTable& nt) {
    double dfact[5];
    dfact[0] = 1.0;
    double dx = 1.0;
    for (int i = 1; i < 5; ++i) {
        dfact[i] = dfact[i - 1] * dx;
        dx *= (2 * i + 1);
    }
    for (int l = 0; l <= LMAX; ++l)
        for (int c = 0; c < ncart(l); ++c) {
            nt.v[l][c] = 1.0 / std::sqrt(dfact[cart_lx(l, c)] * dfact[cart_ly(l, c)] * dfact[cart_lz(l, c)]);
            nt.f[l][c] = (float)nt.v[l][c];
        }
}

// Algorithmic flops of the Rys kernels (FMA = 2, every +,-,*,/,sqrt = 1), counted from the steps of
// fock_kernels.cuh.  Per primitive quartet past the prefactor cut: setup 20; Rys nodes and weights
// NR * (2 polynomials * deg Horner steps * 2) + 3, deg = the table degree of the precision (RYS_DEG
// for FP64, RYS32_DEG for FP32); per root 10 for B00, B1, B1', then per axis 4 for C, C', the 2D
// recurrence, the two horizontal transfers (2 per step), and 3 per function quartet for the product
// and accumulation; (ss|ss) evaluates only the weight and one FMA.  Per shell quartet: 17 per function
// quartet for normalisation and the six density contractions.
double flops_per_prim(int la, int lb, int lc, int ld, bool fp32 = false) {
    const int L12 = la + lb, L34 = lc + ld, NR = (L12 + L34) / 2 + 1;
    const int NF = ncart(la) * ncart(lb) * ncart(lc) * ncart(ld);
    double vrr = 0;
    if (L12 > 0) vrr += 1;
    for (int i = 1; i < L12; ++i) vrr += 4;
    for (int j = 0; j < L34; ++j)
        for (int i = 0; i <= L12; ++i) vrr += 1 + (j > 0 ? 3 : 0) + (i > 0 ? 3 : 0);
    double hrr = 0;
    for (int b = 1; b <= lb; ++b) hrr += 2.0 * (L12 - b + 1) * (L34 + 1);
    for (int d = 1; d <= ld; ++d) hrr += 2.0 * (la + 1) * (lb + 1) * (L34 - d + 1);
    if (L12 + L34 == 0)  // (ss|ss): the weight F0(T) alone (FP64: one table polynomial; FP32: the closed
                         // form, rsqrt, erf and two products) and one FMA into the integral
        return 20 + (fp32 ? 5.0 : 2.0 * RYS_DEG + 3) + 2;
    const double roots = 2.0 * (fp32 ? RYS32_DEG : RYS_DEG) * 2.0;
    return 20 + NR * roots + 3 + NR * (10 + 3 * (4 + vrr + hrr) + 3.0 * NF);
}
double flops_per_quartet(int la, int lb, int lc, int ld) {
    return 17.0 * ncart(la) * ncart(lb) * ncart(lc) * ncart(ld);
}

// Bump allocation of several arrays in one device buffer (256-byte aligned pieces); a pass with no
// buffer only adds up the sizes (and gives the offsets).
struct Carve {
    char* base = nullptr;
    size_t used = 0;
    size_t next(size_t bytes) {
        const size_t off = (used + 255) & ~size_t(255);
        used = off + std::max<size_t>(bytes, 1);
        return off;
    }
    template <typename T>
    T* take(size_t n) {
        const size_t off = next(sizeof(T) * n);
        return base ? reinterpret_cast<T*>(base + off) : nullptr;
    }
};

// One allocation of at least `bytes`, kept while it is large enough.  Callers make sure that no work
// still reads the old buffer (cudaFree would wait for the whole device anyway).
int ensure_arena(UnomolCtx* ctx, char*& buf, size_t& cap, size_t bytes) {
    if (buf && bytes <= cap) return UNOMOL_OK;
    dfree(buf);
    cap = 0;
    CU(cudaMalloc(&buf, bytes));
    cap = bytes;
    return UNOMOL_OK;
}

int ensure_ws(UnomolCtx* ctx, size_t bytes) {
    if (bytes > ctx->ws_bytes) CU(cudaStreamSynchronize(ctx->stream));  // nothing may still use the old scratch
    return ensure_arena(ctx, ctx->d_ws, ctx->ws_bytes, bytes);
}

ShellsDev shells_dev(const UnomolCtx* ctx) {
    ShellsDev sh;
    sh.nshell = ctx->nshell;
    sh.start_shell = ctx->start_shell;
    sh.sl = ctx->d_sl;
    sh.snp = ctx->d_snp;
    sh.scen = ctx->d_scen;
    sh.soff = ctx->d_soff;
    sh.sprim = ctx->d_sprim;
    sh.alpha = ctx->d_alpha;
    sh.coef = ctx->d_coef;
    sh.centers = ctx->d_centers;
    return sh;
}

// Work lists for the current Schwarz cutoff: the block-pair list on the host (a size set by the number
// of blocks), the staircase of every bra row on the device, one read-back of the per-block-pair totals.
int build_worklists(UnomolCtx* ctx) {
    cudaStream_t s = ctx->stream;
    CU(cudaDeviceSynchronize());  // builds still in flight (on any stream) read the lists rewritten here
    ctx->bps.clear();
    ctx->launches.clear();
    const int nb = (int)ctx->block_begin.size();
    std::vector<BlockPair> all;
    std::vector<int> all_x, all_y;
    long long nrows = 0;
    int64_t total_quartets = 0;
    for (int X = 0; X < nb; ++X)
        for (int Y = 0; Y <= X; ++Y) {
            if (ctx->start_shell > 0 && !ctx->block_new[X] && !ctx->block_new[Y]) continue;
            BlockPair bp{};
            bp.bra_begin = ctx->block_begin[X];
            bp.bra_count = ctx->block_count[X];
            bp.ket_begin = ctx->block_begin[Y];
            bp.ket_count = ctx->block_count[Y];
            bp.triangle = (X == Y);
            bp.prefix_off = (int)std::min<long long>(nrows, INT_MAX);
            nrows += bp.bra_count + 1;
            total_quartets += bp.triangle ? (int64_t)bp.bra_count * (bp.bra_count + 1) / 2
                                          : (int64_t)bp.bra_count * bp.ket_count;
            all.push_back(bp);
            all_x.push_back(X);
            all_y.push_back(Y);
        }
    if (nrows >= INT_MAX) return fail(ctx, UNOMOL_EINVAL, "too many staircase rows for one context");
    ctx->nrows = nrows;
    const int nall = (int)all.size();
    size_t t_scan = 0;
    CU(setup_inclusive_sum(nullptr, t_scan, nullptr, nullptr, (int)std::max<long long>(1, nrows), s));
    auto carve = [&](Carve& w, BlockPair*& d_all, long long*& S, long long*& totals, char*& tmp) {
        d_all = w.take<BlockPair>(nall);
        S = w.take<long long>(nrows);
        totals = w.take<long long>(nall);
        tmp = w.take<char>(t_scan);
    };
    BlockPair* d_all;
    long long *S, *totals;
    char* tmp;
    Carve sizing;
    carve(sizing, d_all, S, totals, tmp);
    int rc = ensure_ws(ctx, sizing.used);
    if (rc) return rc;
    Carve w;
    w.base = ctx->d_ws;
    carve(w, d_all, S, totals, tmp);
    // the lists allocation, sized for every block pair being non-empty
    {
        auto lists = [&](Carve& c) {
            ctx->d_bps = c.take<BlockPair>(nall);
            ctx->d_cnt64 = c.take<long long>(nall);
            ctx->d_cnt32 = c.take<long long>(nall);
            ctx->d_prefix = c.take<long long>(nrows);
            ctx->d_c64 = c.take<long long>(nrows);
            ctx->d_c32 = c.take<long long>(nrows);
            ctx->d_pre64 = c.take<long long>(nrows);
            ctx->d_pre32 = c.take<long long>(nrows);
            ctx->d_rowbp = c.take<int>(nrows);
            ctx->d_mseg = c.take<int>(nrows);
            ctx->d_begin64 = c.take<long long>(nall);
            ctx->d_begin32 = c.take<long long>(nall);
            ctx->d_total64 = c.take<long long>(NPAIRCLASS * NPAIRCLASS);
            ctx->d_total32 = c.take<long long>(NPAIRCLASS * NPAIRCLASS);
            ctx->d_launch_bp = c.take<int>(2 * NPAIRCLASS * NPAIRCLASS);
        };
        Carve lay;
        lists(lay);
        rc = ensure_arena(ctx, ctx->d_lists, ctx->lists_bytes, lay.used);
        if (rc) return rc;
        Carve c;
        c.base = ctx->d_lists;
        lists(c);
    }
    std::vector<long long> tot(nall);
    if (nall > 0) {
        CU(cudaMemcpyAsync(d_all, all.data(), sizeof(BlockPair) * nall, cudaMemcpyHostToDevice, s));
        CU(setup_staircase(d_all, nall, ctx->d_pairs, ctx->schwarz_cut, ctx->d_prefix, s));
        size_t tb = t_scan;
        CU(setup_inclusive_sum(tmp, tb, ctx->d_prefix, S, (int)nrows, s));
        CU(setup_prefix_fix(d_all, nall, S, ctx->d_prefix, totals, s));
        CU(cudaMemcpyAsync(tot.data(), totals, sizeof(long long) * nall, cudaMemcpyDeviceToHost, s));
    }
    CU(cudaStreamSynchronize(s));
    // non-empty block pairs grouped by quartet class, work ranges 32-aligned (warps never straddle)
    int64_t screened = 0, fq = 0, prim_q = 0;
    std::vector<std::vector<BlockPair>> per_class(NPAIRCLASS * NPAIRCLASS);
    for (int k = 0; k < nall; ++k) {
        if (tot[k] == 0) continue;
        BlockPair bp = all[k];
        bp.work_count = tot[k];
        const int X = all_x[k], Y = all_y[k];
        const int bc = ctx->block_class[X], kc = ctx->block_class[Y];
        const int nfq = ncart(pc_la(bc)) * ncart(pc_lb(bc)) * ncart(pc_la(kc)) * ncart(pc_lb(kc));
        screened += tot[k];
        fq += tot[k] * nfq;
        prim_q += tot[k] * (int64_t)ctx->block_nprim[X] * ctx->block_nprim[Y];
        bp.prim_quartets = ctx->block_nprim[X] * ctx->block_nprim[Y];
        per_class[bc * NPAIRCLASS + kc].push_back(bp);
    }
    for (int cls = 0; cls < NPAIRCLASS * NPAIRCLASS; ++cls) {
        auto& v = per_class[cls];
        if (v.empty()) continue;
        // the costliest quartets first: a launch's CTAs start in grid order, so the block pairs whose
        // quartets carry the most primitive quartets (up to 36 x 36) no longer end the launch on a few
        // SMs while the rest are idle
        std::stable_sort(v.begin(), v.end(),
                         [](const BlockPair& x, const BlockPair& y) { return x.prim_quartets > y.prim_quartets; });
        ClassLaunch L{};
        L.bc = cls / NPAIRCLASS;
        L.kc = cls % NPAIRCLASS;
        L.bp_begin = (int)ctx->bps.size();
        L.nbp = (int)v.size();
        long long wk = 0;
        for (auto& bp : v) {
            bp.work_begin = wk;
            wk += (bp.work_count + 31) / 32 * 32;
            L.quartets += bp.work_count;
            ctx->bps.push_back(bp);
        }
        L.nwork = wk;
        ctx->launches.push_back(L);
    }
    ctx->stats.shell_quartets = screened;
    ctx->stats.shell_quartets_total = total_quartets;
    ctx->stats.primitive_quartets = prim_q;
    ctx->stats.function_quartets = fq;
    if (!ctx->bps.empty()) {
        const size_t nbp = ctx->bps.size();
        CU(cudaMemcpyAsync(ctx->d_bps, ctx->bps.data(), sizeof(BlockPair) * nbp, cudaMemcpyHostToDevice, s));
        // row -> block pair map (-1 on the end-of-block-pair entries and on the rows of empty block pairs)
        // and the per-build work-list buffers of the density-screened build
        const size_t nr = (size_t)nrows;
        CU(cudaMemsetAsync(ctx->d_rowbp, 0xff, sizeof(int) * nr, s));
        CU(setup_row_bp(ctx->d_bps, (int)nbp, ctx->d_rowbp, s));
        ctx->launch_bp.clear();
        for (const ClassLaunch& L : ctx->launches) {
            ctx->launch_bp.push_back(L.bp_begin);
            ctx->launch_bp.push_back(L.nbp);
        }
        CU(cudaMemcpyAsync(ctx->d_launch_bp, ctx->launch_bp.data(), sizeof(int) * ctx->launch_bp.size(), cudaMemcpyHostToDevice, s));
        CU(cudaMemsetAsync(ctx->d_c64, 0, sizeof(long long) * nr, s));
        CU(cudaMemsetAsync(ctx->d_c32, 0, sizeof(long long) * nr, s));
        CU(cudaMemsetAsync(ctx->d_mseg, 0, sizeof(int) * nr, s));
    }
    CU(cudaStreamSynchronize(s));
    return UNOMOL_OK;
}

// Pairs, Schwarz bounds, block structure and work lists for the current geometry, built on the device.
int build_setup(UnomolCtx* ctx) {
    cudaStream_t s = ctx->stream;
    CU(cudaDeviceSynchronize());  // builds still in flight (on any stream) read the pairs rewritten here
    const int ns = ctx->nshell;
    const long long np64 = (long long)ns * (ns + 1) / 2;
    if (np64 > (1ll << 28)) return fail(ctx, UNOMOL_EINVAL, "too many shell pairs for one context");
    const int P = (int)np64;
    long long nprims = 0;
    for (int i = 0; i < ns; ++i)
        for (int j = 0; j <= i; ++j)
            nprims += i == j ? (long long)ctx->snp[i] * (ctx->snp[i] + 1) / 2 : (long long)ctx->snp[i] * ctx->snp[j];
    if (nprims >= INT_MAX) return fail(ctx, UNOMOL_EINVAL, "too many primitive pairs for one context");
    ctx->npairs = P;
    ctx->nprims = nprims;
    ctx->stats.npairs = P;
    CU(cudaMemcpyAsync(ctx->d_centers, ctx->centers.data(), sizeof(double) * 3 * ctx->ncen, cudaMemcpyHostToDevice, s));
    {
        auto recs = [&](Carve& c) {
            ctx->d_pairs = c.take<ShellPair>(P);
            ctx->d_prims = c.take<PrimPair>(nprims);
            ctx->d_prims32 = c.take<PrimPair32>(nprims);
        };
        Carve lay;
        recs(lay);
        const int rc = ensure_arena(ctx, ctx->d_setup, ctx->setup_bytes, lay.used);
        if (rc) return rc;
        Carve c;
        c.base = ctx->d_setup;
        recs(c);
    }
    // library scratch sizes (the segmented sort's for the largest possible number of blocks)
    size_t t_scan = 0, t_sort = 0, t_rle = 0, t_seg = 0;
    CU(setup_exclusive_sum(nullptr, t_scan, nullptr, nullptr, P, s));
    CU(setup_sort_keys(nullptr, t_sort, nullptr, nullptr, nullptr, nullptr, P, s));
    CU(setup_run_length(nullptr, t_rle, nullptr, nullptr, nullptr, nullptr, P, s));
    CU(setup_sort_desc_segments(nullptr, t_seg, nullptr, nullptr, nullptr, nullptr, P, P, nullptr, nullptr, s));
    const size_t t_max = std::max(std::max(t_scan, t_sort), std::max(t_rle, t_seg));
    struct Arrays {
        unsigned *key0, *key1, *uniq;
        int *np, *poff, *iota, *perm1, *perm2, *counts, *nruns, *seg;
        ShellPair *raw, *sorted1;
        double *q, *q2;
        unsigned long long* qbits;
        PrimPair* prims_c;      // primitive pairs in canonical order (before the interleave by block)
        PrimPair32* prims32_c;
        int *bbegin, *bcount;
        long long* bprim;
        char* tmp;
    } a{};
    auto carve = [&](Carve& w) {
        a.key0 = w.take<unsigned>(P);
        a.key1 = w.take<unsigned>(P);
        a.uniq = w.take<unsigned>(P);
        a.np = w.take<int>(P);
        a.poff = w.take<int>(P);
        a.iota = w.take<int>(P);
        a.perm1 = w.take<int>(P);
        a.perm2 = w.take<int>(P);
        a.counts = w.take<int>(P);
        a.nruns = w.take<int>(1);
        a.seg = w.take<int>((size_t)P + 1);
        a.raw = w.take<ShellPair>(P);
        a.sorted1 = w.take<ShellPair>(P);
        a.q = w.take<double>(P);
        a.q2 = w.take<double>(P);
        a.qbits = w.take<unsigned long long>(P);
        a.prims_c = w.take<PrimPair>(nprims);
        a.prims32_c = w.take<PrimPair32>(nprims);
        a.bbegin = w.take<int>(P);
        a.bcount = w.take<int>(P);
        a.bprim = w.take<long long>(P);
        a.tmp = w.take<char>(t_max);
    };
    Carve sizing;
    carve(sizing);
    int rc = ensure_ws(ctx, sizing.used);
    if (rc) return rc;
    Carve w;
    w.base = ctx->d_ws;
    carve(w);
    // pairs in canonical order, their primitive pairs, and the sort by (class, new/old, primitive pairs)
    const ShellsDev sh = shells_dev(ctx);
    size_t tb = t_max;
    CU(setup_pair_keys(sh, P, a.key0, a.np, a.iota, s));
    CU(setup_exclusive_sum(a.tmp, tb, a.np, a.poff, P, s));
    CU(setup_build_pairs(sh, P, a.poff, a.raw, a.prims_c, a.prims32_c, s));
    tb = t_max;
    CU(setup_sort_keys(a.tmp, tb, a.key0, a.key1, a.iota, a.perm1, P, s));
    tb = t_max;
    CU(setup_run_length(a.tmp, tb, a.key1, a.uniq, a.counts, a.nruns, P, s));
    CU(setup_gather_pairs(a.raw, a.perm1, nullptr, P, a.sorted1, s));
    // block boundaries and keys to the host
    int nb = 0;
    const int head = std::min(P, 4096);
    std::vector<unsigned> ukeys(head);
    std::vector<int> ucnt(head);
    CU(cudaMemcpyAsync(&nb, a.nruns, sizeof(int), cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(ukeys.data(), a.uniq, sizeof(unsigned) * head, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(ucnt.data(), a.counts, sizeof(int) * head, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    if (nb < 1 || nb > P) return fail(ctx, UNOMOL_ECUDA, "shell-pair sort returned no blocks");
    if (nb > head) {
        ukeys.resize(nb);
        ucnt.resize(nb);
        CU(cudaMemcpyAsync(ukeys.data(), a.uniq, sizeof(unsigned) * nb, cudaMemcpyDeviceToHost, s));
        CU(cudaMemcpyAsync(ucnt.data(), a.counts, sizeof(int) * nb, cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
    }
    ctx->block_begin.clear();
    ctx->block_count.clear();
    ctx->block_class.clear();
    ctx->block_nprim.clear();
    ctx->block_new.clear();
    std::vector<int> seg(nb + 1);
    int off = 0;
    for (int k = 0; k < nb; ++k) {
        seg[k] = off;
        ctx->block_begin.push_back(off);
        ctx->block_count.push_back(ucnt[k]);
        ctx->block_class.push_back((int)pair_key_class(ukeys[k]));
        ctx->block_new.push_back((char)pair_key_new(ukeys[k]));
        ctx->block_nprim.push_back((int)pair_key_nprim(ukeys[k]));
        off += ucnt[k];
    }
    seg[nb] = off;
    if (off != P) return fail(ctx, UNOMOL_ECUDA, "shell-pair blocks do not cover the pairs");
    // Schwarz diagonal, one launch per class run of the class-sorted pairs
    for (int k = 0; k < nb;) {
        int k2 = k;
        while (k2 < nb && ctx->block_class[k2] == ctx->block_class[k]) ++k2;
        const int cls = ctx->block_class[k], begin = ctx->block_begin[k];
        const int count = ctx->block_begin[k2 - 1] + ctx->block_count[k2 - 1] - begin;
        if (cls < NTMPLCLASS)
            CU(launch_schwarz(cls, a.sorted1, a.prims_c, begin, count, ctx->nt, ctx->d_rys, a.q, s));
        else
            CU(launch_schwarz_high(pc_la(cls), pc_lb(cls), a.sorted1, a.prims_c, begin, count, ctx->nt, ctx->d_rys, a.q,
                                   a.qbits, s));
        k = k2;
    }
    // descending bound inside every block (stable: equal bounds keep the canonical order)
    size_t t_need = 0;
    CU(setup_sort_desc_segments(nullptr, t_need, nullptr, nullptr, nullptr, nullptr, P, nb, nullptr, nullptr, s));
    if (t_need > t_max) return fail(ctx, UNOMOL_ECUDA, "segmented sort needs more scratch than reserved");
    CU(cudaMemcpyAsync(a.seg, seg.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, s));
    tb = t_max;
    CU(setup_sort_desc_segments(a.tmp, tb, a.q, a.q2, a.iota, a.perm2, P, nb, a.seg, a.seg + 1, s));
    CU(setup_gather_pairs(a.sorted1, a.perm2, a.q2, P, ctx->d_pairs, s));
    // primitive pairs interleaved by block in the final order: adjacent pairs, adjacent records
    {
        std::vector<long long> bprim(nb);
        long long o = 0;
        for (int k = 0; k < nb; ++k) {
            bprim[k] = o;
            o += (long long)ctx->block_count[k] * ctx->block_nprim[k];
        }
        if (o != nprims) return fail(ctx, UNOMOL_ECUDA, "primitive pairs of the blocks do not add up");
        CU(cudaMemcpyAsync(a.bbegin, ctx->block_begin.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, s));
        CU(cudaMemcpyAsync(a.bcount, ctx->block_count.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, s));
        CU(cudaMemcpyAsync(a.bprim, bprim.data(), sizeof(long long) * nb, cudaMemcpyHostToDevice, s));
        CU(setup_interleave_prims(ctx->d_pairs, P, a.bbegin, a.bcount, a.bprim, nb, a.prims_c, a.prims32_c, ctx->d_prims,
                                  ctx->d_prims32, s));
        CU(cudaStreamSynchronize(s));  // the host arrays above are copied from pageable memory
    }
    return build_worklists(ctx);
}

// packed lower triangle -> dense symmetric N x N
__global__ void expand_packed(const double* __restrict__ pk, double* __restrict__ full, int n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * n) return;
    const int i = (int)(t / n), j = (int)(t % n);
    const int hi = i > j ? i : j, lo = i > j ? j : i;
    full[t] = pk[(long long)hi * (hi + 1) / 2 + lo];
}

// G_packed[ij] += T[i][j] + T[j][i]
__global__ void fold_packed(const double* __restrict__ T, double* __restrict__ G, int n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n2 = (long long)n * (n + 1) / 2;
    if (t >= n2) return;
    // invert t = i(i+1)/2 + j
    int i = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((long long)i * (i + 1) / 2 > t) --i;
    while ((long long)(i + 1) * (i + 2) / 2 <= t) ++i;
    const int j = (int)(t - (long long)i * (i + 1) / 2);
    G[t] += T[(long long)i * n + j] + T[(long long)j * n + i];
}

int ensure_density_buffers(UnomolCtx* ctx, bool uhf) {
    const size_t n2 = (size_t)ctx->nbf * ctx->nbf;
    const size_t np = (size_t)ctx->nbf * (ctx->nbf + 1) / 2;
    if (!ctx->d_Pa) {
        CU(cudaMalloc(&ctx->d_Pa, n2 * sizeof(double)));
        CU(cudaMalloc(&ctx->d_Ta, n2 * sizeof(double)));
        CU(cudaMalloc(&ctx->d_Ga, np * sizeof(double)));
        CU(cudaMalloc(&ctx->d_pk_a, np * sizeof(double)));
    }
    if (uhf && !ctx->d_Pb) {
        CU(cudaMalloc(&ctx->d_Pb, n2 * sizeof(double)));
        CU(cudaMalloc(&ctx->d_Tb, n2 * sizeof(double)));
        CU(cudaMalloc(&ctx->d_Gb, np * sizeof(double)));
        CU(cudaMalloc(&ctx->d_pk_b, np * sizeof(double)));
    }
    if (ctx->prec_mode == UNOMOL_PREC_MIXED) {
        if (!ctx->d_Pa32) CU(cudaMalloc(&ctx->d_Pa32, n2 * sizeof(float)));
        if (uhf && !ctx->d_Pb32) CU(cudaMalloc(&ctx->d_Pb32, n2 * sizeof(float)));
    }
    return UNOMOL_OK;
}

// One class launch with the reference's choice of integral method (TwoElectronInts.cpp:658-666): MD
// for la+lb+lc+ld > 8 and for every class in the MD mode; otherwise Rys, by the templated kernels for
// the s/p/d classes they cover and by the runtime-L kernel for the rest.
static cudaError_t launch_class_kernel(const UnomolCtx* ctx, const ClassLaunch& L, bool uhf, bool fp32, const FockArgs& A,
                                       cudaStream_t s) {
    const int la = pc_la(L.bc), lb = pc_lb(L.bc), lc = pc_la(L.kc), ld = pc_lb(L.kc);
    if (ctx->eri_method == UNOMOL_ERI_MD || la + lb + lc + ld > 8) return launch_fock_md(la, lb, lc, ld, uhf, A, ctx->nt, s);
    if (L.bc < NTMPLCLASS && L.kc < NTMPLCLASS)
        return fp32 ? launch_fock_fp32(L.bc, L.kc, uhf, A, ctx->nt, ctx->d_rys32, s)
                    : launch_fock_fp64(L.bc, L.kc, uhf, A, ctx->nt, ctx->d_rys, s);
    return launch_fock_generic(la, lb, lc, ld, uhf, fp32, A, ctx->nt, ctx->d_rys, ctx->d_rys32, s);
}

// Fock build from the stored integral matrix (unomol_gpu_store_integrals / _store_records).
int store_build(UnomolCtx* ctx, const double* dPa, const double* dPb, double* dGa, double* dGb, cudaStream_t s) {
    if (dPb && store_kind(ctx->store) != UNOMOL_STORE_UHF)
        return fail(ctx, UNOMOL_EINVAL, "UHF build on an RHF store: store the integrals with UNOMOL_STORE_UHF");
    int launches = 0;
    CU(cudaEventRecord(ctx->ev[0], s));
    CU(cudaEventRecord(ctx->ev[1], s));
    CU(store_fock(ctx->store, dPa, dPb, dGa, dGb, s, &launches));
    CU(cudaEventRecord(ctx->ev[2], s));
    CU(cudaEventRecord(ctx->ev[3], s));
    ctx->stats.kernel_launches = launches;
    return UNOMOL_OK;
}

// The Fock build proper: packed device P in, packed device G added into.
int fock_device(UnomolCtx* ctx, const double* dPa, const double* dPb, double* dGa, double* dGb, cudaStream_t s) {
    if (ctx->store) return store_build(ctx, dPa, dPb, dGa, dGb, s);
    const bool uhf = dPb != nullptr;
    int rc = ensure_density_buffers(ctx, uhf);
    if (rc) return rc;
    const int n = ctx->nbf;
    const long long n2 = (long long)n * n, np = (long long)n * (n + 1) / 2;
    int launches = 0;
    CU(cudaEventRecord(ctx->ev[0], s));
    expand_packed<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(dPa, ctx->d_Pa, n);
    ++launches;
    if (uhf) {
        expand_packed<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(dPb, ctx->d_Pb, n);
        ++launches;
    }
    CU(cudaMemsetAsync(ctx->d_Ta, 0, n2 * sizeof(double), s));
    if (uhf) CU(cudaMemsetAsync(ctx->d_Tb, 0, n2 * sizeof(double), s));
    CU(cudaGetLastError());
    CU(cudaEventRecord(ctx->ev[1], s));
    FockArgs A{};
    A.pairs = ctx->d_pairs;
    A.prims = ctx->d_prims;
    A.prims32 = ctx->d_prims32;
    A.nbf = n;
    A.Pa = ctx->d_Pa;
    A.Pb = uhf ? ctx->d_Pb : nullptr;
    A.Ta = ctx->d_Ta;
    A.Tb = uhf ? ctx->d_Tb : nullptr;
    A.thr_int = STORE_CUT;
    A.prim_cut = PRIM_CUT;
    A.thr_int32 = (float)STORE_CUT;
    A.prim_cut32 = (float)PRIM_CUT;
    A.fp32_cut = ctx->fp32_cut;
    A.nshell = ctx->nshell;
    A.rys_compat = ctx->rys_mode == UNOMOL_RYS_REFERENCE;
    A.pmax = ctx->d_pmax;
    A.status = ctx->d_status;
    const bool mixed = ctx->prec_mode == UNOMOL_PREC_MIXED;
    if (mixed && !ctx->bps.empty()) {
        // this build's work lists: density bound per shell-pair block, split of every staircase row
        // into FP64 / FP32 / skipped segments, scan per block pair (all on the device, no host sync)
        if (!ctx->d_pmax) CU(cudaMalloc(&ctx->d_pmax, sizeof(float) * ctx->nshell * ctx->nshell));
        if (!ctx->d_dmax) CU(cudaMalloc(&ctx->d_dmax, sizeof(float)));
        A.pmax = ctx->d_pmax;
        CU(cudaMemsetAsync(ctx->d_dmax, 0, sizeof(float), s));
        CU(wl_shell_pmax(ctx->d_Pa, A.Pb, ctx->d_soff, ctx->d_sl, ctx->nshell, n, ctx->d_pmax, ctx->d_dmax, s));
        CU(wl_split_rows(ctx->d_pairs, ctx->d_bps, ctx->d_rowbp, ctx->d_prefix, ctx->nrows, ctx->d_dmax,
                         std::max(ctx->fp32_cut, ctx->skip_cut), ctx->skip_cut, ctx->d_c64, ctx->d_c32, ctx->d_mseg, s));
        CU(wl_scan_rows(ctx->d_bps, (int)ctx->bps.size(), ctx->d_c64, ctx->d_c32, ctx->d_pre64, ctx->d_pre32, ctx->d_cnt64,
                        ctx->d_cnt32, s));
        CU(wl_scan_launches(ctx->d_launch_bp, (int)ctx->launches.size(), ctx->d_cnt64, ctx->d_cnt32, ctx->d_begin64,
                            ctx->d_begin32, ctx->d_total64, ctx->d_total32, s));
        launches += 4;
        A.dmax = ctx->d_dmax;
        A.skip_cut = ctx->skip_cut;
        A.skip_cut32 = (float)ctx->skip_cut;
        A.fp32_cut32 = ctx->fp32_cut > ctx->skip_cut ? (float)ctx->fp32_cut : 0.f;  // per-quartet FP32 choice (fused kernel)
        A.dyn_mseg = ctx->d_mseg;
        CU(wl_to_float(ctx->d_Pa, ctx->d_Pa32, n2, s));
        A.Pa32 = ctx->d_Pa32;
        if (uhf) {
            CU(wl_to_float(ctx->d_Pb, ctx->d_Pb32, n2, s));
            A.Pb32 = ctx->d_Pb32;
        }
    }
    const int ncls = NPAIRCLASS * NPAIRCLASS;
    A.counters = nullptr;
    if (ctx->counting) {
        // per class and part, 32 slots each: primitive quartets (FP64, FP32), screened quartets (FP64, FP32),
        // quartets of the FP64 part's lists run in FP32
        if (!ctx->d_counters) CU(cudaMalloc(&ctx->d_counters, sizeof(unsigned long long) * 5 * ncls * 32));
        CU(cudaMemsetAsync(ctx->d_counters, 0, sizeof(unsigned long long) * 5 * ncls * 32, s));
        A.counters = ctx->d_counters;
    }
    // one class: the reference's integral method (Rys for la+lb+lc+ld <= 8, MD above:
    // TwoElectronInts.cpp:658-666; MD everywhere in the MD mode), templated kernels for s/p/d
#ifndef UGB_FUSED_MIXED
#define UGB_FUSED_MIXED 1
#endif
#ifndef UGB_FUSE_MAXL
#define UGB_FUSE_MAXL -1  // classes with la+lb+lc+ld above this run their two parts as separate kernels
#endif                    // (-1: every class; the batched build keeps fused launches for (ss|ss), (ps|ss))
    // mixed builds: the FP64-part kernels on a high-priority stream, the FP32 kernels on a second one, so
    // that the FP64 CTAs take the SMs first and the FP32 CTAs fill the rest (213 vs 206 builds/s with the
    // classes alternating over two equal-priority streams); plain builds alternate their classes over two
    // streams
    const bool split = mixed && ctx->fp32_cut > ctx->skip_cut;
    const bool fused = split && UGB_FUSED_MIXED && ctx->eri_method != UNOMOL_ERI_MD;
    cudaStream_t ls[2] = {s, s};  // streams of the FP64 and FP32 launches (plain builds: alternate classes)
    if (!ctx->counting) {
        CU(cudaEventRecord(ctx->fork, s));
        ls[0] = ctx->part_stream[mixed ? 0 : 1];
        ls[1] = ctx->part_stream[mixed ? 1 : 2];
        for (int k = 0; k < 2; ++k) CU(cudaStreamWaitEvent(ls[k], ctx->fork, 0));
    }
    auto launch_class = [&](const ClassLaunch& L, bool fp32, bool side = false) -> cudaError_t {
        return launch_class_kernel(ctx, L, uhf, fp32, A, ls[(fp32 || side) ? 1 : 0]);
    };
    for (size_t lk = 0; lk < ctx->launches.size(); ++lk) {
        const size_t li = ctx->reverse_launches ? ctx->launches.size() - 1 - lk : lk;
        const ClassLaunch& L = ctx->launches[li];
        A.bps = ctx->d_bps + L.bp_begin;
        A.prefix = ctx->d_prefix;
        A.nbp = L.nbp;
        A.nwork = L.nwork;
        A.counter_base = (L.bc * NPAIRCLASS + L.kc) * 32;  // FP32 launches use the second half
        if (!mixed) {
            A.mode = 0;
            CU(launch_class(L, false, (li & 1) != 0));
            ++launches;
        } else {
            A.mode = 1;
            A.dyn_prefix = ctx->d_pre64;
            A.dyn_count = ctx->d_cnt64 + L.bp_begin;
            A.dyn_begin = ctx->d_begin64 + L.bp_begin;
            A.dyn_total = ctx->d_total64 + li;
            const int lsum = pc_la(L.bc) + pc_lb(L.bc) + pc_la(L.kc) + pc_lb(L.kc);
            if (fused && fock_mixed_fused(L.bc, L.kc) && lsum <= 8) {
                FockArgs A32 = A;
                A32.mode = 2;
                A32.dyn_prefix = ctx->d_pre32;
                A32.dyn_count = ctx->d_cnt32 + L.bp_begin;
                A32.dyn_begin = ctx->d_begin32 + L.bp_begin;
                A32.dyn_total = ctx->d_total32 + li;
                A32.counter_base += ncls * 32;
                if (lsum <= UGB_FUSE_MAXL) {
                    CU(launch_fock_mixed(L.bc, L.kc, uhf, A, A32, ctx->nt, ctx->d_rys, ctx->d_rys32, ls[0]));
                    ++launches;
                } else {
                    // classes whose FP32 code needs far fewer registers than their FP64 code: the FP64 part
                    // (four lanes per quartet) and the FP32 part as two kernels on the two streams, each
                    // at its own register count
                    CU(launch_fock_fp64_part(L.bc, L.kc, uhf, A, A32, ctx->nt, ctx->d_rys, ctx->d_rys32, ctx->nsm * 4,
                                             ls[0]));
                    CU(launch_class_kernel(ctx, L, uhf, true, A32, ls[1]));
                    launches += 2;
                }
                continue;
            }
            CU(launch_class(L, false));
            if (ctx->fp32_cut > ctx->skip_cut) {
                A.mode = 2;
                A.dyn_prefix = ctx->d_pre32;
                A.dyn_count = ctx->d_cnt32 + L.bp_begin;
                A.dyn_begin = ctx->d_begin32 + L.bp_begin;
                A.dyn_total = ctx->d_total32 + li;
                A.counter_base += ncls * 32;
                CU(launch_class(L, true));
                ++launches;
            }
            ++launches;
        }
    }
    if (ls[0] != s) {  // join the two parts back into the build's stream
        for (int k = 0; k < 2; ++k) {
            CU(cudaEventRecord(ctx->join[k], ls[k]));
            CU(cudaStreamWaitEvent(s, ctx->join[k], 0));
        }
    }
    CU(cudaEventRecord(ctx->ev[2], s));
    fold_packed<<<(unsigned)((np + 255) / 256), 256, 0, s>>>(ctx->d_Ta, dGa, n);
    ++launches;
    if (uhf) {
        fold_packed<<<(unsigned)((np + 255) / 256), 256, 0, s>>>(ctx->d_Tb, dGb, n);
        ++launches;
    }
    CU(cudaEventRecord(ctx->ev[3], s));
    CU(cudaGetLastError());
    ctx->stats.kernel_launches = launches;
    if (ctx->counting) {
        std::vector<unsigned long long> c(5 * ncls * 32);
        CU(cudaMemcpyAsync(c.data(), ctx->d_counters, sizeof(unsigned long long) * c.size(), cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        // shell quartets of this build per block pair: in the density-screened and mixed builds the
        // FP64 and FP32 parts of this build's lists (quartets below the skip cutoff do no work),
        // otherwise the static staircase of every class (ClassLaunch::quartets)
        const bool parts = mixed && !ctx->bps.empty();
        const bool has32 = ctx->fp32_cut > ctx->skip_cut;
        std::vector<long long> q64, q32;
        if (parts) {
            q64.assign(ctx->bps.size(), 0);
            q32.assign(ctx->bps.size(), 0);
            CU(cudaMemcpy(q64.data(), ctx->d_cnt64, sizeof(long long) * q64.size(), cudaMemcpyDeviceToHost));
            if (has32)
                CU(cudaMemcpy(q32.data(), ctx->d_cnt32, sizeof(long long) * q32.size(), cudaMemcpyDeviceToHost));
        }
        int64_t prims = 0, s64 = 0, s32 = 0, fq_done = 0, screened = 0, demoted = 0;
        double fl = 0.0, fl32 = 0.0;
        for (const ClassLaunch& L : ctx->launches) {
            const int cls = L.bc * NPAIRCLASS + L.kc;
            const int la = pc_la(L.bc), lb = pc_lb(L.bc), lc = pc_la(L.kc), ld = pc_lb(L.kc);
            const int64_t nf = (int64_t)ncart(la) * ncart(lb) * ncart(lc) * ncart(ld);
            for (int half = 0; half < 2; ++half) {
                unsigned long long n = 0;
                for (int k = 0; k < 32; ++k) n += c[(half * ncls + cls) * 32 + k];
                prims += (int64_t)n;
                const double f = (double)n * flops_per_prim(la, lb, lc, ld, half != 0);
                if (half) fl32 += f; else fl += f;
            }
            // quartet-level work (normalisation and density contraction) in the precision of the
            // kernel that does it
            long long n64 = L.quartets, n32 = 0;
            if (parts) {
                n64 = 0;
                for (int k = L.bp_begin; k < L.bp_begin + L.nbp; ++k) {
                    n64 += q64[k];
                    n32 += q32[k];
                }
                // quartets the per-quartet density screen dropped do no quartet-level work; quartets of
                // the FP64 part's lists that the fused kernel ran in FP32 count as FP32
                long long d64 = 0, d32 = 0, dem = 0;
                for (int k = 0; k < 32; ++k) {
                    d64 += (long long)c[(2 * ncls + cls) * 32 + k];
                    d32 += (long long)c[(3 * ncls + cls) * 32 + k];
                    dem += (long long)c[(4 * ncls + cls) * 32 + k];
                }
                n64 -= d64 + dem;
                n32 += dem - d32;
                screened += d64 + d32;
                demoted += dem;
            }
            fl += (double)n64 * flops_per_quartet(la, lb, lc, ld);
            fl32 += (double)n32 * flops_per_quartet(la, lb, lc, ld);
            s64 += n64;
            s32 += n32;
            fq_done += (n64 + n32) * nf;
        }
        ctx->stats.primitive_quartets_computed = prims;
        ctx->stats.function_quartets_computed = fq_done;
        ctx->stats.eri_flops = fl + fl32;
        ctx->stats.eri_flops_fp32 = fl32;
        if (parts) {
            ctx->stats.shell_quartets = s64 + s32;
            ctx->stats.shell_quartets_fp32 = s32;
        }
        ctx->stats.shell_quartets_screened = screened;
        ctx->stats.shell_quartets_demoted = demoted;
    }
    return UNOMOL_OK;
}

int finish_timing(UnomolCtx* ctx) {
    CU(cudaEventSynchronize(ctx->ev[3]));
    float ms_eri = 0.f, ms_tot = 0.f;
    CU(cudaEventElapsedTime(&ms_eri, ctx->ev[1], ctx->ev[2]));
    CU(cudaEventElapsedTime(&ms_tot, ctx->ev[0], ctx->ev[3]));
    ctx->stats.ms_eri = ms_eri;
    ctx->stats.ms_total = ms_tot;
    return UNOMOL_OK;
}

}  // namespace

namespace ugb {

CtxView ctx_view(const UnomolCtx* c) {
    CtxView v;
    v.nbf = c->nbf;
    v.nshell = c->nshell;
    v.rys_compat = c->rys_mode == UNOMOL_RYS_REFERENCE;
    v.eri_method = c->eri_method;
    v.d_pairs = c->d_pairs;
    v.npairs = c->npairs;
    v.d_prims = c->d_prims;
    v.d_prims32 = c->d_prims32;
    v.nprims = c->nprims;
    v.d_prefix = c->d_prefix;
    v.d_bps = c->d_bps;
    v.nrows = c->nrows;
    v.bps = &c->bps;
    v.block_begin = &c->block_begin;
    v.block_count = &c->block_count;
    v.block_class = &c->block_class;
    v.soff = &c->soff;
    v.sl = &c->sl;
    v.stream = c->stream;
    for (const ClassLaunch& L : c->launches) v.launches.push_back({L.bc, L.kc, L.bp_begin, L.nbp, L.nwork, L.quartets});
    v.nt = c->nt;
    v.d_rys = c->d_rys;
    v.d_rys32 = c->d_rys32;
    return v;
}

}  // namespace ugb

namespace {

// The Rys tables of every context on one device: file-scope device arrays of the library's image,
// filled once per device (rows re-laid with the padded strides of the kernels, zeros in the padding:
// 16-byte loads), then the large-T limits.
constexpr int RYS64_LEN = rys_table_len(RysStride<double>::value, RYS_H);
constexpr int RYS32_LEN = rys_table_len(RysStride<float>::value, RYS32_H);
static __device__ __align__(32) double g_rys64[RYS64_LEN];  // 64-byte rows: two 256-bit loads each
static __device__ __align__(32) float g_rys32[RYS32_LEN];  // 32-byte rows: one 256-bit load each
constexpr int RYS_MAX_DEVICES = 64;
double* g_rys64_ptr[RYS_MAX_DEVICES] = {nullptr};
float* g_rys32_ptr[RYS_MAX_DEVICES] = {nullptr};
std::mutex g_rys_mu;

int rys_tables(int dev, double*& d64, float*& d32, std::string& err) {
    static_assert(rys_table_len(RYS_DEG + 1, RYS_H) == RYS_TABLE_SIZE + 50, "layout of rys_tables.inc");
    static_assert(rys_table_len(RYS32_DEG + 1, RYS32_H) == RYS32_TABLE_SIZE + 50, "layout of rys_tables.inc");
    if (dev < 0 || dev >= RYS_MAX_DEVICES) {
        err = "device index out of range";
        return UNOMOL_EINVAL;
    }
    std::lock_guard<std::mutex> lock(g_rys_mu);
    if (!g_rys64_ptr[dev]) {
        constexpr int S64 = RysStride<double>::value, S32 = RysStride<float>::value;
        std::vector<double> t64(RYS64_LEN, 0.0);
        std::vector<float> t32(RYS32_LEN, 0.f);
        const int rows64 = RYS_TABLE_SIZE / (RYS_DEG + 1), rows32 = RYS32_TABLE_SIZE / (RYS32_DEG + 1);
        for (int r = 0; r < rows64; ++r)
            for (int d = 0; d <= RYS_DEG; ++d) t64[(size_t)r * S64 + d] = RYS_TABLE_H[(size_t)r * (RYS_DEG + 1) + d];
        for (int r = 0; r < rows32; ++r)
            for (int d = 0; d <= RYS32_DEG; ++d) t32[(size_t)r * S32 + d] = RYS32_TABLE_H[(size_t)r * (RYS32_DEG + 1) + d];
        const size_t h64 = t64.size() - 50, h32 = t32.size() - 50;
        for (int n = 0; n < 5; ++n)
            for (int i = 0; i < 5; ++i) {
                t64[h64 + n * 5 + i] = RYS_HERMITE_X_H[n][i];
                t64[h64 + 25 + n * 5 + i] = RYS_HERMITE_W_H[n][i];
                t32[h32 + n * 5 + i] = (float)RYS_HERMITE_X_H[n][i];
                t32[h32 + 25 + n * 5 + i] = (float)RYS_HERMITE_W_H[n][i];
            }
        void *p64 = nullptr, *p32 = nullptr;
        cudaError_t e = cudaMemcpyToSymbol(g_rys64, t64.data(), sizeof(double) * t64.size());
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_rys32, t32.data(), sizeof(float) * t32.size());
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&p64, g_rys64);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&p32, g_rys32);
        if (e != cudaSuccess) {
            err = std::string("Rys tables: ") + cudaGetErrorString(e);
            return UNOMOL_ECUDA;
        }
        g_rys64_ptr[dev] = static_cast<double*>(p64);
        g_rys32_ptr[dev] = static_cast<float*>(p32);
    }
    d64 = g_rys64_ptr[dev];
    d32 = g_rys32_ptr[dev];
    return UNOMOL_OK;
}

// Stream, events, Rys tables, the basis on the device and the first set-up of a new context.
int init_device(UnomolCtx* ctx, int np) {
    CU(cudaGetDevice(&ctx->dev));
    CU(cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, ctx->dev));
    CU(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    for (auto& e : ctx->ev) CU(cudaEventCreate(&e));
    {
        // the FP64 part's stream at the highest priority: its CTAs take the SMs first and the FP32 part's
        // CTAs fill what they leave (measured: 9 % faster mixed builds than equal priorities); plain
        // builds alternate their classes over two streams of equal priority
        int lo = 0, hi = 0;  // numerically lower = higher priority
        CU(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        CU(cudaStreamCreateWithPriority(&ctx->part_stream[0], cudaStreamNonBlocking, hi));
        CU(cudaStreamCreateWithPriority(&ctx->part_stream[1], cudaStreamNonBlocking, lo));
        CU(cudaStreamCreateWithPriority(&ctx->part_stream[2], cudaStreamNonBlocking, lo));
    }
    CU(cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming));
    for (auto& e : ctx->join) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    {
        const int rc = rys_tables(ctx->dev, ctx->d_rys, ctx->d_rys32, ctx->err);
        if (rc) return fail(ctx, rc, ctx->err);
    }
    // the basis in one allocation (status flag, shell arrays, exponents, coefficients, centres), from a
    // host image of the same layout
    {
        const int ns = ctx->nshell;
        Carve lay;
        const size_t o_status = lay.next(sizeof(int)), o_soff = lay.next(sizeof(int) * ns), o_sl = lay.next(sizeof(int) * ns),
                     o_snp = lay.next(sizeof(int) * ns), o_scen = lay.next(sizeof(int) * ns),
                     o_sprim = lay.next(sizeof(int) * ns), o_alpha = lay.next(sizeof(double) * np),
                     o_coef = lay.next(sizeof(double) * np), o_cen = lay.next(sizeof(double) * 3 * ctx->ncen);
        std::vector<char> img(lay.used, 0);
        auto put = [&](size_t off, const void* src, size_t bytes) { std::memcpy(img.data() + off, src, bytes); };
        put(o_soff, ctx->soff.data(), sizeof(int) * ns);
        put(o_sl, ctx->sl.data(), sizeof(int) * ns);
        put(o_snp, ctx->snp.data(), sizeof(int) * ns);
        put(o_scen, ctx->scen.data(), sizeof(int) * ns);
        put(o_sprim, ctx->sprim.data(), sizeof(int) * ns);
        put(o_alpha, ctx->alpha.data(), sizeof(double) * np);
        put(o_coef, ctx->coef.data(), sizeof(double) * np);
        put(o_cen, ctx->centers.data(), sizeof(double) * 3 * ctx->ncen);
        CU(cudaMalloc(&ctx->d_basis, img.size()));
        CU(cudaMemcpy(ctx->d_basis, img.data(), img.size(), cudaMemcpyHostToDevice));
        char* base = ctx->d_basis;
        ctx->d_status = reinterpret_cast<int*>(base + o_status);
        ctx->d_soff = reinterpret_cast<int*>(base + o_soff);
        ctx->d_sl = reinterpret_cast<int*>(base + o_sl);
        ctx->d_snp = reinterpret_cast<int*>(base + o_snp);
        ctx->d_scen = reinterpret_cast<int*>(base + o_scen);
        ctx->d_sprim = reinterpret_cast<int*>(base + o_sprim);
        ctx->d_alpha = reinterpret_cast<double*>(base + o_alpha);
        ctx->d_coef = reinterpret_cast<double*>(base + o_coef);
        ctx->d_centers = reinterpret_cast<double*>(base + o_cen);
    }
    return build_setup(ctx);
}

}  // namespace

extern "C" {

const char* unomol_gpu_version(void) { return "unomol_gb300 0.1 (sm_103a)"; }

const char* unomol_gpu_last_error(const UnomolCtx* ctx) {
    if (ctx && !ctx->err.empty()) return ctx->err.c_str();
    return g_last_error.c_str();
}

int unomol_gpu_create(const UnomolBasisDesc* b, int start_shell, UnomolCtx** out) {
    UnomolCtx* ctx = nullptr;
    if (!b || !out) return fail(nullptr, UNOMOL_EINVAL, "null argument");
    *out = nullptr;
    if (b->nshell <= 0 || b->ncen <= 0 || b->norb <= 0 || !b->shell_l || !b->shell_nprim || !b->shell_center ||
        !b->shell_offset || !b->alpha || !b->coef || !b->centers)
        return fail(nullptr, UNOMOL_EINVAL, "incomplete basis description");
    std::unique_ptr<UnomolCtx> c(new UnomolCtx());
    ctx = c.get();
    ctx->nshell = b->nshell;
    ctx->nbf = b->norb;
    ctx->ncen = b->ncen;
    ctx->start_shell = start_shell < 0 ? 0 : start_shell;
    int np = 0, off = 0;
    for (int i = 0; i < b->nshell; ++i) {
        const int l = b->shell_l[i];
        if (l < 0 || l > LMAX) return fail(nullptr, UNOMOL_EINVAL, "shell angular momentum above 4 (g) is not supported (Basis.hpp:222)");
        if (b->shell_nprim[i] <= 0) return fail(nullptr, UNOMOL_EINVAL, "shell with no primitives");
        if (b->shell_nprim[i] > 255) return fail(nullptr, UNOMOL_EINVAL, "shell with more than 255 primitives");
        if (b->shell_center[i] < 0 || b->shell_center[i] >= b->ncen) return fail(nullptr, UNOMOL_EINVAL, "shell centre out of range");
        if (b->shell_offset[i] != off) return fail(nullptr, UNOMOL_EINVAL, "shell offsets must follow shell order");
        ctx->sl.push_back(l);
        ctx->snp.push_back(b->shell_nprim[i]);
        ctx->scen.push_back(b->shell_center[i]);
        ctx->soff.push_back(b->shell_offset[i]);
        ctx->sprim.push_back(np);
        np += b->shell_nprim[i];
        off += ncart(l);
        ctx->maxl = std::max(ctx->maxl, l);
    }
    if (off != b->norb) return fail(nullptr, UNOMOL_EINVAL, "norb does not match the shells");
    // the basis is checked first, so that a bad description is reported as such on any machine
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(nullptr, UNOMOL_ENODEV, "no CUDA device: the GB300 Fock build has no CPU fallback");
    ctx->alpha.assign(b->alpha, b->alpha + np);
    ctx->coef.assign(b->coef, b->coef + np);
    ctx->centers.assign(b->centers, b->centers + 3 * b->ncen);
    build_norms(ctx->nt);
    ctx->stats.nbf = ctx->nbf;
    // device resources and the set-up; on failure everything created so far is released
    const int rc = init_device(ctx, np);
    if (rc) {
        g_last_error = ctx->err;
        unomol_gpu_destroy(c.release());
        return rc;
    }
    *out = c.release();
    return UNOMOL_OK;
}

int unomol_gpu_recalculate(UnomolCtx* ctx, const double* centers) {
    if (!ctx || !centers) return fail(ctx, UNOMOL_EINVAL, "null argument");
    ctx->centers.assign(centers, centers + 3 * ctx->ncen);
    const int rc = build_setup(ctx);
    if (rc || !ctx->store) return rc;
    // the reference's recalculate recomputes its stored integrals (TwoElectronInts.hpp:94-96)
    const int kind = store_kind(ctx->store);
    const double max_gib = store_max_gib(ctx->store);
    store_free(ctx->store);
    ctx->store = nullptr;
    return unomol_gpu_store_integrals(ctx, kind, max_gib);
}

// The context's device current for the length of a call, the caller's restored after it.
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceScope() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

int unomol_gpu_store_integrals(UnomolCtx* ctx, int kind, double max_gib) {
    if (!ctx) return fail(ctx, UNOMOL_EINVAL, "null context");
    DeviceScope scope(ctx->dev);
    IntStore* st = nullptr;
    std::string err;
    const int rc = store_from_integrals(ctx_view(ctx), kind, max_gib, &st, err);
    if (rc) return fail(ctx, rc, err);
    store_free(ctx->store);
    ctx->store = st;
    return UNOMOL_OK;
}

int unomol_gpu_store_records(UnomolCtx* ctx, const char* path, int kind, double max_gib) {
    if (!ctx || !path) return fail(ctx, UNOMOL_EINVAL, "null argument");
    DeviceScope scope(ctx->dev);
    IntStore* st = nullptr;
    std::string err;
    const int rc = store_from_file(ctx_view(ctx), path, kind, max_gib, &st, err);
    if (rc) return fail(ctx, rc, err);
    store_free(ctx->store);
    ctx->store = st;
    return UNOMOL_OK;
}

int unomol_gpu_drop_store(UnomolCtx* ctx) {
    if (!ctx) return fail(ctx, UNOMOL_EINVAL, "null context");
    if (ctx->store) {
        CU(cudaStreamSynchronize(ctx->stream));
        store_free(ctx->store);
        ctx->store = nullptr;
    }
    return UNOMOL_OK;
}

int unomol_gpu_store_info(const UnomolCtx* ctx, UnomolStoreInfo* out) {
    if (!ctx || !out) return UNOMOL_EINVAL;
    store_info(ctx->store, out);
    return UNOMOL_OK;
}

int unomol_gpu_write_records(UnomolCtx* ctx, const char* path, int64_t* count) {
    if (!ctx || !path || !count) return fail(ctx, UNOMOL_EINVAL, "null argument");
    DeviceScope scope(ctx->dev);
    long long n = 0;
    std::string err;
    const int rc = write_records(ctx_view(ctx), path, &n, err);
    if (rc) return fail(ctx, rc, err);
    *count = n;
    return UNOMOL_OK;
}

int unomol_gpu_set_screening(UnomolCtx* ctx, double cut) {
    if (!ctx || !(cut >= 0.0)) return fail(ctx, UNOMOL_EINVAL, "bad screening cutoff");
    ctx->schwarz_cut = cut;
    return build_worklists(ctx);
}

int unomol_gpu_set_precision(UnomolCtx* ctx, int mode, double fp32_cut) {
    if (!ctx) return fail(ctx, UNOMOL_EINVAL, "null context");
    if (mode != UNOMOL_PREC_FP64 && mode != UNOMOL_PREC_MIXED) return fail(ctx, UNOMOL_EINVAL, "unknown precision mode");
    if (!(fp32_cut >= 0.0)) return fail(ctx, UNOMOL_EINVAL, "bad FP32 cutoff");
    ctx->prec_mode = mode;
    ctx->fp32_cut = fp32_cut;
    return UNOMOL_OK;
}

int unomol_gpu_set_density_screening(UnomolCtx* ctx, double skip_cut) {
    if (!ctx || !(skip_cut >= 0.0)) return fail(ctx, UNOMOL_EINVAL, "bad density screening cutoff");
    ctx->skip_cut = skip_cut;
    return UNOMOL_OK;
}

int unomol_gpu_set_eri_method(UnomolCtx* ctx, int method) {
    if (!ctx) return fail(ctx, UNOMOL_EINVAL, "null context");
    if (method != UNOMOL_ERI_REFERENCE && method != UNOMOL_ERI_MD) return fail(ctx, UNOMOL_EINVAL, "unknown ERI method");
    ctx->eri_method = method;
    return UNOMOL_OK;
}

int unomol_gpu_set_rys_mode(UnomolCtx* ctx, int mode) {
    if (!ctx) return fail(ctx, UNOMOL_EINVAL, "null context");
    if (mode != UNOMOL_RYS_REFERENCE && mode != UNOMOL_RYS_EXACT) return fail(ctx, UNOMOL_EINVAL, "unknown Rys mode");
    ctx->rys_mode = mode;
    return UNOMOL_OK;
}

int unomol_gpu_last_build_ms(UnomolCtx* ctx, double* ms_eri, double* ms_total) {
    if (!ctx || !ms_eri || !ms_total) return fail(ctx, UNOMOL_EINVAL, "null argument");
    int rc = finish_timing(ctx);
    if (rc) return rc;
    *ms_eri = ctx->stats.ms_eri;
    *ms_total = ctx->stats.ms_total;
    return UNOMOL_OK;
}

int unomol_gpu_set_launch_order(UnomolCtx* ctx, int reversed) {
    if (!ctx) return fail(ctx, UNOMOL_EINVAL, "null context");
    ctx->reverse_launches = reversed ? 1 : 0;
    return UNOMOL_OK;
}

int unomol_gpu_set_counting(UnomolCtx* ctx, int on) {
    if (!ctx) return fail(ctx, UNOMOL_EINVAL, "null context");
    ctx->counting = on ? 1 : 0;
    return UNOMOL_OK;
}

int unomol_gpu_get_stats(const UnomolCtx* ctx, UnomolStats* out) {
    if (!ctx || !out) return UNOMOL_EINVAL;
    *out = ctx->stats;
    return UNOMOL_OK;
}

int unomol_gpu_fock_rhf_device(UnomolCtx* ctx, const double* dP, double* dG, void* stream) {
    if (!ctx || !dP || !dG) return fail(ctx, UNOMOL_EINVAL, "null argument");
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    return fock_device(ctx, dP, nullptr, dG, nullptr, s);
}

int unomol_gpu_fock_uhf_device(UnomolCtx* ctx, const double* dPa, const double* dPb, double* dGa, double* dGb,
                               void* stream) {
    if (!ctx || !dPa || !dPb || !dGa || !dGb) return fail(ctx, UNOMOL_EINVAL, "null argument");
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    return fock_device(ctx, dPa, dPb, dGa, dGb, s);
}

int unomol_gpu_fock_rhf(UnomolCtx* ctx, const double* P, double* G) {
    if (!ctx || !P || !G) return fail(ctx, UNOMOL_EINVAL, "null argument");
    int rc = ensure_density_buffers(ctx, false);
    if (rc) return rc;
    const size_t np = (size_t)ctx->nbf * (ctx->nbf + 1) / 2;
    CU(cudaMemcpyAsync(ctx->d_pk_a, P, np * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaMemcpyAsync(ctx->d_Ga, G, np * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    rc = fock_device(ctx, ctx->d_pk_a, nullptr, ctx->d_Ga, nullptr, ctx->stream);
    if (rc) return rc;
    CU(cudaMemcpyAsync(G, ctx->d_Ga, np * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));  // G is the caller's host array: wait for the copy back
    return finish_timing(ctx);
}

int unomol_gpu_fock_uhf(UnomolCtx* ctx, const double* Pa, const double* Pb, double* Ga, double* Gb) {
    if (!ctx || !Pa || !Pb || !Ga || !Gb) return fail(ctx, UNOMOL_EINVAL, "null argument");
    int rc = ensure_density_buffers(ctx, true);
    if (rc) return rc;
    const size_t np = (size_t)ctx->nbf * (ctx->nbf + 1) / 2;
    CU(cudaMemcpyAsync(ctx->d_pk_a, Pa, np * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaMemcpyAsync(ctx->d_pk_b, Pb, np * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaMemcpyAsync(ctx->d_Ga, Ga, np * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaMemcpyAsync(ctx->d_Gb, Gb, np * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    rc = fock_device(ctx, ctx->d_pk_a, ctx->d_pk_b, ctx->d_Ga, ctx->d_Gb, ctx->stream);
    if (rc) return rc;
    CU(cudaMemcpyAsync(Ga, ctx->d_Ga, np * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaMemcpyAsync(Gb, ctx->d_Gb, np * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));  // G is the caller's host array: wait for the copy back
    return finish_timing(ctx);
}

void unomol_gpu_destroy(UnomolCtx* ctx) {
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    store_free(ctx->store);
    ctx->store = nullptr;
    dfree(ctx->d_basis);
    dfree(ctx->d_setup);
    dfree(ctx->d_lists);
    dfree(ctx->d_ws);
    dfree(ctx->d_Pa);
    dfree(ctx->d_Pb);
    dfree(ctx->d_Ta);
    dfree(ctx->d_Tb);
    dfree(ctx->d_Ga);
    dfree(ctx->d_Gb);
    dfree(ctx->d_pk_a);
    dfree(ctx->d_pk_b);
    dfree(ctx->d_pmax);
    dfree(ctx->d_counters);
    dfree(ctx->d_dmax);
    dfree(ctx->d_Pa32);
    dfree(ctx->d_Pb32);
    for (auto& e : ctx->ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {ctx->fork, ctx->join[0], ctx->join[1]})
        if (e) cudaEventDestroy(e);
    for (cudaStream_t st : ctx->part_stream)
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Allocation-free RHF Fock build.
//
// The regular build keeps its per-build scratch (the dense copy of P and the N x N accumulator T) in
// device buffers that it allocates on first use.  Some callers cannot let a library call cudaMalloc
// once they are running: a host framework that owns every device allocation after start-up (a fixed
// memory allowance, its own pool), or an iteration loop that must not take cudaMalloc's implicit device
// synchronisation.  For them the allocation-free build keeps that scratch in one file-scope device
// array instead.
// The array is part of the library's device image, so every GPU on which the library's kernels are
// loaded holds it (NOALLOC_SCRATCH_BYTES) until the process exits.
// ---------------------------------------------------------------------------------------------
namespace {

constexpr int NOALLOC_MAX_NBF = 1024;  // largest basis the static scratch holds
constexpr size_t NOALLOC_SCRATCH_DOUBLES = 2ull * NOALLOC_MAX_NBF * NOALLOC_MAX_NBF;  // 16 MiB

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

constexpr int NOALLOC_MAX_DEVICES = 64;
double* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {nullptr};  // device address of the array, per device
std::mutex g_noalloc_mu;

}  // namespace

extern "C" int unomol_gpu_fock_rhf_noalloc(UnomolCtx* ctx, const double* dP, double* dG, void* stream) {
    if (!ctx || !dP || !dG) return fail(ctx, UNOMOL_EINVAL, "null argument");
    const int n = ctx->nbf;
    if (n > NOALLOC_MAX_NBF)
        return fail(ctx, UNOMOL_EINVAL,
                    "unomol_gpu_fock_rhf_noalloc: " + std::to_string(n) + " basis functions exceed the " +
                        std::to_string(NOALLOC_MAX_NBF) + " that its static scratch holds");
    if (ctx->prec_mode != UNOMOL_PREC_FP64)
        return fail(ctx, UNOMOL_EINVAL, "unomol_gpu_fock_rhf_noalloc runs the FP64 build only");
    if (ctx->counting)
        return fail(ctx, UNOMOL_EINVAL,
                    "unomol_gpu_fock_rhf_noalloc does not count work (its counters would need an allocation): "
                    "switch counting off or use unomol_gpu_fock_rhf_device");
    int dev = -1;
    CU(cudaGetDevice(&dev));
    if (dev != ctx->dev) return fail(ctx, UNOMOL_EINVAL, "unomol_gpu_fock_rhf_noalloc: current device is not the context's");
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return fail(ctx, UNOMOL_EINVAL, "device index out of range");
    double* scratch = nullptr;
    {
        // once per device, with that device current: the host-side name of the array is only a
        // stand-in, the kernels need its device address
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess)
                return fail(ctx, UNOMOL_ECUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
            g_noalloc_ptr[dev] = static_cast<double*>(p);
        }
        scratch = g_noalloc_ptr[dev];
    }
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    const long long n2 = (long long)n * n, np = (long long)n * (n + 1) / 2;
    double* Pfull = scratch;
    double* T = scratch + n2;
    int launches = 0;
    CU(cudaEventRecord(ctx->ev[0], s));
    expand_packed<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(dP, Pfull, n);
    ++launches;
    CU(cudaGetLastError());
    CU(cudaMemsetAsync(T, 0, n2 * sizeof(double), s));  // the array keeps the previous call's sums
    CU(cudaEventRecord(ctx->ev[1], s));
    FockArgs A{};
    A.pairs = ctx->d_pairs;
    A.prims = ctx->d_prims;
    A.prims32 = ctx->d_prims32;
    A.nbf = n;
    A.Pa = Pfull;
    A.Pb = nullptr;
    A.Ta = T;
    A.Tb = nullptr;
    A.thr_int = STORE_CUT;
    A.prim_cut = PRIM_CUT;
    A.thr_int32 = (float)STORE_CUT;
    A.prim_cut32 = (float)PRIM_CUT;
    A.nshell = ctx->nshell;
    A.rys_compat = ctx->rys_mode == UNOMOL_RYS_REFERENCE;
    A.counters = nullptr;
    A.mode = 0;
    for (const ClassLaunch& L : ctx->launches) {
        A.bps = ctx->d_bps + L.bp_begin;
        A.prefix = ctx->d_prefix;
        A.nbp = L.nbp;
        A.nwork = L.nwork;
        // the regular build's method selection: MD mode, runtime-L and MD classes included
        CU(launch_class_kernel(ctx, L, false, false, A, s));
        ++launches;
    }
    CU(cudaEventRecord(ctx->ev[2], s));
    fold_packed<<<(unsigned)((np + 255) / 256), 256, 0, s>>>(T, dG, n);
    ++launches;
    CU(cudaEventRecord(ctx->ev[3], s));
    CU(cudaGetLastError());
    // unomol_gpu_get_stats / unomol_gpu_last_build_ms then describe this build
    ctx->stats.kernel_launches = launches;
    return UNOMOL_OK;
}
