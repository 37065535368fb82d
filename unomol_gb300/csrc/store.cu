// Conventional Fock build from stored integrals: the GPU form of the reference's integral cache
// (cache.hpp:18-386, filled by TwoElectronInts::calculate, TwoElectronInts.cpp:511-697) and of its
// cached formGmatrix (TwoElectronInts.cpp:822-869).
//
// Record pass.  The class kernels of the direct build evaluate every shell quartet of the Schwarz work
// lists once, in FP64, and append the canonical function quartets with |v| > 1e-14 as 24-byte records
// (TwoInts: val, i, j, k, l; the labels and the storage cut of TwoElectronInts.cpp:622-671).
//
// Assembly.  A record is one unique integral v = (ij|kl).  With d = 1/2 for each coincidence (i = j,
// k = l, (ij) = (kl)) it adds to the N x N accumulator T, whose T + T^T is G, the six terms
//     T_ij += c d v P_kl   T_kl += c d v P_ij                                     (Coulomb, c = 4 RHF / 2 UHF)
//     T_ik -= d v P_jl   T_jk -= d v P_il   T_il -= d v P_jk   T_jl -= d v P_ik   (exchange)
// which sum to the reference's scatter (TwoElectronInts.cpp:699-820) over the record's permutations.
// Each term is one element of a sparse matrix M over packed indices: row = packed (x, y) of its T
// element, column = packed (z, w) of its P element, value doubled when x = y (G_xx = 2 T_xx); then
// G_packed += M P_packed.  RHF stores the one matrix of G = 2J - K; UHF stores J (rows [0, np)) and K
// (rows [np, 2 np)), with Ga = J (Pa + Pb) + K Pa, Gb = J (Pa + Pb) + K Pb, and RHF G = 2 J P + K P.
// The terms are made per slab of rows (slab rows x np fits a 32-bit key), radix-sorted by (row, column)
// and summed per key (CUB), which leaves one CSR matrix per slab with sorted columns and one element per
// distinct (row, column).
//
// Build.  One warp per row piece (rows longer than PIECE_MAX elements are split into near-equal pieces,
// so that no warp of the last wave streams a much longer row than the others) streams the values and
// columns from HBM (cache-streaming loads, read once per build) and gathers P, which stays in L2.  No
// integral is recomputed; in the RHF store a whole row's sum is its G element (a plain add), the pieces
// of split rows add theirs atomically.
#include <cub/cub.cuh>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "fock_dispatch.cuh"
#include "fock_kernels.cuh"
#include "store.h"
#include "store_emit.cuh"

namespace ugb {

// A piece of one row for one warp of the build: rows longer than a piece's limit are split, so that the
// warps of a build get similar element counts (the last wave does not wait on a few long rows).
struct RowPiece {
    int row;    // row within the slab
    int begin;  // element range [begin, end) of the slab
    int end;
    int whole;  // 1: the piece is the whole row (its sum is the row's G element)
};

struct StoreSlab {
    long long r0 = 0, r1 = 0;  // rows [r0, r1) of the matrix
    long long nnz = 0;
    char* mem = nullptr;       // row offsets (int, r1 - r0 + 1), columns (int), values (double)
    int* rowptr = nullptr;
    int* col = nullptr;
    double* val = nullptr;
    RowPiece* pieces = nullptr;  // separate allocation
    int npieces = 0;
};

struct IntStore {
    int kind = 0, nbf = 0;
    long long np = 0;  // packed size N (N + 1) / 2
    long long records = 0, nnz = 0, bytes = 0;
    double ms_records = 0.0, ms_assemble = 0.0, max_gib = 0.0;
    std::vector<StoreSlab> slabs;
};

namespace {

constexpr int NBUCKET = 1024;  // row buckets of the term histogram (slabs are runs of buckets)
#ifndef UGB_PIECE_MAX
#define UGB_PIECE_MAX 4096
#endif
constexpr int PIECE_MAX = UGB_PIECE_MAX;  // elements per warp piece of a build

__device__ __forceinline__ long long packed(int x, int y) {
    return x >= y ? (long long)x * (x + 1) / 2 + y : (long long)y * (y + 1) / 2 + x;
}

// The six matrix terms of one canonical record (see the file comment).
__device__ __forceinline__ void record_terms(const UnomolRecord& r, int kind, long long np, long long* row, long long* col,
                                             double* val) {
    const int i = r.i, j = r.j, k = r.k, l = r.l;
    double d = 1.0;
    if (i == j) d *= 0.5;
    if (k == l) d *= 0.5;
    if (i == k && j == l) d *= 0.5;
    const double cj = (kind == UNOMOL_STORE_RHF ? 4.0 : 2.0) * d * r.val;
    const double ck = -d * r.val;
    const long long koff = kind == UNOMOL_STORE_RHF ? 0 : np;
    const int tx[6] = {i, k, i, j, i, j}, ty[6] = {j, l, k, k, l, l};
    const int pz[6] = {k, i, j, i, j, i}, pw[6] = {l, j, l, l, k, k};
#pragma unroll
    for (int t = 0; t < 6; ++t) {
        const double c = t < 2 ? cj : ck;
        row[t] = packed(tx[t], ty[t]) + (t < 2 ? 0 : koff);
        col[t] = packed(pz[t], pw[t]);
        val[t] = tx[t] == ty[t] ? 2.0 * c : c;
    }
}

// Record pass of one templated class: one thread per shell quartet, its integrals in registers
// (shell_quartet_eri, as the direct build), then the canonical elements of its rectangle with
// |v| > 1e-14 appended as records.
template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) store_records_kernel(const FockArgs A, const NormTable nt, const double* __restrict__ rys,
                                                            const RecSink S) {
    using Q = QClass<LA, LB, LC, LD>;
    constexpr bool UNIT_NORMS = LA < 2 && LB < 2 && LC < 2 && LD < 2;
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int bi = 0, ki = 0;
    const bool ok = decode_work_warp<false>(A, g, bi, ki);  // warp-collective
    double acc[Q::NF];
    ShellPair bra{}, ket{};
    if (ok) {
        bra = A.pairs[bi];
        ket = A.pairs[ki];
        shell_quartet_eri<LA, LB, LC, LD, double, PrimPair>(bra, ket, A.prims, rys, A.prim_cut, A.prim_cut32, A.rys_compat != 0,
                                                            acc);
    }
    unsigned n = 0;
    for (int pass = 0; pass < 2; ++pass) {  // count, then write
        unsigned long long slot = 0;
        if (pass == 1) slot = reserve_records(S, n);
        if (!ok) continue;
#pragma unroll
        for (int ia = 0; ia < Q::NA; ++ia)
#pragma unroll
            for (int ib = 0; ib < Q::NB; ++ib)
#pragma unroll
                for (int ic = 0; ic < Q::NC; ++ic)
#pragma unroll
                    for (int id = 0; id < Q::ND; ++id) {
                        double v = acc[((ia * Q::NB + ib) * Q::NC + ic) * Q::ND + id];
                        if constexpr (!UNIT_NORMS) v *= nt.v[LA][ia] * nt.v[LB][ib] * nt.v[LC][ic] * nt.v[LD][id];
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

template <int BC, int KC>
cudaError_t store_one(const FockArgs& A, const NormTable& nt, const double* rys, const RecSink& S, cudaStream_t s) {
    constexpr int LA = pc_la(BC), LB = pc_lb(BC), LC = pc_la(KC), LD = pc_lb(KC);
    if (A.nwork <= 0) return cudaSuccess;
    if constexpr (QClass<LA, LB, LC, LD>::NF <= 81) {
        store_records_kernel<LA, LB, LC, LD><<<(unsigned)((A.nwork + 127) / 128), 128, 0, s>>>(A, nt, rys, S);
        return cudaGetLastError();
    } else {
        return launch_store_generic(LA, LB, LC, LD, A, nt, rys, S, s);
    }
}

#define UGB_CASE(BC, KC) \
    case (BC) * 8 + (KC): \
        return store_one<BC, KC>(A, nt, rys, S, s);

// The record pass of one class with the direct build's method selection (TwoElectronInts.cpp:658-666).
cudaError_t store_class(const CtxView& v, const ClassLaunchInfo& L, const FockArgs& A, const RecSink& S, cudaStream_t s) {
    const int la = pc_la(L.bc), lb = pc_lb(L.bc), lc = pc_la(L.kc), ld = pc_lb(L.kc);
    const NormTable& nt = v.nt;
    const double* rys = v.d_rys;
    if (v.eri_method == UNOMOL_ERI_MD || la + lb + lc + ld > 8) return launch_store_md(la, lb, lc, ld, A, nt, S, s);
    if (L.bc < NTMPLCLASS && L.kc < NTMPLCLASS) {
        switch (L.bc * 8 + L.kc) {
#include "fock_cases.inc"
            default:
                break;
        }
    }
    return launch_store_generic(la, lb, lc, ld, A, nt, rys, S, s);
}
#undef UGB_CASE

// Terms per row bucket (shared-memory histogram per block).
__global__ void __launch_bounds__(256) term_histogram(const UnomolRecord* __restrict__ rec, long long n, int kind, long long np,
                                                      long long bucket_rows, unsigned long long* __restrict__ hist) {
    __shared__ unsigned sh[NBUCKET];
    for (int b = threadIdx.x; b < NBUCKET; b += blockDim.x) sh[b] = 0u;
    __syncthreads();
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        long long row[6], col[6];
        double val[6];
        record_terms(rec[t], kind, np, row, col, val);
#pragma unroll
        for (int e = 0; e < 6; ++e) atomicAdd(&sh[row[e] / bucket_rows], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < NBUCKET; b += blockDim.x)
        if (sh[b]) atomicAdd(hist + b, (unsigned long long)sh[b]);
}

// The terms of one slab [r0, r1) as (32-bit key = (row - r0) * np + column, value), appended compactly.
__global__ void __launch_bounds__(256) slab_terms(const UnomolRecord* __restrict__ rec, long long n, int kind, long long np,
                                                  long long r0, long long r1, unsigned* __restrict__ keys,
                                                  double* __restrict__ vals, unsigned long long* cursor, unsigned long long cap,
                                                  int* overflow) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long t0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); t0 < n; t0 += stride) {
        const long long t = t0 + (threadIdx.x & 31);
        long long row[6], col[6];
        double val[6];
        unsigned m = 0;
        if (t < n) {
            record_terms(rec[t], kind, np, row, col, val);
#pragma unroll
            for (int e = 0; e < 6; ++e) m += (row[e] >= r0 && row[e] < r1) ? 1u : 0u;
        }
        unsigned long long slot = warp_reserve(cursor, m);  // whole warps: every lane reaches it
        if (!m) continue;
#pragma unroll
        for (int e = 0; e < 6; ++e) {
            if (row[e] < r0 || row[e] >= r1) continue;
            if (slot >= cap) {
                atomicExch(overflow, 1);
                break;
            }
            keys[slot] = (unsigned)((row[e] - r0) * np + col[e]);
            vals[slot] = val[e];
            ++slot;
        }
    }
}

// Sorted unique keys and their sums -> CSR of the slab (row offsets from the first key of every row).
__global__ void __launch_bounds__(256) slab_csr(const unsigned* __restrict__ ukeys, const double* __restrict__ sums, long long nruns,
                                                long long np, int nrows, int* __restrict__ rowptr, int* __restrict__ col,
                                                double* __restrict__ val) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nruns; t += (long long)gridDim.x * blockDim.x) {
        const long long key = ukeys[t];
        const int row = (int)(key / np);
        col[t] = (int)(key - (long long)row * np);
        val[t] = sums[t];
        const int prev = t == 0 ? -1 : (int)((long long)ukeys[t - 1] / np);
        for (int r = prev + 1; r <= row; ++r) rowptr[r] = (int)t;
        if (t == nruns - 1)
            for (int r = row + 1; r <= nrows; ++r) rowptr[r] = (int)nruns;
    }
}

// Record checks of a file: labels inside the basis and canonical (i >= j, k >= l, (i,j) >= (k,l)),
// finite values.  bad[0] = 1 + index of a failing record (the smallest is not guaranteed).
__global__ void check_records(const UnomolRecord* __restrict__ rec, long long n, int nbf, unsigned long long* bad) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const UnomolRecord r = rec[t];
        const bool inside = r.l >= 0 && r.j >= 0 && r.i < nbf && r.k < nbf;
        const bool canon = r.j <= r.i && r.l <= r.k && (r.k < r.i || (r.k == r.i && r.l <= r.j));
        if (!(inside && canon && isfinite(r.val))) atomicMax(bad, (unsigned long long)(t + 1));
    }
}

struct AddOp {
    __device__ __forceinline__ double operator()(double a, double b) const { return a + b; }
};

// Build: one warp per row piece of a slab (whole rows, and the pieces of long rows).  MODE 0: RHF
// store, RHF build; 1: UHF store, RHF build; 2: UHF store, UHF build.
template <int MODE>
__global__ void __launch_bounds__(256) store_spmv(const RowPiece* __restrict__ pieces, int npieces, const int* __restrict__ col,
                                                  const double* __restrict__ val, long long r0, long long np,
                                                  const double* __restrict__ Pa, const double* __restrict__ Pb,
                                                  double* __restrict__ Ga, double* __restrict__ Gb) {
    const int lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    for (int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < npieces; w += nwarps) {
        const RowPiece pc = pieces[w];
        const long long r = r0 + pc.row;
        const bool krow = MODE != 0 && r >= np;
        double sa = 0.0, sb = 0.0;
        auto add = [&](double v, int c) {
            if constexpr (MODE == 2) {
                if (krow) {
                    sa = fma(v, __ldg(Pa + c), sa);
                    sb = fma(v, __ldg(Pb + c), sb);
                } else {
                    sa = fma(v, __ldg(Pa + c) + __ldg(Pb + c), sa);
                }
            } else {
                sa = fma(v, __ldg(Pa + c), sa);
            }
        };
        const int end = pc.end;
        int k = pc.begin + lane;
        for (; k + 96 < end; k += 128) {  // four independent loads per lane in flight
            double v[4];
            int c[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                v[u] = __ldcs(val + k + 32 * u);
                c[u] = __ldcs(col + k + 32 * u);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) add(v[u], c[u]);
        }
        for (; k < end; k += 32) add(__ldcs(val + k), __ldcs(col + k));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sa += __shfl_xor_sync(0xffffffffu, sa, o);
            if constexpr (MODE == 2) sb += __shfl_xor_sync(0xffffffffu, sb, o);
        }
        if (lane != 0) continue;
        if constexpr (MODE == 0) {
            if (pc.whole) Ga[r] += sa;  // the row's one warp
            else atomicAdd(Ga + r, sa);
        } else if constexpr (MODE == 1) {
            if (krow) atomicAdd(Ga + (r - np), sa);
            else atomicAdd(Ga + r, 2.0 * sa);
        } else {
            if (krow) {
                atomicAdd(Ga + (r - np), sa);
                atomicAdd(Gb + (r - np), sb);
            } else {
                atomicAdd(Ga + r, sa);
                atomicAdd(Gb + r, sa);
            }
        }
    }
}

// Device scratch released on every path out of a construction.
struct Scratch {
    std::vector<void*> ptrs;
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <typename T>
    cudaError_t alloc(T** p, size_t n) {
        cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
        if (e == cudaSuccess) ptrs.push_back(*p);
        return e;
    }
};

#define SCU(call)                                                                           \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);                       \
            return e_ == cudaErrorMemoryAllocation ? UNOMOL_ENOMEM : UNOMOL_ECUDA;          \
        }                                                                                   \
    } while (0)

double budget_bytes(double max_gib) { return (max_gib > 0.0 ? max_gib : 64.0) * 1073741824.0; }

int grid_for(long long n, int threads) {
    int dev = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    return (int)std::max<long long>(1, std::min<long long>((n + threads - 1) / threads, (long long)nsm * 8));
}

// Records -> CSR slabs of st (kind, nbf, np set).  used: device bytes already held (the records).
int assemble(IntStore* st, const UnomolRecord* d_rec, long long nrec, double budget, double used, cudaStream_t s,
             std::string& err) {
    const long long np = st->np;
    const long long nrow = st->kind == UNOMOL_STORE_RHF ? np : 2 * np;
    const long long max_rows = (long long)(0xffffffffull / (unsigned long long)np);  // 32-bit keys
    const long long bucket_rows = (nrow + NBUCKET - 1) / NBUCKET;
    if (bucket_rows > max_rows) {
        err = "stored build: " + std::to_string(st->nbf) + " basis functions are too many for its 32-bit slab keys";
        return UNOMOL_EINVAL;
    }
    Scratch tmp;
    unsigned long long *d_hist = nullptr, *d_cursor = nullptr;
    long long* d_nruns = nullptr;
    int* d_over = nullptr;
    SCU(tmp.alloc(&d_hist, NBUCKET));
    SCU(tmp.alloc(&d_cursor, 1));
    SCU(tmp.alloc(&d_nruns, 1));
    SCU(tmp.alloc(&d_over, 1));
    SCU(cudaMemsetAsync(d_hist, 0, sizeof(unsigned long long) * NBUCKET, s));
    SCU(cudaMemsetAsync(d_over, 0, sizeof(int), s));
    if (nrec > 0) term_histogram<<<grid_for(nrec, 256), 256, 0, s>>>(d_rec, nrec, st->kind, np, bucket_rows, d_hist);
    SCU(cudaGetLastError());
    std::vector<unsigned long long> hist(NBUCKET);
    SCU(cudaMemcpyAsync(hist.data(), d_hist, sizeof(unsigned long long) * NBUCKET, cudaMemcpyDeviceToHost, s));
    SCU(cudaStreamSynchronize(s));
    unsigned long long total = 0, biggest = 0;
    for (unsigned long long h : hist) {
        total += h;
        biggest = std::max(biggest, h);
    }
    // slab capacity: the sort buffers (two keys and two values per term) take at most half of what the
    // budget leaves; the finished slabs (12 bytes per element) need the rest
    const double avail = budget - used;
    unsigned long long cap = (unsigned long long)std::max(0.0, avail / 2.0 / 24.0);
    cap = std::min<unsigned long long>(std::max(cap, biggest), std::max<unsigned long long>(total, 1));
    // CUB item counts are int; the build's element indices (int) step past a slab's end by < 128
    cap = std::min<unsigned long long>(cap, (unsigned long long)INT_MAX - 1024ull);
    if (biggest > cap) {
        err = "stored build: a row bucket of " + std::to_string(biggest) + " terms exceeds one sort (2^31 items)";
        return UNOMOL_EINVAL;
    }
    if ((double)cap * 24.0 > avail) {
        err = "stored build: a row bucket of " + std::to_string(biggest) + " terms does not fit the memory budget";
        return UNOMOL_ENOMEM;
    }
    // slabs: runs of buckets within the capacity and the 32-bit key range
    struct Range {
        long long r0, r1;
        unsigned long long terms;
    };
    std::vector<Range> ranges;
    for (int b = 0; b < NBUCKET;) {
        const long long r0 = (long long)b * bucket_rows;
        if (r0 >= nrow) break;
        unsigned long long terms = 0;
        int e = b;
        while (e < NBUCKET && (long long)e * bucket_rows < nrow && terms + hist[e] <= cap &&
               std::min(nrow, (long long)(e + 1) * bucket_rows) - r0 <= max_rows) {
            terms += hist[e];
            ++e;
        }
        if (e == b) {  // cannot happen (cap >= biggest, bucket_rows <= max_rows); guards the loop
            err = "stored build: slab formation failed";
            return UNOMOL_ECUDA;
        }
        ranges.push_back({r0, std::min(nrow, (long long)e * bucket_rows), terms});
        b = e;
    }
    unsigned* d_keys[2] = {nullptr, nullptr};
    double* d_vals[2] = {nullptr, nullptr};
    for (int t = 0; t < 2; ++t) {
        SCU(tmp.alloc(&d_keys[t], cap));
        SCU(tmp.alloc(&d_vals[t], cap));
    }
    size_t sort_bytes = 0, red_bytes = 0;
    {
        cub::DoubleBuffer<unsigned> kb(d_keys[0], d_keys[1]);
        cub::DoubleBuffer<double> vb(d_vals[0], d_vals[1]);
        SCU(cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, kb, vb, (int)std::min<unsigned long long>(cap, INT_MAX), 0, 32, s));
        SCU(cub::DeviceReduce::ReduceByKey(nullptr, red_bytes, d_keys[0], d_keys[1], d_vals[0], d_vals[1], d_nruns, AddOp(),
                                           (long long)cap, s));
    }
    void* d_cub = nullptr;
    const size_t cub_bytes = std::max(sort_bytes, red_bytes);
    SCU(tmp.alloc((char**)&d_cub, cub_bytes));
    double held = used + (double)cap * 24.0 + (double)cub_bytes;
    for (const Range& R : ranges) {
        if (R.terms > (unsigned long long)INT_MAX) {
            err = "stored build: a slab of more than 2^31 terms";
            return UNOMOL_EINVAL;
        }
        const int nt = (int)R.terms;
        const int rows = (int)(R.r1 - R.r0);
        SCU(cudaMemsetAsync(d_cursor, 0, sizeof(unsigned long long), s));
        slab_terms<<<grid_for(nrec, 256), 256, 0, s>>>(d_rec, nrec, st->kind, np, R.r0, R.r1, d_keys[0], d_vals[0], d_cursor, cap,
                                                        d_over);
        SCU(cudaGetLastError());
        int end_bit = 1;
        while (end_bit < 32 && ((unsigned long long)rows * (unsigned long long)np) > (1ull << end_bit)) ++end_bit;
        cub::DoubleBuffer<unsigned> kb(d_keys[0], d_keys[1]);
        cub::DoubleBuffer<double> vb(d_vals[0], d_vals[1]);
        size_t b1 = cub_bytes;
        SCU(cub::DeviceRadixSort::SortPairs(d_cub, b1, kb, vb, nt, 0, end_bit, s));
        size_t b2 = cub_bytes;
        SCU(cub::DeviceReduce::ReduceByKey(d_cub, b2, kb.Current(), kb.Alternate(), vb.Current(), vb.Alternate(), d_nruns, AddOp(),
                                           (long long)nt, s));
        long long nruns = 0;
        int over = 0;
        SCU(cudaMemcpyAsync(&nruns, d_nruns, sizeof(long long), cudaMemcpyDeviceToHost, s));
        SCU(cudaMemcpyAsync(&over, d_over, sizeof(int), cudaMemcpyDeviceToHost, s));
        SCU(cudaStreamSynchronize(s));
        if (over) {
            err = "stored build: slab term count exceeded its histogram (internal error)";
            return UNOMOL_ECUDA;
        }
        StoreSlab sl;
        sl.r0 = R.r0;
        sl.r1 = R.r1;
        sl.nnz = nruns;
        const size_t off_col = ((size_t)(rows + 1) * sizeof(int) + 255) & ~size_t(255);
        const size_t off_val = (off_col + (size_t)nruns * sizeof(int) + 255) & ~size_t(255);
        const size_t bytes = off_val + (size_t)nruns * sizeof(double);
        if (held + (double)bytes > budget) {
            err = "stored build: the matrix does not fit the memory budget (" + std::to_string((long long)((held + bytes) / 1048576.0)) +
                  " MiB needed so far)";
            return UNOMOL_ENOMEM;
        }
        SCU(cudaMalloc(&sl.mem, bytes));
        st->slabs.push_back(sl);  // owned by the store from here on (freed with it on failure)
        StoreSlab& S = st->slabs.back();
        S.rowptr = reinterpret_cast<int*>(S.mem);
        S.col = reinterpret_cast<int*>(S.mem + off_col);
        S.val = reinterpret_cast<double*>(S.mem + off_val);
        if (nruns == 0) {
            SCU(cudaMemsetAsync(S.rowptr, 0, sizeof(int) * (rows + 1), s));
        } else {
            slab_csr<<<grid_for(nruns, 256), 256, 0, s>>>(kb.Alternate(), vb.Alternate(), nruns, np, rows, S.rowptr, S.col, S.val);
            SCU(cudaGetLastError());
        }
        held += (double)bytes;
        st->nnz += nruns;
        st->bytes += (long long)bytes;
    }
    SCU(cudaStreamSynchronize(s));
    // the warps' pieces of every slab, from its row offsets
    for (StoreSlab& S : st->slabs) {
        const int rows = (int)(S.r1 - S.r0);
        std::vector<int> rp(rows + 1);
        SCU(cudaMemcpy(rp.data(), S.rowptr, sizeof(int) * (rows + 1), cudaMemcpyDeviceToHost));
        std::vector<RowPiece> pc;
        for (int r = 0; r < rows; ++r) {
            const int b = rp[r], e = rp[r + 1];
            if (e <= b) continue;
            const int n = (e - b + PIECE_MAX - 1) / PIECE_MAX;
            for (int t = 0; t < n; ++t)
                pc.push_back({r, b + (int)((long long)(e - b) * t / n), b + (int)((long long)(e - b) * (t + 1) / n), n == 1 ? 1 : 0});
        }
        S.npieces = (int)pc.size();
        if (S.npieces) {
            SCU(cudaMalloc(&S.pieces, sizeof(RowPiece) * pc.size()));
            SCU(cudaMemcpy(S.pieces, pc.data(), sizeof(RowPiece) * pc.size(), cudaMemcpyHostToDevice));
        }
        st->bytes += (long long)(sizeof(RowPiece) * pc.size());
    }
    return UNOMOL_OK;
}

// Record pass over every class launch of the context into a device array (capacity: every element of
// every work item's rectangle).  *d_rec is owned by the caller's scratch.
int record_pass(const CtxView& v, Scratch& tmp, UnomolRecord** d_rec, long long* nrec, double budget, double* used,
                cudaStream_t s, std::string& err) {
    unsigned long long cap = 0;
    for (const ClassLaunchInfo& L : v.launches)
        cap += (unsigned long long)L.nwork * ncart(pc_la(L.bc)) * ncart(pc_lb(L.bc)) * ncart(pc_la(L.kc)) * ncart(pc_lb(L.kc));
    cap = std::max<unsigned long long>(cap, 1);
    if ((double)cap * sizeof(UnomolRecord) > budget) {
        err = "stored build: room for " + std::to_string(cap) + " records (" + std::to_string((long long)(cap * 24.0 / 1048576.0)) +
              " MiB) exceeds the memory budget";
        return UNOMOL_ENOMEM;
    }
    unsigned long long* d_count = nullptr;
    int* d_over = nullptr;
    SCU(tmp.alloc(d_rec, cap));
    SCU(tmp.alloc(&d_count, 1));
    SCU(tmp.alloc(&d_over, 1));
    SCU(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), s));
    SCU(cudaMemsetAsync(d_over, 0, sizeof(int), s));
    RecSink S{*d_rec, d_count, cap, d_over};
    FockArgs A{};
    A.pairs = v.d_pairs;
    A.prims = v.d_prims;
    A.prims32 = v.d_prims32;
    A.prefix = v.d_prefix;
    A.nbf = v.nbf;
    A.nshell = v.nshell;
    A.thr_int = STORE_CUT;
    A.prim_cut = PRIM_CUT;
    A.thr_int32 = (float)STORE_CUT;
    A.prim_cut32 = (float)PRIM_CUT;
    A.rys_compat = v.rys_compat;
    A.mode = 0;
    for (const ClassLaunchInfo& L : v.launches) {
        A.bps = v.d_bps + L.bp_begin;
        A.nbp = L.nbp;
        A.nwork = L.nwork;
        SCU(store_class(v, L, A, S, s));
    }
    unsigned long long count = 0;
    int over = 0;
    SCU(cudaMemcpyAsync(&count, d_count, sizeof(count), cudaMemcpyDeviceToHost, s));
    SCU(cudaMemcpyAsync(&over, d_over, sizeof(int), cudaMemcpyDeviceToHost, s));
    SCU(cudaStreamSynchronize(s));
    if (over || count > cap) {
        err = "stored build: record pass overflowed its capacity (internal error)";
        return UNOMOL_ECUDA;
    }
    *nrec = (long long)count;
    *used = (double)cap * sizeof(UnomolRecord);
    return UNOMOL_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

struct Events {
    cudaEvent_t e[3] = {nullptr, nullptr, nullptr};
    Events() {
        for (auto& x : e) cudaEventCreate(&x);
    }
    ~Events() {
        for (auto& x : e)
            if (x) cudaEventDestroy(x);
    }
};

int check_kind(int kind, std::string& err) {
    if (kind != UNOMOL_STORE_RHF && kind != UNOMOL_STORE_UHF) {
        err = "unknown store kind (UNOMOL_STORE_RHF or UNOMOL_STORE_UHF)";
        return UNOMOL_EINVAL;
    }
    return UNOMOL_OK;
}

}  // namespace

int store_from_integrals(const CtxView& v, int kind, double max_gib, IntStore** out, std::string& err) {
    *out = nullptr;
    if (int rc = check_kind(kind, err)) return rc;
    const double budget = budget_bytes(max_gib);
    cudaStream_t s = v.stream;
    Events ev;
    Scratch tmp;
    UnomolRecord* d_rec = nullptr;
    long long nrec = 0;
    double used = 0.0;
    SCU(cudaEventRecord(ev.e[0], s));
    int rc = record_pass(v, tmp, &d_rec, &nrec, budget, &used, s, err);
    if (rc) return rc;
    SCU(cudaEventRecord(ev.e[1], s));
    IntStore* st = new IntStore();
    st->kind = kind;
    st->nbf = v.nbf;
    st->np = (long long)v.nbf * (v.nbf + 1) / 2;
    st->records = nrec;
    st->max_gib = max_gib;
    rc = assemble(st, d_rec, nrec, budget, used, s, err);
    if (rc) {
        store_free(st);
        return rc;
    }
    cudaEventRecord(ev.e[2], s);
    cudaEventSynchronize(ev.e[2]);
    st->ms_records = elapsed(ev.e[0], ev.e[1]);
    st->ms_assemble = elapsed(ev.e[1], ev.e[2]);
    *out = st;
    return UNOMOL_OK;
}

int store_from_file(const CtxView& v, const char* path, int kind, double max_gib, IntStore** out, std::string& err) {
    *out = nullptr;
    if (int rc = check_kind(kind, err)) return rc;
    FILE* f = fopen(path, "rb");
    if (!f) {
        err = std::string("cannot open record file ") + path;
        return UNOMOL_EINVAL;
    }
    std::unique_ptr<FILE, int (*)(FILE*)> guard(f, fclose);
    if (fseeko(f, 0, SEEK_END) != 0) {
        err = "cannot size the record file";
        return UNOMOL_EINVAL;
    }
    const long long size = (long long)ftello(f);
    fseeko(f, 0, SEEK_SET);
    if (size < 0 || size % (long long)sizeof(UnomolRecord)) {
        err = "record file size is not a multiple of 24 bytes";
        return UNOMOL_EINVAL;
    }
    const long long nrec = size / (long long)sizeof(UnomolRecord);
    const double budget = budget_bytes(max_gib);
    if ((double)size > budget) {
        err = "record file larger than the memory budget";
        return UNOMOL_ENOMEM;
    }
    cudaStream_t s = v.stream;
    Events ev;
    Scratch tmp;
    UnomolRecord* d_rec = nullptr;
    unsigned long long* d_bad = nullptr;
    SCU(tmp.alloc(&d_rec, (size_t)std::max<long long>(nrec, 1)));
    SCU(tmp.alloc(&d_bad, 1));
    SCU(cudaEventRecord(ev.e[0], s));
    {
        const long long chunk = 1 << 20;  // records per read
        std::vector<UnomolRecord> buf((size_t)std::min(chunk, std::max<long long>(nrec, 1)));
        for (long long done = 0; done < nrec;) {
            const long long m = std::min(chunk, nrec - done);
            if ((long long)fread(buf.data(), sizeof(UnomolRecord), (size_t)m, f) != m) {
                err = "short read of the record file";
                return UNOMOL_EINVAL;
            }
            SCU(cudaMemcpyAsync(d_rec + done, buf.data(), (size_t)m * sizeof(UnomolRecord), cudaMemcpyHostToDevice, s));
            SCU(cudaStreamSynchronize(s));  // the host buffer is reused
            done += m;
        }
    }
    SCU(cudaMemsetAsync(d_bad, 0, sizeof(unsigned long long), s));
    if (nrec > 0) check_records<<<grid_for(nrec, 256), 256, 0, s>>>(d_rec, nrec, v.nbf, d_bad);
    SCU(cudaGetLastError());
    unsigned long long bad = 0;
    SCU(cudaMemcpyAsync(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost, s));
    SCU(cudaStreamSynchronize(s));
    if (bad) {
        err = "record " + std::to_string(bad - 1) + " of the file is not a canonical record of this basis (i >= j, k >= l, "
              "(i,j) >= (k,l), labels below " + std::to_string(v.nbf) + ", finite value)";
        return UNOMOL_EINVAL;
    }
    SCU(cudaEventRecord(ev.e[1], s));
    IntStore* st = new IntStore();
    st->kind = kind;
    st->nbf = v.nbf;
    st->np = (long long)v.nbf * (v.nbf + 1) / 2;
    st->records = nrec;
    st->max_gib = max_gib;
    const int rc = assemble(st, d_rec, nrec, budget, (double)size, s, err);
    if (rc) {
        store_free(st);
        return rc;
    }
    cudaEventRecord(ev.e[2], s);
    cudaEventSynchronize(ev.e[2]);
    st->ms_records = elapsed(ev.e[0], ev.e[1]);
    st->ms_assemble = elapsed(ev.e[1], ev.e[2]);
    *out = st;
    return UNOMOL_OK;
}

int write_records(const CtxView& v, const char* path, long long* count, std::string& err) {
    cudaStream_t s = v.stream;
    Scratch tmp;
    UnomolRecord* d_rec = nullptr;
    long long nrec = 0;
    double used = 0.0;
    int rc = record_pass(v, tmp, &d_rec, &nrec, budget_bytes(0.0), &used, s, err);
    if (rc) return rc;
    FILE* f = fopen(path, "wb");
    if (!f) {
        err = std::string("cannot create record file ") + path;
        return UNOMOL_EINVAL;
    }
    std::unique_ptr<FILE, int (*)(FILE*)> guard(f, fclose);
    const long long chunk = 1 << 20;
    std::vector<UnomolRecord> buf((size_t)std::min(chunk, std::max<long long>(nrec, 1)));
    for (long long done = 0; done < nrec;) {
        const long long m = std::min(chunk, nrec - done);
        SCU(cudaMemcpyAsync(buf.data(), d_rec + done, (size_t)m * sizeof(UnomolRecord), cudaMemcpyDeviceToHost, s));
        SCU(cudaStreamSynchronize(s));
        if ((long long)fwrite(buf.data(), sizeof(UnomolRecord), (size_t)m, f) != m) {
            err = std::string("short write to ") + path;
            return UNOMOL_EINVAL;
        }
        done += m;
    }
    if (fflush(f) != 0) {
        err = std::string("cannot flush ") + path;
        return UNOMOL_EINVAL;
    }
    *count = nrec;
    return UNOMOL_OK;
}

cudaError_t store_fock(const IntStore* st, const double* dPa, const double* dPb, double* dGa, double* dGb, cudaStream_t s,
                       int* launches) {
    const bool uhf = dPb != nullptr;
    if (uhf && st->kind != UNOMOL_STORE_UHF) return cudaErrorInvalidValue;
    const int mode = st->kind == UNOMOL_STORE_RHF ? 0 : (uhf ? 2 : 1);
    for (const StoreSlab& S : st->slabs) {
        if (S.npieces <= 0) continue;
        const unsigned blocks = (unsigned)((S.npieces + 7) / 8);  // eight warps (pieces) per CTA
        if (mode == 0)
            store_spmv<0><<<blocks, 256, 0, s>>>(S.pieces, S.npieces, S.col, S.val, S.r0, st->np, dPa, dPb, dGa, dGb);
        else if (mode == 1)
            store_spmv<1><<<blocks, 256, 0, s>>>(S.pieces, S.npieces, S.col, S.val, S.r0, st->np, dPa, dPb, dGa, dGb);
        else
            store_spmv<2><<<blocks, 256, 0, s>>>(S.pieces, S.npieces, S.col, S.val, S.r0, st->np, dPa, dPb, dGa, dGb);
        ++*launches;
    }
    return cudaGetLastError();
}

int store_kind(const IntStore* st) { return st ? st->kind : 0; }

double store_max_gib(const IntStore* st) { return st ? st->max_gib : 0.0; }

void store_info(const IntStore* st, UnomolStoreInfo* out) {
    std::memset(out, 0, sizeof(*out));
    if (!st) return;
    out->kind = st->kind;
    out->slabs = (int)st->slabs.size();
    out->records = st->records;
    out->nonzeros = st->nnz;
    out->bytes = st->bytes;
    out->ms_records = st->ms_records;
    out->ms_assemble = st->ms_assemble;
}

void store_free(IntStore* st) {
    if (!st) return;
    for (StoreSlab& S : st->slabs) {
        if (S.mem) cudaFree(S.mem);
        if (S.pieces) cudaFree(S.pieces);
    }
    delete st;
}

}  // namespace ugb
