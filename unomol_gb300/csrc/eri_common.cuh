// Shared device/host definitions of the direct Fock build: data layout of shell pairs and primitive
// pairs in HBM, Cartesian component tables, and the Rys root/weight evaluation.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ugb {

constexpr int LMAX = 4;                 // largest shell angular momentum (g; Basis.hpp:222)
constexpr int LTMPL = 2;                // shells up to d have class-templated Rys kernels
constexpr int NPAIRCLASS = (LMAX + 1) * (LMAX + 2) / 2;  // (la >= lb) pair classes
constexpr int NTMPLCLASS = (LTMPL + 1) * (LTMPL + 2) / 2;
constexpr double SRTERM = 34.9868366552497250;  // 2 pi^{5/2} (TwoElectronInts.cpp:427)
constexpr double PRIM_CUT = 1.e-12;     // primitive prefactor cut (TwoElectronInts.cpp:428,478-479)
constexpr double STORE_CUT = 1.e-14;    // integral storage cut (TwoElectronInts.cpp:517,668)

__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }
__host__ __device__ constexpr int pair_class(int la, int lb) { return la * (la + 1) / 2 + lb; }

// Cartesian exponents of component c of a shell with angular momentum l, in the reference's order:
// lx descending, then ly descending (AuxFunctions.hpp:35-43).
// Closed form (components with lx = l - i form the i-th block of i+1 entries, ly descending), so
// that unrolled kernels fold it to constants without evaluating loops.
__host__ __device__ constexpr int cart_blk(int c) { return (c >= 1) + (c >= 3) + (c >= 6) + (c >= 10); }
__host__ __device__ constexpr int cart_lx(int l, int c) { return l - cart_blk(c); }
__host__ __device__ constexpr int cart_ly(int l, int c) {
    return cart_blk(c) - (c - cart_blk(c) * (cart_blk(c) + 1) / 2);
}
__host__ __device__ constexpr int cart_lz(int l, int c) { return l - cart_lx(l, c) - cart_ly(l, c); }

// One primitive pair of a shell pair (a has the larger L after the swap of
// TwoElectronInts.cpp:563-579); the kernels read it through the read-only path.
struct __align__(16) PrimPair {
    double p;          // alpha_a + alpha_b
    double rp;         // 1 / p
    double P[3];       // Gaussian product centre
    double PA[3];      // P - A
    double E;          // exp(-alpha_a alpha_b |AB|^2 / p) / p, coefficient free (prefactor screen)
    double cc;         // c_a c_b, times 2 for the i != j half of a same-shell pair
                       // (TwoElectronInts.cpp:444-449)
    double Ecc;        // sqrt(2 pi^{5/2}) E cc: a primitive quartet's prefactor is Ecc_ab Ecc_cd / sqrt(p + q)
    float pf, Ef;      // p and E in FP32, for a cheap pre-screen (96 bytes: six 16-byte loads)
};

struct __align__(16) PrimPair32 {
    float p, rp, P[3], PA[3], E, cc;
    float Ecc;      // sqrt(2 pi^{5/2}) E cc, as PrimPair::Ecc
    float pad_;     // 48 bytes: three 16-byte loads
};

constexpr double SQRT_SRTERM = 5.914967172795613;  // sqrt(2 pi^{5/2})
static_assert(SQRT_SRTERM * SQRT_SRTERM - SRTERM < 1e-13 && SRTERM - SQRT_SRTERM * SQRT_SRTERM < 1e-13, "sqrt of SRTERM");

// One shell pair, sorted into blocks of equal (class, primitive-pair count), within a block by
// descending Schwarz bound.
struct ShellPair {
    int a_off, b_off;      // first AO of shell a (larger L) and of shell b
    int la, lb;            // la >= lb
    int prim_begin, nprim; // primitive pair ik of this pair at prim_begin + ik * prim_stride
    int prim_stride;       // pairs of one block (equal nprim) interleave their primitive pairs: the
                           // stride is the block's pair count, so consecutive pairs' records are adjacent
    int same;              // ish == jsh
    double AB[3];          // A - B
    double q;              // Schwarz bound: max over functions of sqrt|(ab|ab)|
    int ish, jsh;          // shell indices (ish >= jsh)
    int maxsh;             // max(ish, jsh)
    int pad;
    float ABf[3];          // A - B and q in FP32, for the FP32 kernels (no FP64 work or conversion there)
    float qf;
};

// A rectangle (or triangle, when bra block == ket block) of quartets between two pair blocks,
// trimmed by the Schwarz staircase: bra pair i pairs with the first cnt[i] ket pairs of its block.
struct BlockPair {
    int bra_begin, bra_count;   // pair index range of the bra block
    int ket_begin, ket_count;   // pair index range of the ket block
    int triangle;               // bra block == ket block: ket index <= bra index
    int prefix_off;             // offset of this block pair's prefix array (bra_count + 1 entries)
    int prim_quartets;          // primitive quartets of each of its shell quartets (nprim bra x nprim ket)
    long long work_begin;       // first work item (multiple of 32, so warps never straddle)
    long long work_count;       // quartets in this block pair
};

// Kernel arguments shared by every class instance.
struct FockArgs {
    const ShellPair* pairs;
    const PrimPair* prims;
    const PrimPair32* prims32;
    const BlockPair* bps;
    const long long* prefix;    // concatenated staircase prefix sums
    int nbp;                    // block pairs of this launch
    long long nwork;            // work items of this launch (padded)
    int nbf;
    const double* Pa;           // full N x N density (RHF: P; UHF: Pa)
    const double* Pb;           // UHF: Pb; RHF: nullptr
    const float* Pa32;          // FP32 copies of Pa / Pb for the FP32 kernels' density contraction
    const float* Pb32;
    const float* pmax;          // shell-pair max |P| (nshell x nshell), for density screening
    double* Ta;                 // N x N accumulators; G = T + T^T
    double* Tb;                 // UHF beta accumulator
    double thr_int;             // per-integral cut (1e-14)
    double prim_cut;            // primitive prefactor cut (1e-12)
    float thr_int32, prim_cut32, skip_cut32;  // the same cuts in FP32, for the FP32 kernels
    float fp32_cut32;           // mixed mode: a quartet with bound * max|P| of its blocks below this runs in FP32
    double fp32_cut;            // mixed mode: bound * max|P| below this -> FP32 part, else FP64 part
    int mode;                   // 0 all quartets; 1 only "large" (FP64 part); 2 only "small" (FP32 part)
    int nshell;
    int rys_compat;             // reference-compatible two-root Rys regime (FP64 only)
    unsigned long long* counters;  // optional: primitive quartets past the prefactor cut, 32 slots per launch
    int counter_base;           // first slot of this launch (class id * 32)
    // density-screened / mixed-precision builds (mode 1 = FP64 part, mode 2 = FP32 part): per-build
    // work lists made on the device (split_rows + scan_rows)
    const long long* dyn_prefix;  // per bra row, exclusive prefix of this part's quartets (prefix layout)
    const long long* dyn_count;   // per block pair of this launch: quartets of this part
    const long long* dyn_begin;   // per block pair of this launch: its first item in this part's compact
                                  // numbering (counts rounded up to 32 and summed over the launch)
    const long long* dyn_total;   // [0]: items of this part in the launch (the compact numbering's end)
    const int* dyn_mseg;          // per bra row: length of its FP64 segment (the FP32 segment follows it)
    const float* dmax;            // [0]: max |P| over all shell-pair blocks
    double skip_cut;              // quartets with bound * max|P| below this are skipped
    // batches of molecules: ShellPair::pad holds the molecule; its dense P / T start at mol_base and
    // have mol_nbf rows (nullptr: one molecule, A.nbf rows at offset 0)
    const int* mol_nbf;
    const long long* mol_base;
    const int* mol_nshell;        // batches in the screened build: shells of the molecule and the first
    const long long* mol_pmax;    // entry of its shell-pair max|P| blocks in pmax
    unsigned long long* tile_counter;  // persistent launches: next tile of this launch
    int* status;                // device error flag
};

}  // namespace ugb
