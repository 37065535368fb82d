/*
 * unomol_gb300 -- C ABI of the GB300 (sm_103a) direct two-electron Fock build.
 *
 * This is the drop-in boundary for unomol's TwoElectronInts class (TwoElectronInts.hpp:79-110).
 * The reference computes every unique integral once in its constructor, stores them in a cache and
 * streams the cache on every formGmatrix call.  Here the constructor uploads the basis and builds
 * shell pairs and Schwarz bounds on the GPU; every formGmatrix call recomputes the integrals on the
 * GPU and contracts them directly into G (direct SCF), unless the context holds a store of the
 * integrals (unomol_gpu_store_integrals below: the reference's conventional scheme, in device memory).
 *
 * Conventions (identical to the reference):
 *   - packed lower triangle, row major: element (i, j), j <= i, at i*(i+1)/2 + j, N*(N+1)/2 doubles;
 *   - AO order = shell order of the basis; Cartesian components of a shell ordered lx descending,
 *     then ly descending (AuxFunctions.hpp:35-43);
 *   - centres in bohr; contraction coefficients already normalised as Basis::normalize leaves them
 *     (Basis.hpp:56-75);
 *   - P is the reference's RHF density C_occ C_occ^T (RHF.hpp:192-203), G = 2 J(P) - K(P);
 *     UHF: Ga = J(Pa + Pb) - K(Pa), Gb = J(Pa + Pb) - K(Pb) (TwoElectronInts.cpp:749-820);
 *   - formGmatrix ADDS into the caller's G (the callers zero it first: RHF.hpp:89-90, UHF.hpp:103-107).
 *
 * Every entry point returns 0 on success and a negative UNOMOL_E* code on failure; the message is
 * available from unomol_gpu_last_error().  There is no CPU fallback: without a usable GPU the calls
 * fail with UNOMOL_ENODEV.
 */
#ifndef UNOMOL_GB300_H
#define UNOMOL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UNOMOL_OK 0
#define UNOMOL_EINVAL (-1)   /* bad argument (sizes, L > supported, null pointers) */
#define UNOMOL_ENODEV (-2)   /* no CUDA device / driver */
#define UNOMOL_ECUDA (-3)    /* a CUDA runtime or library call failed */
#define UNOMOL_ENOMEM (-4)   /* device allocation failed */
#define UNOMOL_ETIMEOUT (-5) /* a bounded device wait gave up */
#define UNOMOL_ESCF (-6)     /* SCF driver: singular overlap, eigen-solver failure */

/* Precision modes (unomol_gpu_set_precision). */
#define UNOMOL_PREC_FP64 0  /* every quartet in FP64 (the plain path; the default) */
#define UNOMOL_PREC_MIXED 1 /* quartets with Schwarz bound * max|P| below the cutoff in FP32 */

/* Flat description of a basis (the data of unomol::Basis, Basis.hpp:157-170). */
typedef struct UnomolBasisDesc {
    int nshell;               /* number of shells */
    int norb;                 /* number of basis functions (sum of (L+1)(L+2)/2) */
    int ncen;                 /* number of centres */
    const int* shell_l;       /* [nshell] angular momentum, 0..4 */
    const int* shell_nprim;   /* [nshell] primitives per shell */
    const int* shell_center;  /* [nshell] centre index */
    const int* shell_offset;  /* [nshell] first AO of the shell (Basis::offset, Basis.hpp:226-232) */
    const double* alpha;      /* [sum nprim] exponents, shell after shell */
    const double* coef;       /* [sum nprim] normalised contraction coefficients */
    const double* centers;    /* [ncen*3] positions in bohr */
} UnomolBasisDesc;

typedef struct UnomolCtx UnomolCtx;

/* Counters of the last Fock build (for throughput figures). */
typedef struct UnomolStats {
    int64_t shell_quartets;        /* unique shell quartets after Schwarz screening */
    int64_t shell_quartets_fp32;   /* of which evaluated in FP32 (mixed mode) */
    int64_t shell_quartets_total;  /* unique shell quartets before screening */
    int64_t function_quartets;     /* unique function quartets after screening (canonical count) */
    int64_t primitive_quartets;    /* primitive quartets after Schwarz screening (before the 1e-12 cut) */
    double ms_eri;                 /* device time of the last build's ERI + J/K kernels */
    double ms_total;               /* device time of the last build (including P expand / G fold) */
    int nbf;                       /* basis functions */
    int npairs;                    /* shell pairs kept */
    int kernel_launches;           /* kernels launched by the last build */
    int pad_;
    /* filled only while counting is on (unomol_gpu_set_counting): */
    int64_t primitive_quartets_computed; /* primitive quartets past the 1e-12 prefactor cut */
    double eri_flops;              /* algorithmic flops of the ERI + J/K kernels (FMA = 2): per primitive
                                      quartet its setup, roots, recurrences and transfers, per shell
                                      quartet its density contraction, counted from the kernels' steps */
    double eri_flops_fp32;         /* of which in the FP32 kernels (mixed mode) */
    int64_t function_quartets_computed; /* function quartets of the last build's work lists (in the
                                           density-screened and mixed builds: its FP64 and FP32 parts,
                                           without the quartets the per-quartet density screen drops) */
    int64_t shell_quartets_screened;    /* density-screened and mixed builds: quartets of the work lists
                                           dropped by the per-quartet density screen (max |P| of the six
                                           blocks a quartet contracts with, times its bound) */
    int64_t shell_quartets_demoted;     /* mixed builds: quartets of the FP64 part's work lists run in FP32
                                           because their own density bound (as above) is below the FP32
                                           cutoff (included in shell_quartets_fp32) */
} UnomolStats;

/* TwoElectronInts(basis, start_shell, label) -- TwoElectronInts.hpp:83-88.
 * Uploads the basis, builds shell pairs, Schwarz bounds and the class work lists on device 0 (or
 * the current device).  start_shell: only quartets whose largest shell index is >= start_shell
 * contribute (TwoElectronInts.cpp:541; used by the DPM path, RHF.hpp:315). */
int unomol_gpu_create(const UnomolBasisDesc* basis, int start_shell, UnomolCtx** out);

/* TwoElectronInts::recalculate(basis) -- TwoElectronInts.hpp:94-96 (centre moved: RHF.hpp:354).
 * centers: [ncen*3] new positions in bohr; shells and exponents are unchanged. */
int unomol_gpu_recalculate(UnomolCtx* ctx, const double* centers);

/* TwoElectronInts::formGmatrix(P, G) -- TwoElectronInts.cpp:822-844.  Host pointers, packed. */
int unomol_gpu_fock_rhf(UnomolCtx* ctx, const double* P, double* G);

/* TwoElectronInts::formGmatrix(Pa, Pb, Ga, Gb) -- TwoElectronInts.cpp:846-869.  Host pointers. */
int unomol_gpu_fock_uhf(UnomolCtx* ctx, const double* Pa, const double* Pb, double* Ga, double* Gb);

/* Device-resident variants of the two calls above: all pointers are device pointers (packed),
 * `stream` is a cudaStream_t (NULL = the context's own stream).  G is added into, as above. */
int unomol_gpu_fock_rhf_device(UnomolCtx* ctx, const double* dP, double* dG, void* stream);
int unomol_gpu_fock_uhf_device(UnomolCtx* ctx, const double* dPa, const double* dPb, double* dGa,
                               double* dGb, void* stream);

/* Precision form (no reference counterpart; the reference is FP64 only).
 * UNOMOL_PREC_FP64 (default): every quartet that passes the integral Schwarz cut, in FP64.
 * UNOMOL_PREC_MIXED: density-screened build made per call on the device.  With b = sqrt((ab|ab))
 *   sqrt((cd|cd)) and D = max |P| over the density passed in: quartets with b*D >= fp32_cutoff run in
 *   FP64, quartets with skip_cut <= b*D < fp32_cutoff in FP32 (Rys roots, recurrences, contraction and
 *   the density contraction of each quartet in FP32; its J/K sums added into G in FP64), the rest (and
 *   quartets whose six density blocks are all small) are skipped.  Meant for incremental builds
 *   G(P) = G(P_old) + G(dP),
 *   where |dP| shrinks as the SCF converges.  fp32_cutoff <= skip_cut gives a density-screened FP64
 *   build. */
int unomol_gpu_set_precision(UnomolCtx* ctx, int mode, double fp32_cutoff);

/* skip_cut of the density-screened build (default 1e-13: at 1e-12 the skipped quartets of a 416-function
 * cluster left ~1e-9 Eh of noise per incremental build, too much for a 1e-10 Eh convergence test). */
int unomol_gpu_set_density_screening(UnomolCtx* ctx, double skip_cut);

/* Rys quadrature of the two-root classes (unomol_gpu_set_rys_mode).
 * UNOMOL_RYS_REFERENCE (default): for 15 < T <= 40 the two-root nodes and weights follow the
 *   reference's own fit (Rys::root2, Rys.cpp:611-623), which departs from the exact quadrature by up
 *   to 3.5e-4 relative at T = 15; G and energies then match the reference's.
 * UNOMOL_RYS_EXACT: exact quadrature at every T (all other root counts are exact in both modes;
 *   the reference's root1 and root3..5 agree with exact quadrature to ~1e-13). */
#define UNOMOL_RYS_REFERENCE 0
#define UNOMOL_RYS_EXACT 1
int unomol_gpu_set_rys_mode(UnomolCtx* ctx, int mode);

/* Integral method (unomol_gpu_set_eri_method).
 * UNOMOL_ERI_REFERENCE (default): Rys quadrature for la+lb+lc+ld <= 8 and McMurchie-Davidson above,
 *   as the reference's default build (TwoElectronInts.cpp:658-666).
 * UNOMOL_ERI_MD: McMurchie-Davidson for every quartet, as the reference built with -DUNOMOL_MD_INTS.
 * The MD integrals use the reference's Boys evaluation (MD_Rfunction.hpp:2185-2206). */
#define UNOMOL_ERI_REFERENCE 0
#define UNOMOL_ERI_MD 1
int unomol_gpu_set_eri_method(UnomolCtx* ctx, int method);

/* Schwarz cutoff on sqrt((ab|ab)) sqrt((cd|cd)).  Default 1e-14: the reference drops stored
 * integrals with |v| <= 1e-14 (TwoElectronInts.cpp:668), so quartets whose bound is below that
 * contribute nothing there either.  Rebuilds the work lists. */
int unomol_gpu_set_screening(UnomolCtx* ctx, double schwarz_cutoff);

int unomol_gpu_get_stats(const UnomolCtx* ctx, UnomolStats* out);

/* Work counting for throughput figures (no reference counterpart): while on, every Fock build counts
 * the primitive quartets its kernels evaluate and fills the counting fields of UnomolStats; the build
 * then synchronises its stream before returning. */
int unomol_gpu_set_counting(UnomolCtx* ctx, int on);

/* Order of the class launches of a Fock build (no reference counterpart; a diagnostic control):
 * 0 (default) in class order, non-zero in reverse.  The J/K contributions meet in FP64 atomics, so the
 * order of the additions, and with it the rounding of G, changes from launch order to launch order and
 * from run to run; the determinism tests bound that difference. */
int unomol_gpu_set_launch_order(UnomolCtx* ctx, int reversed);

/* Device time of the last Fock build, from CUDA events recorded on the build's stream (no reference
 * counterpart): ms_eri covers the ERI + J/K kernels, ms_total the whole build.  Waits for the build. */
int unomol_gpu_last_build_ms(UnomolCtx* ctx, double* ms_eri, double* ms_total);

/* FMA throughput of the current device (no reference counterpart): TFLOP/s of a dependent-chain FMA
 * kernel over every SM, FP64 (fp64 = 1) or FP32 (fp64 = 0).  The roofline denominator of the Fock
 * kernels, which are bound by the FP64 (or FP32) pipe. */
int unomol_gpu_fma_peak(int fp64, double* tflops);
/* L2 figures of the J/K scatter, measured on the current device: read bandwidth of an L2-resident 32 MiB
 * buffer (GB/s) and FP64 atomicAdd throughput on a 416 x 416 accumulator (10^9 atomics/s). */
int unomol_gpu_l2_peak(double* read_gbs, double* atomic_gops);

/* Allocation-free RHF Fock build.  No counterpart in the reference (its Fock build runs on the host).
 * Same contract as unomol_gpu_fock_rhf_device (device pointers, packed P in, packed G added into,
 * NULL stream = the context's stream), for callers that must not trigger cudaMalloc once they run:
 * a host framework that owns every device allocation after start-up, or an iteration loop that must
 * not take cudaMalloc's implicit device synchronisation.  Create the context during start-up; this
 * call then allocates nothing: its per-build scratch (dense P and the N x N accumulator) lives in a
 * 16 MiB static device array of the library, which every GPU that loads the library's kernels holds
 * until exit.  Limits: at most 1024 basis functions (larger bases return UNOMOL_EINVAL with a
 * message) and the FP64 precision mode only.  Every integral method of the regular build runs: the
 * Rys kernels for s/p/d/f/g classes up to la+lb+lc+ld = 8, MD above that and in UNOMOL_ERI_MD mode.
 * Counting mode (unomol_gpu_set_counting) is rejected with UNOMOL_EINVAL (its counters would need an
 * allocation); the build's launch count and event timings (unomol_gpu_get_stats,
 * unomol_gpu_last_build_ms) describe the last call.  The first call on a device looks up the array's
 * device address; make that first call before any stream capture.  Every call shares the one array,
 * so calls that overlap on the GPU (other streams, other host threads) race; serialise them. */
int unomol_gpu_fock_rhf_noalloc(UnomolCtx* ctx, const double* dP, double* dG, void* stream);

/* ---- Conventional build from stored integrals ----
 * The reference computes every unique integral once (TwoElectronInts.cpp:511-697), keeps each one with
 * |v| > 1e-14 as a 24-byte record {double val; int i, j, k, l} (TwoInts, TwoElectronInts.hpp:20-23) in
 * an 8 GiB memory cache that spills to its integral file (cache.hpp:18-386), and streams the records
 * through its scatter on every formGmatrix call (TwoElectronInts.cpp:699-869).  These calls give the
 * same two things on the GPU:
 *   - the records: unomol_gpu_write_records computes the canonical integrals (i >= j, k >= l,
 *     (i,j) >= (k,l) in that order, the reference's labels and storage cut; the same set the reference
 *     stores, in another order) and writes them as raw 24-byte records, the layout of the reference's
 *     integral file;
 *   - a stored build: unomol_gpu_store_integrals computes the records on the GPU (or
 *     unomol_gpu_store_records reads them from such a file) and turns them into the sparse matrix of
 *     the linear map P -> G over packed indices, kept in device memory.  While a context holds a
 *     store, unomol_gpu_fock_rhf/uhf and their _device variants stream that matrix (FP64, no
 *     integrals recomputed); the precision, density-screening and integral-method settings then play
 *     no part.  unomol_gpu_recalculate rebuilds the store for the new centres; unomol_gpu_drop_store
 *     returns to the direct build.  The allocation-free build always runs the direct build.
 * The store holds one matrix element per distinct (row, column) pair: for RHF (UNOMOL_STORE_RHF) the
 * matrix of G = 2J - K; for UHF (UNOMOL_STORE_UHF) the J and the K matrices, which serve RHF builds
 * as well.  Its size grows with the square of the surviving shell quartets: for the 32-water 6-31G
 * cluster (416 functions) about 10^9 elements, 12 bytes each.  max_gib bounds the device memory that
 * building the store may hold at once (0: 64 GiB); a store that does not fit returns UNOMOL_ENOMEM. */
typedef struct UnomolRecord {
    double val;
    int32_t i, j, k, l;
} UnomolRecord; /* TwoInts (TwoElectronInts.hpp:20-23): 24 bytes */

#define UNOMOL_STORE_RHF 1
#define UNOMOL_STORE_UHF 2

typedef struct UnomolStoreInfo {
    int kind;            /* 0 (no store), UNOMOL_STORE_RHF or UNOMOL_STORE_UHF */
    int slabs;           /* row ranges the matrix is kept in */
    int64_t records;     /* integral records the store was made from */
    int64_t nonzeros;    /* stored matrix elements */
    int64_t bytes;       /* device bytes of the store (values, columns, row offsets) */
    double ms_records;   /* device time of the integral pass (or of reading and checking the records) */
    double ms_assemble;  /* device time of turning the records into the matrix (sorts and merges) */
} UnomolStoreInfo;

/* TwoElectronInts::calculate (TwoElectronInts.cpp:511-697) into a store on the device; see above. */
int unomol_gpu_store_integrals(UnomolCtx* ctx, int kind, double max_gib);
/* The same from a file of 24-byte records (the reference's integral file layout, or the output of
 * unomol_gpu_write_records); the records must be canonical and index the context's basis. */
int unomol_gpu_store_records(UnomolCtx* ctx, const char* path, int kind, double max_gib);
/* Back to the direct build; frees the store. */
int unomol_gpu_drop_store(UnomolCtx* ctx);
int unomol_gpu_store_info(const UnomolCtx* ctx, UnomolStoreInfo* out);
/* Computes the canonical records of the context's basis on the GPU and writes them to `path` as raw
 * 24-byte records (cache.hpp:298-327 writes the same layout); *count = records written. */
int unomol_gpu_write_records(UnomolCtx* ctx, const char* path, int64_t* count);

void unomol_gpu_destroy(UnomolCtx* ctx);

/* ---- Batches of molecules (no reference counterpart: the reference handles one molecule) ----
 * Many molecules of uneven size share one launch per quartet class: their shell pairs and Schwarz
 * staircases are merged, and a persistent kernel per class pulls tiles of work from an atomic counter.
 * The batch owns a packed P and a packed G buffer on the device (molecule m at packed_offsets[m]);
 * a build writes G = G(P) for every molecule (RHF, FP64, shells up to d). */
typedef struct UnomolBatch UnomolBatch;
#define UNOMOL_BATCH_GRAPH 0      /* the batched build captured once as a CUDA graph, then replayed */
#define UNOMOL_BATCH_LAUNCHES 1   /* the batched build as plain launches on the stream */
#define UNOMOL_BATCH_SEQUENTIAL 2 /* one molecule after the other (the single-molecule path), for comparison */
int unomol_gpu_batch_create(const UnomolBasisDesc* bases, int nmol, UnomolBatch** out);
int unomol_gpu_batch_buffers(UnomolBatch* batch, double** dP, double** dG, const long long** packed_offsets,
                             int64_t* packed_total);
int unomol_gpu_batch_fock(UnomolBatch* batch, int mode, void* stream);
/* The same on caller-owned device buffers: packed densities of all molecules in (dP, copied into the
 * batch's buffer on `stream`), packed G out (dG, copied from it); either may be the batch's own buffer
 * or NULL (use the batch's buffer). */
int unomol_gpu_batch_fock_device(UnomolBatch* batch, const double* dP, double* dG, int mode, void* stream);
int unomol_gpu_batch_size(const UnomolBatch* batch);  /* molecules in the batch */
/* Autotuner: times every (CTA size 64/128/256, CTAs per SM 1/2/4/8) per class launch on the current P
 * and keeps the fastest; chosen (optional, 3 ints per launch): class id, CTA size, CTAs per SM.
 * Returns the number of launches (>= 0) or an error code. */
int unomol_gpu_batch_autotune(UnomolBatch* batch, int reps, int* chosen);
/* Precision form of the batched build, as unomol_gpu_set_precision and unomol_gpu_set_density_screening
 * for one context: UNOMOL_PREC_MIXED splits every molecule's quartets per build into FP64 (Schwarz bound
 * x max|P| of its six density blocks >= fp32_cutoff), FP32 (>= skip_cutoff) and skipped parts; the
 * persistent kernels run both parts.  The batch's CUDA graph is captured again on its next use. */
int unomol_gpu_batch_set_precision(UnomolBatch* batch, int mode, double fp32_cutoff, double skip_cutoff);
/* host copies of the batch's packed P (in) and G (out), all molecules concatenated */
int unomol_gpu_batch_set_density(UnomolBatch* batch, const double* P);
int unomol_gpu_batch_get_fock(UnomolBatch* batch, double* G);
void unomol_gpu_batch_destroy(UnomolBatch* batch);
const char* unomol_gpu_batch_last_error(const UnomolBatch* batch);

/* ---- SCF layer (the callers of the Fock build) ---- */

/* One-electron integrals S, T and H = T + V, packed (the data of OneElectronInts, OneElectronInts.cpp:
 * 6-202; computed on the host).  charges: [ncen] nuclear charges. */
int unomol_one_electron(const UnomolBasisDesc* basis, const double* charges, double* S, double* T, double* H);

/* The same integrals on the GPU for ngeom geometries of one basis in one launch (one thread per packed
 * element and geometry; the reference computes them on the host once per geometry,
 * OneElectronInts.cpp:6-202).  centers: [ngeom][ncen][3] bohr (NULL: the basis's own, ngeom = 1);
 * S, T, H: host [ngeom][no2] (T may be NULL).  Shells up to l = 4. */
int unomol_gpu_one_electron(const UnomolBasisDesc* basis, const double* charges, int ngeom, const double* centers,
                            double* S, double* T, double* H);
const char* unomol_gpu_one_electron_last_error(void);

/* Dipole and quadrupole integrals about the origin (the data MomentInts writes to RMOM.DAT,
 * Moments.cpp:98-181): M[k][no2] packed, k = dx, dy, dz, qxx, qxy, qxz, qyy, qyz, qzz, unweighted. */
int unomol_gpu_moment_ints(const UnomolBasisDesc* basis, double* M);

typedef struct UnomolScfInput {
    int norb;            /* basis functions */
    int nelec;           /* electrons: even -> RHF, odd -> UHF (Unomol.cc:13-24) */
    double nucrep;       /* nuclear repulsion energy */
    const double* S;     /* packed overlap */
    const double* H;     /* packed core Hamiltonian */
} UnomolScfInput;

#define UNOMOL_SCF_DAMPED 0 /* the reference's averaging (RHF.hpp:536-569); flag 1 behaves the same */
#define UNOMOL_SCF_DIIS 2   /* Pulay DIIS on F (new) */

typedef struct UnomolScfOptions {
    int maxits;          /* iteration cap (patin.dat maxits) */
    double eps;          /* convergence threshold (Basis::scf_eps) */
    int conv_type;       /* scf_flag[0]: 0 energy, 1 density, 2 both (RHF.hpp:390-402) */
    int accel;           /* UNOMOL_SCF_DAMPED or UNOMOL_SCF_DIIS */
    int guess;           /* 0 core Hamiltonian (RHF.hpp:205-211), 1 the P passed in (PMATRIX.DAT form),
                            2 the P passed in, McWeeny-purified and trace-checked, core Hamiltonian if it
                            fails (UNOMOL_GUESS_PURIFY; for the learned guess) */
    int diis_size;       /* DIIS subspace (default 8) */
    double diis_tol;     /* DIIS: max |X^T (FPS - SPF) X| at convergence */
    double diis_start;   /* DIIS: extrapolate once the error is below this (<= 0: from the start) */
    double level_shift;  /* DIIS: virtual-orbital shift sigma (0: none) ... */
    double level_shift_until; /* ... applied while the DIIS error is above this */
    int incremental;     /* 1: G(P) = G(P_prev) + G(P - P_prev) between full builds (new) */
    int rebuild_every;   /* incremental: a full build every this many builds (<= 0: 8) */
    int loop;            /* UNOMOL_SCF_LOOP_GROUND: the loop of findEnergy (two updates, then the
                            convergence test; RHF.hpp:138-162); UNOMOL_SCF_LOOP_DPM: the loop of
                            findPolarizationPotential (one update, then the test; RHF.hpp:323-329) */
    int density;         /* new density from F: UNOMOL_DENSITY_DIAG (default: eigen-solve, C_occ C_occ^T,
                            RHF.hpp:178-203), UNOMOL_DENSITY_SP2 (no reference counterpart: second-order
                            spectral projection of X^T F X by matrix products, the same projector when a
                            gap separates the occupied states; an iteration without that gap, and the
                            final orbital energies, use the eigen-solve) or UNOMOL_DENSITY_PSEUDO (no
                            reference counterpart: pseudo-diagonalisation, the occupied-virtual block of F
                            in the last orbitals rotated away to first order by matrix products; the
                            eigen-solve for the first density of each spin, for steps with a rotation
                            above 0.2 or a gap below 1e-3 Eh, and for the final orbital energies) */
} UnomolScfOptions;

#define UNOMOL_DENSITY_DIAG 0
#define UNOMOL_DENSITY_SP2 1
#define UNOMOL_DENSITY_PSEUDO 2

#define UNOMOL_SCF_LOOP_GROUND 0
#define UNOMOL_SCF_LOOP_DPM 1

typedef struct UnomolScfResult {
    int status;
    char message[256];
    double energy;        /* final total energy (electronic + nuclear repulsion) */
    double e_electronic;
    double init_energy;   /* energy of the first iteration (short.gs.out line 1) */
    double ediff, pdiff, diis_error;
    double seconds;       /* wall time of the SCF */
    int iterations, converged, fock_builds;
    double* energies;     /* optional [energies_cap]: total energy after every update */
    int energies_cap;
    double fock_ms;       /* device time of all Fock builds (CUDA events) */
    double* densities;    /* optional [densities_cap][no2 (UHF: 2*no2)]: the density of every build */
    int densities_cap;
    int guess_used;       /* UNOMOL_GUESS_USED_*: what the SCF started from */
    int purify_iterations;
    double purify_error;  /* guess 2: ||Q^2 - Q||_F at the end of the purification (per spin: max) */
    double guess_trace;   /* guess 2: tr Q after the purification (alpha spin for UHF) */
    double seconds_setup; /* wall time of the parts of the SCF: set-up (handles, X, guess), */
    double seconds_fock;  /* Fock builds (host call to result on the host), */
    double seconds_diis;  /* DIIS error and extrapolation (+ level shift), */
    double seconds_diag;  /* diagonalisation and new density */
    int sp2_steps;        /* UNOMOL_DENSITY_SP2: projection steps over the whole SCF */
    int sp2_fallbacks;    /* UNOMOL_DENSITY_SP2: densities that needed the eigen-solve (no gap) */
    int pseudo_steps;     /* UNOMOL_DENSITY_PSEUDO: densities by the pseudo-diagonalisation step */
} UnomolScfResult;

#define UNOMOL_GUESS_CORE 0
#define UNOMOL_GUESS_GIVEN 1
#define UNOMOL_GUESS_PURIFY 2
#define UNOMOL_GUESS_USED_CORE 0       /* core Hamiltonian (asked for) */
#define UNOMOL_GUESS_USED_GIVEN 1      /* the caller's P as given */
#define UNOMOL_GUESS_USED_PURIFIED 2   /* the caller's P after McWeeny purification */
#define UNOMOL_GUESS_USED_FALLBACK 3   /* purification or trace check failed: core Hamiltonian */

/* SCF on the GPU: the loop of RestrictedHartreeFock / UnRestrictedHartreeFock::findEnergy (RHF.hpp:
 * 114-176, UHF.hpp:137-177) with every Fock build on this context and the FP64 linear algebra in
 * cuSOLVER (syevd) / cuBLAS.  P_io: [no2] (RHF) or [2*no2] (UHF: Pa then Pb) -- the guess when
 * options->guess == 1, the final density on return.  orbital_energies: optional [norb] (UHF: 2*norb). */
int unomol_scf(UnomolCtx* ctx, const UnomolScfInput* input, const UnomolScfOptions* options, UnomolScfResult* result,
               double* P_io, double* orbital_energies);

/* RHF SCF of every molecule of the batch at once: each iteration is one batched Fock build plus the
 * DIIS update of the single-molecule driver (F = H + G, energy, X^T (FPS - SPF) X, Pulay extrapolation,
 * X^T F X, batched eigen-solve, P = C_occ C_occ^T) for all molecules, with converged molecules frozen;
 * with graph != 0 the iteration is captured once as a CUDA graph and replayed (graph_used reports
 * whether the capture succeeded; unomol_gpu_batch_scf_last_error then names what stopped it).
 * inputs: [nmol] (S, H packed, nelec even); options: maxits, eps, conv_type, accel (UNOMOL_SCF_DIIS:
 * the DIIS update and test of unomol_scf; otherwise the reference's damping and is_converged),
 * guess (core Hamiltonian, or UNOMOL_GUESS_GIVEN: the densities in P_io), loop (ground-state or DPM
 * loop order), diis_size, diis_tol, incremental, rebuild_every and density (UNOMOL_DENSITY_PSEUDO with
 * UNOMOL_SCF_DIIS: from the third iteration on, pseudo-diagonalisation steps by grouped matrix products
 * whenever every active molecule's step passes the check of unomol_scf (rotation at most 0.2, occupied
 * and virtual levels 1e-3 Eh apart), the batched eigen-solve for all molecules otherwise; other values:
 * the batched eigen-solve).  P_io: the batch's packed densities (in: the guess when given; out: the
 * final densities; may be NULL with the core-Hamiltonian guess). */
typedef struct UnomolBatchScfResult {
    double energy, e_electronic, diis_error;
    int iterations, converged;
    double init_energy;   /* energy after the first update (short.gs.out line 1; vpol's E_init) */
    double ediff, pdiff;  /* of the last update */
} UnomolBatchScfResult;
int unomol_gpu_batch_scf(UnomolBatch* batch, const UnomolScfInput* inputs, int nmol, const UnomolScfOptions* options,
                         int graph, UnomolBatchScfResult* results, double* P_io, double* seconds, int* graph_used);
const char* unomol_gpu_batch_scf_last_error(void);
/* Fock builds of the last batched SCF on this thread: their device time (CUDA events around each
 * iteration's build, also inside a replayed graph) and their number.  With options->incremental the
 * batched SCF builds G(P - P_prev) added to the G it keeps, a full build every options->rebuild_every
 * (the single-molecule scheme; the build count is kept on the device), so that in the precision form
 * the density bound of each build shrinks as the molecules converge. */
int unomol_gpu_batch_scf_last_builds(double* fock_ms, int* builds);
/* Iterations of the last batched SCF on this thread (UNOMOL_DENSITY_PSEUDO) whose densities came from
 * the pseudo-diagonalisation step (steps) and those where a molecule's check sent every molecule to the
 * eigen-solve (refused). */
int unomol_gpu_batch_scf_last_pseudo(int* steps, int* refused);

/* ---- Learned initial density (no reference counterpart; the reference starts from the core
 * Hamiltonian, RHF.hpp:205-211, or reads PMATRIX.DAT, RHF.hpp:120-123) ----
 * A per-atom-pair MLP maps (element of i, element of j, 16 radial basis functions of r_ij) to
 * Slater-Koster-like coefficients of the density blocks in the bond frame; the blocks are rotated
 * into place and summed into the RHF half density P (trace(PS) = nocc, the PMATRIX.DAT form).  Training
 * and inference run on the GPU: BF16 GEMMs on the tensor cores with FP32 accumulation, FP32 master
 * weights and Adam.  Bases: s and p shells, every centre of an element with the same shell list. */

/* the network alone: y = W_L silu(... silu(W_0 x + b_0) ...) + b_L; parameters (fp32, host order):
 * per linear map W [dout x din] row major, then b [dout] */
typedef struct UnomolMlp UnomolMlp;
int unomol_mlp_create(int n_in, int hidden, int layers, int n_out, unsigned long long seed, UnomolMlp** out);
long long unomol_mlp_num_params(const UnomolMlp* m);
int unomol_mlp_get_params(UnomolMlp* m, float* out);
int unomol_mlp_set_params(UnomolMlp* m, const float* in);
/* x: device fp32 [rows x n_in]; y: device fp32 [rows x n_out] */
int unomol_mlp_forward(UnomolMlp* m, const float* x, int rows, float* y, void* stream);
/* gradients of sum(dy * y) for the rows of the last forward; dy: device fp32 [rows x n_out] */
int unomol_mlp_backward(UnomolMlp* m, const float* dy, void* stream);
int unomol_mlp_get_grads(UnomolMlp* m, float* out);
int unomol_mlp_adam(UnomolMlp* m, float lr, float beta1, float beta2, float eps, float weight_decay, void* stream);
void unomol_mlp_destroy(UnomolMlp* m);
const char* unomol_mlp_last_error(const UnomolMlp* m);
/* C[M x N] (fp32, device) = A[M x K] . B[N x K]^T, A and B bf16 row major on the device (the tensor-core
 * GEMM of the network); status: device int set to 1 if a bounded wait gave up. */
int unomol_tc_gemm_bf16(const void* A, const void* B, int M, int N, int K, float* C, int* status, void* stream);
/* Poll limit of the tensor-core GEMMs' pipeline waits, for every GEMM the process launches afterwards
 * (no reference counterpart; a failure-detection control).  0 (default): 2^22 polls.  Negative: the
 * producer's and the MMA issuer's waits give up at their first wait, so the call reports a timeout
 * (status word 1, UNOMOL_ETIMEOUT from the network calls) after draining the copies it issued and
 * releasing its tensor memory; the next call with the default works normally. */
int unomol_tc_set_wait_polls(int polls);

typedef struct UnomolGuess UnomolGuess;
typedef struct UnomolGuessConfig {
    int hidden;                /* hidden width (<= 0: 256) */
    int layers;                /* hidden layers (<= 0: 3) */
    int n_rbf;                 /* radial basis functions (<= 1: 16), centres k * r_cut / (n_rbf - 1) */
    double r_cut;              /* pair cutoff in bohr (<= 0: 15) */
    unsigned long long seed;   /* weight initialisation */
} UnomolGuessConfig;
typedef struct UnomolGuessTrainOptions {
    int first, count;          /* molecules [first, first + count) of the model's data set */
    int epochs;
    int batch_molecules;       /* molecules per Adam step (<= 0: 16) */
    float lr, lr_final;        /* cosine schedule from lr to lr_final (<= 0: lr / 100) */
    float weight_decay;
    unsigned long long seed;   /* mini-batch order */
} UnomolGuessTrainOptions;
/* The model's elements and their shell lists come from this basis; charges: [ncen] nuclear charges. */
int unomol_guess_create(const UnomolGuessConfig* cfg, const UnomolBasisDesc* basis, const int* charges,
                        UnomolGuess** out);
int unomol_guess_info(const UnomolGuess* g, int* n_in, int* n_out, long long* n_params, int* n_elements);
/* append a molecule and its converged RHF density (packed, PMATRIX.DAT form) to the data set */
int unomol_guess_add_molecule(UnomolGuess* g, const UnomolBasisDesc* basis, const int* charges, const double* P);
int unomol_guess_num_molecules(const UnomolGuess* g);
/* Adam on the mean over molecules of sum (P_pred - P)^2; loss_history: optional [epochs] */
int unomol_guess_train(UnomolGuess* g, const UnomolGuessTrainOptions* opt, double* loss_history);
/* loss of molecules [first, first + count) and, if grads != NULL, its gradient (host order) */
int unomol_guess_loss(UnomolGuess* g, int first, int count, int batch_molecules, double* loss, float* grads);
/* predicted P (packed) for a molecule; hand it to unomol_scf with guess = UNOMOL_GUESS_PURIFY */
int unomol_guess_predict(UnomolGuess* g, const UnomolBasisDesc* basis, const int* charges, double* P);
int unomol_guess_get_params(UnomolGuess* g, float* out);
int unomol_guess_set_params(UnomolGuess* g, const float* in);
void unomol_guess_destroy(UnomolGuess* g);
const char* unomol_guess_last_error(const UnomolGuess* g);

/* DPM polarisation-potential integrals (GDPMInts.cpp:86-143): H -= sum_k c_k (mu nu | g_k), with
 * g_k = exp(-a_k |r - q|^2) the six-Gaussian positron charge at q (bohr), over the context's basis
 * (packed H on the host, subtracted in place).  Shells up to d. */
int unomol_gpu_gdpm(UnomolCtx* ctx, const double* q, double* H);
const char* unomol_gpu_gdpm_last_error(void);

/* Last error of this context (ctx may be NULL for errors raised before a context existed). */
const char* unomol_gpu_last_error(const UnomolCtx* ctx);

/* Library version string. */
const char* unomol_gpu_version(void);

#ifdef __cplusplus
}
#endif
#endif /* UNOMOL_GB300_H */
