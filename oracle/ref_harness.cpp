// Test infrastructure only: a C ABI over the reference's own objects, compiled unchanged from the
// reference sources by oracle/Makefile. The tests, the golden-fixture generator and bench.py's
// CPU-baseline leg load it through ctypes; nothing in the product links it.
//
// What it exposes (reference file:line in brackets):
//   * the Basis reader and normaliser               [Basis.hpp:181-255]
//   * the integral pass and its stored records      [TwoElectronInts.cpp:511-697, cache.hpp]
//   * G(P) for RHF and UHF                           [TwoElectronInts.cpp:822-869]
//   * one-electron S, T, H                          [OneElectronInts.cpp]
//   * the stock RHF / UHF SCF                       [RHF.hpp:114-176, UHF.hpp:137-177]
//   * the DPM one-electron matrices                 [OneElectronInts.cpp, GDPMInts.cpp:86-143]
//   * the stock SCF trajectory, iteration by iteration, from the reference's own members
//                                                   [RHF.hpp:114-166, UHF.hpp:137-163]
//   * a Pulay DIIS loop (test-only) on the reference's formGmatrix, one-electron integrals, X matrix
//     and eigen-solver, for molecules where the stock damped loop does not converge
//                                                   [TwoElectronInts.cpp:822-869, RHF.hpp:87-112,
//                                                    UHF.hpp:101-134, SymmPack.cpp:67-348]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <cfloat>
#include <cstdint>
#include <string>
#include <vector>
#include <iostream>
#include <fstream>
#include <iomanip>
#include <filesystem>
#include <functional>
#include <unistd.h>
#include <chrono>
#include <algorithm>
#include <type_traits>

// The reference keeps the integral store, the SCF state and the basis behind `private:`; the harness
// reads them directly so that the fixtures come from the reference's own records.
#define private public
#include "Basis.hpp"
#include "TwoElectronInts.hpp"
#include "RHF.hpp"
#include "UHF.hpp"
#undef private

using unomol::Basis;
using unomol::TwoElectronInts;
using unomol::TwoInts;

extern "C" {

void* refh_basis_new(const char* path) { return new Basis(std::string(path)); }

void refh_basis_free(void* b) { delete static_cast<Basis*>(b); }

// dims = {nshell, norb, ncen, maxl, nelec, maxits}
void refh_basis_dims(void* vb, int* dims) {
    Basis* b = static_cast<Basis*>(vb);
    dims[0] = b->number_of_shells();
    dims[1] = b->number_of_orbitals();
    dims[2] = b->number_of_centers();
    dims[3] = b->maxLvalue();
    dims[4] = b->number_of_electrons();
    dims[5] = b->maximum_iterations();
}

// Per shell: {L, nprim, centre, offset}; alpha/coef after the reference's normalisation; centres
// as {charge, x, y, z}. Arrays are sized by the caller from refh_basis_dims and the prim count.
int refh_basis_export(void* vb, int* shell_info, double* alpha, double* coef, double* centres) {
    Basis* b = static_cast<Basis*>(vb);
    const unomol::Shell* sh = b->shell_ptr();
    int np = 0;
    for (int i = 0; i < b->number_of_shells(); ++i) {
        shell_info[4 * i + 0] = sh[i].Lvalue();
        shell_info[4 * i + 1] = sh[i].number_of_prims();
        shell_info[4 * i + 2] = sh[i].center();
        shell_info[4 * i + 3] = b->offset(i);
        for (int k = 0; k < sh[i].number_of_prims(); ++k, ++np) {
            alpha[np] = sh[i].alf(k);
            coef[np] = sh[i].cof(k);
        }
    }
    const unomol::Center* c = b->center_ptr();
    for (int i = 0; i < b->number_of_centers(); ++i) {
        centres[4 * i + 0] = c[i].charge();
        for (int k = 0; k < 3; ++k) centres[4 * i + 1 + k] = c[i].position(k);
    }
    return np;
}

void* refh_tints_new(void* vb, int start_shell, const char* label) {
    return new TwoElectronInts(*static_cast<Basis*>(vb), start_shell, std::string(label));
}

void refh_tints_free(void* t) { delete static_cast<TwoElectronInts*>(t); }

long long refh_tints_count(void* vt) {
    TwoElectronInts* t = static_cast<TwoElectronInts*>(vt);
    return (long long)(t->cache.total_size() / (long long)sizeof(TwoInts));
}

// Copies the stored records (val, i, j, k, l) in the order the reference wrote them.
long long refh_tints_dump(void* vt, double* vals, int* ijkl, long long cap) {
    TwoElectronInts* t = static_cast<TwoElectronInts*>(vt);
    long long n = refh_tints_count(vt);
    if (n > cap) n = cap;
    std::vector<TwoInts> buf(4096);
    t->cache.open_for_reading();
    long long done = 0;
    while (done < n) {
        long long m = std::min<long long>(4096, n - done);
        t->cache.read(buf.data(), m);
        for (long long q = 0; q < m; ++q) {
            vals[done + q] = buf[q].val;
            ijkl[4 * (done + q) + 0] = buf[q].i;
            ijkl[4 * (done + q) + 1] = buf[q].j;
            ijkl[4 * (done + q) + 2] = buf[q].k;
            ijkl[4 * (done + q) + 3] = buf[q].l;
        }
        done += m;
    }
    t->cache.close();
    return done;
}

void refh_form_g(void* vt, const double* P, double* G) {
    static_cast<TwoElectronInts*>(vt)->formGmatrix(P, G);
}

void refh_form_g_uhf(void* vt, const double* Pa, const double* Pb, double* Ga, double* Gb) {
    static_cast<TwoElectronInts*>(vt)->formGmatrix(Pa, Pb, Ga, Gb);
}

void refh_one_electron(void* vb, double* S, double* T, double* H) {
    unomol::OneElectronInts(*static_cast<Basis*>(vb), S, T, H);
}

// Runs the stock SCF of Unomol.cc:8-26 (RHF for even, UHF for odd electron counts) inside `workdir`
// (the reference writes its output files into the current directory).
// out = {final energy, initial energy, iterations, ediff, pdiff, nucrep, seconds_ints, seconds_scf}
// P_out receives the final packed density (RHF: no2 values; UHF: Pa then Pb).
int refh_scf(const char* patin, const char* workdir, double* out, double* P_out) {
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd))) return -1;
    if (chdir(workdir) != 0) return -2;
    Basis bas{std::string(patin)};
    auto t0 = std::chrono::steady_clock::now();
    TwoElectronInts t(bas, 0, std::string("MINTS.DAT"));
    auto t1 = std::chrono::steady_clock::now();
    int no2 = bas.number_of_orbitals() * (bas.number_of_orbitals() + 1) / 2;
    if (bas.number_of_electrons() % 2) {
        unomol::UnRestrictedHartreeFock uhf(&bas, &t);
        uhf.findEnergy();
        out[0] = uhf.energy + uhf.nucrep;
        out[2] = uhf.iteration;
        out[3] = uhf.ediff;
        out[4] = uhf.pdiff;
        out[5] = uhf.nucrep;
        if (P_out) {
            std::memcpy(P_out, uhf.PmatA, sizeof(double) * no2);
            std::memcpy(P_out + no2, uhf.PmatB, sizeof(double) * no2);
        }
    } else {
        unomol::RestrictedHartreeFock rhf(&bas, &t);
        rhf.findEnergy();
        out[0] = rhf.energy + rhf.nucrep;
        out[2] = rhf.iteration;
        out[3] = rhf.ediff;
        out[4] = rhf.pdiff;
        out[5] = rhf.nucrep;
        if (P_out) std::memcpy(P_out, rhf.Pmat, sizeof(double) * no2);
    }
    auto t2 = std::chrono::steady_clock::now();
    // initial energy is the first line of short.gs.out (RHF.hpp:405-409)
    out[1] = NAN;
    if (FILE* f = fopen("short.gs.out", "r")) {
        if (fscanf(f, "%lf", &out[1]) != 1) out[1] = NAN;
        fclose(f);
    }
    out[6] = std::chrono::duration<double>(t1 - t0).count();
    out[7] = std::chrono::duration<double>(t2 - t1).count();
    if (chdir(cwd) != 0) return -3;
    return 0;
}

// DPM one-electron matrices [OneElectronInts.cpp, GDPMInts.cpp:86-143]: in directory `dir` (patin.dat
// with int_flag[0] = 1 and posin.bas), the basis augmented with the positron shells (Basis.hpp:341-345),
// the positron centre at q (Basis.hpp:346-348); H_plain = T + V over all centres (the positron a +1
// point charge), H_dpm = H_plain minus the DPM potential integrals.  Packed over the augmented basis.
int refh_dpm_h(const char* dir, const double* q, double* S, double* H_plain, double* H_dpm, int* dims) {
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd))) return -1;
    if (chdir(dir) != 0) return -2;
    {
        Basis b(std::string("patin.dat"));
        const int pcen = b.skip_center();
        b.dpm_augment();
        b.SetCenterPosition(q[0], q[1], q[2], pcen);
        const int no = b.number_of_orbitals(), no2 = no * (no + 1) / 2;
        dims[0] = b.number_of_shells();
        dims[1] = no;
        dims[2] = b.number_of_centers();
        if (S) {
            std::vector<double> T(no2);
            unomol::OneElectronInts(b, S, T.data(), H_plain);
            std::memcpy(H_dpm, H_plain, sizeof(double) * no2);
            unomol::GDPMInts(b, H_dpm);
        }
    }
    if (chdir(cwd) != 0) return -3;
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------------
// SCF set-up shared by the trace and the DIIS loop: the opening of findEnergy (RHF.hpp:115-126,
// UHF.hpp:138-149) without the files it writes (moments, intsout), which do not touch the SCF state.
template <class HF>
static void scf_setup(HF& hf, const double* P0) {
    hf.nucrep = hf.nuclear_repulsion_energy(hf.ncen, hf.basis.center_ptr());
    unomol::OneElectronInts(hf.basis, hf.Smat, hf.Tmat, hf.Hmat);
    hf.formXmatrix();
    if constexpr (std::is_same_v<HF, unomol::RestrictedHartreeFock>) {
        if (P0) std::memcpy(hf.Pmat, P0, sizeof(double) * hf.no2);
        else hf.PmatrixGuess();
    } else {
        if (P0) {
            std::memcpy(hf.PmatA, P0, sizeof(double) * hf.no2);
            std::memcpy(hf.PmatB, P0 + hf.no2, sizeof(double) * hf.no2);
        } else {
            hf.PmatrixGuess();
        }
    }
}

// The stock loop of findEnergy (RHF.hpp:140-166, UHF.hpp:150-163), energy + nucrep after every
// update.  The UHF loop resets eold before its second update (UHF.hpp:157-159), so its second
// ediff is the whole energy and the first damping step is skipped; both loops are kept as written.
template <class HF>
static int stock_trace(HF& hf, int kmax, double* e_out) {
    int k = 0;
    hf.iteration = 0;
    hf.extrap = 0;
    hf.eold = 0.0;
    hf.update();
    e_out[k++] = hf.energy + hf.nucrep;
    if (k >= kmax) return k;
    hf.iteration = 1;
    if constexpr (!std::is_same_v<HF, unomol::RestrictedHartreeFock>) {
        hf.extrap = 0;
        hf.eold = 0.0;
    }
    hf.update();
    e_out[k++] = hf.energy + hf.nucrep;
    while (k < kmax && hf.iteration < hf.maxits) {
        hf.scf_converger();
        hf.update();
        e_out[k++] = hf.energy + hf.nucrep;
        if (hf.is_converged()) break;
    }
    return k;
}

// packed lower triangle (i(i+1)/2 + j) -> full symmetric row-major
static void unpack(int n, const double* p, double* f) {
    for (int i = 0, ij = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j, ++ij) f[i * n + j] = f[j * n + i] = p[ij];
}

// c = a b (row-major n x n), i-k-j order
static void matmul(int n, const double* a, const double* b, double* c) {
    std::fill(c, c + (size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < n; ++k) {
            const double aik = a[(size_t)i * n + k];
            const double* bk = b + (size_t)k * n;
            double* ci = c + (size_t)i * n;
            for (int j = 0; j < n; ++j) ci[j] += aik * bk[j];
        }
}

// Pulay coefficients: [B -1; -1 0][c; l] = [0; -1], Gaussian elimination with partial pivoting.
// Returns false when the system is singular to working precision.
static bool pulay_solve(int m, const std::vector<double>& B, std::vector<double>& c) {
    const int d = m + 1;
    std::vector<double> A((size_t)d * d), r(d, 0.0);
    double scale = 0.0;
    for (int i = 0; i < m; ++i) scale = std::max(scale, std::fabs(B[(size_t)i * m + i]));
    if (!(scale > 0.0)) scale = 1.0;
    for (int i = 0; i < m; ++i) {
        for (int j = 0; j < m; ++j) A[(size_t)i * d + j] = B[(size_t)i * m + j] / scale;
        A[(size_t)i * d + m] = -1.0;
        A[(size_t)m * d + i] = -1.0;
    }
    A[(size_t)m * d + m] = 0.0;
    r[m] = -1.0;
    for (int col = 0; col < d; ++col) {
        int piv = col;
        for (int i = col + 1; i < d; ++i)
            if (std::fabs(A[(size_t)i * d + col]) > std::fabs(A[(size_t)piv * d + col])) piv = i;
        if (std::fabs(A[(size_t)piv * d + col]) < 1e-300) return false;
        if (piv != col) {
            for (int j = 0; j < d; ++j) std::swap(A[(size_t)piv * d + j], A[(size_t)col * d + j]);
            std::swap(r[piv], r[col]);
        }
        for (int i = col + 1; i < d; ++i) {
            const double f = A[(size_t)i * d + col] / A[(size_t)col * d + col];
            for (int j = col; j < d; ++j) A[(size_t)i * d + j] -= f * A[(size_t)col * d + j];
            r[i] -= f * r[col];
        }
    }
    std::vector<double> x(d);
    for (int i = d - 1; i >= 0; --i) {
        double s = r[i];
        for (int j = i + 1; j < d; ++j) s -= A[(size_t)i * d + j] * x[j];
        x[i] = s / A[(size_t)i * d + i];
    }
    c.assign(x.begin(), x.begin() + m);
    for (double v : c)
        if (!std::isfinite(v)) return false;
    return true;
}

// Pulay DIIS over the reference's own pieces: G from tints.formGmatrix (the cached build,
// TwoElectronInts.cpp:822-869), energies as update() forms them (RHF.hpp:94-96, UHF.hpp:111-114),
// F = H + G, the error F P S - S P F, extrapolation of F over the last `nkeep`
// iterations, then the reference's diagonalisation step (sp_trans, rsp, formCmatrix,
// formPmatrix: RHF.hpp:103-109).  Converged when |dE| < eps_e and max|error| < eps_err.
// The error is taken to the orthonormal basis of the reference's X, X^T (FPS - SPF) X.
// out = {E total, iterations, converged, max error, last |dE|, nucrep, seconds, max|X^T S X - 1|}
template <class HF>
static void diis_loop(HF& hf, int maxits, int nkeep, double eps_e, double eps_err, double* out,
                      double* P_out) {
    constexpr bool rhf = std::is_same_v<HF, unomol::RestrictedHartreeFock>;
    constexpr int ns = rhf ? 1 : 2;
    const int n = hf.no, n2 = hf.no2;
    const size_t nn = (size_t)n * n;
    double* P[2];
    double* G[2];
    double* Cm[2];
    double* Ev[2];
    int nocc[2];
    if constexpr (rhf) {
        P[0] = hf.Pmat; G[0] = hf.Gmat; Cm[0] = hf.Cmat; Ev[0] = hf.Evals; nocc[0] = hf.nocc;
    } else {
        P[0] = hf.PmatA; G[0] = hf.GmatA; Cm[0] = hf.CmatA; Ev[0] = hf.EvalsA; nocc[0] = hf.noccA;
        P[1] = hf.PmatB; G[1] = hf.GmatB; Cm[1] = hf.CmatB; Ev[1] = hf.EvalsB; nocc[1] = hf.noccB;
    }
    std::vector<double> S(nn), Pf(nn), Ff(nn), T1(nn), T2(nn), X(hf.Xmat, hf.Xmat + nn), XT(nn);
    unpack(n, hf.Smat, S.data());
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) XT[(size_t)j * n + i] = X[(size_t)i * n + j];
    {   // the reference's X (RHF.hpp:214-233) must satisfy X^T S X = 1
        matmul(n, XT.data(), S.data(), T1.data());
        matmul(n, T1.data(), X.data(), T2.data());
        double dev = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) dev = std::max(dev, std::fabs(T2[(size_t)i * n + j] - (i == j ? 1.0 : 0.0)));
        out[7] = dev;
    }
    std::vector<std::vector<double>> Fh, Eh;  // history: per entry ns packed F, ns full errors
    std::vector<double> F(n2 * ns);
    auto t0 = std::chrono::steady_clock::now();
    double e_old = 0.0, de = 1e30, err = 1e30, e_total = 0.0;
    int it = 0, conv = 0;
    for (it = 1; it <= maxits; ++it) {
        for (int s = 0; s < ns; ++s) std::fill(G[s], G[s] + n2, 0.0);
        if constexpr (rhf) hf.tints.formGmatrix(P[0], G[0]);
        else hf.tints.formGmatrix(P[0], P[1], G[0], G[1]);
        double e;
        if constexpr (rhf) {
            e = unomol::SymmPack::TraceSymmPackProduct(P[0], hf.Hmat, n) * 2.0 +
                unomol::SymmPack::TraceSymmPackProduct(P[0], G[0], n);
        } else {
            e = unomol::SymmPack::TraceSymmPackProduct(P[0], hf.Hmat, n) +
                unomol::SymmPack::TraceSymmPackProduct(P[1], hf.Hmat, n) +
                0.5 * (unomol::SymmPack::TraceSymmPackProduct(P[0], G[0], n) +
                       unomol::SymmPack::TraceSymmPackProduct(P[1], G[1], n));
        }
        e_total = e + hf.nucrep;
        de = std::fabs(e - e_old);
        e_old = e;
        std::vector<double> errs(ns * nn);
        err = 0.0;
        for (int s = 0; s < ns; ++s) {
            for (int q = 0; q < n2; ++q) F[(size_t)s * n2 + q] = hf.Hmat[q] + G[s][q];
            unpack(n, F.data() + (size_t)s * n2, Ff.data());
            unpack(n, P[s], Pf.data());
            matmul(n, Ff.data(), Pf.data(), T1.data());   // F P
            matmul(n, T1.data(), S.data(), T2.data());    // F P S
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) T1[(size_t)i * n + j] = T2[(size_t)i * n + j] - T2[(size_t)j * n + i];
            // FPS - SPF = FPS - (FPS)^T, taken to the orthonormal basis: X^T (FPS - SPF) X
            matmul(n, T1.data(), X.data(), T2.data());
            double* es = errs.data() + s * nn;
            matmul(n, XT.data(), T2.data(), es);
            for (size_t q = 0; q < nn; ++q) err = std::max(err, std::fabs(es[q]));
        }
        if (it > 2 && de < eps_e && err < eps_err) {
            conv = 1;
            break;
        }
        Fh.push_back(F);
        Eh.push_back(std::move(errs));
        if ((int)Fh.size() > nkeep) {
            Fh.erase(Fh.begin());
            Eh.erase(Eh.begin());
        }
        std::vector<double> c;
        while (true) {
            const int m = (int)Fh.size();
            std::vector<double> B((size_t)m * m);
            for (int i = 0; i < m; ++i)
                for (int j = 0; j <= i; ++j) {
                    double d = 0.0;
                    for (size_t q = 0; q < ns * nn; ++q) d += Eh[i][q] * Eh[j][q];
                    B[(size_t)i * m + j] = B[(size_t)j * m + i] = d;
                }
            if (pulay_solve(m, B, c) || m == 1) break;
            Fh.erase(Fh.begin());
            Eh.erase(Eh.begin());
        }
        if (Fh.size() < 2 || c.size() != Fh.size()) c.assign(Fh.size(), 0.0), c.back() = 1.0;
        for (int s = 0; s < ns; ++s) {
            for (int q = 0; q < n2; ++q) {
                double v = 0.0;
                for (size_t h = 0; h < Fh.size(); ++h) v += c[h] * Fh[h][(size_t)s * n2 + q];
                hf.Fock[q] = v;
            }
            unomol::SymmPack::sp_trans(n, hf.Fock, hf.Xmat, hf.Wrka);
            unomol::SymmPack::rsp(n, hf.Fock, hf.Wmat, Ev[s], hf.Wrka);
            hf.formCmatrix(Cm[s]);
            hf.formPmatrix(P[s], Cm[s], nocc[s]);
        }
    }
    auto t1 = std::chrono::steady_clock::now();
    out[0] = e_total;
    out[1] = it;
    out[2] = conv;
    out[3] = err;
    out[4] = de;
    out[5] = hf.nucrep;
    out[6] = std::chrono::duration<double>(t1 - t0).count();
    if (P_out)
        for (int s = 0; s < ns; ++s) std::memcpy(P_out + (size_t)s * n2, P[s], sizeof(double) * n2);
}

extern "C" {

// Stock SCF trajectory: the first kmax energies (energy + nucrep after each update) of findEnergy's
// loop on basis `vb` with the integrals of `vt` (a TwoElectronInts over the same shells), core-H
// guess.  Returns the number of energies written (fewer when the loop converged earlier).
// perturb != 0 scales the starting density by (1 + perturb): a probe of how strongly the trajectory
// amplifies a difference in its input.
int refh_scf_trace(void* vb, void* vt, const char* workdir, int kmax, double* e_out, double perturb) {
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd))) return -1;
    if (chdir(workdir) != 0) return -2;
    Basis* b = static_cast<Basis*>(vb);
    TwoElectronInts* t = static_cast<TwoElectronInts*>(vt);
    int k;
    if (b->number_of_electrons() % 2) {
        unomol::UnRestrictedHartreeFock hf(b, t);
        scf_setup(hf, nullptr);
        for (int i = 0; i < hf.no2; ++i) hf.PmatA[i] *= 1.0 + perturb, hf.PmatB[i] *= 1.0 + perturb;
        k = stock_trace(hf, kmax, e_out);
    } else {
        unomol::RestrictedHartreeFock hf(b, t);
        scf_setup(hf, nullptr);
        for (int i = 0; i < hf.no2; ++i) hf.Pmat[i] *= 1.0 + perturb;
        k = stock_trace(hf, kmax, e_out);
    }
    if (chdir(cwd) != 0) return -3;
    return k;
}

// DIIS SCF (test-only) on basis `vb` with the integrals of `vt`.  P0: the starting density (RHF: no2
// values, UHF: Pa then Pb) or null for the reference's core-Hamiltonian guess.  out as diis_loop.
int refh_scf_diis(void* vb, void* vt, const char* workdir, const double* P0, int maxits, int nkeep,
                  double eps_e, double eps_err, double* out, double* P_out) {
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd))) return -1;
    if (chdir(workdir) != 0) return -2;
    Basis* b = static_cast<Basis*>(vb);
    TwoElectronInts* t = static_cast<TwoElectronInts*>(vt);
    if (b->number_of_electrons() % 2) {
        unomol::UnRestrictedHartreeFock hf(b, t);
        scf_setup(hf, P0);
        diis_loop(hf, maxits, nkeep, eps_e, eps_err, out, P_out);
    } else {
        unomol::RestrictedHartreeFock hf(b, t);
        scf_setup(hf, P0);
        diis_loop(hf, maxits, nkeep, eps_e, eps_err, out, P_out);
    }
    if (chdir(cwd) != 0) return -3;
    return 0;
}

}  // extern "C"
