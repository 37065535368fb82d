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
