// Drop-in replacement for unomol's TwoElectronInts.hpp (TwoElectronInts.hpp:79-110): the same class
// name, namespace, constructor and methods, backed by the GB300 direct Fock build of
// libunomol_gb300.so (C ABI: unomol_gb300.h).
//
// Use: put this directory ahead of the reference tree on the include path, so that RHF.hpp, UHF.hpp
// and Unomol.cc pick up this header for "TwoElectronInts.hpp"; compile every reference source except
// TwoElectronInts.cpp; link libunomol_gb300.so.  The SCF driver, SymmPack storage, Moments and the
// DPM / finite-field paths stay as they are.
//
// Differences a caller can observe:
//   * no integral store by default: the constructor builds shell pairs and Schwarz bounds on the GPU,
//     and every formGmatrix recomputes the integrals (direct SCF); `label` (the cache file name) is
//     unused.  The reference's conventional scheme is one call away:
//     unomol_gpu_store_integrals(context(), UNOMOL_STORE_UHF, 0.0) keeps every integral in device
//     memory and later formGmatrix calls stream it; unomol_gpu_write_records writes the records in
//     the layout of the reference's integral file;
//   * directFormGMatrix is exact (the reference's variant drops pairs with |AB|^2 > 20 bohr^2,
//     TwoElectronInts.cpp:920,961);
//   * errors end the program through the reference's convention (message on stderr, exit(EXIT_FAILURE),
//     Util.cpp:6-9).
// The basis type is a template parameter so that any class with the accessors of unomol::Basis
// (Basis.hpp:157-337) works.
#ifndef UNOMOL_TWOELEC_HPP
#define UNOMOL_TWOELEC_HPP

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../unomol_gb300.h"

namespace unomol {

class TwoElectronInts {
  public:
    TwoElectronInts() = delete;
    TwoElectronInts(const TwoElectronInts&) = delete;
    TwoElectronInts& operator=(const TwoElectronInts&) = delete;

    // TwoElectronInts(basis, start_shell, label) -- TwoElectronInts.hpp:83-88
    template <class BasisT>
    TwoElectronInts(const BasisT& basis, int start_shell, const std::string& label)
        : start_(start_shell), label_(label) {
        calculate(basis);
    }

    ~TwoElectronInts() {
        if (ctx_) unomol_gpu_destroy(ctx_);
    }

    // calculate(basis): set-up for this basis and geometry (TwoElectronInts.cpp:511)
    template <class BasisT>
    void calculate(const BasisT& basis) {
        if (ctx_) {
            unomol_gpu_destroy(ctx_);
            ctx_ = nullptr;
        }
        const int ns = basis.number_of_shells();
        l_.resize(ns);
        np_.resize(ns);
        cen_.resize(ns);
        off_.resize(ns);
        alpha_.clear();
        coef_.clear();
        for (int i = 0; i < ns; ++i) {
            const auto& sh = basis.shell_ptr()[i];
            l_[i] = sh.Lvalue();
            np_[i] = sh.number_of_prims();
            cen_[i] = sh.center();
            off_[i] = basis.offset(i);
            for (int k = 0; k < np_[i]; ++k) {
                alpha_.push_back(sh.alf_ptr()[k]);
                coef_.push_back(sh.cof_ptr()[k]);
            }
        }
        ncen_ = basis.number_of_centers();
        xyz_.resize(3 * ncen_);
        for (int c = 0; c < ncen_; ++c)
            for (int k = 0; k < 3; ++k) xyz_[3 * c + k] = basis.center_ptr()[c].r_vec()[k];
        UnomolBasisDesc d;
        d.nshell = ns;
        d.norb = basis.number_of_orbitals();
        d.ncen = ncen_;
        d.shell_l = l_.data();
        d.shell_nprim = np_.data();
        d.shell_center = cen_.data();
        d.shell_offset = off_.data();
        d.alpha = alpha_.data();
        d.coef = coef_.data();
        d.centers = xyz_.data();
        check(unomol_gpu_create(&d, start_, &ctx_));
    }

    // recalculate(basis): a centre moved (RHF.hpp:354); shells are unchanged
    template <class BasisT>
    void recalculate(const BasisT& basis) {
        if (!ctx_ || basis.number_of_centers() != ncen_) {
            calculate(basis);
            return;
        }
        for (int c = 0; c < ncen_; ++c)
            for (int k = 0; k < 3; ++k) xyz_[3 * c + k] = basis.center_ptr()[c].r_vec()[k];
        check(unomol_gpu_recalculate(ctx_, xyz_.data()));
    }

    // formGmatrix(P, G): G += 2 J(P) - K(P), packed (TwoElectronInts.cpp:822-844)
    void formGmatrix(const double* Pmat, double* Gmat) { check(unomol_gpu_fock_rhf(ctx_, Pmat, Gmat)); }

    // formGmatrix(Pa, Pb, Ga, Gb): UHF (TwoElectronInts.cpp:846-869)
    void formGmatrix(const double* PmatA, const double* PmatB, double* GmatA, double* GmatB) {
        check(unomol_gpu_fock_uhf(ctx_, PmatA, PmatB, GmatA, GmatB));
    }

    // directFormGMatrix(P, G, basis) (TwoElectronInts.cpp:871-1055): the same exact direct build
    template <class BasisT>
    void directFormGMatrix(const double* Pmat, double* Gmat, const BasisT&) {
        formGmatrix(Pmat, Gmat);
    }

    // access to the GPU context (precision form, screening, statistics)
    UnomolCtx* context() const { return ctx_; }

  private:
    void check(int rc) const {
        if (rc != UNOMOL_OK) {
            std::fprintf(stderr, "%s\n", unomol_gpu_last_error(ctx_));
            std::exit(EXIT_FAILURE);
        }
    }
    UnomolCtx* ctx_ = nullptr;
    int start_;
    std::string label_;
    int ncen_ = 0;
    std::vector<int> l_, np_, cen_, off_;
    std::vector<double> alpha_, coef_, xyz_;
};

}  // namespace unomol
#endif
