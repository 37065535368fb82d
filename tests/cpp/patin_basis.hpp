// Test helper: a minimal reader of unomol's patin.dat with the accessors of unomol::Basis that the
// drop-in TwoElectronInts uses (Basis.hpp:157-337), so that the drop-in can be exercised from C++ on
// machines without the reference sources.  Normalisation as Shell::normalize (Basis.hpp:56-75).
#pragma once
#include <cmath>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace testbasis {

struct Shell {
    int npr = 0, lsh = 0, cen = 0;
    std::vector<double> al, co;
    int Lvalue() const { return lsh; }
    int number_of_prims() const { return npr; }
    int center() const { return cen; }
    const double* alf_ptr() const { return al.data(); }
    const double* cof_ptr() const { return co.data(); }
    void normalize() {
        const double lpow = 1.5 + lsh;
        double sum = 0.0;
        for (int i = 0; i < npr; ++i)
            for (int j = 0; j < npr; ++j) sum += co[i] * co[j] * std::pow(std::sqrt(al[i] * al[j]) / (al[i] + al[j]), lpow);
        sum = 1.0 / std::sqrt(sum * 2.8284271247461903);
        for (int i = 0; i < npr; ++i) co[i] = co[i] * sum * std::sqrt(std::pow(2 * al[i], lpow) / 5.568327996831707);
    }
};

struct Center {
    double chg = 0, r[3] = {0, 0, 0};
    const double* r_vec() const { return r; }
    double charge() const { return chg; }
};

class Basis {
  public:
    explicit Basis(const std::string& path) {
        std::ifstream in(path);
        if (!in) throw std::runtime_error("cannot open " + path);
        int maxl, maxits, f;
        double eps;
        in >> nshell_ >> norb_ >> ncen_ >> maxl >> nelec_ >> maxits >> eps;
        for (int k = 0; k < 8; ++k) in >> f;
        centers_.resize(ncen_);
        for (auto& c : centers_) in >> c.chg >> c.r[0] >> c.r[1] >> c.r[2];
        shells_.resize(nshell_);
        int off = 0;
        for (auto& s : shells_) {
            in >> s.npr >> s.lsh >> s.cen;
            s.al.resize(s.npr);
            s.co.resize(s.npr);
            for (int k = 0; k < s.npr; ++k) in >> s.al[k] >> s.co[k];
            s.normalize();
            offsets_.push_back(off);
            off += (s.lsh + 1) * (s.lsh + 2) / 2;
        }
    }
    int number_of_shells() const { return nshell_; }
    int number_of_orbitals() const { return norb_; }
    int number_of_centers() const { return ncen_; }
    int number_of_electrons() const { return nelec_; }
    const Shell* shell_ptr() const { return shells_.data(); }
    const Center* center_ptr() const { return centers_.data(); }
    int offset(int i) const { return offsets_[i]; }

  private:
    int nshell_ = 0, norb_ = 0, ncen_ = 0, nelec_ = 0;
    std::vector<Shell> shells_;
    std::vector<Center> centers_;
    std::vector<int> offsets_;
};

}  // namespace testbasis
