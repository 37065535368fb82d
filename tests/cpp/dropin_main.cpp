// Test driver of the C++ drop-in (include/unomol_gb300/TwoElectronInts.hpp):
//   dropin_main patin.dat P.bin G.bin            RHF: G = formGmatrix(P)
//   dropin_main patin.dat Pa.bin Pb.bin Ga.bin Gb.bin   UHF
// P/G files are raw packed doubles.  G arrays start at zero (the callers zero them, RHF.hpp:89-90).
#include <cstdio>
#include <fstream>
#include <vector>

#include "patin_basis.hpp"
#include "unomol_gb300/TwoElectronInts.hpp"

static std::vector<double> load(const char* p, size_t n) {
    std::vector<double> v(n);
    std::ifstream in(p, std::ios::binary);
    in.read(reinterpret_cast<char*>(v.data()), n * sizeof(double));
    return v;
}
static void save(const char* p, const std::vector<double>& v) {
    std::ofstream out(p, std::ios::binary);
    out.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(double));
}

int main(int argc, char** argv) {
    if (argc != 4 && argc != 6) {
        std::fprintf(stderr, "usage: %s patin P G | patin Pa Pb Ga Gb\n", argv[0]);
        return 2;
    }
    testbasis::Basis basis(argv[1]);
    const size_t no2 = (size_t)basis.number_of_orbitals() * (basis.number_of_orbitals() + 1) / 2;
    unomol::TwoElectronInts tints(basis, 0, "MINTS.DAT");
    if (argc == 4) {
        std::vector<double> P = load(argv[2], no2), G(no2, 0.0);
        tints.formGmatrix(P.data(), G.data());
        save(argv[3], G);
    } else {
        std::vector<double> Pa = load(argv[2], no2), Pb = load(argv[3], no2), Ga(no2, 0.0), Gb(no2, 0.0);
        tints.formGmatrix(Pa.data(), Pb.data(), Ga.data(), Gb.data());
        save(argv[4], Ga);
        save(argv[5], Gb);
    }
    return 0;
}
