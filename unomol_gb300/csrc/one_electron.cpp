// One-electron integrals S, T and H = T + V over the basis (packed lower triangle, reference AO order).
// They feed the SCF driver of this library; in the drop-in setting the caller's own
// OneElectronInts (OneElectronInts.cpp:6-202) provides them.  O(N^2) host work, once per geometry.
//
// Overlap and kinetic energy: Obara-Saika 1D recurrences per Cartesian axis,
//   S(i+1, j) = PA S(i, j) + (i S(i-1, j) + j S(i, j-1)) / 2p,  S(i, j+1) likewise with PB,
//   T(i, j) = 1/2 [i j S(i-1, j-1) + 4 a b S(i+1, j+1) - 2 a j S(i+1, j-1) - 2 b i S(i-1, j+1)]
// (the same identity as OneElectronInts.cpp:74-115).  Nuclear attraction: McMurchie-Davidson,
//   V = -sum_C Z_C 2 pi / p  sum_{tuv} E_t^x E_u^y E_v^z R_{tuv}(p, P - C),
// with the Boys functions from a series and downward recursion (asymptotic form for T > 40).
// Contraction coefficients arrive normalised (Basis.hpp:56-75); the component factors of
// AuxFunctions.hpp:48-63 multiply each element as in the reference.
#include <cmath>
#include <vector>

#include "../../include/unomol_gb300.h"

namespace {

constexpr int LM = 4;

int ncart(int l) { return (l + 1) * (l + 2) / 2; }

void cart(int l, int c, int* v) {
    int k = 0;
    for (int x = l; x >= 0; --x)
        for (int y = l - x; y >= 0; --y) {
            if (k == c) {
                v[0] = x;
                v[1] = y;
                v[2] = l - x - y;
                return;
            }
            ++k;
        }
}

double comp_norm(int l, int c) {
    double dfact[LM + 1];
    dfact[0] = 1.0;
    double dx = 1.0;
    for (int i = 1; i <= LM; ++i) {
        dfact[i] = dfact[i - 1] * dx;
        dx *= (2 * i + 1);
    }
    int v[3];
    cart(l, c, v);
    return 1.0 / std::sqrt(dfact[v[0]] * dfact[v[1]] * dfact[v[2]]);
}

// Boys F_m(T), m = 0..mmax, evaluated as the reference's nuclear-attraction path does
// (MD_Rfunction::Fgamma, MD_Rfunction.hpp:2185-2206): the large-T form above T = 20 and the series
// for F_mmax stopped once a term drops below 1e-12, then downward recursion.  Both cut-offs leave
// errors (up to ~1e-9 relative at T just above 20) that the reference's H carries; keeping them keeps
// the SCF energies on the reference's.
void boys(int mmax, double T, double* F) {
    if (T > 20.0) {
        F[0] = 0.88622692545275801365 / std::sqrt(T);
        for (int m = 1; m <= mmax; ++m) F[m] = F[m - 1] * (m - 0.5) / T;
        return;
    }
    const double mph = mmax + 0.5;
    double term = 0.5 / mph, sum = term;
    for (int k = 1; k <= 200; ++k) {
        term *= T / (mph + k);
        sum += term;
        if (term < 1.e-12) break;
    }
    const double e = std::exp(-T);
    F[mmax] = sum * e;
    for (int m = mmax - 1; m >= 0; --m) F[m] = (F[m + 1] * 2.0 * T + e) / (m + m + 1.0);
}

// Hermite expansion coefficients E[i][j][t] of one axis (McMurchie-Davidson)
struct Herm {
    double E[LM + 2][LM + 2][2 * LM + 5];
};

void hermite(int la, int lb, double p, double PA, double PB, double Kab, Herm& H) {
    const double o = 0.5 / p;
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= lb; ++j)
            for (int t = 0; t <= i + j + 1; ++t) H.E[i][j][t] = 0.0;
    H.E[0][0][0] = Kab;
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= lb; ++j) {
            if (i == 0 && j == 0) continue;
            for (int t = 0; t <= i + j; ++t) {
                double v;
                if (i > 0) {
                    v = PA * H.E[i - 1][j][t];
                    if (t > 0) v += o * H.E[i - 1][j][t - 1];
                    if (t + 1 <= i + j - 1) v += (t + 1) * H.E[i - 1][j][t + 1];
                } else {
                    v = PB * H.E[i][j - 1][t];
                    if (t > 0) v += o * H.E[i][j - 1][t - 1];
                    if (t + 1 <= i + j - 1) v += (t + 1) * H.E[i][j - 1][t + 1];
                }
                H.E[i][j][t] = v;
            }
        }
}

}  // namespace

extern "C" int unomol_one_electron(const UnomolBasisDesc* b, const double* charges, double* S, double* T, double* H) {
    if (!b || !charges || !S || !T || !H) return UNOMOL_EINVAL;
    const int ns = b->nshell;
    std::vector<int> p0(ns);
    int np = 0;
    for (int s = 0; s < ns; ++s) {
        if (b->shell_l[s] < 0 || b->shell_l[s] > LM) return UNOMOL_EINVAL;
        p0[s] = np;
        np += b->shell_nprim[s];
    }
    const int n = b->norb;
    const size_t no2 = (size_t)n * (n + 1) / 2;
    for (size_t k = 0; k < no2; ++k) S[k] = T[k] = H[k] = 0.0;
    for (int sa = 0; sa < ns; ++sa)
        for (int sb = 0; sb <= sa; ++sb) {
            const int la = b->shell_l[sa], lb = b->shell_l[sb];
            const double* A = b->centers + 3 * b->shell_center[sa];
            const double* B = b->centers + 3 * b->shell_center[sb];
            const int na = ncart(la), nb = ncart(lb);
            std::vector<double> sv(na * nb, 0.0), tv(na * nb, 0.0), vv(na * nb, 0.0);
            const int L = la + lb;
            for (int ia = 0; ia < b->shell_nprim[sa]; ++ia)
                for (int ib = 0; ib < b->shell_nprim[sb]; ++ib) {
                    const double a = b->alpha[p0[sa] + ia], bb = b->alpha[p0[sb] + ib];
                    const double cab = b->coef[p0[sa] + ia] * b->coef[p0[sb] + ib];
                    const double p = a + bb, mu = a * bb / p;
                    double P[3], PA[3], PB[3], s1[3][LM + 3][LM + 3];
                    for (int k = 0; k < 3; ++k) {
                        P[k] = (a * A[k] + bb * B[k]) / p;
                        PA[k] = P[k] - A[k];
                        PB[k] = P[k] - B[k];
                        const double X = A[k] - B[k];
                        double(*s)[LM + 3] = s1[k];
                        s[0][0] = std::sqrt(M_PI / p) * std::exp(-mu * X * X);
                        for (int i = 0; i <= la + 1; ++i)
                            for (int j = 0; j <= lb + 1; ++j) {
                                if (i == 0 && j == 0) continue;
                                double v;
                                if (i > 0) {
                                    v = PA[k] * s[i - 1][j];
                                    if (i > 1) v += (i - 1) * s[i - 2][j] / (2 * p);
                                    if (j > 0) v += j * s[i - 1][j - 1] / (2 * p);
                                } else {
                                    v = PB[k] * s[i][j - 1];
                                    if (j > 1) v += (j - 1) * s[i][j - 2] / (2 * p);
                                }
                                s[i][j] = v;
                            }
                    }
                    auto kin = [&](int k, int i, int j) {
                        const double(*s)[LM + 3] = s1[k];
                        double v = 4.0 * a * bb * s[i + 1][j + 1];
                        if (i > 0 && j > 0) v += i * j * s[i - 1][j - 1];
                        if (j > 0) v -= 2.0 * a * j * s[i + 1][j - 1];
                        if (i > 0) v -= 2.0 * bb * i * s[i - 1][j + 1];
                        return 0.5 * v;
                    };
                    Herm Ex, Ey, Ez;
                    hermite(la, lb, p, PA[0], PB[0], 1.0, Ex);
                    hermite(la, lb, p, PA[1], PB[1], 1.0, Ey);
                    hermite(la, lb, p, PA[2], PB[2], 1.0, Ez);
                    const double Kab = std::exp(-mu * ((A[0] - B[0]) * (A[0] - B[0]) + (A[1] - B[1]) * (A[1] - B[1]) +
                                                       (A[2] - B[2]) * (A[2] - B[2])));
                    // R_{tuv} summed over nuclei, weighted by -Z
                    std::vector<double> Rsum((L + 1) * (L + 1) * (L + 1), 0.0);
                    for (int c = 0; c < b->ncen; ++c) {
                        const double Z = charges[c];
                        if (Z == 0.0) continue;
                        const double* Cc = b->centers + 3 * c;
                        const double PC[3] = {P[0] - Cc[0], P[1] - Cc[1], P[2] - Cc[2]};
                        const double Tt = p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]);
                        double F[2 * LM + 2];
                        boys(L, Tt, F);
                        // R^{n}_{tuv} by the MD recursion, n from L down to 0
                        std::vector<double> R((L + 1) * (L + 1) * (L + 1) * (L + 1), 0.0);
                        auto idx = [&](int nn, int t, int u, int v) { return ((nn * (L + 1) + t) * (L + 1) + u) * (L + 1) + v; };
                        double m2p = 1.0;
                        for (int nn = 0; nn <= L; ++nn) {
                            R[idx(nn, 0, 0, 0)] = m2p * F[nn];
                            m2p *= -2.0 * p;
                        }
                        for (int nn = L - 1; nn >= 0; --nn)
                            for (int t = 0; t <= L - nn; ++t)
                                for (int u = 0; u <= L - nn - t; ++u)
                                    for (int v = 0; v <= L - nn - t - u; ++v) {
                                        if (t + u + v == 0) continue;
                                        double r;
                                        if (t > 0) {
                                            r = PC[0] * R[idx(nn + 1, t - 1, u, v)];
                                            if (t > 1) r += (t - 1) * R[idx(nn + 1, t - 2, u, v)];
                                        } else if (u > 0) {
                                            r = PC[1] * R[idx(nn + 1, t, u - 1, v)];
                                            if (u > 1) r += (u - 1) * R[idx(nn + 1, t, u - 2, v)];
                                        } else {
                                            r = PC[2] * R[idx(nn + 1, t, u, v - 1)];
                                            if (v > 1) r += (v - 1) * R[idx(nn + 1, t, u, v - 2)];
                                        }
                                        R[idx(nn, t, u, v)] = r;
                                    }
                        for (int t = 0; t <= L; ++t)
                            for (int u = 0; u <= L - t; ++u)
                                for (int v = 0; v <= L - t - u; ++v)
                                    Rsum[(t * (L + 1) + u) * (L + 1) + v] -= Z * R[idx(0, t, u, v)];
                    }
                    for (int ca = 0; ca < na; ++ca)
                        for (int cb = 0; cb < nb; ++cb) {
                            int va[3], vb[3];
                            cart(la, ca, va);
                            cart(lb, cb, vb);
                            const double sx = s1[0][va[0]][vb[0]], sy = s1[1][va[1]][vb[1]], sz = s1[2][va[2]][vb[2]];
                            sv[ca * nb + cb] += cab * sx * sy * sz;
                            tv[ca * nb + cb] += cab * (kin(0, va[0], vb[0]) * sy * sz + sx * kin(1, va[1], vb[1]) * sz +
                                                       sx * sy * kin(2, va[2], vb[2]));
                            double v = 0.0;
                            for (int t = 0; t <= va[0] + vb[0]; ++t)
                                for (int u = 0; u <= va[1] + vb[1]; ++u)
                                    for (int w = 0; w <= va[2] + vb[2]; ++w)
                                        v += Ex.E[va[0]][vb[0]][t] * Ey.E[va[1]][vb[1]][u] * Ez.E[va[2]][vb[2]][w] *
                                             Rsum[(t * (L + 1) + u) * (L + 1) + w];
                            vv[ca * nb + cb] += cab * 2.0 * M_PI / p * Kab * v;
                        }
                }
            for (int ca = 0; ca < na; ++ca)
                for (int cb = 0; cb < nb; ++cb) {
                    const int i = b->shell_offset[sa] + ca, j = b->shell_offset[sb] + cb;
                    if (j > i) continue;  // within a diagonal shell block keep the lower triangle
                    const double nrm = comp_norm(la, ca) * comp_norm(lb, cb);
                    const size_t k = (size_t)i * (i + 1) / 2 + j;
                    S[k] = sv[ca * nb + cb] * nrm;
                    T[k] = tv[ca * nb + cb] * nrm;
                    H[k] = (tv[ca * nb + cb] + vv[ca * nb + cb]) * nrm;
                }
        }
    return UNOMOL_OK;
}
