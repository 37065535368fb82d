// Test infrastructure: an exact replacement for the reference's two-root Rys fit, linked over a copy
// of the reference's Rys.o whose Rys::root2 symbol is made weak (oracle/Makefile).  The result is the
// reference with every other line unchanged and Rys::root2 exact, the oracle of the GPU path's
// "exact" Rys mode.
//
// Why: Rys::root2 (Rys.cpp:414-631) uses, for 15 < T <= 40, a large-T form whose e^{-T} corrections
// leave errors of up to 3.5e-4 relative at T = 15 (1e-12 near T = 31); root1 and root3..5 agree with
// exact quadrature to ~1e-13.
//
// Method: n = 2 Rys quadrature from the moments F_0..F_3 (Boys functions, long double): the monic
// orthogonal polynomial x^2 + a x + b has int p x^k = 0 for k = 0, 1; its roots are the nodes
// x_i = t_i^2 and the weights follow from w1 + w2 = F_0, w1 x1 + w2 x2 = F_1.  Stored as the
// reference stores them: roots u = t^2 / (1 - t^2) (Rys.cpp:307-310).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "Rys.hpp"

namespace {

// F_m(T) for m = 0..mmax by the series for F_mmax and downward recursion (long double).
void boys_ld(int mmax, long double T, long double* F) {
    const long double e = expl(-T);
    long double term = 1.0L / (2 * mmax + 1), sum = term;
    for (int k = 1; k < 2000; ++k) {
        term *= 2.0L * T / (2 * mmax + 2 * k + 1);
        sum += term;
        if (term < sum * 1e-21L) break;
    }
    F[mmax] = sum * e;
    for (int m = mmax; m > 0; --m) F[m - 1] = (2.0L * T * F[m] + e) / (2 * m - 1);
}

}  // namespace

namespace unomol {

void Rys::root2(double T) noexcept {
    if (T >= 48.0) {
        // large-T limit: half-line Gauss-Hermite (H_4) nodes r^2 / T and weights W / sqrt(T); exact
        // to double rounding from T = 48 on (the moment series below would overflow at T ~ 1e4)
        const long double x1 = 0.2752551286084109509014L / T, x2 = 2.724744871391589049099L / T;
        const long double s = 1.0L / sqrtl((long double)T);
        roots[0] = (double)(x1 / (1.0L - x1));
        roots[1] = (double)(x2 / (1.0L - x2));
        weights[0] = (double)(0.804914090005512836506L * s);
        weights[1] = (double)(0.08131283544724517714303L * s);
        return;
    }
    long double F[4];
    boys_ld(3, (long double)T, F);
    // mu2 + a mu1 + b mu0 = 0 ; mu3 + a mu2 + b mu1 = 0
    const long double det = F[1] * F[1] - F[2] * F[0];
    const long double a = (F[3] * F[0] - F[2] * F[1]) / det;
    const long double b = (F[2] * F[2] - F[3] * F[1]) / det;
    const long double disc = sqrtl(a * a - 4.0L * b);
    // stable quadratic roots
    const long double q = -0.5L * (a + (a >= 0 ? disc : -disc));
    long double x1 = q, x2 = b / q;
    if (x1 > x2) {
        long double t = x1;
        x1 = x2;
        x2 = t;
    }
    const long double w2 = (F[1] - x1 * F[0]) / (x2 - x1);
    const long double w1 = F[0] - w2;
    roots[0] = (double)(x1 / (1.0L - x1));
    roots[1] = (double)(x2 / (1.0L - x2));
    weights[0] = (double)w1;
    weights[1] = (double)w2;
}

}  // namespace unomol
