"""Generates rys_tables.inc: piecewise polynomial fits of the Rys quadrature nodes and weights.

For n roots, the Rys quadrature of the weight e^{-T t^2} on t in [0, 1] is exact for polynomials in
x = t^2 of degree <= 2n-1:  int_0^1 f(t^2) e^{-T t^2} dt = sum_i w_i f(x_i).  The moments of that
weight are the Boys functions F_k(T) = int_0^1 t^{2k} e^{-T t^2} dt.

Construction (all in 60-digit arithmetic with mpmath, so the ill-conditioning of power moments does
not matter):
  1. F_k(T) from the lower incomplete gamma function;
  2. recurrence coefficients of the orthogonal polynomials by Chebyshev's algorithm
     (W. Gautschi, "Orthogonal Polynomials: Computation and Approximation", 2004, sec. 2.1.7);
  3. nodes and weights from the eigen-decomposition of the Jacobi matrix (Golub & Welsch, 1969).

On [0, TMAX) the nodes x_i(T) and weights w_i(T) are fitted interval by interval (width H for the
FP64 table, H32 for the FP32 one) with
Chebyshev interpolants, converted to monomials in y = 2 (T - T_k)/H - 1 in [-1, 1] and evaluated by
Horner's rule.  For T >= TMAX the large-T limit is used: the weight function is then a half-line
Gaussian, so x_i = r_i^2 / T and w_i = W_i / sqrt(T), with r_i > 0 the roots of the Hermite
polynomial H_{2n} and W_i their Gauss-Hermite weights.  TMAX is chosen per n so that this limit is
accurate to double rounding.

The reference fits the same functions with its own tables (Rys.cpp:314-2197, regime boundaries 33 to
59); these fits are independent of them and are checked against the reference's integrals through
the golden fixtures.

Output arrays (C source included by the CUDA kernels):
  RYS_NMAX, RYS_H (interval width), RYS_DEG (polynomial degree), RYS_TMAX[n],
  RYS_TABLE_H[n][interval][2n][RYS_DEG+1]  (node i at 2i, weight i at 2i+1; highest power first),
  RYS_HERMITE_X_H[n][i], RYS_HERMITE_W_H[n][i].
A float table with its own interval width and lower degree (RYS32_H, RYS32_DEG) serves the FP32
kernels.

Run: python gen_rys_tables.py  (a few minutes; writes rys_tables.inc next to this file)
"""
from __future__ import annotations

import os
import sys

import mpmath as mp
import numpy as np

mp.mp.dps = 60
NMAX = 5
H = 0.25         # FP64 interval width in T
DEG = 7          # FP64 Horner degree (8 coefficients; 3e-15 relative at H = 0.25; degree 9 at H = 0.5
                 # gives 2e-16 with 2 more FMAs per polynomial, degree 8 at H = 0.5 1e-14)
H32 = 0.5        # FP32 interval width (the FP32 kernels read the table per lane: it stays small)
DEG32 = 5        # FP32 Horner degree (1.1e-7 relative at H32 = 0.5)
NCHEB = 24       # interpolation nodes per interval for the fit


def boys(k: int, T) -> mp.mpf:
    T = mp.mpf(T)
    if T == 0:
        return mp.mpf(1) / (2 * k + 1)
    a = k + mp.mpf(1) / 2
    return mp.gammainc(a, 0, T) / (2 * mp.power(T, a))


def rys_exact(n: int, T):
    """Nodes x_i = t_i^2 (ascending) and weights w_i for n roots at T, high precision."""
    mu = [boys(k, T) for k in range(2 * n)]
    alpha = [mp.mpf(0)] * n
    beta = [mp.mpf(0)] * n
    sig_prev = [mp.mpf(0)] * (2 * n)
    sig = list(mu)
    alpha[0] = mu[1] / mu[0]
    beta[0] = mu[0]
    for k in range(1, n):
        sig_new = [mp.mpf(0)] * (2 * n)
        for l in range(k, 2 * n - k):
            sig_new[l] = sig[l + 1] - alpha[k - 1] * sig[l] - beta[k - 1] * sig_prev[l]
        alpha[k] = sig_new[k + 1] / sig_new[k] - sig[k] / sig[k - 1]
        beta[k] = sig_new[k] / sig[k - 1]
        sig_prev, sig = sig, sig_new
    J = mp.zeros(n, n)
    for k in range(n):
        J[k, k] = alpha[k]
        if k + 1 < n:
            J[k, k + 1] = J[k + 1, k] = mp.sqrt(beta[k + 1])
    E, Q = mp.eigsy(J)
    pairs = sorted((E[i], beta[0] * Q[0, i] ** 2) for i in range(n))
    return [p[0] for p in pairs], [p[1] for p in pairs]


def hermite_half(n: int):
    """Positive roots r_i of H_{2n} (ascending, squared) and their Gauss-Hermite weights."""
    m = 2 * n
    J = mp.zeros(m, m)
    for k in range(m - 1):
        J[k, k + 1] = J[k + 1, k] = mp.sqrt(mp.mpf(k + 1) / 2)
    E, Q = mp.eigsy(J)
    pos = sorted((E[i], mp.sqrt(mp.pi) * Q[0, i] ** 2) for i in range(m) if E[i] > 0)
    return [p[0] ** 2 for p in pos], [p[1] for p in pos]


def asym_tmax(n: int) -> float:
    """Smallest integer T (multiple of H) from which the large-T limit matches to ~1e-16 relative."""
    hx, hw = hermite_half(n)
    for T in range(20, 200):
        ok = True
        for TT in (T, T + 0.5, T + 1):
            x, w = rys_exact(n, TT)
            for i in range(n):
                ex = abs(hx[i] / TT - x[i]) / x[i]
                ew = abs(hw[i] / mp.sqrt(TT) - w[i]) / w[i]
                if ex > 2e-17 or ew > 2e-17:
                    ok = False
        if ok:
            return float(T)
    raise RuntimeError("no TMAX")


def cheb_fit(fvals, deg):
    """Chebyshev interpolation at NCHEB first-kind nodes, truncated to deg, as monomials in y."""
    N = len(fvals)
    c = []
    for j in range(N):
        s = mp.mpf(0)
        for k in range(N):
            s += fvals[k] * mp.cos(mp.pi * j * (k + mp.mpf(1) / 2) / N)
        c.append(s * (2 if j else 1) / N)
    c = c[: deg + 1]
    # Chebyshev -> monomial (T_0 = 1, T_1 = y, T_{k+1} = 2y T_k - T_{k-1})
    Tk = [[mp.mpf(1)], [mp.mpf(0), mp.mpf(1)]]
    for k in range(2, deg + 1):
        a = [mp.mpf(0)] + [2 * v for v in Tk[k - 1]]
        b = Tk[k - 2] + [mp.mpf(0)] * (len(a) - len(Tk[k - 2]))
        Tk.append([a[i] - b[i] for i in range(len(a))])
    mono = [mp.mpf(0)] * (deg + 1)
    for k, ck in enumerate(c):
        for i, v in enumerate(Tk[k]):
            mono[i] += ck * v
    return mono  # lowest power first


def horner(coefs_high_first, y, dtype):
    r = dtype(coefs_high_first[0])
    y = dtype(y)
    for c in coefs_high_first[1:]:
        r = dtype(r * y + dtype(c))
    return r


def fit_table(n: int, tmax: float, h: float, deg: int, dtype):
    """Per interval of width h on [0, tmax): the degree-deg fits of the n nodes and weights, and the
    worst relative error of their Horner evaluation in dtype at off-node points."""
    nint = int(round(tmax / h))
    tab = np.zeros((nint, 2 * n, deg + 1))
    worst = 0.0
    nodes = [mp.cos(mp.pi * (j + mp.mpf(1) / 2) / NCHEB) for j in range(NCHEB)]
    for k in range(nint):
        a = k * h
        samples = [rys_exact(n, a + (y + 1) * h / 2) for y in nodes]
        for i in range(n):
            for which in (0, 1):
                f = [s[which][i] for s in samples]
                tab[k, 2 * i + which, :] = [float(v) for v in reversed(cheb_fit(f, deg))]
        for y in np.linspace(-1, 1, 9):
            ex = rys_exact(n, a + (mp.mpf(y) + 1) * h / 2)
            for i in range(n):
                for which in (0, 1):
                    tv = ex[which][i]
                    v = horner(tab[k, 2 * i + which], dtype(y), dtype)
                    worst = max(worst, float(abs(mp.mpf(float(v)) - tv) / abs(tv)))
    return tab, worst


def build(n: int, tmax: float):
    tab64, worst64 = fit_table(n, tmax, H, DEG, np.float64)
    tab32, worst32 = fit_table(n, tmax, H32, DEG32, np.float32)
    return tab64, tab32, worst64, worst32


def fmt(v):
    return repr(float(v))


def main():
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rys_tables.inc")
    lines = ["// Generated by gen_rys_tables.py -- do not edit. Rys nodes x=t^2 and weights, piecewise",
             "// polynomials in y = 2 (T - k H)/H - 1 on [k H, (k+1) H), highest power first.",
             f"#define RYS_NMAX {NMAX}", f"#define RYS_H {H!r}", f"#define RYS_DEG {DEG}",
             f"#define RYS32_H {H32!r}", f"#define RYS32_DEG {DEG32}"]
    tmaxes, offs, offs32 = [], [], []
    body64, body32 = [], []
    hx_all, hw_all = [], []
    o = 0
    o32 = 0
    for n in range(1, NMAX + 1):
        tmax = asym_tmax(n)
        t64, t32, e64, e32 = build(n, tmax)
        print(f"n={n}: TMAX={tmax} intervals={t64.shape[0]}/{t32.shape[0]} worst rel err fp64={e64:.2e} "
              f"fp32={e32:.2e}", file=sys.stderr, flush=True)
        tmaxes.append(tmax)
        offs.append(o)
        offs32.append(o32)
        body64.extend(fmt(v) for v in t64.ravel())
        body32.extend(fmt(v) + "f" for v in t32.ravel())
        o += t64.size
        o32 += t32.size
        hx, hw = hermite_half(n)
        hx_all.append([float(v) for v in hx] + [0.0] * (NMAX - n))
        hw_all.append([float(v) for v in hw] + [0.0] * (NMAX - n))
    for n, t in enumerate(tmaxes, 1):
        lines.append(f"#define RYS_TMAX_{n} {t!r}")
    lines.append("static const double RYS_TMAX_H[RYS_NMAX] = {" + ", ".join(fmt(t) for t in tmaxes) + "};")
    lines.append("static const int RYS_OFF_H[RYS_NMAX] = {" + ", ".join(map(str, offs)) + "};")
    lines.append("static const int RYS32_OFF_H[RYS_NMAX] = {" + ", ".join(map(str, offs32)) + "};")
    lines.append(f"#define RYS_TABLE_SIZE {o}")
    lines.append(f"#define RYS32_TABLE_SIZE {o32}")
    lines.append("static const double RYS_HERMITE_X_H[RYS_NMAX][RYS_NMAX] = {"
                 + ", ".join("{" + ", ".join(fmt(v) for v in r) + "}" for r in hx_all) + "};")
    lines.append("static const double RYS_HERMITE_W_H[RYS_NMAX][RYS_NMAX] = {"
                 + ", ".join("{" + ", ".join(fmt(v) for v in r) + "}" for r in hw_all) + "};")
    lines.append("static const double RYS_TABLE_H[RYS_TABLE_SIZE] = {")
    for i in range(0, len(body64), 4):
        lines.append("  " + ", ".join(body64[i:i + 4]) + ",")
    lines.append("};")
    lines.append("static const float RYS32_TABLE_H[RYS32_TABLE_SIZE] = {")
    for i in range(0, len(body32), 4):
        lines.append("  " + ", ".join(body32[i:i + 4]) + ",")
    lines.append("};")
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", out, file=sys.stderr)


if __name__ == "__main__":
    main()
