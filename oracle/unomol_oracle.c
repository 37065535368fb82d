/*
 * Test infrastructure: a CPU restatement, in C, of the reference's two-electron Fock build.  It is the
 * oracle of the GPU path on machines without the reference sources, and the "port" CPU baseline of
 * bench.py.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use it; the product never
 * links or calls it.
 *
 * Followed step by step (reference file:line):
 *   shell / function quartet enumeration with the L swaps and 4-bit component keys
 *                                                     TwoElectronInts.cpp:511-653
 *   primitive loops, same-shell symmetry, prefactor cut, Rys recurrence and shift
 *                                                     TwoElectronInts.cpp:420-509, Rys.hpp:85-212
 *   storage cut |v| > 1e-14                           TwoElectronInts.cpp:667-671
 *   RHF and UHF scatter into packed G                 TwoElectronInts.cpp:699-820
 * The Rys nodes and weights come from the piecewise fits of unomol_gb300/csrc/rys_tables.inc (exact
 * quadrature to ~2e-16); in the reference-compatible mode the two-root regime 15 < T <= 40 follows the
 * reference's fit (Rys.cpp:611-623), as in the GPU path.  The reference's own root fits are not
 * restated.  Parity of this oracle with the reference is pinned by tests/test_oracle.py against the
 * golden fixtures generated from the reference itself.
 *
 * Work can be split for a bounded CPU sample: only shell quartets whose running index q satisfies
 * q % stride == offset are computed.  OpenMP threads split the ish loop.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../unomol_gb300/csrc/rys_tables.inc"

typedef struct {
    int nshell, norb, ncen;
    const int *shell_l, *shell_nprim, *shell_center, *shell_offset;
    const double *alpha, *coef, *centers;
} orc_basis;

#define MAXL 2
#define MAXR (2 * MAXL + 1)
#define MAXROOT 5
#define MAXLST 6
#define MAXINTS (MAXLST * MAXLST * MAXLST * MAXLST)

static double binom[MAXR + 1][MAXR + 1];
static double nfact[MAXL + 1][MAXLST];
static int lxyz[MAXL + 1][MAXLST][3];
static int tables_ready = 0;

/* AuxFunctions.hpp:21-67: component order lx descending, ly descending; 1/sqrt of the reference's
 * double-factorial table (1, 1, 3 for l <= 2). */
static void init_tables(void) {
    if (tables_ready) return;
    double fact[MAXR + 2];
    fact[0] = 1.0;
    for (int i = 1; i <= MAXR + 1; ++i) fact[i] = fact[i - 1] * i;
    for (int i = 0; i <= MAXR; ++i)
        for (int j = 0; j <= i; ++j) binom[i][j] = fact[i] / fact[i - j] / fact[j];
    double dfact[MAXL + 1];
    dfact[0] = 1.0;
    double dx = 1.0;
    for (int i = 1; i <= MAXL; ++i) {
        dfact[i] = dfact[i - 1] * dx;
        dx *= (2 * i + 1);
    }
    for (int l = 0; l <= MAXL; ++l) {
        int k = 0;
        for (int x = l; x >= 0; --x)
            for (int y = l - x; y >= 0; --y) {
                lxyz[l][k][0] = x;
                lxyz[l][k][1] = y;
                lxyz[l][k][2] = l - x - y;
                nfact[l][k] = 1.0 / sqrt(dfact[x] * dfact[y] * dfact[l - x - y]);
                ++k;
            }
    }
    tables_ready = 1;
}

static const double tmax_tab[5] = {RYS_TMAX_1, RYS_TMAX_2, RYS_TMAX_3, RYS_TMAX_4, RYS_TMAX_5};

/* Rys nodes x = t^2 and weights for n roots at T. */
static void roots_weights(int n, double T, int compat, double* x, double* w) {
    if (compat && n == 2 && T > 15.0 && T <= 40.0) {
        const double r12 = .275255128608411, r22 = 2.72474487139158, w22 = .0917517095361369;
        const double g = exp(-T), w0 = sqrt(.785398163397448 / T);
        const double u0 = (T * -.87894730749888 + 10.9243702330261) * g + r12 / (T - r12);
        const double u1 = (T * -9.28903924275977 + 81.0642367843811) * g + r22 / (T - r22);
        const double w1 = (T * 4.468573893084 - 77.9250653461045) * g + w22 * w0;
        x[0] = u0 / (1.0 + u0);
        x[1] = u1 / (1.0 + u1);
        w[0] = w0 - w1;
        w[1] = w1;
        return;
    }
    if (T < tmax_tab[n - 1]) {
        const double Ts = T * (1.0 / RYS_H);
        int k = (int)Ts;
        double y = 2.0 * (Ts - k) - 1.0;
        const double* c = RYS_TABLE_H + RYS_OFF_H[n - 1] + k * (2 * n * (RYS_DEG + 1));
        for (int i = 0; i < n; ++i) {
            const double* cx = c + 2 * i * (RYS_DEG + 1);
            const double* cw = cx + (RYS_DEG + 1);
            double vx = cx[0], vw = cw[0];
            for (int d = 1; d <= RYS_DEG; ++d) {
                vx = vx * y + cx[d];
                vw = vw * y + cw[d];
            }
            x[i] = vx;
            w[i] = vw;
        }
    } else {
        double rT = 1.0 / T, s = sqrt(rT);
        for (int i = 0; i < n; ++i) {
            x[i] = RYS_HERMITE_X_H[n - 1][i] * rT;
            w[i] = RYS_HERMITE_W_H[n - 1][i] * s;
        }
    }
}

typedef struct {
    double G[MAXROOT][3][MAXR][MAXR];
    double w[MAXROOT];
} rys_ws;

/* Rys.hpp:113-143 and 194-212 (Recur / RecurKernel), with x = t^2 directly. */
static void recur(rys_ws* ws, const double* p, const double* q, const double* pa, const double* qc, double pxp,
                  double qxp, double txp, int l12, int l34, int nroots, int compat) {
    double pq[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
    double pq2 = pq[0] * pq[0] + pq[1] * pq[1] + pq[2] * pq[2];
    double T = pxp * qxp / txp * pq2;
    double x[MAXROOT];
    roots_weights(nroots, T, compat, x, ws->w);
    for (int r = 0; r < nroots; ++r) {
        double fff = x[r] / txp;
        double B00 = 0.5 * fff, B1 = (0.5 - B00 * qxp) / pxp, B1p = (0.5 - B00 * pxp) / qxp;
        for (int ax = 0; ax < 3; ++ax) {
            double C = pa[ax] - qxp * pq[ax] * fff, Cp = qc[ax] + pxp * pq[ax] * fff;
            double(*G)[MAXR] = ws->G[r][ax];
            G[0][0] = 1.0;
            G[0][1] = Cp;
            G[1][0] = C;
            G[1][1] = B00 + C * Cp;
            if (l12 < 2 && l34 < 2) continue;
            for (int j = 1; j < l34; ++j) {
                G[0][j + 1] = j * B1p * G[0][j - 1] + Cp * G[0][j];
                G[1][j + 1] = j * B1p * G[1][j - 1] + B00 * G[0][j] + Cp * G[1][j];
            }
            for (int i = 2; i <= l12; ++i) {
                G[i][0] = (i - 1) * B1 * G[i - 2][0] + C * G[i - 1][0];
                G[i][1] = i * B00 * G[i - 1][0] + Cp * G[i][0];
                for (int j = 1; j < l34; ++j) G[i][j + 1] = j * B1p * G[i][j - 1] + i * B00 * G[i - 1][j] + Cp * G[i][j];
            }
        }
    }
}

/* Rys.hpp:173-192 (ShiftKernel): horizontal transfer by binomial sums. */
static double shift1(double (*G)[MAXR], double abx, double cdx, int l12, int l2, int l34, int l4) {
    double sum = 0.0, x12t = 1.0;
    for (int i = 0; i <= l2; ++i) {
        double x34t = binom[l2][i] * x12t;
        for (int j = 0; j <= l4; ++j) {
            sum += binom[l4][j] * x34t * G[l12 - i][l34 - j];
            x34t *= cdx;
        }
        x12t *= abx;
    }
    return sum;
}

typedef struct {
    const double *a, *b, *c, *d;
    int n1, l1, n2, l2, n3, l3, n4, l4;
    const double *al1, *co1, *al2, *co2, *al3, *co3, *al4, *co4;
    int same12, same34;
    int len;
    unsigned keys[MAXINTS];
    double norms[MAXINTS];
    double val[MAXINTS];
} quartet;

/* TwoElectronInts.cpp:420-509. */
static void eri_rys(quartet* sq, rys_ws* ws, int compat, long long* nprim) {
    const double SRterm = 34.9868366552497250, threshold = 1.e-12;
    double ab[3], cd[3], p[3], q[3], pa[3], qc[3];
    for (int k = 0; k < 3; ++k) {
        ab[k] = sq->a[k] - sq->b[k];
        cd[k] = sq->c[k] - sq->d[k];
    }
    double ab2 = ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2];
    double cd2 = cd[0] * cd[0] + cd[1] * cd[1] + cd[2] * cd[2];
    int lvt12 = sq->l1 + sq->l2, lvt34 = sq->l3 + sq->l4, nroots = (lvt12 + lvt34) / 2 + 1;
    for (int kc = 0; kc < sq->len; ++kc) sq->val[kc] = 0.0;
    for (int i = 0; i < sq->n1; ++i) {
        double axp = sq->al1[i], c1 = sq->co1[i];
        int jend = sq->same12 ? i + 1 : sq->n2;
        for (int j = 0; j < jend; ++j) {
            double f12 = (sq->same12 && i != j) ? 2.0 : 1.0;
            double c12 = c1 * f12 * sq->co2[j], bxp = sq->al2[j], pxp = axp + bxp, abi = 1.0 / pxp;
            double s12 = exp(-axp * bxp * ab2 * abi);
            for (int k = 0; k < 3; ++k) {
                p[k] = (axp * sq->a[k] + bxp * sq->b[k]) * abi;
                pa[k] = p[k] - sq->a[k];
            }
            for (int k3 = 0; k3 < sq->n3; ++k3) {
                double cxp = sq->al3[k3], c3 = sq->co3[k3];
                int lend = sq->same34 ? k3 + 1 : sq->n4;
                for (int l = 0; l < lend; ++l) {
                    double f34 = (sq->same34 && k3 != l) ? 2.0 : 1.0;
                    double c34 = c3 * f34 * sq->co4[l], dxp = sq->al4[l], qxp = cxp + dxp, cdi = 1.0 / qxp;
                    double s34 = exp(-cxp * dxp * cd2 * cdi), txp = pxp + qxp;
                    double sr = SRterm * s12 * s34 * abi * cdi / sqrt(txp);
                    if (sr < threshold) continue;
                    sr *= c12 * c34;
                    ++*nprim;
                    for (int k = 0; k < 3; ++k) {
                        q[k] = (cxp * sq->c[k] + dxp * sq->d[k]) * cdi;
                        qc[k] = q[k] - sq->c[k];
                    }
                    recur(ws, p, q, pa, qc, pxp, qxp, txp, lvt12, lvt34, nroots, compat);
                    for (int kc = 0; kc < sq->len; ++kc) {
                        unsigned key = sq->keys[kc];
                        int lls = key & 0xF, kls = (key >> 4) & 0xF, jls = (key >> 8) & 0xF, ils = (key >> 12) & 0xF;
                        const int *v1 = lxyz[sq->l1][ils], *v2 = lxyz[sq->l2][jls], *v3 = lxyz[sq->l3][kls], *v4 = lxyz[sq->l4][lls];
                        double sum = 0.0;
                        for (int r = 0; r < nroots; ++r) {
                            double s = ws->w[r];
                            for (int ax = 0; ax < 3; ++ax)
                                s *= shift1(ws->G[r][ax], ab[ax], cd[ax], v1[ax] + v2[ax], v2[ax], v3[ax] + v4[ax], v4[ax]);
                            sum += s;
                        }
                        sq->val[kc] += sum * sr * sq->norms[kc];
                    }
                }
            }
        }
    }
}

/* TwoElectronInts.cpp:699-747 (formGMatrixKernel) and 749-820 (formGMatrixKernel2). */
static void scatter(double val, int i, int j, int k, int l, const double* Pa, const double* Pb, double* Ga, double* Gb) {
    int ii = i * (i + 1) / 2, ij = ii + j, ik = ii + k, il = ii + l, jk, jl;
    int kk = k * (k + 1) / 2, kl = kk + l;
    if (j >= k) {
        int jj = j * (j + 1) / 2;
        jk = jj + k;
        jl = jj + l;
    } else {
        jk = kk + j;
        jl = (j > l) ? j * (j + 1) / 2 + l : l * (l + 1) / 2 + j;
    }
    const int uhf = Pb != NULL;
    double da = uhf ? val * (Pa[ij] + Pb[ij]) : val * 2.0 * Pa[ij];
    double db = uhf ? val * (Pa[kl] + Pb[kl]) : val * 2.0 * Pa[kl];
    for (int s = 0; s < (uhf ? 2 : 1); ++s) {
        const double* P = s ? Pb : Pa;
        double* G = s ? Gb : Ga;
        double d_a = da, d_b = db;
        double sjl = val * P[ik], sjk = val * P[il], sik = val * P[jl], sil = val * P[jk];
        if (k != l) {
            d_b += d_b;
            G[ik] -= sik;
            if (i != j && j >= k) G[jk] -= sjk;
        }
        G[il] -= sil;
        G[ij] += d_b;
        if (i != j && j >= l) G[jl] -= sjl;
        if (ij != kl) {
            if (i != j) d_a += d_a;
            if (j <= k) {
                G[jk] -= sjk;
                if (i != j && i <= k) G[ik] -= sik;  /* RHF kernel writes i == k; equal under j <= k, i != j? see note */
                if (k != l && j <= l) G[jl] -= sjl;
            }
            G[kl] += d_a;
        }
    }
}

/* splitmix64 finaliser: a well-mixed 64-bit hash of the quartet index (for the hashed sample) */
static unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Full G over the canonical quartets of TwoElectronInts::calculate, or a sample of them: stride > 1
 * keeps the quartets with q % stride == offset (q = running index of the canonical enumeration);
 * stride < -1 keeps those with hash(q) % |stride| == offset, a pseudo-random 1/|stride| of every
 * class, and the |stride| offsets partition the build.
 * Pb == NULL: RHF (G += 2J - K); else UHF (Ga, Gb).  rys_mode 0 = reference-compatible, 1 = exact.
 * counts (optional): [0] shell quartets done, [1] function quartets, [2] primitive quartets,
 * [3] stored integrals.  Returns 0, or -1 for an unsupported basis (L > 2). */
/* Record sink of orc_records: the stored integrals (TwoInts val, i, j, k, l) instead of the scatter. */
typedef struct {
    double* val;
    int* ijkl;
    long long cap, n;
} rec_sink;

static int fock_pass(const orc_basis* B, int start, const double* Pa, const double* Pb, double* Ga, double* Gb, int rys_mode,
                     long long stride, long long offset, int nthreads, long long* counts, rec_sink* sink) {
    init_tables();
    for (int s = 0; s < B->nshell; ++s)
        if (B->shell_l[s] > MAXL) return -1;
    const int no2 = B->norb * (B->norb + 1) / 2;
    int* sp0 = (int*)malloc(sizeof(int) * B->nshell);
    int np = 0;
    for (int s = 0; s < B->nshell; ++s) {
        sp0[s] = np;
        np += B->shell_nprim[s];
    }
    const int hashed = stride < -1;
    if (hashed) stride = -stride;
    if (stride < 1) stride = 1;
    long long tot[4] = {0, 0, 0, 0};
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        double* ga = (double*)calloc(no2, sizeof(double));
        double* gb = Pb ? (double*)calloc(no2, sizeof(double)) : NULL;
        quartet* sq = (quartet*)malloc(sizeof(quartet));
        rys_ws* ws = (rys_ws*)malloc(sizeof(rys_ws));
        long long cnt[4] = {0, 0, 0, 0};
#pragma omp for schedule(dynamic, 1)
        for (int ish = start; ish < B->nshell; ++ish) {
            /* running quartet index of the first quartet of this ish (for the strided sample) */
            long long q = 0;
            for (int s = start; s < ish; ++s) q += (long long)(s + 1) * (s + 1) * (s + 2) / 2;
            for (int jsh = 0; jsh <= ish; ++jsh) {
                for (int ksh = 0; ksh <= ish; ++ksh) {
                    for (int lsh = 0; lsh <= ksh; ++lsh, ++q) {
                        if (stride > 1 && (long long)((hashed ? mix64((unsigned long long)q) : (unsigned long long)q) %
                                                      (unsigned long long)stride) != offset)
                            continue;
                        int sh[4] = {ish, jsh, ksh, lsh};
                        int off[4], lv[4], nls[4];
                        for (int t = 0; t < 4; ++t) {
                            off[t] = B->shell_offset[sh[t]];
                            lv[t] = B->shell_l[sh[t]];
                            nls[t] = (lv[t] + 1) * (lv[t] + 2) / 2;
                        }
                        /* TwoElectronInts.cpp:563-579, 604-620: larger L first in each pair */
                        int sw12 = lv[0] < lv[1], sw34 = lv[2] < lv[3];
                        int a = sw12 ? jsh : ish, b = sw12 ? ish : jsh, c = sw34 ? lsh : ksh, d = sw34 ? ksh : lsh;
                        sq->a = B->centers + 3 * B->shell_center[a];
                        sq->b = B->centers + 3 * B->shell_center[b];
                        sq->c = B->centers + 3 * B->shell_center[c];
                        sq->d = B->centers + 3 * B->shell_center[d];
                        sq->n1 = B->shell_nprim[a]; sq->l1 = B->shell_l[a]; sq->al1 = B->alpha + sp0[a]; sq->co1 = B->coef + sp0[a];
                        sq->n2 = B->shell_nprim[b]; sq->l2 = B->shell_l[b]; sq->al2 = B->alpha + sp0[b]; sq->co2 = B->coef + sp0[b];
                        sq->n3 = B->shell_nprim[c]; sq->l3 = B->shell_l[c]; sq->al3 = B->alpha + sp0[c]; sq->co3 = B->coef + sp0[c];
                        sq->n4 = B->shell_nprim[d]; sq->l4 = B->shell_l[d]; sq->al4 = B->alpha + sp0[d]; sq->co4 = B->coef + sp0[d];
                        sq->same12 = (ish == jsh);
                        sq->same34 = (ksh == lsh);
                        int knt = 0;
                        int idx[MAXINTS][4];
                        for (int ils = 0; ils < nls[0]; ++ils) {
                            int ir = off[0] + ils;
                            for (int jls = 0; jls < nls[1]; ++jls) {
                                int jr = off[1] + jls;
                                if (jr > ir) break;
                                for (int kls = 0; kls < nls[2]; ++kls) {
                                    int kr = off[2] + kls;
                                    if (kr > ir) break;
                                    for (int lls = 0; lls < nls[3]; ++lls) {
                                        int lr = off[3] + lls;
                                        if (lr > kr || (ir == kr && lr > jr)) break;
                                        unsigned l12 = sw12 ? (jls << 4) + ils : (ils << 4) + jls;
                                        unsigned l34 = sw34 ? (lls << 4) + kls : (kls << 4) + lls;
                                        sq->keys[knt] = (l12 << 8) + l34;
                                        sq->norms[knt] = nfact[lv[0]][ils] * nfact[lv[1]][jls] * nfact[lv[2]][kls] * nfact[lv[3]][lls];
                                        idx[knt][0] = ir; idx[knt][1] = jr; idx[knt][2] = kr; idx[knt][3] = lr;
                                        ++knt;
                                    }
                                }
                            }
                        }
                        if (!knt) continue;
                        sq->len = knt;
                        cnt[0] += 1;
                        cnt[1] += knt;
                        eri_rys(sq, ws, rys_mode == 0, &cnt[2]);
                        for (int kc = 0; kc < knt; ++kc) {
                            if (fabs(sq->val[kc]) > 1.e-14) {
                                ++cnt[3];
                                if (sink) {
#pragma omp critical
                                    {
                                        if (sink->n < sink->cap) {
                                            sink->val[sink->n] = sq->val[kc];
                                            for (int t = 0; t < 4; ++t) sink->ijkl[4 * sink->n + t] = idx[kc][t];
                                        }
                                        ++sink->n;
                                    }
                                } else {
                                    scatter(sq->val[kc], idx[kc][0], idx[kc][1], idx[kc][2], idx[kc][3], Pa, Pb, ga, gb);
                                }
                            }
                        }
                    }
                }
            }
        }
#pragma omp critical
        {
            for (int t = 0; t < no2; ++t) Ga[t] += ga[t];
            if (Pb)
                for (int t = 0; t < no2; ++t) Gb[t] += gb[t];
            for (int t = 0; t < 4; ++t) tot[t] += cnt[t];
        }
        free(ga);
        free(gb);
        free(sq);
        free(ws);
    }
    if (counts)
        for (int t = 0; t < 4; ++t) counts[t] = tot[t];
    free(sp0);
    return 0;
}

int orc_fock(const orc_basis* B, int start, const double* Pa, const double* Pb, double* Ga, double* Gb, int rys_mode,
             long long stride, long long offset, int nthreads, long long* counts) {
    return fock_pass(B, start, Pa, Pb, Ga, Gb, rys_mode, stride, offset, nthreads, counts, NULL);
}

/* The stored integrals of TwoElectronInts::calculate (TwoElectronInts.cpp:622-671): the canonical
 * function quartets with |v| > 1e-14 as (val, i, j, k, l), at most cap of them written into val[] and
 * ijkl[4 * cap]; returns the count (which may exceed cap), or -1 for an unsupported basis. */
long long orc_records(const orc_basis* B, int start, int rys_mode, double* val, int* ijkl, long long cap) {
    const int no2 = B->norb * (B->norb + 1) / 2;
    double* P = (double*)calloc(no2, sizeof(double));
    double* G = (double*)calloc(no2, sizeof(double));
    rec_sink sink = {val, ijkl, cap, 0};
    const int rc = fock_pass(B, start, P, NULL, G, NULL, rys_mode, 1, 0, 0, NULL, &sink);
    free(P);
    free(G);
    return rc ? -1 : sink.n;
}
