// One-electron integrals S, T and H = T + V on the GPU, for many geometries of one basis in one launch
// (the data of OneElectronInts, OneElectronInts.cpp:6-202; same algorithms and conventions as the host
// version in one_electron.cpp):
//   * overlap and kinetic energy by Obara-Saika 1D recurrences per Cartesian axis, the kinetic energy
//     from the overlap table by T(i, j) = [i j S(i-1, j-1) + 4 a b S(i+1, j+1) - 2 a j S(i+1, j-1)
//     - 2 b i S(i-1, j+1)] / 2 (the identity of OneElectronInts.cpp:74-115);
//   * nuclear attraction by McMurchie-Davidson, V = -sum_C Z_C 2 pi / p K_ab sum_tuv E^x_t E^y_u E^z_v
//     R_tuv(p, P - C), with the reference's Boys function (MD_Rfunction.hpp:2185-2206: large-T form above
//     T = 20, series stopped at a term < 1e-12, downward recursion), which keeps H on the reference's;
//   * component factors 1 / sqrt(df(lx) df(ly) df(lz)) with the reference's table df = 1, 1, 3, 45, 4725
//     (AuxFunctions.hpp:48-63).
// Work decomposition: one thread per (packed matrix element, geometry).  Element (i, j), j <= i, comes
// from one shell pair and one component pair; the thread loops over the primitive pairs and the nuclei.
// The per-geometry cost is O(N^2 K^2 N_atoms) with everything in registers (L <= 2 * LM).
#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/unomol_gb300.h"

namespace {

struct OneItem {
    int sa, sb, ca, cb;
};

struct OneArgs {
    const OneItem* items;
    int nitems;
    const int *sl, *snp, *sc, *sp0;
    const long long* kpk;       // packed index of every item
    const double *alpha, *coef;
    const double* centers;      // [ngeom][ncen][3]
    const double* charges;      // [ncen]
    int ncen;
    long long no2;
    double *S, *T, *H;          // [ngeom][no2]
};

__device__ __forceinline__ void cart_of(int l, int c, int& x, int& y, int& z) {
    // lx descending, then ly descending (AuxFunctions.hpp:35-43)
    int k = 0;
    for (int a = l; a >= 0; --a)
        for (int b = l - a; b >= 0; --b) {
            if (k == c) {
                x = a, y = b, z = l - a - b;
                return;
            }
            ++k;
        }
    x = y = z = 0;
}

__device__ __forceinline__ double dfact_ref(int l) {
    return l <= 1 ? 1.0 : l == 2 ? 3.0 : l == 3 ? 45.0 : 4725.0;
}

// the reference's Boys function (MD_Rfunction.hpp:2185-2206)
__device__ void boys_ref(int mmax, double T, double* F) {
    if (T > 20.0) {
        F[0] = 0.88622692545275801365 / sqrt(T);
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
    const double e = exp(-T);
    F[mmax] = sum * e;
    for (int m = mmax - 1; m >= 0; --m) F[m] = (F[m + 1] * 2.0 * T + e) / (m + m + 1.0);
}

// 1D overlap table s[i][j], i <= ni, j <= nj (Obara-Saika)
template <int LM>
__device__ __forceinline__ void os_table(double s[LM + 2][LM + 2], int ni, int nj, double s00, double PA, double PB,
                                         double o2p) {
    s[0][0] = s00;
    for (int i = 0; i <= ni; ++i)
        for (int j = 0; j <= nj; ++j) {
            if (i == 0 && j == 0) continue;
            double v;
            if (i > 0) {
                v = PA * s[i - 1][j];
                if (i > 1) v += (i - 1) * s[i - 2][j] * o2p;
                if (j > 0) v += j * s[i - 1][j - 1] * o2p;
            } else {
                v = PB * s[i][j - 1];
                if (j > 1) v += (j - 1) * s[i][j - 2] * o2p;
            }
            s[i][j] = v;
        }
}

template <int LM>
__device__ __forceinline__ double kin1(const double s[LM + 2][LM + 2], int i, int j, double a, double b) {
    double v = 4.0 * a * b * s[i + 1][j + 1];
    if (i > 0 && j > 0) v += i * j * s[i - 1][j - 1];
    if (j > 0) v -= 2.0 * a * j * s[i + 1][j - 1];
    if (i > 0) v -= 2.0 * b * i * s[i - 1][j + 1];
    return 0.5 * v;
}

// Hermite coefficients E^{i0 j0}_t, t <= i0 + j0, of one axis (K_ab = 1)
template <int LM>
__device__ __forceinline__ void hermite1(int i0, int j0, double PA, double PB, double o, double* Et) {
    double E[LM + 1][LM + 1][2 * LM + 2];
    for (int i = 0; i <= i0; ++i)
        for (int j = 0; j <= j0; ++j)
            for (int t = 0; t <= i + j + 1; ++t) E[i][j][t] = 0.0;
    E[0][0][0] = 1.0;
    for (int i = 0; i <= i0; ++i)
        for (int j = 0; j <= j0; ++j) {
            if (i == 0 && j == 0) continue;
            for (int t = 0; t <= i + j; ++t) {
                double v;
                if (i > 0) {
                    v = PA * E[i - 1][j][t];
                    if (t > 0) v += o * E[i - 1][j][t - 1];
                    if (t + 1 <= i + j - 1) v += (t + 1) * E[i - 1][j][t + 1];
                } else {
                    v = PB * E[i][j - 1][t];
                    if (t > 0) v += o * E[i][j - 1][t - 1];
                    if (t + 1 <= i + j - 1) v += (t + 1) * E[i][j - 1][t + 1];
                }
                E[i][j][t] = v;
            }
        }
    for (int t = 0; t <= i0 + j0; ++t) Et[t] = E[i0][j0][t];
}

template <int LM>
__global__ void __launch_bounds__(128) k_one_electron(const OneArgs a) {
    constexpr int L2 = 2 * LM;
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= a.nitems) return;
    const long long g = blockIdx.y;
    const OneItem w = a.items[it];
    const double* cen = a.centers + g * 3LL * a.ncen;
    const int la = a.sl[w.sa], lb = a.sl[w.sb];
    int ax, ay, az, bx, by, bz;
    cart_of(la, w.ca, ax, ay, az);
    cart_of(lb, w.cb, bx, by, bz);
    const double* A = cen + 3 * a.sc[w.sa];
    const double* B = cen + 3 * a.sc[w.sb];
    const double AB2 = (A[0] - B[0]) * (A[0] - B[0]) + (A[1] - B[1]) * (A[1] - B[1]) + (A[2] - B[2]) * (A[2] - B[2]);
    const int L = la + lb;
    double sv = 0.0, tv = 0.0, vv = 0.0;
    for (int ia = 0; ia < a.snp[w.sa]; ++ia)
        for (int ib = 0; ib < a.snp[w.sb]; ++ib) {
            const double al = a.alpha[a.sp0[w.sa] + ia], be = a.alpha[a.sp0[w.sb] + ib];
            const double cab = a.coef[a.sp0[w.sa] + ia] * a.coef[a.sp0[w.sb] + ib];
            const double p = al + be, mu = al * be / p, o2p = 0.5 / p;
            double P[3], PA[3], PB[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                P[k] = (al * A[k] + be * B[k]) / p;
                PA[k] = P[k] - A[k];
                PB[k] = P[k] - B[k];
            }
            double sx[LM + 2][LM + 2], sy[LM + 2][LM + 2], sz[LM + 2][LM + 2];
            const double rp = sqrt(3.14159265358979323846 / p);
            os_table<LM>(sx, ax + 1, bx + 1, rp * exp(-mu * (A[0] - B[0]) * (A[0] - B[0])), PA[0], PB[0], o2p);
            os_table<LM>(sy, ay + 1, by + 1, rp * exp(-mu * (A[1] - B[1]) * (A[1] - B[1])), PA[1], PB[1], o2p);
            os_table<LM>(sz, az + 1, bz + 1, rp * exp(-mu * (A[2] - B[2]) * (A[2] - B[2])), PA[2], PB[2], o2p);
            const double Sx = sx[ax][bx], Sy = sy[ay][by], Sz = sz[az][bz];
            sv += cab * Sx * Sy * Sz;
            tv += cab * (kin1<LM>(sx, ax, bx, al, be) * Sy * Sz + Sx * kin1<LM>(sy, ay, by, al, be) * Sz +
                         Sx * Sy * kin1<LM>(sz, az, bz, al, be));
            double Ex[L2 + 1], Ey[L2 + 1], Ez[L2 + 1];
            hermite1<LM>(ax, bx, PA[0], PB[0], o2p, Ex);
            hermite1<LM>(ay, by, PA[1], PB[1], o2p, Ey);
            hermite1<LM>(az, bz, PA[2], PB[2], o2p, Ez);
            const int tx = ax + bx, ty = ay + by, tz = az + bz;
            double vsum = 0.0;
            for (int c = 0; c < a.ncen; ++c) {
                const double Z = a.charges[c];
                if (Z == 0.0) continue;
                const double PC[3] = {P[0] - cen[3 * c], P[1] - cen[3 * c + 1], P[2] - cen[3 * c + 2]};
                const double Tt = p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]);
                double F[L2 + 1];
                boys_ref(L, Tt, F);
                // R^n_tuv, n from L down to 0; level n keeps t <= tx, u <= ty, v <= tz, t + u + v <= L - n
                double R[2][L2 + 1][L2 + 1][L2 + 1];
                int cur = 0;
                double m2p = 1.0;
                for (int n = 0; n < L; ++n) m2p *= -2.0 * p;
                R[cur][0][0][0] = m2p * F[L];
                for (int n = L - 1; n >= 0; --n) {
                    const int nx = cur ^ 1;
                    m2p /= -2.0 * p;
                    for (int t = 0; t <= tx; ++t)
                        for (int u = 0; u <= ty; ++u)
                            for (int v = 0; v <= tz; ++v) {
                                if (t + u + v > L - n) continue;
                                double r;
                                if (t + u + v == 0) {
                                    r = m2p * F[n];
                                } else if (t > 0) {
                                    r = PC[0] * R[cur][t - 1][u][v];
                                    if (t > 1) r += (t - 1) * R[cur][t - 2][u][v];
                                } else if (u > 0) {
                                    r = PC[1] * R[cur][t][u - 1][v];
                                    if (u > 1) r += (u - 1) * R[cur][t][u - 2][v];
                                } else {
                                    r = PC[2] * R[cur][t][u][v - 1];
                                    if (v > 1) r += (v - 1) * R[cur][t][u][v - 2];
                                }
                                R[nx][t][u][v] = r;
                            }
                    cur = nx;
                }
                double vc = 0.0;
                for (int t = 0; t <= tx; ++t)
                    for (int u = 0; u <= ty; ++u)
                        for (int v = 0; v <= tz; ++v) vc += Ex[t] * Ey[u] * Ez[v] * R[cur][t][u][v];
                vsum -= Z * vc;
            }
            vv += cab * 2.0 * 3.14159265358979323846 / p * exp(-mu * AB2) * vsum;
        }
    const double nrm = 1.0 / sqrt(dfact_ref(ax) * dfact_ref(ay) * dfact_ref(az) * dfact_ref(bx) * dfact_ref(by) *
                                  dfact_ref(bz));
    const long long o = g * a.no2 + a.kpk[it];
    a.S[o] = sv * nrm;
    if (a.T) a.T[o] = tv * nrm;
    a.H[o] = (tv + vv) * nrm;
}

// Dipole and quadrupole integrals about the origin (the data of MomentInts, Moments.cpp:5-181; the
// reference expands them with McMurchie-Davidson D functions, here with the same Obara-Saika tables,
// x = (x - A_x) + A_x):  <a|x|b> = S(a+1, b) + A_x S(a, b),  <a|x^2|b> = S(a+2, b) + 2 A_x S(a+1, b) + A_x^2 S(a, b).
// Output M[k][packed] for k = dx, dy, dz, qxx, qxy, qxz, qyy, qyz, qzz (RMOM.DAT order, unweighted).
template <int LM>
__global__ void __launch_bounds__(128) k_moments(const OneArgs a, double* __restrict__ M) {
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= a.nitems) return;
    const OneItem w = a.items[it];
    const double* cen = a.centers;
    const int la = a.sl[w.sa], lb = a.sl[w.sb];
    int lx[2][3];
    cart_of(la, w.ca, lx[0][0], lx[0][1], lx[0][2]);
    cart_of(lb, w.cb, lx[1][0], lx[1][1], lx[1][2]);
    const double* A = cen + 3 * a.sc[w.sa];
    const double* B = cen + 3 * a.sc[w.sb];
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int ia = 0; ia < a.snp[w.sa]; ++ia)
        for (int ib = 0; ib < a.snp[w.sb]; ++ib) {
            const double al = a.alpha[a.sp0[w.sa] + ia], be = a.alpha[a.sp0[w.sb] + ib];
            const double cab = a.coef[a.sp0[w.sa] + ia] * a.coef[a.sp0[w.sb] + ib];
            const double p = al + be, mu = al * be / p, o2p = 0.5 / p;
            const double rp = sqrt(3.14159265358979323846 / p);
            double m0[3], m1[3], m2[3];  // per axis: <a|1|b>, <a|x|b>, <a|x^2|b>
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double Pk = (al * A[k] + be * B[k]) / p;
                double t[LM + 3][LM + 2];
                const int i0 = lx[0][k], j0 = lx[1][k];
                t[0][0] = rp * exp(-mu * (A[k] - B[k]) * (A[k] - B[k]));
                for (int i = 0; i <= i0 + 2; ++i)
                    for (int j = 0; j <= j0; ++j) {
                        if (i == 0 && j == 0) continue;
                        double v;
                        if (i > 0) {
                            v = (Pk - A[k]) * t[i - 1][j];
                            if (i > 1) v += (i - 1) * t[i - 2][j] * o2p;
                            if (j > 0) v += j * t[i - 1][j - 1] * o2p;
                        } else {
                            v = (Pk - B[k]) * t[i][j - 1];
                            if (j > 1) v += (j - 1) * t[i][j - 2] * o2p;
                        }
                        t[i][j] = v;
                    }
                m0[k] = t[i0][j0];
                m1[k] = t[i0 + 1][j0] + A[k] * t[i0][j0];
                m2[k] = t[i0 + 2][j0] + 2.0 * A[k] * t[i0 + 1][j0] + A[k] * A[k] * t[i0][j0];
            }
            acc[0] += cab * m1[0] * m0[1] * m0[2];
            acc[1] += cab * m0[0] * m1[1] * m0[2];
            acc[2] += cab * m0[0] * m0[1] * m1[2];
            acc[3] += cab * m2[0] * m0[1] * m0[2];
            acc[4] += cab * m1[0] * m1[1] * m0[2];
            acc[5] += cab * m1[0] * m0[1] * m1[2];
            acc[6] += cab * m0[0] * m2[1] * m0[2];
            acc[7] += cab * m0[0] * m1[1] * m1[2];
            acc[8] += cab * m0[0] * m0[1] * m2[2];
        }
    const double nrm = 1.0 / sqrt(dfact_ref(lx[0][0]) * dfact_ref(lx[0][1]) * dfact_ref(lx[0][2]) * dfact_ref(lx[1][0]) *
                                  dfact_ref(lx[1][1]) * dfact_ref(lx[1][2]));
#pragma unroll
    for (int k = 0; k < 9; ++k) M[k * a.no2 + a.kpk[it]] = acc[k] * nrm;
}

thread_local std::string g_one_err;

template <class T>
struct Dv {
    T* p = nullptr;
    ~Dv() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)); }
};

// host part of both entry points: M != NULL computes the moment integrals (one geometry) instead of S, T, H
int one_electron_impl(const UnomolBasisDesc* b, const double* charges, int ngeom, const double* centers, double* S,
                      double* T, double* H, double* M) {
    const int ns = b->nshell, nc = b->ncen, n = b->norb;
    int lmax = 0, np = 0;
    std::vector<int> p0(ns);
    for (int s = 0; s < ns; ++s) {
        if (b->shell_l[s] < 0 || b->shell_l[s] > 4 || b->shell_nprim[s] <= 0 || b->shell_center[s] < 0 ||
            b->shell_center[s] >= nc) {
            g_one_err = "one-electron: bad shell";
            return UNOMOL_EINVAL;
        }
        lmax = std::max(lmax, b->shell_l[s]);
        p0[s] = np;
        np += b->shell_nprim[s];
    }
    const long long no2 = (long long)n * (n + 1) / 2;
    std::vector<OneItem> items;
    std::vector<long long> kpk;
    items.reserve((size_t)no2);
    for (int sa = 0; sa < ns; ++sa)
        for (int sb = 0; sb <= sa; ++sb) {
            const int na = (b->shell_l[sa] + 1) * (b->shell_l[sa] + 2) / 2, nb = (b->shell_l[sb] + 1) * (b->shell_l[sb] + 2) / 2;
            for (int ca = 0; ca < na; ++ca)
                for (int cb = 0; cb < nb; ++cb) {
                    const long long i = b->shell_offset[sa] + ca, j = b->shell_offset[sb] + cb;
                    if (j > i) continue;
                    if (i >= n) {
                        g_one_err = "one-electron: shell offsets beyond norb";
                        return UNOMOL_EINVAL;
                    }
                    items.push_back({sa, sb, ca, cb});
                    kpk.push_back(i * (i + 1) / 2 + j);
                }
        }
    if ((long long)items.size() != no2) {
        g_one_err = "one-electron: the shells do not cover every basis function once";
        return UNOMOL_EINVAL;
    }
    Dv<OneItem> d_items;
    Dv<long long> d_kpk;
    Dv<int> d_sl, d_snp, d_sc, d_sp0;
    Dv<double> d_alpha, d_coef, d_cen, d_chg, d_S, d_T, d_H;
    const size_t out = (size_t)ngeom * (size_t)no2;
    cudaError_t e = cudaSuccess;
    auto ck = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    ck(d_items.alloc(items.size()));
    ck(d_kpk.alloc(kpk.size()));
    ck(d_sl.alloc(ns)), ck(d_snp.alloc(ns)), ck(d_sc.alloc(ns)), ck(d_sp0.alloc(ns));
    ck(d_alpha.alloc(np)), ck(d_coef.alloc(np));
    ck(d_cen.alloc((size_t)ngeom * nc * 3)), ck(d_chg.alloc(nc));
    if (M) ck(d_S.alloc((size_t)9 * no2));
    else ck(d_S.alloc(out)), ck(d_H.alloc(out));
    if (T && !M) ck(d_T.alloc(out));
    if (e != cudaSuccess) {
        g_one_err = std::string("one-electron: ") + cudaGetErrorString(e);
        return UNOMOL_ENOMEM;
    }
    ck(cudaMemcpy(d_items.p, items.data(), items.size() * sizeof(OneItem), cudaMemcpyHostToDevice));
    ck(cudaMemcpy(d_kpk.p, kpk.data(), kpk.size() * sizeof(long long), cudaMemcpyHostToDevice));
    ck(cudaMemcpy(d_sl.p, b->shell_l, ns * sizeof(int), cudaMemcpyHostToDevice));
    ck(cudaMemcpy(d_snp.p, b->shell_nprim, ns * sizeof(int), cudaMemcpyHostToDevice));
    ck(cudaMemcpy(d_sc.p, b->shell_center, ns * sizeof(int), cudaMemcpyHostToDevice));
    ck(cudaMemcpy(d_sp0.p, p0.data(), ns * sizeof(int), cudaMemcpyHostToDevice));
    ck(cudaMemcpy(d_alpha.p, b->alpha, np * sizeof(double), cudaMemcpyHostToDevice));
    ck(cudaMemcpy(d_coef.p, b->coef, np * sizeof(double), cudaMemcpyHostToDevice));
    ck(cudaMemcpy(d_cen.p, centers ? centers : b->centers, (size_t)ngeom * nc * 3 * sizeof(double), cudaMemcpyHostToDevice));
    if (charges) ck(cudaMemcpy(d_chg.p, charges, nc * sizeof(double), cudaMemcpyHostToDevice));
    OneArgs a{};
    a.items = d_items.p, a.nitems = (int)items.size(), a.sl = d_sl.p, a.snp = d_snp.p, a.sc = d_sc.p, a.sp0 = d_sp0.p;
    a.kpk = d_kpk.p, a.alpha = d_alpha.p, a.coef = d_coef.p, a.centers = d_cen.p, a.charges = d_chg.p, a.ncen = nc;
    a.no2 = no2, a.S = d_S.p, a.T = T ? d_T.p : nullptr, a.H = d_H.p;
    const dim3 grid((unsigned)((items.size() + 127) / 128), (unsigned)ngeom);
    if (e == cudaSuccess && M) {
        if (lmax <= 1) k_moments<1><<<grid, 128>>>(a, d_S.p);
        else if (lmax == 2) k_moments<2><<<grid, 128>>>(a, d_S.p);
        else k_moments<4><<<grid, 128>>>(a, d_S.p);
        ck(cudaGetLastError());
        ck(cudaMemcpy(M, d_S.p, (size_t)9 * no2 * sizeof(double), cudaMemcpyDeviceToHost));
    } else if (e == cudaSuccess) {
        if (lmax <= 1) k_one_electron<1><<<grid, 128>>>(a);
        else if (lmax == 2) k_one_electron<2><<<grid, 128>>>(a);
        else k_one_electron<4><<<grid, 128>>>(a);
        ck(cudaGetLastError());
        ck(cudaMemcpy(S, d_S.p, out * sizeof(double), cudaMemcpyDeviceToHost));
        ck(cudaMemcpy(H, d_H.p, out * sizeof(double), cudaMemcpyDeviceToHost));
        if (T) ck(cudaMemcpy(T, d_T.p, out * sizeof(double), cudaMemcpyDeviceToHost));
    }
    if (e != cudaSuccess) {
        g_one_err = std::string("one-electron: ") + cudaGetErrorString(e);
        return UNOMOL_ECUDA;
    }
    return UNOMOL_OK;
}

}  // namespace

extern "C" int unomol_gpu_one_electron(const UnomolBasisDesc* b, const double* charges, int ngeom, const double* centers,
                                       double* S, double* T, double* H) {
    if (!b || !charges || !S || !H || ngeom <= 0 || (!centers && ngeom != 1)) return UNOMOL_EINVAL;
    return one_electron_impl(b, charges, ngeom, centers, S, T, H, nullptr);
}

extern "C" int unomol_gpu_moment_ints(const UnomolBasisDesc* b, double* M) {
    if (!b || !M) return UNOMOL_EINVAL;
    return one_electron_impl(b, nullptr, 1, nullptr, nullptr, nullptr, nullptr, M);
}

extern "C" const char* unomol_gpu_one_electron_last_error(void) { return g_one_err.c_str(); }
