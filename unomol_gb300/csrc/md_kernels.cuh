// McMurchie-Davidson two-electron integrals (FP64): the reference's path for quartets with
// la+lb+lc+ld > 8 (f and g shells; TwoElectronInts.cpp:658-666) and, in the MD mode, for every
// quartet (the reference's -DUNOMOL_MD_INTS build).
//
// One thread per (shell quartet, function quartet): high angular momentum classes have up to 15^4
// function quartets, too many to hold per thread, so each thread contracts one function quartet over
// the primitive quartets and scatters its J/K contributions.  Per primitive quartet:
//   (ab|cd) += sr sum_{tuv} E^{ab}_t E^{ab}_u E^{ab}_v sum_{t'u'v'} (-1)^{t'+u'+v'} E^{cd}_{t'} E^{cd}_{u'}
//              E^{cd}_{v'} R_{t+t', u+u', v+v'}
// with the Hermite expansion coefficients E (MD_Dfunction.hpp:39-72) per Cartesian axis for the
// thread's components only, and R_{tuv} (MD_Rfunction.hpp:2208-2319) by the downward recursion over
// the auxiliary index inside the box t <= Tx, u <= Ty, v <= Tz of this function quartet, keeping two
// levels.  The Boys function follows the reference's MD_Rfunction::Fgamma (MD_Rfunction.hpp:2185-2206):
// large-T form above T = 20, series for F_L stopped at a term below 1e-12, downward recursion --
// so that the integrals carry the same approximation as the reference's.  The MD path has no
// primitive prefactor cut (TwoElectronInts.cpp:269-418).
#pragma once
#include "eri_common.cuh"
#include "fock_kernels.cuh"

namespace ugb {

constexpr int MD_LMAX = 4;
constexpr int MD_LT = 4 * MD_LMAX;  // largest total angular momentum

__device__ __forceinline__ void md_boys_reference(int L, double T, double* F) {
    if (T > 20.0) {
        F[0] = 0.88622692545275801365 / sqrt(T);
        for (int m = 1; m <= L; ++m) F[m] = F[m - 1] * (m - 0.5) / T;
        return;
    }
    const double mph = L + 0.5;
    double term = 0.5 / mph, sum = term;
    for (int k = 1; k <= 200; ++k) {
        term *= T / (mph + k);
        sum += term;
        if (term < 1.e-12) break;
    }
    const double e = exp(-T);
    F[L] = sum * e;
    for (int m = L - 1; m >= 0; --m) F[m] = (F[m + 1] * 2.0 * T + e) / (m + m + 1.0);
}

// Hermite coefficients E^{i j}_t, t = 0..i+j, for one axis (abi = 1/(2p), PA = P - A, PB = P - B)
__device__ __forceinline__ void md_hermite(int li, int lj, double abi, double PA, double PB, double* E) {
    double T[(MD_LMAX + 1) * (MD_LMAX + 1) * (2 * MD_LMAX + 1)];
    auto at = [&](int i, int j, int t) -> double& { return T[(i * (MD_LMAX + 1) + j) * (2 * MD_LMAX + 1) + t]; };
    at(0, 0, 0) = 1.0;
    for (int j = 1; j <= lj; ++j)
        for (int t = 0; t <= j; ++t) {
            double v = PB * (t <= j - 1 ? at(0, j - 1, t) : 0.0);
            if (t > 0) v += abi * at(0, j - 1, t - 1);
            if (t + 1 <= j - 1) v += (t + 1) * at(0, j - 1, t + 1);
            at(0, j, t) = v;
        }
    for (int i = 1; i <= li; ++i)
        for (int j = 0; j <= lj; ++j)
            for (int t = 0; t <= i + j; ++t) {
                double v = PA * (t <= i - 1 + j ? at(i - 1, j, t) : 0.0);
                if (t > 0) v += abi * at(i - 1, j, t - 1);
                if (t + 1 <= i - 1 + j) v += (t + 1) * at(i - 1, j, t + 1);
                at(i, j, t) = v;
            }
    for (int t = 0; t <= li + lj; ++t) E[t] = at(li, lj, t);
}

// One contracted function quartet by McMurchie-Davidson (components c1..c4 of shells with angular
// momenta la..ld; the bra pair's A is its first shell, B = A - AB), without the component
// normalisation factors.
__device__ double md_function_quartet(const ShellPair& bra, const ShellPair& ket, const PrimPair* __restrict__ prims,
                                      int la, int lb, int lc, int ld, int c1, int c2, int c3, int c4) {
    int va[3], vb[3], vc[3], vd[3];
    va[0] = cart_lx(la, c1); va[1] = cart_ly(la, c1); va[2] = cart_lz(la, c1);
    vb[0] = cart_lx(lb, c2); vb[1] = cart_ly(lb, c2); vb[2] = cart_lz(lb, c2);
    vc[0] = cart_lx(lc, c3); vc[1] = cart_ly(lc, c3); vc[2] = cart_lz(lc, c3);
    vd[0] = cart_lx(ld, c4); vd[1] = cart_ly(ld, c4); vd[2] = cart_lz(ld, c4);
    int T12[3], T34[3], Tb[3];
    for (int k = 0; k < 3; ++k) {
        T12[k] = va[k] + vb[k];
        T34[k] = vc[k] + vd[k];
        Tb[k] = T12[k] + T34[k];
    }
    const int L = la + lb + lc + ld;
    double Rn[2][(MD_LT / 3 + 2) * (MD_LT / 3 + 2) * (MD_LT / 3 + 2) + 64];  // two levels of the box
    auto bidx = [&](int t, int u, int v) { return (t * (Tb[1] + 1) + u) * (Tb[2] + 1) + v; };
    double sum = 0.0;
    const PrimPair* pb = prims + bra.prim_begin;
    const PrimPair* pk = prims + ket.prim_begin;
    for (int i = 0; i < bra.nprim; ++i) {
        const double p = pb[i * bra.prim_stride].p;
        double Eab[3][2 * MD_LMAX + 1];
        for (int k = 0; k < 3; ++k) md_hermite(va[k], vb[k], 0.5 * pb[i * bra.prim_stride].rp, pb[i * bra.prim_stride].PA[k], pb[i * bra.prim_stride].PA[k] + bra.AB[k], Eab[k]);
        for (int j = 0; j < ket.nprim; ++j) {
            const double q = pk[j * ket.prim_stride].p;
            double Ecd[3][2 * MD_LMAX + 1];
            for (int k = 0; k < 3; ++k) md_hermite(vc[k], vd[k], 0.5 * pk[j * ket.prim_stride].rp, pk[j * ket.prim_stride].PA[k], pk[j * ket.prim_stride].PA[k] + ket.AB[k], Ecd[k]);
            const double sr = SRTERM * pb[i * bra.prim_stride].E * pk[j * ket.prim_stride].E * pb[i * bra.prim_stride].cc * pk[j * ket.prim_stride].cc / sqrt(p + q);
            const double rho = p * q / (p + q);
            const double PQ[3] = {pb[i * bra.prim_stride].P[0] - pk[j * ket.prim_stride].P[0], pb[i * bra.prim_stride].P[1] - pk[j * ket.prim_stride].P[1], pb[i * bra.prim_stride].P[2] - pk[j * ket.prim_stride].P[2]};
            double F[MD_LT + 1];
            md_boys_reference(L, rho * (PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2]), F);
            // R^{(n)}_{tuv} for n = L .. 0 inside the box, t + u + v <= L - n
            int cur = 0;
            double m2r = 1.0;
            for (int n = 0; n < L; ++n) m2r *= -2.0 * rho;
            for (int n = L; n >= 0; --n) {
                double* Rc = Rn[cur];
                const double* Rp = Rn[cur ^ 1];
                for (int t = 0; t <= Tb[0]; ++t)
                    for (int u = 0; u <= Tb[1]; ++u)
                        for (int v = 0; v <= Tb[2]; ++v) {
                            if (t + u + v > L - n) continue;
                            double r;
                            if (t + u + v == 0) r = m2r * F[n];
                            else if (t > 0) r = PQ[0] * Rp[bidx(t - 1, u, v)] + (t > 1 ? (t - 1) * Rp[bidx(t - 2, u, v)] : 0.0);
                            else if (u > 0) r = PQ[1] * Rp[bidx(t, u - 1, v)] + (u > 1 ? (u - 1) * Rp[bidx(t, u - 2, v)] : 0.0);
                            else r = PQ[2] * Rp[bidx(t, u, v - 1)] + (v > 1 ? (v - 1) * Rp[bidx(t, u, v - 2)] : 0.0);
                            Rc[bidx(t, u, v)] = r;
                        }
                if (n > 0) m2r /= -2.0 * rho;
                cur ^= 1;
            }
            const double* R0 = Rn[cur ^ 1];
            double acc = 0.0;
            for (int t = 0; t <= T12[0]; ++t)
                for (int u = 0; u <= T12[1]; ++u)
                    for (int v = 0; v <= T12[2]; ++v) {
                        const double e12 = Eab[0][t] * Eab[1][u] * Eab[2][v];
                        double s = 0.0;
                        for (int t2 = 0; t2 <= T34[0]; ++t2)
                            for (int u2 = 0; u2 <= T34[1]; ++u2)
                                for (int v2 = 0; v2 <= T34[2]; ++v2) {
                                    const double e34 = Ecd[0][t2] * Ecd[1][u2] * Ecd[2][v2];
                                    const double sg = ((t2 + u2 + v2) & 1) ? -1.0 : 1.0;
                                    s += sg * e34 * R0[bidx(t + t2, u + u2, v + v2)];
                                }
                        acc += e12 * s;
                    }
            sum += sr * acc;
        }
    }
    return sum;
}

// Fock kernel of one class by MD: g = (quartet work item) * NF + function quartet.
template <bool UHF>
__global__ void __launch_bounds__(128) fock_jk_md(const FockArgs A, const NormTable nt, int la, int lb, int lc, int ld,
                                                  long long nthreads) {
    const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
    const long long NF = (long long)NA * NB * NC * ND;
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < nthreads; g += (long long)gridDim.x * blockDim.x) {
        const long long w = g / NF;
        const int f = (int)(g % NF);
        int bi, ki;
        if (!(A.mode == 0 ? decode_work(A, w, bi, ki) : decode_work_dyn(A, w, bi, ki))) continue;
        const ShellPair bra = A.pairs[bi];
        const ShellPair ket = A.pairs[ki];
        if (A.mode != 0 && quartet_bound(A, bra, ket) < A.skip_cut32) continue;
        const int id = f % ND, ic = (f / ND) % NC, ib = (f / (ND * NC)) % NB, ia = f / (ND * NC * NB);
        double v = md_function_quartet(bra, ket, A.prims, la, lb, lc, ld, ia, ib, ic, id);
        v *= nt.v[la][ia] * nt.v[lb][ib] * nt.v[lc][ic] * nt.v[ld][id];
        if (!above_cut(v, A.thr_int)) continue;  // TwoElectronInts.cpp:668
        double deg = 1.0;
        if (bra.same) deg *= 0.5;
        if (ket.same) deg *= 0.5;
        if (bi == ki) deg *= 0.5;
        v *= deg;
        const int N = A.nbf;
        const int a = bra.a_off + ia, b = bra.b_off + ib, c = ket.a_off + ic, d = ket.b_off + id;
        const double* Pa = A.Pa;
        const double* Pb = A.Pb;
        const double jf = UHF ? 2.0 : 4.0;
        double Pab = Pa[a * N + b], Pcd = Pa[c * N + d];
        if (UHF) {
            Pab += Pb[a * N + b];
            Pcd += Pb[c * N + d];
        }
        atomicAdd(A.Ta + a * N + b, jf * v * Pcd);
        atomicAdd(A.Ta + c * N + d, jf * v * Pab);
        atomicAdd(A.Ta + a * N + c, -v * Pa[b * N + d]);
        atomicAdd(A.Ta + a * N + d, -v * Pa[b * N + c]);
        atomicAdd(A.Ta + b * N + c, -v * Pa[a * N + d]);
        atomicAdd(A.Ta + b * N + d, -v * Pa[a * N + c]);
        if (UHF) {
            atomicAdd(A.Tb + a * N + b, jf * v * Pcd);
            atomicAdd(A.Tb + c * N + d, jf * v * Pab);
            atomicAdd(A.Tb + a * N + c, -v * Pb[b * N + d]);
            atomicAdd(A.Tb + a * N + d, -v * Pb[b * N + c]);
            atomicAdd(A.Tb + b * N + c, -v * Pb[a * N + d]);
            atomicAdd(A.Tb + b * N + d, -v * Pb[a * N + c]);
        }
    }
}

// Schwarz diagonal by MD for pairs whose (ab|ab) has la+lb > 4: one thread per (pair, component
// pair); q holds the bit pattern of max |(ab|ab)| (non-negative doubles order as integers).
__global__ void __launch_bounds__(128) schwarz_md(const ShellPair* __restrict__ pairs, const PrimPair* __restrict__ prims,
                                                  int begin, int count, const NormTable nt, unsigned long long* qbits) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const ShellPair& s0 = pairs[begin];
    const int nab = ncart(s0.la) * ncart(s0.lb);
    if (g >= (long long)count * nab) return;
    const int t = (int)(g / nab), f = (int)(g % nab);
    const ShellPair sp = pairs[begin + t];
    const int ia = f / ncart(sp.lb), ib = f % ncart(sp.lb);
    double v = md_function_quartet(sp, sp, prims, sp.la, sp.lb, sp.la, sp.lb, ia, ib, ia, ib);
    const double n = nt.v[sp.la][ia] * nt.v[sp.lb][ib];
    v = fabs(v) * n * n;
    atomicMax(qbits + begin + t, (unsigned long long)__double_as_longlong(v));
}

}  // namespace ugb
