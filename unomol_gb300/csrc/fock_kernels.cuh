// Direct J/K Fock build: one thread per unique shell quartet, templated on the angular class
// (la lb | lc ld) and on the arithmetic type (double for the plain path, float for the FP32 part
// of the mixed-precision path).  Per primitive quartet: Rys roots and weights from piecewise
// polynomials (registers), the 2D Rys recurrence and the horizontal transfer per Cartesian axis
// (registers), and the contracted integrals accumulated in registers.  After the primitive loops
// the integrals are contracted with the density and the six J/K contributions of every function
// quartet are summed in registers and scattered with FP64 atomics into a dense N x N accumulator T,
// whose symmetrisation T + T^T is the G matrix.
//
// Reference: TwoElectronInts.cpp:420-509 (calc_two_electron_ints_rys), Rys.hpp:85-212 (Recur,
// Shift, RecurKernel, ShiftKernel), TwoElectronInts.cpp:699-820 (formGMatrixKernel{,2}).
#pragma once
#include "eri_common.cuh"
#include "rys_tables.inc"

namespace ugb {

template <typename R> struct RysDeg;
template <> struct RysDeg<double> { static constexpr int value = RYS_DEG; };
template <> struct RysDeg<float> { static constexpr int value = RYS32_DEG; };
// Row length of one polynomial in the device tables: the coefficients padded to a multiple of 16
// bytes, so that a row is read with 16-byte loads (FP64: 10 doubles; FP32: 6 floats padded to 8).
template <typename R> struct RysStride;
template <> struct RysStride<double> { static constexpr int value = (RYS_DEG + 2) / 2 * 2; };
template <> struct RysStride<float> { static constexpr int value = (RYS32_DEG + 4) / 4 * 4; };
// Interval width in T of each precision's table (a power of two: T / H is exact).
template <typename R> struct RysH;
template <> struct RysH<double> { static constexpr double value = RYS_H; };
template <> struct RysH<float> { static constexpr double value = RYS32_H; };

__host__ __device__ constexpr double rys_tmax(int n) {
    return n == 1 ? RYS_TMAX_1 : n == 2 ? RYS_TMAX_2 : n == 3 ? RYS_TMAX_3 : n == 4 ? RYS_TMAX_4 : RYS_TMAX_5;
}
// Offset of the n-root block in a table of interval width h whose polynomial rows hold `stride`
// coefficients (rys_tables.inc with stride = degree + 1; the device tables with the padded strides of
// RysStride).
__host__ __device__ constexpr int rys_off(int n, int stride, double h) {
    int o = 0;
    for (int m = 1; m < n; ++m) o += int(rys_tmax(m) / h) * 2 * m * stride;
    return o;
}
// Size of a device table: polynomial blocks, then hermite x[5][5] and w[5][5].
__host__ __device__ constexpr int rys_table_len(int stride, double h) { return rys_off(RYS_NMAX + 1, stride, h) + 50; }

// one FP64 polynomial row (8 doubles, 64 bytes, 32-byte aligned) into registers with two 256-bit loads
static_assert(RysStride<double>::value == 8, "two 256-bit loads per FP64 row");
__device__ __forceinline__ void load_row(const double* __restrict__ c, double (&v)[RysStride<double>::value]) {
    asm("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];" : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3]) : "l"(c));
    asm("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];" : "=d"(v[4]), "=d"(v[5]), "=d"(v[6]), "=d"(v[7]) : "l"(c + 4));
}
// FP32 rows are 8 floats (32 bytes, 32-byte aligned): one 256-bit load, half the load instructions of
// two 16-byte loads (the FP32 kernels are bound by the L1 wavefronts of these per-lane rows)
static_assert(RysStride<float>::value == 8, "one 256-bit load per FP32 row");
__device__ __forceinline__ void load_row(const float* __restrict__ c, float (&v)[RysStride<float>::value]) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
        : "l"(c));
}

// |v| > cut (cut >= 0) compared as IEEE bit patterns: integer pipe, no FP64 compare
__device__ __forceinline__ bool above_cut(double v, double cut) {
    return (__double_as_longlong(v) & 0x7fffffffffffffffLL) > __double_as_longlong(cut);
}
__device__ __forceinline__ bool above_cut(float v, float cut) {
    return (__float_as_int(v) & 0x7fffffff) > __float_as_int(cut);
}

// FP32 -> FP64 on the integer pipe.  The FP64 pipe of this GPU runs at 1/64 of the FP32 rate and also
// executes the F2F conversions, so the FP32 kernels convert their J/K sums by moving the fields: the
// sign in place, the exponent rebiased by 1023 - 127, the 23 mantissa bits to the top of the 52.  Exact
// for every normal float; zero and subnormal floats (|f| < 1.2e-38, below every cut of the build) give
// a signed zero.  (The kernels produce no infinities or NaN from finite inputs.)
__device__ __forceinline__ double f32_to_f64(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned hi = (u & 0x80000000u) | (e ? (((e + 896u) << 20) | ((u >> 3) & 0xfffffu)) : 0u);
    const unsigned lo = e ? (u << 29) : 0u;
    return __hiloint2double((int)hi, (int)lo);
}
__device__ __forceinline__ double to_f64(double v) { return v; }
__device__ __forceinline__ double to_f64(float v) { return f32_to_f64(v); }

// J_ab flush of the FP32 kernels: the lanes of a warp mostly hold one bra pair, so their J_ab sums go
// to one element of T, and 32 FP64 atomics on one address serialise in L2.  When the whole warp is
// converged on one element, the sums are added by shuffles and one lane issues the atomic; otherwise
// every lane adds its own.  (The FP64 kernels keep plain atomics: their FP64 pipe, not L2, binds them,
// and the shuffles cost more there than they save: 13.98 -> 13.56 plain builds/s.)
template <typename R>
__device__ __forceinline__ void add_bra_sum(double* addr, R v) {
    if constexpr (sizeof(R) == 4) {
        const unsigned m = __activemask();
        const unsigned peers = __match_any_sync(m, (unsigned long long)addr);
        if (m == 0xffffffffu && peers == m) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(m, v, o);
            if ((threadIdx.x & 31) == 0) atomicAdd(addr, to_f64(v));
            return;
        }
    }
    atomicAdd(addr, to_f64(v));
}

// Taylor coefficients of F1(T) = int_0^1 t^2 e^{-T t^2} dt = sum_k (-T)^k / (k! (2k + 3))
__host__ __device__ constexpr double boys1_coef(int k) {
    double f = 1.0;
    for (int i = 2; i <= k; ++i) f *= i;
    return (k & 1 ? -1.0 : 1.0) / (f * (2 * k + 3));
}

// One-root Rys rule in FP32 without tables: weight w = F0(T) and node x = t^2 = F1(T) / F0(T), from
// the Boys functions F_m(T) = int_0^1 t^{2m} e^{-T t^2} dt.  For T >= 1, F0 = sqrt(pi / T) erf(sqrt T) / 2
// and F1 = (F0 - e^{-T}) / (2 T) (at T >= 1 the difference loses at most a factor 2); below 1, F1 from
// its Taylor series (12 terms: the first one left out is below 1e-8 of F1) and F0 = 2 T F1 + e^{-T}
// (the same relation, now a sum of two positive terms).  About 2e-7 relative, as the FP32 tables
// (1.1e-7), with no table row read per lane.
template <bool NEED_X>
__device__ __forceinline__ void rys1_f32(float T, float& x, float& w) {
    const float e = expf(-T);
    float F0, F1 = 0.f;
    if (T < 1.f) {
        F1 = float(boys1_coef(11));
#pragma unroll
        for (int k = 10; k >= 0; --k) F1 = fmaf(F1, T, float(boys1_coef(k)));
        F0 = fmaf(2.f * T, F1, e);
    } else {
        const float r = rsqrtf(T);
        F0 = 0.886226925452758f * r * erff(T * r);  // sqrt(pi) / 2 / sqrt(T) * erf(sqrt(T))
        if (NEED_X) F1 = (F0 - e) * (0.5f * r * r);
    }
    w = F0;
    if (NEED_X) x = __fdividef(F1, F0);
}

// Reference-compatible two-root regime.  For 15 < T <= 40 the reference's Rys::root2 evaluates a
// large-T form with fitted e^{-T} corrections (Rys.cpp:611-623) that departs from the exact
// quadrature by up to 3.5e-4 relative at T = 15 (below 1e-12 from T ~ 31 on); the golden energies of
// the reference carry that departure.  The same form is evaluated here when the context runs in the
// reference-compatible Rys mode, so that the drop-in reproduces the reference's G and energies.
// Constants: the Hermite limit r12, r22, w22 and pi/4 as the reference writes them (Rys.cpp:416-419)
// and the six fitted coefficients of that regime.
__device__ __forceinline__ void rys2_reference_regime(double T, double* x, double* w) {
    const double r12 = .275255128608411, r22 = 2.72474487139158, w22 = .0917517095361369;
    const double g = exp(-T);
    const double w0 = sqrt(.785398163397448 / T);
    const double u0 = (T * -.87894730749888 + 10.9243702330261) * g + r12 / (T - r12);
    const double u1 = (T * -9.28903924275977 + 81.0642367843811) * g + r22 / (T - r22);
    const double w1 = (T * 4.468573893084 - 77.9250653461045) * g + w22 * w0;
    x[0] = u0 / (1.0 + u0);  // the reference stores u = t^2 / (1 - t^2) (Rys.cpp:307-310)
    x[1] = u1 / (1.0 + u1);
    w[0] = w0 - w1;
    w[1] = w1;
}

// log2(1 / H) of the FP64 table's interval width H (a power of two)
__host__ __device__ constexpr int rys_h_shift64() {
    int sft = 0;
    for (double h = RYS_H; h < 1.0; h *= 2.0) ++sft;
    return sft;
}
static_assert(RYS_H * (1 << rys_h_shift64()) == 1.0, "the FP64 table interval is 2^-s");

// Interval index k = floor(T / H) and local coordinate y = 2 (T / H - k) - 1 in [-1, 1) of the FP64
// table, from the IEEE bits of T >= 0 with integer operations and one DFMA: T / H = 1.m x 2^E, k is the
// integer part of the shifted mantissa, 1 + frac is the double whose mantissa field is the remaining bits,
// and y = 2 (1 + frac) - 3 (exact).  Below one interval (E < 0) k = 0 and y = 2 T / H - 1.  Returns
// T < tmax (compared as bit patterns; a NaN T compares above, as before).
__device__ __forceinline__ bool rys_index64(double T, double tmax, int& k, double& y) {
    constexpr int S = rys_h_shift64();
    const long long u = __double_as_longlong(T);
    const int E = (int)((u >> 52) & 0x7ff) - 1023 + S;  // exponent of T * 2^S
    if (E < 0) {
        k = 0;
        y = fma(T, double(1 << (S + 1)), -1.0);
    } else {
        const long long M = (u & 0xfffffffffffffLL) | 0x10000000000000LL;
        const int sh = 52 - min(E, 52);
        k = (int)(M >> sh);
        const long long fb = M & ((1LL << sh) - 1);
        y = fma(2.0, __longlong_as_double(0x3ff0000000000000LL | (fb << (52 - sh))), -3.0);
    }
    return u < __double_as_longlong(tmax);
}

// Rys nodes x_r = t_r^2 and weights w_r at T (NR roots).  compat: reference-compatible two-root
// regime (FP64 only; see rys2_reference_regime).
template <int NR, typename R>
__device__ __forceinline__ void rys_roots(R T, const R* __restrict__ tab, R* x, R* w, bool compat = false) {
    constexpr int DEG = RysDeg<R>::value;
    constexpr R TMAX = R(rys_tmax(NR));
    if constexpr (NR == 1 && sizeof(R) == 4) {  // one root in FP32: closed form, no table
        rys1_f32<true>(T, x[0], w[0]);
        return;
    }
    if constexpr (NR == 2 && sizeof(R) == 8) {
        if (compat && T > R(15) && T <= R(40)) {
            rys2_reference_regime(T, x, w);
            return;
        }
    }
    int k;
    R y;
    bool in_table;
    if constexpr (sizeof(R) == 8) {
        // FP64: the interval and the local coordinate from the bits of T on the integer pipe (the FP64
        // pipe, 1/64 of the FP32 rate on this GPU, also runs compares and int/double conversions)
        in_table = rys_index64(T, TMAX, k, y);
    } else {
        in_table = T < TMAX;
        const R Ts = T * R(1.0 / RysH<R>::value);  // intervals of width H (a power of two: exact)
        k = (int)Ts;
        y = R(2) * (Ts - R(k)) - R(1);
    }
    if (in_table) {
        constexpr int ST = RysStride<R>::value;
        const R* c = tab + rys_off(NR, ST, RysH<R>::value) + k * (2 * NR * ST);
#pragma unroll
        for (int i = 0; i < NR; ++i) {
            R cx[ST], cw[ST];
            load_row(c + (2 * i) * ST, cx);
            load_row(c + (2 * i + 1) * ST, cw);
            R vx = cx[0], vw = cw[0];
#pragma unroll
            for (int d = 1; d <= DEG; ++d) {
                vx = fma(vx, y, cx[d]);
                vw = fma(vw, y, cw[d]);
            }
            x[i] = vx;
            w[i] = vw;
        }
    } else {  // large-T limit (also taken by a NaN T, which keeps the table index in range)
        const R* herm = tab + rys_table_len(RysStride<R>::value, RysH<R>::value) - 50;
        R rT = R(1) / T;
        R s = sqrt(rT);
#pragma unroll
        for (int i = 0; i < NR; ++i) {
            x[i] = __ldg(herm + (NR - 1) * 5 + i) * rT;
            w[i] = __ldg(herm + 25 + (NR - 1) * 5 + i) * s;
        }
    }
}

// Per axis: 2D Rys recurrence G[i][j] (i <= la+lb, j <= lc+ld) from G[0][0] = g00, then the
// horizontal transfer to I[a][b][c][d] (a <= la, b <= lb, c <= lc, d <= ld):
//   I(a, b+1) = I(a+1, b) + AB I(a, b), and the same on the ket with CD.
// Rys.hpp:194-212 writes the same recurrence; Rys.hpp:173-192 applies the transfer by binomial
// sums per function quartet instead.
template <int LA, int LB, int LC, int LD, typename R>
__device__ __forceinline__ void rys_axis(R g00, R C, R Cp, R B00, R B1, R B1p, R AB, R CD,
                                         R (&I)[(LA + 1) * (LB + 1) * (LC + 1) * (LD + 1)]) {
    constexpr int L12 = LA + LB, L34 = LC + LD;
    R G[L12 + 1][L34 + 1];
    G[0][0] = g00;
    if constexpr (L12 > 0) G[1][0] = C * g00;
#pragma unroll
    for (int i = 1; i < L12; ++i) G[i + 1][0] = C * G[i][0] + R(i) * B1 * G[i - 1][0];
#pragma unroll
    for (int j = 0; j < L34; ++j) {
#pragma unroll
        for (int i = 0; i <= L12; ++i) {
            R v = Cp * G[i][j];
            if (j > 0) v = fma(R(j) * B1p, G[i][j - 1], v);
            if (i > 0) v = fma(R(i) * B00, G[i - 1][j], v);
            G[i][j + 1] = v;
        }
    }
    // bra transfer: X[b][a][j], a <= L12 - b
    R X[LB + 1][L12 + 1][L34 + 1];
#pragma unroll
    for (int a = 0; a <= L12; ++a)
#pragma unroll
        for (int j = 0; j <= L34; ++j) X[0][a][j] = G[a][j];
#pragma unroll
    for (int b = 1; b <= LB; ++b)
#pragma unroll
        for (int a = 0; a <= L12 - b; ++a)
#pragma unroll
            for (int j = 0; j <= L34; ++j) X[b][a][j] = fma(AB, X[b - 1][a][j], X[b - 1][a + 1][j]);
    // ket transfer per (a, b)
#pragma unroll
    for (int a = 0; a <= LA; ++a)
#pragma unroll
        for (int b = 0; b <= LB; ++b) {
            R Y[LD + 1][L34 + 1];
#pragma unroll
            for (int c = 0; c <= L34; ++c) Y[0][c] = X[b][a][c];
#pragma unroll
            for (int d = 1; d <= LD; ++d)
#pragma unroll
                for (int c = 0; c <= L34 - d; ++c) Y[d][c] = fma(CD, Y[d - 1][c], Y[d - 1][c + 1]);
#pragma unroll
            for (int c = 0; c <= LC; ++c)
#pragma unroll
                for (int d = 0; d <= LD; ++d) I[((a * (LB + 1) + b) * (LC + 1) + c) * (LD + 1) + d] = Y[d][c];
        }
}

template <int LA, int LB, int LC, int LD>
struct QClass {
    static constexpr int L12 = LA + LB, L34 = LC + LD, NR = (L12 + L34) / 2 + 1;
    static constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    static constexpr int NF = NA * NB * NC * ND;
    static constexpr int NI = (LA + 1) * (LB + 1) * (LC + 1) * (LD + 1);
    __host__ __device__ static constexpr int iidx(int a, int b, int c, int d) {
        return ((a * (LB + 1) + b) * (LC + 1) + c) * (LD + 1) + d;
    }
};

// Contracted integrals (ab|cd) of one shell quartet, without the component normalisation factors,
// accumulated into acc[NF] (function quartet f = ((ia*NB + ib)*NC + ic)*ND + id).  With nparts > 1 only
// the primitive quartets t = part, part + nparts, ... (bra-major) are summed: the caller's threads
// split one shell quartet and add their partial sums afterwards.
template <int LA, int LB, int LC, int LD, typename R, typename PP>
__device__ __forceinline__ void shell_quartet_eri(const ShellPair& bra, const ShellPair& ket,
                                                  const PP* __restrict__ prims,
                                                  const R* __restrict__ rys, R prim_cut, float prim_cut32, bool compat,
                                                  R (&acc)[QClass<LA, LB, LC, LD>::NF], unsigned* npass = nullptr,
                                                  int part = 0, int nparts = 1) {
    using Q = QClass<LA, LB, LC, LD>;
    constexpr int NR = Q::NR;
#pragma unroll
    for (int f = 0; f < Q::NF; ++f) acc[f] = R(0);
    R ABx, ABy, ABz, CDx, CDy, CDz;
    if constexpr (sizeof(R) == 4) {  // the pairs' FP32 copies: no conversion on the FP64 pipe
        ABx = bra.ABf[0], ABy = bra.ABf[1], ABz = bra.ABf[2];
        CDx = ket.ABf[0], CDy = ket.ABf[1], CDz = ket.ABf[2];
    } else {
        ABx = bra.AB[0], ABy = bra.AB[1], ABz = bra.AB[2];
        CDx = ket.AB[0], CDy = ket.AB[1], CDz = ket.AB[2];
    }
    const PP* pb = prims + bra.prim_begin;
    const PP* pk = prims + ket.prim_begin;
    const int nb = bra.nprim, nk = ket.nprim, sb = bra.prim_stride, sk = ket.prim_stride;
    // one surviving primitive quartet: bra record bp, ket record kp, rs = 1/sqrt(p+q), and its prefactor
    // with the contraction coefficients, sr = Ecc_ab Ecc_cd rs (TwoElectronInts.cpp:472-480)
    auto primitive = [&](const PP& bp, const PP& kp, R rs, R sr) {
        const R p = bp.p, rp = bp.rp;
        const R Px = bp.P[0], Py = bp.P[1], Pz = bp.P[2];
        const R PAx = bp.PA[0], PAy = bp.PA[1], PAz = bp.PA[2];
        const R q = kp.p, rq = kp.rp;
        const R rpq = rs * rs;
        if (npass) ++*npass;
        const R QCx = kp.PA[0], QCy = kp.PA[1], QCz = kp.PA[2];
        const R PQx = Px - R(kp.P[0]), PQy = Py - R(kp.P[1]), PQz = Pz - R(kp.P[2]);
        const R T = p * q * rpq * (PQx * PQx + PQy * PQy + PQz * PQz);
        R x[NR], w[NR];
        if constexpr (LA + LB + LC + LD == 0 && sizeof(R) == 4) {
            // (ss|ss) in FP32 needs only F0(T) = sqrt(pi / T) erf(sqrt T) / 2: one branch-free form for every
            // T (T kept away from 0, where erf(x) / x is still accurate to a few ulps)
            const float Tc = fmaxf(T, 1e-30f);
            const float r = rsqrtf(Tc);
            acc[0] = fmaf(0.886226925452758f * r * erff(Tc * r), sr, acc[0]);
            return;
        }
        rys_roots<NR, R>(T, rys, x, w, compat);
        if constexpr (LA + LB + LC + LD == 0) {  // (ss|ss): the integral is the weight times the prefactor
            acc[0] = fma(w[0], sr, acc[0]);
        } else {
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                const R fff = x[r] * rpq;  // t^2 / (p + q)   (Rys.hpp:126-129)
                const R B00 = R(0.5) * fff;
                const R B1 = (R(0.5) - B00 * q) * rp;
                const R B1p = (R(0.5) - B00 * p) * rq;
                const R qf = q * fff, pf = p * fff;
                R Ix[Q::NI], Iy[Q::NI], Iz[Q::NI];
                rys_axis<LA, LB, LC, LD, R>(R(1), PAx - qf * PQx, QCx + pf * PQx, B00, B1, B1p, ABx, CDx, Ix);
                rys_axis<LA, LB, LC, LD, R>(R(1), PAy - qf * PQy, QCy + pf * PQy, B00, B1, B1p, ABy, CDy, Iy);
                rys_axis<LA, LB, LC, LD, R>(w[r] * sr, PAz - qf * PQz, QCz + pf * PQz, B00, B1, B1p, ABz, CDz, Iz);
#pragma unroll
                for (int ia = 0; ia < Q::NA; ++ia)
#pragma unroll
                    for (int ibb = 0; ibb < Q::NB; ++ibb)
#pragma unroll
                        for (int ic = 0; ic < Q::NC; ++ic)
#pragma unroll
                            for (int id = 0; id < Q::ND; ++id) {
                                const int f = ((ia * Q::NB + ibb) * Q::NC + ic) * Q::ND + id;
                                const int jx = Q::iidx(cart_lx(LA, ia), cart_lx(LB, ibb), cart_lx(LC, ic), cart_lx(LD, id));
                                const int jy = Q::iidx(cart_ly(LA, ia), cart_ly(LB, ibb), cart_ly(LC, ic), cart_ly(LD, id));
                                const int jz = Q::iidx(cart_lz(LA, ia), cart_lz(LB, ibb), cart_lz(LC, ic), cart_lz(LD, id));
                                acc[f] = fma(Ix[jx] * Iy[jy], Iz[jz], acc[f]);
                            }
            }
        }
    };
    if (nparts > 1) {
        for (int t = part; t < nb * nk; t += nparts) {
            const int ib = t / nk, ik = t - ib * nk;
            const PP bp = pb[ib * sb];
            const PP kp = pk[ik * sk];
            const R rs = rsqrt(bp.p + kp.p);
            const R sr = R(SRTERM) * bp.E * kp.E * rs;
            if (!above_cut(sr, prim_cut)) continue;  // TwoElectronInts.cpp:478-479
            primitive(bp, kp, rs, R(bp.Ecc) * R(kp.Ecc) * rs);
        }
        return;
    }
    if constexpr (sizeof(R) == 8) {
        // FP64: each lane walks its primitive quartets (bra-major, as the reference) and first looks
        // ahead for the next one past the prefactor screen (TwoElectronInts.cpp:478-479).  The screen
        // runs on float copies of p and E (within ~1e-6 of the FP64 value): quartets more than 0.1 %
        // below the cut are dropped and quartets more than 0.1 % above it kept without FP64 work; the
        // few in between take the exact FP64 test, so the surviving set is the one the FP64 test
        // gives.  The warp then evaluates one surviving quartet per lane and round, so lanes whose
        // quartets were screened out do not sit idle through another lane's FP64 work.
        const float lo32 = prim_cut32 * 0.999f, hi32 = prim_cut32 * 1.001f;
        int ib = 0, ik = 0, cb = -1;
        PP bp = pb[0];
        for (;;) {
            PP kp;
            R rs = R(0), sr = R(0);
            bool found = false;
            while (ib < nb) {
                if (ib != cb) {
                    bp = pb[ib * sb];  // whole 16-byte-aligned records: vector loads
                    cb = ib;
                }
                kp = pk[ik * sk];
                if (++ik == nk) {
                    ik = 0;
                    ++ib;
                }
                const float v32 = float(SRTERM) * bp.Ef * kp.Ef * rsqrtf(bp.pf + kp.pf);
                if (v32 < lo32) continue;
                // one reciprocal square root gives both 1/sqrt(p+q) and 1/(p+q) (the FP64 pipe of this
                // GPU is 1/64 of the FP32 one: a division and a square root cost twice as much)
                rs = rsqrt(bp.p + kp.p);
                if (v32 <= hi32 && !above_cut(R(SRTERM) * bp.E * kp.E * rs, prim_cut)) continue;
                found = true;
                break;
            }
            if (!found) break;
            primitive(bp, kp, rs, bp.Ecc * kp.Ecc * rs);
        }
    } else {
        // FP32 (bound by its loads, not by divergence): the plain nested loops, ket records outer (the
        // lanes of a warp hold different ket pairs but mostly one bra pair, whose records are then
        // broadcast loads in the inner loop)
        for (int ik = 0; ik < nk; ++ik) {
            const PP kp = pk[ik * sk];
            for (int ib = 0; ib < nb; ++ib) {
                const PP bp = pb[ib * sb];
                const R rs = rsqrt(bp.p + kp.p);
                const R sr = R(SRTERM) * bp.E * kp.E * rs;
                if (!above_cut(sr, prim_cut)) continue;  // TwoElectronInts.cpp:478-479
                primitive(bp, kp, rs, R(bp.Ecc) * R(kp.Ecc) * rs);
            }
        }
    }
}

// Decode work item g of a launch into (bra pair, ket pair).  Returns false for padding.
__device__ __forceinline__ bool decode_work(const FockArgs& A, long long g, int& bra_idx, int& ket_idx) {
    if (g >= A.nwork) return false;
    int lo = 0, hi = A.nbp - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (A.bps[mid].work_begin <= g) lo = mid; else hi = mid - 1;
    }
    const BlockPair& bp = A.bps[lo];
    long long w = g - bp.work_begin;
    if (w >= bp.work_count) return false;
    const long long* pre = A.prefix + bp.prefix_off;
    int a = 0, b = bp.bra_count - 1;  // largest i with pre[i] <= w
    while (a < b) {
        int mid = (a + b + 1) >> 1;
        if (pre[mid] <= w) a = mid; else b = mid - 1;
    }
    bra_idx = bp.bra_begin + a;
    ket_idx = bp.ket_begin + (int)(w - pre[a]);
    return true;
}

// Decode for the per-build work lists of the density-screened / mixed-precision build: this part
// (FP64: mode 1, FP32: mode 2) has dyn_count quartets in every block pair, numbered compactly over the
// launch (block pair k from dyn_begin[k], counts rounded up to 32), so that items past dyn_total end at
// once.  Bra row i's FP64 segment is ket [0, mseg_i), its FP32 segment ket [mseg_i, mseg_i + n32_i).
__device__ __forceinline__ bool decode_work_dyn(const FockArgs& A, long long g, int& bra_idx, int& ket_idx) {
    if (g >= *A.dyn_total) return false;
    int lo = 0, hi = A.nbp - 1;  // largest block pair with dyn_begin <= g (dyn_begin[0] = 0)
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (A.dyn_begin[mid] <= g) lo = mid; else hi = mid - 1;
    }
    const BlockPair& bp = A.bps[lo];
    const long long w = g - A.dyn_begin[lo];
    if (w >= A.dyn_count[lo]) return false;
    const long long* pre = A.dyn_prefix + bp.prefix_off;
    int a = 0, b = bp.bra_count - 1;
    while (a < b) {
        int mid = (a + b + 1) >> 1;
        if (pre[mid] <= w) a = mid; else b = mid - 1;
    }
    bra_idx = bp.bra_begin + a;
    int j = (int)(w - pre[a]);
    if (A.mode == 2) j += A.dyn_mseg[bp.prefix_off + a];
    ket_idx = bp.ket_begin + j;
    return true;
}

// Warp-cooperative decode (all 32 lanes must call it).  Work ranges are 32-aligned per block pair, so
// the lanes of a warp hold 32 consecutive items of one block pair: the warp finds that block pair and
// the bra row of its first item with 32-way ballot searches (each round narrows the range 32-fold, one
// load per lane), and every lane then steps forward to its own row.  The result is that of
// decode_work / decode_work_dyn (DYN) with ~3 rounds of loads instead of two serial binary searches.
// decode_warp_items: the same for warps whose lanes hold fewer items: the warp's items start at g0 (all
// of them inside one 32-aligned range) and the lane decodes item g0 + item.
template <bool DYN>
__device__ __forceinline__ bool decode_warp_items(const FockArgs& A, long long g0, int item, int& bra_idx, int& ket_idx) {
    const int lane = threadIdx.x & 31;
    if (g0 >= (DYN ? *A.dyn_total : A.nwork)) return false;  // uniform over the warp
    int lo = 0, hi = A.nbp - 1;  // largest block pair whose first item is <= g0 (block pair 0 starts at 0)
    while (lo < hi) {
        const int step = (hi - lo + 32) >> 5;
        const int idx = lo + lane * step;
        bool le = false;
        if (idx <= hi) le = (DYN ? A.dyn_begin[idx] : A.bps[idx].work_begin) <= g0;
        const unsigned m = __ballot_sync(0xffffffffu, le);
        lo += (31 - __clz(m)) * step;
        hi = min(hi, lo + step - 1);
    }
    const BlockPair& bp = A.bps[lo];
    const long long* pre = (DYN ? A.dyn_prefix : A.prefix) + bp.prefix_off;
    const long long w0 = g0 - (DYN ? A.dyn_begin[lo] : bp.work_begin);
    const long long count = DYN ? A.dyn_count[lo] : bp.work_count;
    if (w0 >= count) return false;  // the whole warp lies past this part's quartets of the block pair
    int a = 0, b = bp.bra_count - 1;  // largest row with pre[row] <= w0 (pre[0] = 0)
    while (a < b) {
        const int step = (b - a + 32) >> 5;
        const int idx = a + lane * step;
        const unsigned m = __ballot_sync(0xffffffffu, idx <= b && pre[idx] <= w0);
        a += (31 - __clz(m)) * step;
        b = min(b, a + step - 1);
    }
    const long long w = w0 + item;
    if (w >= count) return false;
    while (a + 1 < bp.bra_count && pre[a + 1] <= w) ++a;
    bra_idx = bp.bra_begin + a;
    int j = (int)(w - pre[a]);
    if (DYN && A.mode == 2) j += A.dyn_mseg[bp.prefix_off + a];
    ket_idx = bp.ket_begin + j;
    return true;
}

template <bool DYN>
__device__ __forceinline__ bool decode_work_warp(const FockArgs& A, long long g, int& bra_idx, int& ket_idx) {
    const int lane = threadIdx.x & 31;
    return decode_warp_items<DYN>(A, g - lane, lane, bra_idx, ket_idx);
}

// Density-weighted bound of one quartet: its Schwarz bound times the largest |P| of the six shell-pair
// blocks it contracts with (J: ab, cd; K: ac, ad, bc, bd).
__device__ __forceinline__ float quartet_bound(const FockArgs& A, const ShellPair& bra, const ShellPair& ket) {
    const int a = bra.ish, b = bra.jsh, c = ket.ish, d = ket.jsh;
    int n = A.nshell;
    const float* pm = A.pmax;
    if (A.mol_nshell) {  // batch: the blocks of the quartet's molecule
        n = A.mol_nshell[bra.pad];
        pm += A.mol_pmax[bra.pad];
    }
    float m = fmaxf(fmaxf(pm[a * n + b], pm[c * n + d]), fmaxf(pm[a * n + c], pm[a * n + d]));
    m = fmaxf(m, fmaxf(pm[b * n + c], pm[b * n + d]));
    return bra.qf * ket.qf * m;
}

// Density contraction of one shell quartet and scatter into T (G = T + T^T):
//   T[a][b] += 4 v' P_cd   T[c][d] += 4 v' P_ab   (2J)
//   T[a][c] -= v' P_bd  T[b][c] -= v' P_ad  T[a][d] -= v' P_bc  T[b][d] -= v' P_ac   (K)
// with v' = v / |stabiliser of the shell quartet| (1/2 for a == b, c == d, (ab) == (cd) each);
// the sum over the 8 index permutations of every function quartet of the rectangle a x b x c x d
// then counts every ordered (ij|kl) exactly once.  UHF (UHF = true): Ta collects J(Pa + Pb) - K(Pa)
// and Tb collects J(Pa + Pb) - K(Pb) in the same T + T^T form (TwoElectronInts.cpp:749-820).
struct NormTable {
    double v[LMAX + 1][15];
    float f[LMAX + 1][15];  // the same in FP32, for the FP32 kernels
};

template <int LA, int LB, int LC, int LD, bool UHF, typename R>
__device__ __forceinline__ void digest_jk(const FockArgs& A, const ShellPair& bra, const ShellPair& ket,
                                          bool same_pair, const R (&acc)[QClass<LA, LB, LC, LD>::NF],
                                          const NormTable& nt) {
    // The density contraction runs in the kernel's own type R (FP32 in the FP32 kernels, on an FP32
    // copy of P); only the partial sums reach the FP64 accumulator T.  The degeneracy factor is applied
    // to those sums, and the storage cut compares magnitudes as integers (no FP64 compare).
    using Q = QClass<LA, LB, LC, LD>;
    constexpr bool UNIT_NORMS = LA < 2 && LB < 2 && LC < 2 && LD < 2;  // all component factors are 1
    int N = A.nbf;
    long long base = 0;
    if (A.mol_nbf) {  // batch of molecules: this molecule's dense matrices
        N = A.mol_nbf[bra.pad];
        base = A.mol_base[bra.pad];
    }
    double* __restrict__ Ta = A.Ta + base;
    double* __restrict__ Tb = UHF ? A.Tb + base : nullptr;
    R deg = R(1);
    if (bra.same) deg *= R(0.5);
    if (ket.same) deg *= R(0.5);
    if (same_pair) deg *= R(0.5);
    const R* __restrict__ Pa;
    const R* __restrict__ Pb;
    if constexpr (sizeof(R) == 8) {
        Pa = reinterpret_cast<const R*>(A.Pa) + base;
        Pb = UHF ? reinterpret_cast<const R*>(A.Pb) + base : nullptr;
    } else {
        Pa = reinterpret_cast<const R*>(A.Pa32) + base;
        Pb = UHF ? reinterpret_cast<const R*>(A.Pb32) + base : nullptr;
    }
    const R jf = UHF ? R(2) : R(4);
    R thr;
    if constexpr (sizeof(R) == 4) thr = A.thr_int32;
    else thr = A.thr_int;
    R jcd[Q::NC * Q::ND];
    R kbc[Q::NB * Q::NC], kbd[Q::NB * Q::ND];
    R kbcB[UHF ? Q::NB * Q::NC : 1], kbdB[UHF ? Q::NB * Q::ND : 1];
#pragma unroll
    for (int i = 0; i < Q::NC * Q::ND; ++i) jcd[i] = R(0);
#pragma unroll
    for (int i = 0; i < Q::NB * Q::NC; ++i) { kbc[i] = R(0); if constexpr (UHF) kbcB[i] = R(0); }
#pragma unroll
    for (int i = 0; i < Q::NB * Q::ND; ++i) { kbd[i] = R(0); if constexpr (UHF) kbdB[i] = R(0); }
#pragma unroll
    for (int ia = 0; ia < Q::NA; ++ia) {
        const int a = bra.a_off + ia;
        R kac[Q::NC], kad[Q::ND], kacB[UHF ? Q::NC : 1], kadB[UHF ? Q::ND : 1];
#pragma unroll
        for (int i = 0; i < Q::NC; ++i) { kac[i] = R(0); if constexpr (UHF) kacB[i] = R(0); }
#pragma unroll
        for (int i = 0; i < Q::ND; ++i) { kad[i] = R(0); if constexpr (UHF) kadB[i] = R(0); }
#pragma unroll
        for (int ib = 0; ib < Q::NB; ++ib) {
            const int b = bra.b_off + ib;
            R Pab = __ldg(Pa + a * N + b);
            if constexpr (UHF) Pab += __ldg(Pb + a * N + b);
            R jab = R(0);
#pragma unroll
            for (int ic = 0; ic < Q::NC; ++ic) {
                const int c = ket.a_off + ic;
#pragma unroll
                for (int id = 0; id < Q::ND; ++id) {
                    const int d = ket.b_off + id;
                    const int f = ((ia * Q::NB + ib) * Q::NC + ic) * Q::ND + id;
                    R v = acc[f];
                    if constexpr (!UNIT_NORMS) {
                        if constexpr (sizeof(R) == 4) v *= nt.f[LA][ia] * nt.f[LB][ib] * nt.f[LC][ic] * nt.f[LD][id];
                        else v *= nt.v[LA][ia] * nt.v[LB][ib] * nt.v[LC][ic] * nt.v[LD][id];
                    }
                    if (!above_cut(v, thr)) continue;  // TwoElectronInts.cpp:668
                    R Pcd = __ldg(Pa + c * N + d);
                    if constexpr (UHF) Pcd += __ldg(Pb + c * N + d);
                    jab = fma(v, Pcd, jab);
                    jcd[ic * Q::ND + id] = fma(v, Pab, jcd[ic * Q::ND + id]);
                    kac[ic] = fma(v, __ldg(Pa + b * N + d), kac[ic]);
                    kad[id] = fma(v, __ldg(Pa + b * N + c), kad[id]);
                    kbc[ib * Q::NC + ic] = fma(v, __ldg(Pa + a * N + d), kbc[ib * Q::NC + ic]);
                    kbd[ib * Q::ND + id] = fma(v, __ldg(Pa + a * N + c), kbd[ib * Q::ND + id]);
                    if constexpr (UHF) {
                        kacB[ic] = fma(v, __ldg(Pb + b * N + d), kacB[ic]);
                        kadB[id] = fma(v, __ldg(Pb + b * N + c), kadB[id]);
                        kbcB[ib * Q::NC + ic] = fma(v, __ldg(Pb + a * N + d), kbcB[ib * Q::NC + ic]);
                        kbdB[ib * Q::ND + id] = fma(v, __ldg(Pb + a * N + c), kbdB[ib * Q::ND + id]);
                    }
                }
            }
            add_bra_sum<R>(Ta + a * N + b, jf * deg * jab);
            if constexpr (UHF) add_bra_sum<R>(Tb + a * N + b, jf * deg * jab);
        }
#pragma unroll
        for (int ic = 0; ic < Q::NC; ++ic) {
            const int c = ket.a_off + ic;
            atomicAdd(Ta +a * N + c, to_f64(-deg * kac[ic]));
            if constexpr (UHF) atomicAdd(Tb +a * N + c, to_f64(-deg * kacB[ic]));
        }
#pragma unroll
        for (int id = 0; id < Q::ND; ++id) {
            const int d = ket.b_off + id;
            atomicAdd(Ta +a * N + d, to_f64(-deg * kad[id]));
            if constexpr (UHF) atomicAdd(Tb +a * N + d, to_f64(-deg * kadB[id]));
        }
    }
#pragma unroll
    for (int ic = 0; ic < Q::NC; ++ic)
#pragma unroll
        for (int id = 0; id < Q::ND; ++id) {
            const int c = ket.a_off + ic, d = ket.b_off + id;
            const double j = to_f64(jf * deg * jcd[ic * Q::ND + id]);
            atomicAdd(Ta +c * N + d, j);
            if constexpr (UHF) atomicAdd(Tb +c * N + d, j);
        }
#pragma unroll
    for (int ib = 0; ib < Q::NB; ++ib) {
        const int b = bra.b_off + ib;
#pragma unroll
        for (int ic = 0; ic < Q::NC; ++ic) {
            const int c = ket.a_off + ic;
            atomicAdd(Ta +b * N + c, to_f64(-deg * kbc[ib * Q::NC + ic]));
            if constexpr (UHF) atomicAdd(Tb +b * N + c, to_f64(-deg * kbcB[ib * Q::NC + ic]));
        }
#pragma unroll
        for (int id = 0; id < Q::ND; ++id) {
            const int d = ket.b_off + id;
            atomicAdd(Ta +b * N + d, to_f64(-deg * kbd[ib * Q::ND + id]));
            if constexpr (UHF) atomicAdd(Tb +b * N + d, to_f64(-deg * kbdB[ib * Q::ND + id]));
        }
    }
}

// Optional work counter: primitive quartets past the prefactor cut, summed over the converged lanes of
// the warp and added to one of 32 slots of the launch (spread to avoid a hot address).
__device__ __forceinline__ void count_flush(const FockArgs& A, unsigned v) {
    const unsigned m = __activemask();
    const unsigned s = __reduce_add_sync(m, v);
    if ((int)(threadIdx.x & 31) == __ffs(m) - 1 && s)
        atomicAdd(A.counters + A.counter_base + (blockIdx.x & 31), (unsigned long long)s);
}

// Counting mode: quartets of this build's work lists dropped by the per-quartet density screen, per
// warp into one of 32 slots of the launch's class (the third and fourth quarters of the counter array:
// FP64 part, then FP32 part).
__device__ __forceinline__ void count_screened(const FockArgs& A) {
    const unsigned m = __activemask();
    if ((int)(threadIdx.x & 31) == __ffs(m) - 1)
        atomicAdd(A.counters + 2 * NPAIRCLASS * NPAIRCLASS * 32 + A.counter_base + (blockIdx.x & 31),
                  (unsigned long long)__popc(m));
}

// Counting mode: quartets of the FP64 part's work lists that the mixed kernel ran in FP32 (fifth quarter
// of the counter array), per warp into one of 32 slots of the launch's class.
__device__ __forceinline__ void count_demoted(const FockArgs& A) {
    const unsigned m = __activemask();
    if ((int)(threadIdx.x & 31) == __ffs(m) - 1)
        atomicAdd(A.counters + 4 * NPAIRCLASS * NPAIRCLASS * 32 + A.counter_base + (blockIdx.x & 31),
                  (unsigned long long)__popc(m));
}

// Integrals, density contraction and scatter of one shell quartet in the arithmetic type R.
template <int LA, int LB, int LC, int LD, bool UHF, typename R>
__device__ __forceinline__ void quartet_item(const FockArgs& A, const NormTable& nt, const R* __restrict__ rys,
                                             const ShellPair& bra, const ShellPair& ket, bool same_pair) {
    using Q = QClass<LA, LB, LC, LD>;
    unsigned npass = 0;
    R acc[Q::NF];
    if constexpr (sizeof(R) == 8)
        shell_quartet_eri<LA, LB, LC, LD, R, PrimPair>(bra, ket, A.prims, rys, R(A.prim_cut), A.prim_cut32, A.rys_compat != 0, acc,
                                                       A.counters ? &npass : nullptr);
    else
        shell_quartet_eri<LA, LB, LC, LD, R, PrimPair32>(bra, ket, A.prims32, rys, A.prim_cut32, A.prim_cut32, false, acc,
                                                         A.counters ? &npass : nullptr);
    digest_jk<LA, LB, LC, LD, UHF, R>(A, bra, ket, same_pair, acc, nt);
    if (A.counters) count_flush(A, npass);
}

template <int LA, int LB, int LC, int LD, bool UHF, typename R>
__device__ __forceinline__ void fock_item(const FockArgs& A, const NormTable& nt, const R* __restrict__ rys, long long g) {
    int bi, ki;
    if (!(A.mode == 0 ? decode_work_warp<false>(A, g, bi, ki) : decode_work_warp<true>(A, g, bi, ki))) return;
    const ShellPair bra = A.pairs[bi];
    const ShellPair ket = A.pairs[ki];
    if (A.mode != 0 && quartet_bound(A, bra, ket) < A.skip_cut32) {
        if (A.counters) count_screened(A);
        return;
    }
    quartet_item<LA, LB, LC, LD, UHF, R>(A, nt, rys, bra, ket, bi == ki);
}

// FP64 part of a mixed build, with the precision chosen per quartet.  The work lists put a quartet in
// the FP64 part when its Schwarz bound times the largest |P| of the whole density reaches the FP32 cut;
// here a quartet whose bound times the largest |P| of its own six blocks (the density elements it is
// contracted with) is below that cut runs in FP32 (with the FP32 part's arguments A32), under the same
// per-quartet error bound as the FP32 part's own quartets.
template <int LA, int LB, int LC, int LD, bool UHF>
__device__ __forceinline__ void fock_item_fp64_part(const FockArgs& A64, const FockArgs& A32, const NormTable& nt,
                                                    const double* __restrict__ rys64, const float* __restrict__ rys32,
                                                    long long g) {
    int bi, ki;
    if (!decode_work_warp<true>(A64, g, bi, ki)) return;
    const ShellPair bra = A64.pairs[bi];
    const ShellPair ket = A64.pairs[ki];
    const float bound = quartet_bound(A64, bra, ket);
    if (bound < A64.skip_cut32) {
        if (A64.counters) count_screened(A64);
        return;
    }
    if (bound < A64.fp32_cut32) {
        if (A64.counters) count_demoted(A64);
        quartet_item<LA, LB, LC, LD, UHF, float>(A32, nt, rys32, bra, ket, bi == ki);
    } else {
        quartet_item<LA, LB, LC, LD, UHF, double>(A64, nt, rys64, bra, ket, bi == ki);
    }
}

// One shell quartet on a group of NP lanes (mask gmask): lane `part` of the group sums the primitive
// quartets part, part + NP, ...; the group adds its partial integrals with warp shuffles and its first
// lane contracts them with the density.
template <int LA, int LB, int LC, int LD, bool UHF, typename R, int NP>
__device__ __forceinline__ void quartet_item_group(const FockArgs& A, const NormTable& nt, const R* __restrict__ rys,
                                                   const ShellPair& bra, const ShellPair& ket, bool same_pair, int part,
                                                   unsigned gmask) {
    using Q = QClass<LA, LB, LC, LD>;
    unsigned npass = 0;
    R acc[Q::NF];
    if constexpr (sizeof(R) == 8)
        shell_quartet_eri<LA, LB, LC, LD, R, PrimPair>(bra, ket, A.prims, rys, R(A.prim_cut), A.prim_cut32, A.rys_compat != 0, acc,
                                                       A.counters ? &npass : nullptr, part, NP);
    else
        shell_quartet_eri<LA, LB, LC, LD, R, PrimPair32>(bra, ket, A.prims32, rys, A.prim_cut32, A.prim_cut32, false, acc,
                                                         A.counters ? &npass : nullptr, part, NP);
#pragma unroll
    for (int o = 1; o < NP; o <<= 1)
#pragma unroll
        for (int f = 0; f < Q::NF; ++f) acc[f] += __shfl_xor_sync(gmask, acc[f], o);
    if (part == 0) digest_jk<LA, LB, LC, LD, UHF, R>(A, bra, ket, same_pair, acc, nt);
    if (A.counters) count_flush(A, npass);
}

// FP64 part of a mixed build with NP lanes per quartet: the warp holds the 32 / NP items from g0 (the FP64
// part's quartets are few and the costliest of the build, so one lane per quartet leaves most of the
// FP64 pipe's issue slots idle); precision chosen per quartet as in fock_item_fp64_part.
template <int LA, int LB, int LC, int LD, bool UHF, int NP>
__device__ __forceinline__ void fock_group_fp64_part(const FockArgs& A64, const FockArgs& A32, const NormTable& nt,
                                                     const double* __restrict__ rys64, const float* __restrict__ rys32,
                                                     long long g0) {
    const int lane = threadIdx.x & 31, sub = lane / NP, part = lane % NP;
    const unsigned gmask = ((1u << NP) - 1u) << (sub * NP);
    int bi, ki;
    if (!decode_warp_items<true>(A64, g0, sub, bi, ki)) return;  // warp-collective; uniform over a group
    const ShellPair bra = A64.pairs[bi];
    const ShellPair ket = A64.pairs[ki];
    const float bound = quartet_bound(A64, bra, ket);
    if (bound < A64.skip_cut32) {
        if (A64.counters && part == 0) count_screened(A64);
        return;
    }
    if (bound < A64.fp32_cut32) {
        if (A64.counters && part == 0) count_demoted(A64);
        quartet_item_group<LA, LB, LC, LD, UHF, float, NP>(A32, nt, rys32, bra, ket, bi == ki, part, gmask);
    } else {
        quartet_item_group<LA, LB, LC, LD, UHF, double, NP>(A64, nt, rys64, bra, ket, bi == ki, part, gmask);
    }
}

#ifndef UGB_FP64_PARTS
#define UGB_FP64_PARTS 4
#endif
// Lanes per quartet of the FP64 part of a mixed build
template <int LA, int LB, int LC, int LD>
struct Fp64Parts {
    static constexpr int value = UGB_FP64_PARTS;
};

template <int LA, int LB, int LC, int LD, bool UHF, typename R>
__global__ void __launch_bounds__(128) fock_jk_kernel(const FockArgs A, const NormTable nt, const R* __restrict__ rys) {
    fock_item<LA, LB, LC, LD, UHF, R>(A, nt, rys, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// Mixed builds: the FP64 part (A64, mode 1) and the FP32 part (A32, mode 2) of one class in one launch
// of 2 x nblk CTAs, alternating (even CTAs FP64, odd CTAs FP32).  Both parts number their quartets
// compactly from 0, so their working CTAs come first in the grid and an SM holds both kinds at once:
// warps on the FP64 pipe beside warps on the FP32 pipe and the loads.  CTAs past a part's total end at
// their first load.  The FP64 part's quartets whose own density bound is below the FP32 cut run in FP32
// (fock_item_fp64_part).
template <int LA, int LB, int LC, int LD, bool UHF>
__global__ void __launch_bounds__(128) fock_jk_mixed(const FockArgs A64, const FockArgs A32, const NormTable nt,
                                                      const double* __restrict__ rys64,
                                                      const float* __restrict__ rys32) {
    const long long g = (long long)(blockIdx.x >> 1) * blockDim.x + threadIdx.x;
    if (blockIdx.x & 1) {
        fock_item<LA, LB, LC, LD, UHF, float>(A32, nt, rys32, g);
        return;
    }
    constexpr int NP = Fp64Parts<LA, LB, LC, LD>::value;
    if constexpr (NP == 1) {
        fock_item_fp64_part<LA, LB, LC, LD, UHF>(A64, A32, nt, rys64, rys32, g);
    } else {
        // the FP64 CTAs cover 32 / NP items per warp and step over the part's total in whole warps
        const long long per_warp = 32 / NP;
        const long long nwarps = (long long)((gridDim.x + 1) >> 1) * (blockDim.x >> 5);
        const long long total = *A64.dyn_total;
        for (long long wi = (long long)(blockIdx.x >> 1) * (blockDim.x >> 5) + (threadIdx.x >> 5); wi * per_warp < total;
             wi += nwarps)
            fock_group_fp64_part<LA, LB, LC, LD, UHF, NP>(A64, A32, nt, rys64, rys32, wi * per_warp);
    }
}

// The FP64 part of a mixed build alone (NP lanes per quartet, per-quartet precision as in fock_jk_mixed),
// for the classes whose FP32 part runs as its own kernel at the FP32 code's register count: a fixed grid
// whose warps step over the part's quartets.
template <int LA, int LB, int LC, int LD, bool UHF>
__global__ void __launch_bounds__(128) fock_jk_fp64_part(const FockArgs A64, const FockArgs A32, const NormTable nt,
                                                         const double* __restrict__ rys64, const float* __restrict__ rys32) {
    constexpr int NP = Fp64Parts<LA, LB, LC, LD>::value;
    const long long per_warp = 32 / NP;
    const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
    const long long total = *A64.dyn_total;
    for (long long wi = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); wi * per_warp < total; wi += nwarps)
        fock_group_fp64_part<LA, LB, LC, LD, UHF, NP>(A64, A32, nt, rys64, rys32, wi * per_warp);
}

// Persistent form for batches of molecules: a fixed grid of CTAs (a few per SM) pulls tiles of
// blockDim consecutive work items from an atomic counter until the launch's work is done, so that
// molecules of uneven size balance across the GPU in one launch per class.  Tiles follow the work
// order (block pairs of one molecule are contiguous), which keeps a tile's warps uniform.
template <int LA, int LB, int LC, int LD, bool UHF, typename R>
__global__ void __launch_bounds__(256) fock_jk_persistent(const FockArgs A, const NormTable nt, const R* __restrict__ rys) {
    __shared__ long long tile;
    const long long end = A.mode != 0 ? *A.dyn_total : A.nwork;  // screened parts: their compact numbering
    for (;;) {
        if (threadIdx.x == 0) tile = (long long)atomicAdd(A.tile_counter, 1ull);
        __syncthreads();
        const long long g0 = tile * blockDim.x;
        __syncthreads();
        if (g0 >= end) return;
        fock_item<LA, LB, LC, LD, UHF, R>(A, nt, rys, g0 + threadIdx.x);
    }
}

// Schwarz diagonal: q[pair] = sqrt(max_{a,b} |(ab|ab)|) for every pair of one class (no primitive
// cut, so the bound is that of the exact integrals).  One warp per shell pair: the lanes split its
// primitive quartets and add their partial integrals with warp shuffles (one thread per pair would
// leave most SMs idle at these counts and serialise each warp on the FP64 pipe).
template <int LA, int LB>
__global__ void __launch_bounds__(128) schwarz_kernel(const ShellPair* __restrict__ pairs, const PrimPair* __restrict__ prims,
                                                      int begin, int count, const NormTable nt,
                                                      const double* __restrict__ rys, double* __restrict__ q_out) {
    using Q = QClass<LA, LB, LA, LB>;
    const int w = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (w >= count) return;  // whole warps: count is per warp
    const ShellPair sp = pairs[begin + w];
    double acc[Q::NF];
    shell_quartet_eri<LA, LB, LA, LB, double, PrimPair>(sp, sp, prims, rys, 0.0, 0.f, false, acc, nullptr, lane, 32);
    double m = 0.0;
#pragma unroll
    for (int ia = 0; ia < Q::NA; ++ia)
#pragma unroll
        for (int ib = 0; ib < Q::NB; ++ib) {
            const int f = ((ia * Q::NB + ib) * Q::NC + ia) * Q::ND + ib;
            double v = acc[f];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            const double n = nt.v[LA][ia] * nt.v[LB][ib];
            m = fmax(m, fabs(v) * n * n);
        }
    if (lane == 0) q_out[begin + w] = sqrt(m);
}

}  // namespace ugb

namespace ugb {

// ---------------------------------------------------------------------------------------------
// Generic path for the classes with more than 81 function quartets (d shells): the same
// arithmetic with runtime angular momenta and loops, the integrals in thread-local memory.
// ---------------------------------------------------------------------------------------------
constexpr int GEN_LMAX = LMAX;  // shells up to g, classes with la+lb+lc+ld <= 8 (the Rys domain)
constexpr int GEN_L2 = 8;       // largest la+lb (or lc+ld) of such a class
constexpr int GEN_NC = (GEN_LMAX + 1) * (GEN_LMAX + 2) / 2;
constexpr int GEN_NF = 1296;    // most function quartets of a class with la+lb+lc+ld <= 8: (dd|dd)
constexpr int GEN_NI = 81;      // most 1D transfer values (la+1)(lb+1)(lc+1)(ld+1) of such a class

template <typename R>
__device__ void rys_axis_rt(int la, int lb, int lc, int ld, R g00, R C, R Cp, R B00, R B1, R B1p, R AB,
                            R CD, R* I) {
    const int L12 = la + lb, L34 = lc + ld;
    R G[GEN_L2 + 1][GEN_L2 + 1];
    G[0][0] = g00;
    if (L12 > 0) G[1][0] = C * g00;
    for (int i = 1; i < L12; ++i) G[i + 1][0] = C * G[i][0] + R(i) * B1 * G[i - 1][0];
    for (int j = 0; j < L34; ++j)
        for (int i = 0; i <= L12; ++i) {
            R v = Cp * G[i][j];
            if (j > 0) v = fma(R(j) * B1p, G[i][j - 1], v);
            if (i > 0) v = fma(R(i) * B00, G[i - 1][j], v);
            G[i][j + 1] = v;
        }
    R X[GEN_LMAX + 1][GEN_L2 + 1][GEN_L2 + 1];
    for (int a = 0; a <= L12; ++a)
        for (int j = 0; j <= L34; ++j) X[0][a][j] = G[a][j];
    for (int b = 1; b <= lb; ++b)
        for (int a = 0; a <= L12 - b; ++a)
            for (int j = 0; j <= L34; ++j) X[b][a][j] = fma(AB, X[b - 1][a][j], X[b - 1][a + 1][j]);
    for (int a = 0; a <= la; ++a)
        for (int b = 0; b <= lb; ++b) {
            R Y[GEN_LMAX + 1][GEN_L2 + 1];
            for (int c = 0; c <= L34; ++c) Y[0][c] = X[b][a][c];
            for (int d = 1; d <= ld; ++d)
                for (int c = 0; c <= L34 - d; ++c) Y[d][c] = fma(CD, Y[d - 1][c], Y[d - 1][c + 1]);
            for (int c = 0; c <= lc; ++c)
                for (int d = 0; d <= ld; ++d) I[((a * (lb + 1) + b) * (lc + 1) + c) * (ld + 1) + d] = Y[d][c];
        }
}

template <typename R>
__device__ __forceinline__ void rys_roots_rt(int nr, R T, const R* __restrict__ tab, R* x, R* w, bool compat = false) {
    switch (nr) {
        case 1: rys_roots<1, R>(T, tab, x, w); break;
        case 2: rys_roots<2, R>(T, tab, x, w, compat); break;
        case 3: rys_roots<3, R>(T, tab, x, w); break;
        case 4: rys_roots<4, R>(T, tab, x, w); break;
        default: rys_roots<5, R>(T, tab, x, w); break;
    }
}

// Contracted integrals of one shell quartet with runtime angular momenta (classes with f or g shells
// and the large d classes) into acc[NF] (f = ((ia*NB + ib)*NC + ic)*ND + id), without the component
// normalisation factors; npass counts the primitive quartets past the prefactor cut.
template <typename R, typename PP>
__device__ void generic_quartet_eri(const FockArgs& A, const ShellPair& bra, const ShellPair& ket, const R* __restrict__ rys,
                                    const PP* __restrict__ prims, int la, int lb, int lc, int ld, R* acc, unsigned& npass) {
    const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
    const int NF = NA * NB * NC * ND;
    const int nr = (la + lb + lc + ld) / 2 + 1;
    for (int f = 0; f < NF; ++f) acc[f] = R(0);
    const R prim_cut = R(A.prim_cut);
    const PP* pb = prims + bra.prim_begin;
    const PP* pk = prims + ket.prim_begin;
    for (int ib = 0; ib < bra.nprim; ++ib) {
        const R p = pb[ib * bra.prim_stride].p, rp = pb[ib * bra.prim_stride].rp, Eab = pb[ib * bra.prim_stride].E, cab = pb[ib * bra.prim_stride].cc;
        for (int ik = 0; ik < ket.nprim; ++ik) {
            const R q = pk[ik * ket.prim_stride].p, rq = pk[ik * ket.prim_stride].rp, Ecd = pk[ik * ket.prim_stride].E, ccd = pk[ik * ket.prim_stride].cc;
            const R rpq = R(1) / (p + q);
            R sr = R(SRTERM) * Eab * Ecd * sqrt(rpq);
            if (sr < prim_cut) continue;
            sr *= cab * ccd;
            ++npass;
            R PQ[3], x[5], w[5];
            for (int k = 0; k < 3; ++k) PQ[k] = R(pb[ib * bra.prim_stride].P[k]) - R(pk[ik * ket.prim_stride].P[k]);
            const R T = p * q * rpq * (PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2]);
            rys_roots_rt<R>(nr, T, rys, x, w, A.rys_compat != 0);
            for (int r = 0; r < nr; ++r) {
                const R fff = x[r] * rpq;
                const R B00 = R(0.5) * fff;
                const R B1 = (R(0.5) - B00 * q) * rp;
                const R B1p = (R(0.5) - B00 * p) * rq;
                R I[3][GEN_NI];
                for (int k = 0; k < 3; ++k)
                    rys_axis_rt<R>(la, lb, lc, ld, k == 2 ? w[r] * sr : R(1), R(pb[ib * bra.prim_stride].PA[k]) - q * fff * PQ[k],
                                   R(pk[ik * ket.prim_stride].PA[k]) + p * fff * PQ[k], B00, B1, B1p, R(bra.AB[k]), R(ket.AB[k]), I[k]);
                int f = 0;
                for (int ia = 0; ia < NA; ++ia)
                    for (int ibb = 0; ibb < NB; ++ibb)
                        for (int ic = 0; ic < NC; ++ic)
                            for (int id = 0; id < ND; ++id, ++f) {
                                auto idx = [&](int ax, int ca, int cb, int cc, int cd) {
                                    auto comp = [&](int l, int c) {
                                        return ax == 0 ? cart_lx(l, c) : ax == 1 ? cart_ly(l, c) : cart_lz(l, c);
                                    };
                                    return ((comp(la, ca) * (lb + 1) + comp(lb, cb)) * (lc + 1) + comp(lc, cc)) * (ld + 1) + comp(ld, cd);
                                };
                                acc[f] = fma(I[0][idx(0, ia, ibb, ic, id)] * I[1][idx(1, ia, ibb, ic, id)],
                                             I[2][idx(2, ia, ibb, ic, id)], acc[f]);
                            }
            }
        }
    }
}

template <bool UHF, typename R, typename PP>
__global__ void __launch_bounds__(64) fock_jk_generic(const FockArgs A, const NormTable nt, const R* __restrict__ rys,
                                                      const PP* __restrict__ prims, int la, int lb, int lc, int ld) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int bi, ki;
    unsigned npass = 0;
    if (!(A.mode == 0 ? decode_work_warp<false>(A, g, bi, ki) : decode_work_warp<true>(A, g, bi, ki))) return;
    const ShellPair bra = A.pairs[bi];
    const ShellPair ket = A.pairs[ki];
    if (A.mode != 0 && quartet_bound(A, bra, ket) < A.skip_cut32) return;
    const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
    R acc[GEN_NF];
    generic_quartet_eri<R, PP>(A, bra, ket, rys, prims, la, lb, lc, ld, acc, npass);
    // density contraction and scatter, as digest_jk with runtime sizes
    int N = A.nbf;
    long long base = 0;
    if (A.mol_nbf) {
        N = A.mol_nbf[bra.pad];
        base = A.mol_base[bra.pad];
    }
    double* __restrict__ Ta = A.Ta + base;
    double* __restrict__ Tb = UHF ? A.Tb + base : nullptr;
    double deg = 1.0;
    if (bra.same) deg *= 0.5;
    if (ket.same) deg *= 0.5;
    if (bi == ki) deg *= 0.5;
    const double* __restrict__ Pa = A.Pa + base;
    const double* __restrict__ Pb = UHF ? A.Pb + base : nullptr;
    int f = 0;
    for (int ia = 0; ia < NA; ++ia) {
        const int a = bra.a_off + ia;
        for (int ib = 0; ib < NB; ++ib) {
            const int b = bra.b_off + ib;
            double Pab = Pa[a * N + b];
            if (UHF) Pab += Pb[a * N + b];
            double jab = 0.0;
            for (int ic = 0; ic < NC; ++ic) {
                const int c = ket.a_off + ic;
                for (int id = 0; id < ND; ++id, ++f) {
                    const int d = ket.b_off + id;
                    double v = double(acc[f]) * (nt.v[la][ia] * nt.v[lb][ib] * nt.v[lc][ic] * nt.v[ld][id]);
                    if (!(fabs(v) > A.thr_int)) continue;
                    v *= deg;
                    double Pcd = Pa[c * N + d];
                    if (UHF) Pcd += Pb[c * N + d];
                    jab = fma(v, Pcd, jab);
                    const double jf = UHF ? 2.0 : 4.0;
                    atomicAdd(Ta +c * N + d, jf * v * Pab);
                    atomicAdd(Ta +a * N + c, -v * Pa[b * N + d]);
                    atomicAdd(Ta +a * N + d, -v * Pa[b * N + c]);
                    atomicAdd(Ta +b * N + c, -v * Pa[a * N + d]);
                    atomicAdd(Ta +b * N + d, -v * Pa[a * N + c]);
                    if (UHF) {
                        atomicAdd(Tb +c * N + d, jf * v * Pab);
                        atomicAdd(Tb +a * N + c, -v * Pb[b * N + d]);
                        atomicAdd(Tb +a * N + d, -v * Pb[b * N + c]);
                        atomicAdd(Tb +b * N + c, -v * Pb[a * N + d]);
                        atomicAdd(Tb +b * N + d, -v * Pb[a * N + c]);
                    }
                }
            }
            const double jf = UHF ? 2.0 : 4.0;
            atomicAdd(Ta +a * N + b, jf * jab);
            if (UHF) atomicAdd(Tb +a * N + b, jf * jab);
        }
    }
    if (A.counters) count_flush(A, npass);
}

}  // namespace ugb

namespace ugb {

// Schwarz diagonal for the large pair classes (runtime loops, integrals in local memory).
static __global__ void __launch_bounds__(64) schwarz_generic(const ShellPair* __restrict__ pairs, const PrimPair* __restrict__ prims,
                                                      int begin, int count, const NormTable nt,
                                                      const double* __restrict__ rys, double* __restrict__ q_out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const ShellPair sp = pairs[begin + t];
    const int la = sp.la, lb = sp.lb;
    const int NA = ncart(la), NB = ncart(lb);
    const int nr = (2 * la + 2 * lb) / 2 + 1;
    double acc[GEN_NC * GEN_NC];  // only the diagonal (ab|ab) is needed
    for (int f = 0; f < NA * NB; ++f) acc[f] = 0.0;
    const PrimPair* pp = prims + sp.prim_begin;
    for (int ib = 0; ib < sp.nprim; ++ib) {
        const double p = pp[ib * sp.prim_stride].p, rp = pp[ib * sp.prim_stride].rp;
        for (int ik = 0; ik < sp.nprim; ++ik) {
            const double q = pp[ik * sp.prim_stride].p, rq = pp[ik * sp.prim_stride].rp;
            const double rpq = 1.0 / (p + q);
            const double sr = SRTERM * pp[ib * sp.prim_stride].E * pp[ik * sp.prim_stride].E * sqrt(rpq) * pp[ib * sp.prim_stride].cc * pp[ik * sp.prim_stride].cc;
            double PQ[3], x[5], w[5];
            for (int k = 0; k < 3; ++k) PQ[k] = pp[ib * sp.prim_stride].P[k] - pp[ik * sp.prim_stride].P[k];
            const double T = p * q * rpq * (PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2]);
            rys_roots_rt<double>(nr, T, rys, x, w);
            for (int r = 0; r < nr; ++r) {
                const double fff = x[r] * rpq, B00 = 0.5 * fff;
                const double B1 = (0.5 - B00 * q) * rp, B1p = (0.5 - B00 * p) * rq;
                double I[3][GEN_NI];
                for (int k = 0; k < 3; ++k)
                    rys_axis_rt<double>(la, lb, la, lb, k == 2 ? w[r] * sr : 1.0, pp[ib * sp.prim_stride].PA[k] - q * fff * PQ[k],
                                        pp[ik * sp.prim_stride].PA[k] + p * fff * PQ[k], B00, B1, B1p, sp.AB[k], sp.AB[k], I[k]);
                for (int ia = 0; ia < NA; ++ia)
                    for (int ibb = 0; ibb < NB; ++ibb) {
                        const int ix = ((cart_lx(la, ia) * (lb + 1) + cart_lx(lb, ibb)) * (la + 1) + cart_lx(la, ia)) * (lb + 1) + cart_lx(lb, ibb);
                        const int iy = ((cart_ly(la, ia) * (lb + 1) + cart_ly(lb, ibb)) * (la + 1) + cart_ly(la, ia)) * (lb + 1) + cart_ly(lb, ibb);
                        const int iz = ((cart_lz(la, ia) * (lb + 1) + cart_lz(lb, ibb)) * (la + 1) + cart_lz(la, ia)) * (lb + 1) + cart_lz(lb, ibb);
                        acc[ia * NB + ibb] += I[0][ix] * I[1][iy] * I[2][iz];
                    }
            }
        }
    }
    double m = 0.0;
    for (int ia = 0; ia < NA; ++ia)
        for (int ibb = 0; ibb < NB; ++ibb) {
            const double n = nt.v[la][ia] * nt.v[lb][ibb];
            m = fmax(m, fabs(acc[ia * NB + ibb]) * n * n);
        }
    q_out[begin + t] = sqrt(m);
}

}  // namespace ugb
