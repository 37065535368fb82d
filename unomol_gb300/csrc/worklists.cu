// Per-build work lists of the density-screened and mixed-precision Fock builds (see worklists.h).
#include "worklists.h"

namespace ugb {
namespace {

// FP32 copy of a dense density (the FP32 kernels contract with it)
__global__ void to_float(const double* __restrict__ full, float* __restrict__ f32, long long n2) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n2) f32[t] = (float)full[t];
}


// max |P| over every shell pair block (and over all blocks into dmax[0]), for density screening
__global__ void shell_pmax(const double* __restrict__ Pa, const double* __restrict__ Pb, const int* __restrict__ soff,
                           const int* __restrict__ sl, int nshell, int n, float* __restrict__ out, float* dmax) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nshell * nshell) return;
    const int a = t / nshell, b = t % nshell;
    const int na = (sl[a] + 1) * (sl[a] + 2) / 2, nb = (sl[b] + 1) * (sl[b] + 2) / 2;
    double m = 0.0;
    for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j) {
            const long long ix = (long long)(soff[a] + i) * n + soff[b] + j;
            double v = fabs(Pa[ix]);
            if (Pb) v = fmax(v, fabs(Pb[ix]));
            m = fmax(m, v);
        }
    // round up so that the float bound never undercuts the double one
    const float mf = __double2float_ru(m);
    out[t] = mf;
    atomicMax(reinterpret_cast<unsigned*>(dmax), __float_as_uint(mf));  // non-negative floats order as uints
}

// Per bra row of every block pair: lengths of the FP64 segment (bound * max|P| >= cut64) and of the
// FP32 segment (>= skip) of the row's Schwarz staircase, for this build's density (max|P| of the
// pair's molecule in a batch).
__global__ void split_rows(const ShellPair* __restrict__ pairs, const BlockPair* __restrict__ bps,
                           const int* __restrict__ row_bp, const long long* __restrict__ prefix, long long nrows,
                           const float* __restrict__ dmax, double cut64, double skip, long long* __restrict__ c64,
                           long long* __restrict__ c32, int* __restrict__ mseg) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nrows) return;
    const int bpi = row_bp[t];
    if (bpi < 0) return;  // end-of-block-pair sentinel
    const BlockPair bp = bps[bpi];
    const int i = (int)(t - bp.prefix_off);
    const int nstat = (int)(prefix[t + 1] - prefix[t]);  // static (integral-bound) staircase of the row
    const ShellPair& bra = pairs[bp.bra_begin + i];
    const double qd = bra.q * (double)dmax[bra.pad];  // pad: the molecule of a batch (0 for one context)
    const ShellPair* kp = pairs + bp.ket_begin;
    auto count = [&](double cut) {  // ket pairs j < nstat with q_i q_j max|P| >= cut (q descending)
        if (!(qd > 0.0)) return 0;
        const double thr = cut / qd;
        int lo = 0, hi = nstat;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (kp[mid].q >= thr) lo = mid + 1; else hi = mid;
        }
        return lo;
    };
    const int n64 = count(cut64);
    const int nall = cut64 <= skip ? n64 : count(skip);
    c64[t] = n64;
    c32[t] = nall - n64;
    mseg[t] = n64;
}

// Exclusive scan of the two row counts within every block pair (one CUDA block per block pair).
__global__ void __launch_bounds__(1024) scan_rows(const BlockPair* __restrict__ bps, const long long* __restrict__ c64,
                                                  const long long* __restrict__ c32, long long* __restrict__ p64,
                                                  long long* __restrict__ p32, long long* __restrict__ n64,
                                                  long long* __restrict__ n32) {
    __shared__ long long warp_a[32], warp_b[32];
    __shared__ long long run_a, run_b;
    const BlockPair bp = bps[blockIdx.x];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        run_a = 0;
        run_b = 0;
    }
    __syncthreads();
    for (int base = 0; base < bp.bra_count; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const long long va = i < bp.bra_count ? c64[bp.prefix_off + i] : 0;
        const long long vb = i < bp.bra_count ? c32[bp.prefix_off + i] : 0;
        long long sa = va, sb = vb;  // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const long long xa = __shfl_up_sync(0xffffffffu, sa, o), xb = __shfl_up_sync(0xffffffffu, sb, o);
            if (lane >= o) {
                sa += xa;
                sb += xb;
            }
        }
        if (lane == 31) {
            warp_a[wid] = sa;
            warp_b[wid] = sb;
        }
        __syncthreads();
        if (wid == 0) {
            const int nw = blockDim.x >> 5;
            long long ta = lane < nw ? warp_a[lane] : 0, tb = lane < nw ? warp_b[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const long long xa = __shfl_up_sync(0xffffffffu, ta, o), xb = __shfl_up_sync(0xffffffffu, tb, o);
                if (lane >= o) {
                    ta += xa;
                    tb += xb;
                }
            }
            if (lane < nw) {
                warp_a[lane] = ta;  // inclusive sums of the warps
                warp_b[lane] = tb;
            }
        }
        __syncthreads();
        const long long wa = wid > 0 ? warp_a[wid - 1] : 0, wb = wid > 0 ? warp_b[wid - 1] : 0;
        if (i < bp.bra_count) {
            p64[bp.prefix_off + i] = run_a + wa + sa - va;
            p32[bp.prefix_off + i] = run_b + wb + sb - vb;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            run_a += warp_a[(blockDim.x >> 5) - 1];
            run_b += warp_b[(blockDim.x >> 5) - 1];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        n64[blockIdx.x] = run_a;
        n32[blockIdx.x] = run_b;
    }
}


// Compact numbering of both parts per class launch: for the block pairs of launch l (first
// launch_bp[2l], count launch_bp[2l+1]) begin[k] = sum over the launch's earlier block pairs of their
// part's quartets rounded up to 32 (warps never straddle block pairs); total[l] = the sum over all.
// One CTA per launch.
__global__ void __launch_bounds__(1024) scan_launches(const int* __restrict__ launch_bp, const long long* __restrict__ n64,
                                                      const long long* __restrict__ n32, long long* __restrict__ b64,
                                                      long long* __restrict__ b32, long long* __restrict__ t64,
                                                      long long* __restrict__ t32) {
    __shared__ long long warp_a[32], warp_b[32];
    __shared__ long long run_a, run_b;
    const int first = launch_bp[2 * blockIdx.x], count = launch_bp[2 * blockIdx.x + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        run_a = 0;
        run_b = 0;
    }
    __syncthreads();
    for (int base = 0; base < count; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const long long va = i < count ? (n64[first + i] + 31) / 32 * 32 : 0;
        const long long vb = i < count ? (n32[first + i] + 31) / 32 * 32 : 0;
        long long sa = va, sb = vb;  // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const long long xa = __shfl_up_sync(0xffffffffu, sa, o), xb = __shfl_up_sync(0xffffffffu, sb, o);
            if (lane >= o) {
                sa += xa;
                sb += xb;
            }
        }
        if (lane == 31) {
            warp_a[wid] = sa;
            warp_b[wid] = sb;
        }
        __syncthreads();
        if (wid == 0) {
            const int nw = blockDim.x >> 5;
            long long ta = lane < nw ? warp_a[lane] : 0, tb = lane < nw ? warp_b[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const long long xa = __shfl_up_sync(0xffffffffu, ta, o), xb = __shfl_up_sync(0xffffffffu, tb, o);
                if (lane >= o) {
                    ta += xa;
                    tb += xb;
                }
            }
            if (lane < nw) {
                warp_a[lane] = ta;
                warp_b[lane] = tb;
            }
        }
        __syncthreads();
        const long long wa = wid > 0 ? warp_a[wid - 1] : 0, wb = wid > 0 ? warp_b[wid - 1] : 0;
        if (i < count) {
            b64[first + i] = run_a + wa + sa - va;
            b32[first + i] = run_b + wb + sb - vb;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            run_a += warp_a[(blockDim.x >> 5) - 1];
            run_b += warp_b[(blockDim.x >> 5) - 1];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        t64[blockIdx.x] = run_a;
        t32[blockIdx.x] = run_b;
    }
}

// max |P| per shell-pair block for every molecule of a batch (one thread per block)
__global__ void shell_pmax_batch(const double* __restrict__ P, const long long* __restrict__ doff, const int* __restrict__ nbf,
                                 const int* __restrict__ shell0, const int* __restrict__ nshell,
                                 const long long* __restrict__ pmax_off, const int* __restrict__ soff,
                                 const int* __restrict__ sl, int nmol, long long total, float* __restrict__ pmax,
                                 float* __restrict__ dmax) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    int lo = 0, hi = nmol - 1;  // the molecule: last with pmax_off <= t
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pmax_off[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const int ns = nshell[lo], n = nbf[lo];
    const long long r = t - pmax_off[lo];
    const int a = (int)(r / ns), b = (int)(r % ns);
    const int sa = shell0[lo] + a, sb = shell0[lo] + b;
    const int na = (sl[sa] + 1) * (sl[sa] + 2) / 2, nb = (sl[sb] + 1) * (sl[sb] + 2) / 2;
    const double* Pm = P + doff[lo];
    double m = 0.0;
    for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j) m = fmax(m, fabs(Pm[(long long)(soff[sa] + i) * n + soff[sb] + j]));
    const float mf = __double2float_ru(m);
    pmax[t] = mf;
    atomicMax(reinterpret_cast<unsigned*>(dmax + lo), __float_as_uint(mf));
}

unsigned blocks_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

cudaError_t wl_to_float(const double* full, float* f32, long long n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    to_float<<<blocks_for(n, 256), 256, 0, s>>>(full, f32, n);
    return cudaGetLastError();
}

cudaError_t wl_shell_pmax(const double* Pa, const double* Pb, const int* soff, const int* sl, int nshell, int nbf,
                          float* pmax, float* dmax, cudaStream_t s) {
    const long long n2 = (long long)nshell * nshell;
    if (n2 <= 0) return cudaSuccess;
    shell_pmax<<<blocks_for(n2, 256), 256, 0, s>>>(Pa, Pb, soff, sl, nshell, nbf, pmax, dmax);
    return cudaGetLastError();
}

cudaError_t wl_shell_pmax_batch(const double* P, const long long* doff, const int* nbf, const int* shell0,
                                const int* nshell, const long long* pmax_off, const int* soff, const int* sl, int nmol,
                                long long total, float* pmax, float* dmax, cudaStream_t s) {
    if (total <= 0 || nmol <= 0) return cudaSuccess;
    shell_pmax_batch<<<blocks_for(total, 256), 256, 0, s>>>(P, doff, nbf, shell0, nshell, pmax_off, soff, sl, nmol, total,
                                                             pmax, dmax);
    return cudaGetLastError();
}

cudaError_t wl_split_rows(const ShellPair* pairs, const BlockPair* bps, const int* row_bp, const long long* prefix,
                          long long nrows, const float* dmax, double cut64, double skip, long long* c64, long long* c32,
                          int* mseg, cudaStream_t s) {
    if (nrows <= 0) return cudaSuccess;
    split_rows<<<blocks_for(nrows, 256), 256, 0, s>>>(pairs, bps, row_bp, prefix, nrows, dmax, cut64, skip, c64, c32, mseg);
    return cudaGetLastError();
}

cudaError_t wl_scan_rows(const BlockPair* bps, int nbp, const long long* c64, const long long* c32, long long* p64,
                         long long* p32, long long* n64, long long* n32, cudaStream_t s) {
    if (nbp <= 0) return cudaSuccess;
    scan_rows<<<(unsigned)nbp, 512, 0, s>>>(bps, c64, c32, p64, p32, n64, n32);
    return cudaGetLastError();
}

cudaError_t wl_scan_launches(const int* launch_bp, int nlaunch, const long long* n64, const long long* n32,
                             long long* begin64, long long* begin32, long long* total64, long long* total32,
                             cudaStream_t s) {
    if (nlaunch <= 0) return cudaSuccess;
    scan_launches<<<(unsigned)nlaunch, 1024, 0, s>>>(launch_bp, n64, n32, begin64, begin32, total64, total32);
    return cudaGetLastError();
}

}  // namespace ugb
