// Legendre contractions (FP64) and the refinement residual.
//
// Analysis, per m and parity p of l - m:
//   A[l(l+1)/2 + m][c] (+)= sum_r lambda[m][p][li][r] * F[p][m][r][c],  l = m + p + 2 li
// where F[0] = F_north + F_south and F[1] = F_north - F_south (north/south
// symmetry lambda_lm(pi - theta) = (-1)^{l+m} lambda_lm(theta)), so the ring
// sum runs over the 2*nside north rings only.
// Synthesis is the transpose: G[p][m][r][c] = sum_li lambda[m][p][li][r] A[l(li)][c].
// The refinement of map2alm (niter Jacobi steps, reference
// src/healpix_helpers.jl:50-56) is done in ring-Fourier space:
//   R = F - w * nph * cfold * Fold(G)
// where Fold sums the synthesised coefficients that alias onto each m on a
// ring of nph pixels (exactly what the ring FFT of the synthesised map sees).
#include <algorithm>

#include "sfb_internal.h"

namespace sfb {

namespace {
constexpr int BM = 64, BN = 64, BK = 16;

__device__ __forceinline__ int nrows_of(int m, int par, int lmax) {
    return (m + par <= lmax) ? (lmax - m - par) / 2 + 1 : 0;
}
}  // namespace

// Ring range of the sum: rings r < rlim; with nzr, only the ring pairs
// [nzr[0], nzr[1]] (F is zero outside them: the ring transform recorded the
// span of ring pairs holding data; an empty span sums nothing).
template <typename T>
__global__ void __launch_bounds__(256) k_leg_analysis(const T *__restrict__ lam, const int64_t *lam_off,
                                                      int lmax, int nrn, const T *__restrict__ F,
                                                      int64_t ncol, T *__restrict__ A, int accumulate, int rlim,
                                                      const int *__restrict__ nzr) {
    const int z = blockIdx.z;
    const int m = z >> 1, par = z & 1;
    const int nrows = nrows_of(m, par, lmax);
    const int row0 = blockIdx.y * BM;
    if (row0 >= nrows) return;
    const int64_t col0 = (int64_t)blockIdx.x * BN;
    const T *L = lam + lam_off[z];
    const T *B = F + ((int64_t)(par * (lmax + 1) + m) * nrn) * ncol;
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    int kend = min(rlim, nrn), kbeg = 0;
    if (nzr) {
        const int lo = nzr[0], hi = nzr[1];
        kend = min(kend, hi + 1);
        kbeg = lo < kend ? (lo / BK) * BK : kend;
    }
    T acc[4][4] = {};
    for (int k0 = kbeg; k0 < kend; k0 += BK) {
        for (int i = tid; i < BM * BK; i += 256) {
            const int rr = i / BK, kk = i % BK;
            const int row = row0 + rr, k = k0 + kk;
            As[kk][rr] = (row < nrows && k < kend) ? L[(int64_t)row * nrn + k] : T(0);
        }
        for (int i = tid; i < BK * BN; i += 256) {
            const int kk = i / BN, cc = i % BN;
            const int k = k0 + kk;
            const int64_t col = col0 + cc;
            Bs[kk][cc] = (k < kend && col < ncol) ? B[(int64_t)k * ncol + col] : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            T a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int row = row0 + ty * 4 + i;
        if (row >= nrows) continue;
        const int l = m + par + 2 * row;
        const int64_t lm = (int64_t)l * (l + 1) / 2 + m;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t col = col0 + tx + 16 * j;
            if (col >= ncol) continue;
            T *d = A + lm * ncol + col;
            *d = accumulate ? *d + acc[i][j] : acc[i][j];
        }
    }
}

// Only the rings r < rlim are formed.
template <typename T>
__global__ void __launch_bounds__(256) k_leg_synthesis(const T *__restrict__ lam, const int64_t *lam_off,
                                                       int lmax, int nrn, const T *__restrict__ A,
                                                       int64_t ncol, T *__restrict__ G, int rlim) {
    const int z = blockIdx.z;
    const int m = z >> 1, par = z & 1;
    const int nrows = nrows_of(m, par, lmax);   // K dimension
    const int r0 = blockIdx.y * BM;
    if (r0 >= rlim) return;
    const int64_t col0 = (int64_t)blockIdx.x * BN;
    const T *L = lam + lam_off[z];
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    T acc[4][4] = {};
    for (int k0 = 0; k0 < nrows; k0 += BK) {
        for (int i = tid; i < BM * BK; i += 256) {
            const int kk = i / BM, rr = i % BM;
            const int k = k0 + kk, r = r0 + rr;
            As[kk][rr] = (k < nrows && r < nrn) ? L[(int64_t)k * nrn + r] : T(0);
        }
        for (int i = tid; i < BK * BN; i += 256) {
            const int kk = i / BN, cc = i % BN;
            const int k = k0 + kk;
            const int64_t col = col0 + cc;
            T v = T(0);
            if (k < nrows && col < ncol) {
                const int l = m + par + 2 * k;
                v = A[((int64_t)l * (l + 1) / 2 + m) * ncol + col];
            }
            Bs[kk][cc] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            T a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
    T *Gb = G + ((int64_t)(par * (lmax + 1) + m) * nrn) * ncol;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = r0 + ty * 4 + i;
        if (r >= rlim) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t col = col0 + tx + 16 * j;
            if (col < ncol) Gb[(int64_t)r * ncol + col] = acc[i][j];
        }
    }
}

// R[p][m'][r][c] = F[p][m'][r][c] - w * nph * cfold * Fold(G[p][.][r][c])[m']
// Fold(G)_{m'} = sum_{m = m' mod n + t n <= L} G_m e^{i(m-m')phi0}
//              + sum_{m >= 1, m = -m' mod n + t n <= L} conj(G_m) e^{-i(m+m')phi0},
// and (m -/+ m') is a multiple of n, phi0 = pi/den with den in {0, n}, so
// every phase is +1 or (-1)^t.  G_0 enters through its real part.
template <typename T>
__global__ void __launch_bounds__(128) k_fold_residual(const RingGeom *rings, int nrn, int lmax, double w,
                                                      const T *__restrict__ F, const T *__restrict__ G, int64_t ncplx,
                                                      T *__restrict__ R) {
    // one block per (parity, m', ring); threads stride over the complex columns
    const int mp = blockIdx.x;
    const int r = blockIdx.y;
    const int par = blockIdx.z;
    const RingGeom g = rings[r];
    const int n = g.nph;
    const int L1 = lmax + 1;
    const int64_t ld = 2 * ncplx;
    const bool odd_phase = g.phi0_den != 0;   // e^{i t n phi0} = (-1)^t when phi0 = pi/n
    const T f = (T)(w * (double)n * g.cfold);
    const int64_t off = ((int64_t)(par * L1 + mp) * nrn + r) * ld;
    const int k = mp % n;
    const int kk = (n - k) % n;
    if (n > 2 * lmax) {   // no aliasing on this ring: Fold(G)_{m'} = G_{m'} (real part for m' = 0)
        for (int64_t c = threadIdx.x; c < ncplx; c += blockDim.x) {
            const T gx = G[off + 2 * c], gy = mp == 0 ? T(0) : G[off + 2 * c + 1];
            R[off + 2 * c] = F[off + 2 * c] - f * gx;
            R[off + 2 * c + 1] = F[off + 2 * c + 1] - f * gy;
        }
        return;
    }
    for (int64_t c = threadIdx.x; c < ncplx; c += blockDim.x) {
        T sx = 0, sy = 0;
        int t = 0;
        for (int m = k; m <= lmax; m += n, ++t) {
            const T *gp = G + ((int64_t)(par * L1 + m) * nrn + r) * ld + 2 * c;
            const int dt = t - mp / n;                       // (m - m') = dt * n
            const T sgn = (odd_phase && (dt & 1)) ? T(-1) : T(1);
            sx += sgn * gp[0];
            if (m != 0) sy += sgn * gp[1];
        }
        for (int m = (kk == 0 ? n : kk); m <= lmax; m += n) {
            const T *gp = G + ((int64_t)(par * L1 + m) * nrn + r) * ld + 2 * c;
            const int q = (m + mp) / n;                      // (m + m') = q * n
            const T sgn = (odd_phase && (q & 1)) ? T(-1) : T(1);
            sx += sgn * gp[0];
            sy -= sgn * gp[1];
        }
        R[off + 2 * c] = F[off + 2 * c] - f * sx;
        R[off + 2 * c + 1] = F[off + 2 * c + 1] - f * sy;
    }
}

// Few columns (ncol <= 8, e.g. one reference map): matrix-vector shape.
// Analysis: one warp per (block z, row li), lanes stride over the rings
// (coalesced lambda rows), warp-reduced.
template <typename T, int NC>
__global__ void __launch_bounds__(256) k_leg_analysis_narrow(const T *__restrict__ lam, const int64_t *lam_off,
                                                             int lmax, int nrn, int rlim, const T *__restrict__ F,
                                                             T *__restrict__ A, int accumulate) {
    const int z = blockIdx.y;
    const int m = z >> 1, par = z & 1;
    const int nrows = nrows_of(m, par, lmax);
    const int row = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (row >= nrows) return;
    const int lane = threadIdx.x & 31;
    const T *L = lam + lam_off[z] + (int64_t)row * nrn;
    const T *B = F + ((int64_t)(par * (lmax + 1) + m) * nrn) * NC;
    T acc[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] = T(0);
    for (int r = lane; r < rlim; r += 32) {      // rings r >= rlim count as zero
        const T l = L[r];
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[c] = fma(l, B[(int64_t)r * NC + c], acc[c]);
    }
#pragma unroll
    for (int c = 0; c < NC; ++c)
        for (int off = 16; off > 0; off >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], off);
    if (lane < NC) {
        T v = acc[0];
#pragma unroll
        for (int c = 1; c < NC; ++c)
            if (lane == c) v = acc[c];
        const int l = m + par + 2 * row;
        T *d = A + ((int64_t)l * (l + 1) / 2 + m) * NC + lane;
        *d = accumulate ? *d + v : v;
    }
}

// Synthesis: one thread per (block z, ring r), looping over the rows li
// (lambda reads coalesced over r, a_lm broadcast).
template <typename T, int NC>
__global__ void __launch_bounds__(128) k_leg_synthesis_narrow(const T *__restrict__ lam, const int64_t *lam_off,
                                                              int lmax, int nrn, int rlim, const T *__restrict__ A,
                                                              T *__restrict__ G) {
    const int z = blockIdx.y;
    const int m = z >> 1, par = z & 1;
    const int nrows = nrows_of(m, par, lmax);
    const int r = blockIdx.x * 128 + threadIdx.x;
    if (r >= rlim) return;                        // only the first rlim rings are formed
    const T *L = lam + lam_off[z] + r;
    T acc[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] = T(0);
    for (int li = 0; li < nrows; ++li) {
        const T l = L[(int64_t)li * nrn];
        const int ll = m + par + 2 * li;
        const T *a = A + ((int64_t)ll * (ll + 1) / 2 + m) * NC;
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[c] = fma(l, a[c], acc[c]);
    }
    T *g = G + (((int64_t)(par * (lmax + 1) + m) * nrn) + r) * NC;
#pragma unroll
    for (int c = 0; c < NC; ++c) g[c] = acc[c];
}

template <typename T, int NC>
static void narrow_analysis(const Plan &p, const T *lam, const T *F, T *A, bool accumulate, int rlim,
                            cudaStream_t st) {
    const int maxrows = p.lmax / 2 + 1;
    dim3 grid((unsigned)((maxrows + 7) / 8), (unsigned)(2 * (p.lmax + 1)));
    k_leg_analysis_narrow<T, NC><<<grid, 256, 0, st>>>(lam, p.d_lam_off, p.lmax, (int)p.nrn, rlim, F, A,
                                                       accumulate ? 1 : 0);
}

template <typename T, int NC>
static void narrow_synthesis(const Plan &p, const T *lam, const T *A, T *G, int rlim, cudaStream_t st) {
    dim3 grid((unsigned)((rlim + 127) / 128), (unsigned)(2 * (p.lmax + 1)));
    k_leg_synthesis_narrow<T, NC><<<grid, 128, 0, st>>>(lam, p.d_lam_off, p.lmax, (int)p.nrn, rlim, A, G);
}

template <typename T>
static bool narrow_dispatch(const Plan &p, const T *lam, const T *in, int64_t ncol, T *out, bool analysis,
                            bool accumulate, cudaStream_t st, int rlim = -1) {
    if (rlim < 0 || rlim > p.nrn) rlim = (int)p.nrn;
    switch (ncol) {
    case 2:
        if (analysis) narrow_analysis<T, 2>(p, lam, in, out, accumulate, rlim, st);
        else narrow_synthesis<T, 2>(p, lam, in, out, rlim, st);
        return true;
    case 4:
        if (analysis) narrow_analysis<T, 4>(p, lam, in, out, accumulate, rlim, st);
        else narrow_synthesis<T, 4>(p, lam, in, out, rlim, st);
        return true;
    case 8:
        if (analysis) narrow_analysis<T, 8>(p, lam, in, out, accumulate, rlim, st);
        else narrow_synthesis<T, 8>(p, lam, in, out, rlim, st);
        return true;
    default:
        return false;
    }
}

// FP64 Gram refinement step for few columns (the narrow transforms):
//   Anew[l(r)] = A0[l(r)] - sum_li D_z[r][li] Acur[l(li)]   (= Acur + (A0 - M_z Acur))
// one thread per (block z, output row r, column); D_z = M_z - I from the plan's
// FP64 Gram tables (element [li][r] at gram_off[z] + li R + r).
template <int NC>
__global__ void __launch_bounds__(128) k_gram_update_fp64(const double *__restrict__ gram,
                                                          const int64_t *__restrict__ gram_off, int R, int lmax,
                                                          const double *__restrict__ Acur,
                                                          const double *__restrict__ A0, double *__restrict__ Anew) {
    const int z = blockIdx.y;
    const int m = z >> 1, par = z & 1;
    const int nrows = nrows_of(m, par, lmax);
    const int idx = blockIdx.x * 128 + threadIdx.x;
    const int r = idx / NC, c = idx - r * NC;
    if (r >= nrows) return;
    const double *M = gram + gram_off[z] + r;
    double acc = 0.0;
    for (int li = 0; li < nrows; ++li) {
        const int l = m + par + 2 * li;
        acc = fma(M[(int64_t)li * R], Acur[((int64_t)l * (l + 1) / 2 + m) * NC + c], acc);
    }
    const int l = m + par + 2 * r;
    const int64_t o = ((int64_t)l * (l + 1) / 2 + m) * NC + c;
    Anew[o] = A0[o] - acc;
}

// Many columns: the same update as a tiled GEMM per block z (output rows r x
// columns, K = the rows li), with the update in the epilogue.
__global__ void __launch_bounds__(256) k_gram_update_wide(const double *__restrict__ gram,
                                                          const int64_t *__restrict__ gram_off, int R, int lmax,
                                                          const double *__restrict__ Acur,
                                                          const double *__restrict__ A0, int64_t ncol,
                                                          double *__restrict__ Anew) {
    const int z = blockIdx.z;
    const int m = z >> 1, par = z & 1;
    const int nrows = nrows_of(m, par, lmax);
    const int r0 = blockIdx.y * BM;
    if (r0 >= nrows) return;
    const int64_t col0 = (int64_t)blockIdx.x * BN;
    const double *M = gram + gram_off[z];
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < nrows; k0 += BK) {
        for (int i = tid; i < BM * BK; i += 256) {
            const int kk = i / BM, rr = i % BM;
            const int k = k0 + kk, r = r0 + rr;
            As[kk][rr] = (k < nrows && r < nrows) ? M[(int64_t)k * R + r] : 0.0;
        }
        for (int i = tid; i < BK * BN; i += 256) {
            const int kk = i / BN, cc = i % BN;
            const int k = k0 + kk;
            const int64_t col = col0 + cc;
            double v = 0.0;
            if (k < nrows && col < ncol) {
                const int l = m + par + 2 * k;
                v = Acur[((int64_t)l * (l + 1) / 2 + m) * ncol + col];
            }
            Bs[kk][cc] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = r0 + ty * 4 + i;
        if (r >= nrows) continue;
        const int l = m + par + 2 * r;
        const int64_t base = ((int64_t)l * (l + 1) / 2 + m) * ncol;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t col = col0 + tx + 16 * j;
            if (col >= ncol) continue;
            const int64_t o = base + col;
            Anew[o] = A0[o] - acc[i][j];
        }
    }
}

void launch_leg_analysis(const Plan &p, const double *F, int64_t ncol, double *A, bool accumulate,
                         cudaStream_t st, int rlim, const int *nzr) {
    const bool narrow = p.precision == SFB_MIXED
                            ? narrow_dispatch<float>(p, p.d_lam32, (const float *)F, ncol, (float *)A, true, accumulate, st,
                                                     rlim)
                            : narrow_dispatch<double>(p, p.d_lam, F, ncol, A, true, accumulate, st, rlim);
    if (narrow) {
        note_launch();
        return;
    }
    const int maxrows = p.lmax / 2 + 1;
    if (rlim < 0 || rlim > p.nrn) rlim = (int)p.nrn;
    dim3 grid((unsigned)((ncol + BN - 1) / BN), (unsigned)((maxrows + BM - 1) / BM), (unsigned)(2 * (p.lmax + 1)));
    if (p.precision == SFB_MIXED)
        k_leg_analysis<float><<<grid, 256, 0, st>>>(p.d_lam32, p.d_lam_off, p.lmax, (int)p.nrn, (const float *)F,
                                                    ncol, (float *)A, accumulate ? 1 : 0, rlim, nzr);
    else
        k_leg_analysis<double><<<grid, 256, 0, st>>>(p.d_lam, p.d_lam_off, p.lmax, (int)p.nrn, F, ncol, A,
                                                     accumulate ? 1 : 0, rlim, nzr);
    note_launch();
}

void launch_leg_synthesis(const Plan &p, const double *A, int64_t ncol, double *G, cudaStream_t st, int rlim) {
    const bool narrow = p.precision == SFB_MIXED
                            ? narrow_dispatch<float>(p, p.d_lam32, (const float *)A, ncol, (float *)G, false, false, st,
                                                     rlim)
                            : narrow_dispatch<double>(p, p.d_lam, A, ncol, G, false, false, st, rlim);
    if (narrow) {
        note_launch();
        return;
    }
    if (rlim < 0 || rlim > p.nrn) rlim = (int)p.nrn;
    if (rlim == 0) return;
    dim3 grid((unsigned)((ncol + BN - 1) / BN), (unsigned)((rlim + BM - 1) / BM), (unsigned)(2 * (p.lmax + 1)));
    if (p.precision == SFB_MIXED)
        k_leg_synthesis<float><<<grid, 256, 0, st>>>(p.d_lam32, p.d_lam_off, p.lmax, (int)p.nrn, (const float *)A,
                                                     ncol, (float *)G, rlim);
    else
        k_leg_synthesis<double><<<grid, 256, 0, st>>>(p.d_lam, p.d_lam_off, p.lmax, (int)p.nrn, A, ncol, G, rlim);
    note_launch();
}

// Column-major variant: one block per (m', parity, tile of complex columns,
// chunk of FOLD_RC rings), looping over its rings (coalesced over the
// columns).  With Ecol it also raises the scale exponent of every real column
// over the rings (atomicMax; Ecol preset to a value below every exponent),
// the input of the mixed-precision Legendre analysis (as k_colmax computes
// for F).
constexpr int FOLD_RC = 64;

// Mixed precision: F and R are normalised double-float pairs.  r = F - f s with
// the product f s exact (TwoProd) and the sum in double-float.
__device__ __forceinline__ float2 df_resid(float2 F, float f, float s) {
    const float p = -f * s;
    const float e = fmaf(-f, s, -p);
    const float h = F.x + p;
    const float z = h - F.x;
    const float l = ((F.x - (h - z)) + (p - z)) + (F.y + e);
    const float h2 = h + l;
    return make_float2(h2, l - (h2 - h));
}

// Mixed-precision column-major fold (as k_fold_cols): F (nullable) and R double-float, G FP32.
__global__ void __launch_bounds__(128) k_fold_cols_df(const RingGeom *__restrict__ rings, int nrn, int rlim, int lmax,
                                                      double w, const float2 *__restrict__ F,
                                                      const float *__restrict__ G, int64_t ncplx,
                                                      float2 *__restrict__ R, int *__restrict__ Ecol) {
    const int mp = blockIdx.y >> 1, par = blockIdx.y & 1;
    const int rc0 = blockIdx.z * FOLD_RC;
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncplx) return;
    const int L1 = lmax + 1;
    const int64_t ld = 2 * ncplx;
    float mxr = 0.f, mxi = 0.f;
    const int rend = min(rlim, rc0 + FOLD_RC);
    for (int r = rc0; r < rend; ++r) {
        const RingGeom g = rings[r];
        const int n = g.nph;
        const bool odd_phase = g.phi0_den != 0;
        const float f = (float)(w * (double)n * g.cfold);
        const int64_t off = ((int64_t)(par * L1 + mp) * nrn + r) * ld + 2 * c;
        float sx, sy;
        if (n > 2 * lmax) {
            sx = G[off];
            sy = mp == 0 ? 0.f : G[off + 1];
        } else {
            sx = 0.f;
            sy = 0.f;
            const int k = mp % n;
            const int kk = (n - k) % n;
            int tt = 0;
            for (int m = k; m <= lmax; m += n, ++tt) {
                const float *gp = G + ((int64_t)(par * L1 + m) * nrn + r) * ld + 2 * c;
                const int dt = tt - mp / n;
                const float sgn = (odd_phase && (dt & 1)) ? -1.f : 1.f;
                sx += sgn * gp[0];
                if (m != 0) sy += sgn * gp[1];
            }
            for (int m = (kk == 0 ? n : kk); m <= lmax; m += n) {
                const float *gp = G + ((int64_t)(par * L1 + m) * nrn + r) * ld + 2 * c;
                const int q = (m + mp) / n;
                const float sgn = (odd_phase && (q & 1)) ? -1.f : 1.f;
                sx += sgn * gp[0];
                sy -= sgn * gp[1];
            }
        }
        const float2 fx = F ? F[off] : make_float2(0.f, 0.f), fy = F ? F[off + 1] : make_float2(0.f, 0.f);
        const float2 rx = df_resid(fx, f, sx), ry = df_resid(fy, f, sy);
        *reinterpret_cast<float4 *>(R + off) = make_float4(rx.x, rx.y, ry.x, ry.y);
        mxr = fmaxf(mxr, fabsf(rx.x));
        mxi = fmaxf(mxi, fabsf(ry.x));
    }
    if (Ecol) {
        const int lg = 32 - __clz(nrn > 1 ? nrn - 1 : 1);
        const int extra = max(0, lg - 9);
        auto ex = [&](float mx) {
            int E = (mx > 0.f && isfinite(mx)) ? ilogbf(mx) + 1 : 0;
            return max(-90, min(E + extra, 100));
        };
        const int64_t z = 2 * (int64_t)mp + par;
        if (mxr > 0.f) atomicMax(Ecol + z * ld + 2 * c, ex(mxr));      // all-zero ring chunks leave the preset
        if (mxi > 0.f) atomicMax(Ecol + z * ld + 2 * c + 1, ex(mxi));
    }
}

// F == nullptr: R = -w n cfold Fold(G) (the aliased-ring term of the Gram
// refinement).  Only rings r < rlim are written.
template <typename T>
__global__ void __launch_bounds__(128) k_fold_cols(const RingGeom *__restrict__ rings, int nrn, int rlim, int lmax,
                                                   double w, const T *__restrict__ F, const T *__restrict__ G,
                                                   int64_t ncplx, T *__restrict__ R, int *__restrict__ Ecol) {
    const int mp = blockIdx.y >> 1, par = blockIdx.y & 1;
    const int rc0 = blockIdx.z * FOLD_RC;
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncplx) return;
    const int L1 = lmax + 1;
    const int64_t ld = 2 * ncplx;
    float mxr = 0.f, mxi = 0.f;
    const int rend = min(rlim, rc0 + FOLD_RC);
#pragma unroll 4
    for (int r = rc0; r < rend; ++r) {
        const RingGeom g = rings[r];
        const int n = g.nph;
        const bool odd_phase = g.phi0_den != 0;
        const T f = (T)(w * (double)n * g.cfold);
        const int64_t off = ((int64_t)(par * L1 + mp) * nrn + r) * ld + 2 * c;
        T sx, sy;
        if (n > 2 * lmax) {          // no aliasing on this ring
            sx = G[off];
            sy = mp == 0 ? T(0) : G[off + 1];
        } else {
            sx = 0;
            sy = 0;
            const int k = mp % n;
            const int kk = (n - k) % n;
            int tt = 0;
            for (int m = k; m <= lmax; m += n, ++tt) {
                const T *gp = G + ((int64_t)(par * L1 + m) * nrn + r) * ld + 2 * c;
                const int dt = tt - mp / n;
                const T sgn = (odd_phase && (dt & 1)) ? T(-1) : T(1);
                sx += sgn * gp[0];
                if (m != 0) sy += sgn * gp[1];
            }
            for (int m = (kk == 0 ? n : kk); m <= lmax; m += n) {
                const T *gp = G + ((int64_t)(par * L1 + m) * nrn + r) * ld + 2 * c;
                const int q = (m + mp) / n;
                const T sgn = (odd_phase && (q & 1)) ? T(-1) : T(1);
                sx += sgn * gp[0];
                sy -= sgn * gp[1];
            }
        }
        const T rx = (F ? F[off] : T(0)) - f * sx, ry = (F ? F[off + 1] : T(0)) - f * sy;
        R[off] = rx;
        R[off + 1] = ry;
        mxr = fmaxf(mxr, fabsf((float)rx));
        mxi = fmaxf(mxi, fabsf((float)ry));
    }
    if (Ecol) {
        const int lg = 32 - __clz(nrn > 1 ? nrn - 1 : 1);
        const int extra = max(0, lg - 9);
        auto ex = [&](float mx) {
            int E = (mx > 0.f && isfinite(mx)) ? ilogbf(mx) + 1 : 0;
            return max(-90, min(E + extra, 100));
        };
        const int64_t z = 2 * (int64_t)mp + par;
        if (mxr > 0.f) atomicMax(Ecol + z * ld + 2 * c, ex(mxr));      // all-zero ring chunks leave the preset
        if (mxi > 0.f) atomicMax(Ecol + z * ld + 2 * c + 1, ex(mxi));
    }
}

// Aliased-ring fold of the Gram refinement (F = 0, rings r < ral):
//   R[p][m'][r][c] = -w nph cfold Fold(G[p][.][r][c])[m']
// computed per ring through residue buckets instead of per-output alias
// loops: P[k] = sum_{m = k mod n} s_m G[m] (s_m = (-1)^floor(m/n) for rings
// with the half-pixel phase, else 1; m = 0 adds its real part only), then
//   Fold[m'] = s(m') P[m' mod n] + s(c) conj(P'[(n - m' mod n) mod n]),
// c = (kk + m') / n, P' = P without the m = 0 term — the same sums as
// k_fold_cols, O(lmax) per ring and column instead of O(lmax^2 / n).
// Block: parity, FC complex columns, a group of rings; shared memory holds
// the ring's G rows, the buckets and the running column maxima (exponents for
// the analysis).
// MXREG: (lmax + 1) FC <= 256 MXQ, and each thread keeps the maxima of its output elements
// (i = tid + 256 q) in registers instead of shared memory (a smaller footprint, more CTAs per SM).
constexpr int FOLD_MXQ = 8;

template <int FC, bool MXREG>
__global__ void __launch_bounds__(256) k_fold_alias(const RingGeom *__restrict__ rings, int nrn, int ral, int rpb,
                                                    int nbk, int lmax, double w, const float *__restrict__ G,
                                                    int64_t ncplx, float2 *__restrict__ R, int *__restrict__ Ecol) {
    extern __shared__ float2 fsm[];
    const int par = blockIdx.y;
    const int64_t c0 = (int64_t)blockIdx.x * FC;
    const int r0 = blockIdx.z * rpb, r1 = min(ral, r0 + rpb);
    const int L1 = lmax + 1;
    const int64_t ld = 2 * ncplx;
    float2 *P = fsm;                                  // [nbk][FC], nbk = the longest of the rings
    float2 *mx = fsm + (int64_t)nbk * FC;             // [L1][FC] (re, im maxima; not MXREG)
    float2 *Gs = mx + (MXREG ? 0 : (int64_t)L1 * FC); // [L1][FC] the ring's G rows
    const int tid = threadIdx.x;
    float2 mxr[MXREG ? FOLD_MXQ : 1];
#pragma unroll
    for (int q = 0; q < (MXREG ? FOLD_MXQ : 1); ++q) mxr[q] = make_float2(0.f, 0.f);
    if (!MXREG)
        for (int i = tid; i < L1 * FC; i += 256) mx[i] = make_float2(0.f, 0.f);
    // a ring's G rows: element i = m * FC + cc at thread tid + 256 q; FOLD_PF loads per thread in
    // registers, the next ring's issued before this ring's buckets (more rows loop through Gs directly)
    constexpr int FOLD_PF = 8;
    float2 gv[FOLD_PF];
    auto load_ring = [&](int r) {
#pragma unroll
        for (int q = 0; q < FOLD_PF; ++q) {
            const int i = tid + q * 256;
            const int m = i / FC, cc = i - m * FC;
            gv[q] = make_float2(0.f, 0.f);
            if (i < L1 * FC && c0 + cc < ncplx)
                gv[q] = *reinterpret_cast<const float2 *>(G + ((int64_t)(par * L1 + m) * nrn + r) * ld +
                                                          2 * (c0 + cc));
        }
    };
    if (r0 < r1) load_ring(r0);
    for (int r = r0; r < r1; ++r) {
        const RingGeom g = rings[r];
        const int n = min(g.nph, nbk);
        const bool odd = g.phi0_den != 0;
        const float f = (float)(w * (double)n * g.cfold);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < FOLD_PF; ++q)
            if (tid + q * 256 < L1 * FC) Gs[tid + q * 256] = gv[q];
        for (int i = tid + FOLD_PF * 256; i < L1 * FC; i += 256) {
            const int m = i / FC, cc = i - m * FC;
            Gs[i] = c0 + cc < ncplx ? *reinterpret_cast<const float2 *>(G + ((int64_t)(par * L1 + m) * nrn + r) * ld +
                                                                       2 * (c0 + cc))
                                    : make_float2(0.f, 0.f);
        }
        __syncthreads();
        if (r + 1 < r1) load_ring(r + 1);
        // buckets, each summed by one thread in a fixed order (deterministic)
        for (int i = tid; i < n * FC; i += 256) {
            const int k = i / FC, cc = i - k * FC;
            float sx = 0.f, sy = 0.f;
            int t = 0;
            for (int m = k; m <= lmax; m += n, ++t) {
                const float2 gv = Gs[m * FC + cc];
                const float sg = (odd && (t & 1)) ? -1.f : 1.f;
                sx += sg * gv.x;
                if (m != 0) sy += sg * gv.y;
            }
            P[i] = make_float2(sx, sy);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < (MXREG ? FOLD_MXQ : 1 << 30); ++q) {
            const int i = tid + 256 * q;
            if (i >= L1 * FC) break;
            const int mp = i / FC, cc = i - mp * FC;
            const int64_t c = c0 + cc;
            if (c >= ncplx) continue;
            const int k = mp % n;
            const int kk = (n - k) % n;
            const float2 p1 = P[k * FC + cc];
            float2 p2 = P[kk * FC + cc];
            if (kk == 0) p2.x -= Gs[cc].x;                  // P' excludes m = 0
            const float s1 = (odd && ((mp / n) & 1)) ? -1.f : 1.f;
            const float s2 = (odd && (((kk + mp) / n) & 1)) ? -1.f : 1.f;
            const float sx = s1 * p1.x + s2 * p2.x, sy = s1 * p1.y - s2 * p2.y;
            const float rx = -f * sx, ry = -f * sy;
            const int64_t off = ((int64_t)(par * L1 + mp) * nrn + r) * ld + 2 * c;
            // double-float storage: the exact product error as the low word
            *reinterpret_cast<float4 *>(R + off) = make_float4(rx, fmaf(-f, sx, -rx), ry, fmaf(-f, sy, -ry));
            if constexpr (MXREG) {
                mxr[q].x = fmaxf(mxr[q].x, fabsf(rx));
                mxr[q].y = fmaxf(mxr[q].y, fabsf(ry));
            } else {
                float2 m2 = mx[i];
                m2.x = fmaxf(m2.x, fabsf(rx));
                m2.y = fmaxf(m2.y, fabsf(ry));
                mx[i] = m2;
            }
        }
    }
    if (!Ecol) return;
    __syncthreads();
    const int lg = 32 - __clz(nrn > 1 ? nrn - 1 : 1);
    const int extra = max(0, lg - 9);
    auto ex = [&](float v) {
        int E = (v > 0.f && isfinite(v)) ? ilogbf(v) + 1 : 0;
        return max(-90, min(E + extra, 100));
    };
#pragma unroll
    for (int q = 0; q < (MXREG ? FOLD_MXQ : 1 << 30); ++q) {
        const int i = tid + 256 * q;
        if (i >= L1 * FC) break;
        const int mp = i / FC, cc = i - mp * FC;
        const int64_t c = c0 + cc;
        if (c >= ncplx) continue;
        const int64_t z = 2 * (int64_t)mp + par;
        const float2 m2 = MXREG ? mxr[MXREG ? q : 0] : mx[i];
        // a ring group whose residuals are all zero (lambda below the slices at polar rings) leaves the
        // preset: its ex(0) would otherwise override the smaller exponents of the groups with data
        if (m2.x > 0.f) atomicMax(Ecol + z * ld + 2 * c, ex(m2.x));
        if (m2.y > 0.f) atomicMax(Ecol + z * ld + 2 * c + 1, ex(m2.y));
    }
}

// Few columns: one thread per (parity, m', ring, complex column), same sums.
__device__ __forceinline__ double resid_of(const double *F, int64_t off, double f, double s) {
    return (F ? F[off] : 0.0) - f * s;
}
__device__ __forceinline__ float2 resid_of(const float2 *F, int64_t off, float f, float s) {
    return df_resid(F ? F[off] : make_float2(0.f, 0.f), f, s);
}

// TF: element type of F and R (double, or the double-float pairs of the mixed transform)
template <typename T, typename TF>
__global__ void __launch_bounds__(256) k_fold_residual_narrow(const RingGeom *rings, int nrn, int rlim, int lmax,
                                                             double w, const TF *__restrict__ F,
                                                             const T *__restrict__ G, int64_t ncplx,
                                                             TF *__restrict__ R) {
    const int L1 = lmax + 1;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)2 * L1 * rlim * ncplx;     // rings r < rlim only
    if (idx >= total) return;
    const int64_t c = idx % ncplx;
    int64_t t = idx / ncplx;
    const int r = (int)(t % rlim);
    t /= rlim;
    const int mp = (int)(t % L1);
    const int par = (int)(t / L1);
    const RingGeom g = rings[r];
    const int n = g.nph;
    const int64_t ld = 2 * ncplx;
    const bool odd_phase = g.phi0_den != 0;
    const T f = (T)(w * (double)n * g.cfold);
    const int64_t off = ((int64_t)(par * L1 + mp) * nrn + r) * ld + 2 * c;
    T sx = 0, sy = 0;
    const int k = mp % n;
    const int kk = (n - k) % n;
    int tt = 0;
    for (int m = k; m <= lmax; m += n, ++tt) {
        const T *gp = G + ((int64_t)(par * L1 + m) * nrn + r) * ld + 2 * c;
        const int dt = tt - mp / n;
        const T sgn = (odd_phase && (dt & 1)) ? T(-1) : T(1);
        sx += sgn * gp[0];
        if (m != 0) sy += sgn * gp[1];
    }
    for (int m = (kk == 0 ? n : kk); m <= lmax; m += n) {
        const T *gp = G + ((int64_t)(par * L1 + m) * nrn + r) * ld + 2 * c;
        const int q = (m + mp) / n;
        const T sgn = (odd_phase && (q & 1)) ? T(-1) : T(1);
        sx += sgn * gp[0];
        sy -= sgn * gp[1];
    }
    R[off] = resid_of(F, off, f, sx);
    R[off + 1] = resid_of(F, off + 1, f, sy);
}

bool launch_gram_update_fp64(const Plan &p, const double *Acur, const double *A0, int64_t ncol, double *Anew,
                             cudaStream_t st) {
    if (!p.d_gram64) return false;
    const int maxrows = p.lmax / 2 + 1;
    dim3 grid((unsigned)((maxrows * ncol + 127) / 128), (unsigned)(2 * (p.lmax + 1)));
    switch (ncol) {
    case 2: k_gram_update_fp64<2><<<grid, 128, 0, st>>>(p.d_gram64, p.d_gram_off, p.gram_rows, p.lmax, Acur, A0, Anew); break;
    case 4: k_gram_update_fp64<4><<<grid, 128, 0, st>>>(p.d_gram64, p.d_gram_off, p.gram_rows, p.lmax, Acur, A0, Anew); break;
    case 8: k_gram_update_fp64<8><<<grid, 128, 0, st>>>(p.d_gram64, p.d_gram_off, p.gram_rows, p.lmax, Acur, A0, Anew); break;
    default: {
        dim3 wg((unsigned)((ncol + BN - 1) / BN), (unsigned)((maxrows + BM - 1) / BM), (unsigned)(2 * (p.lmax + 1)));
        k_gram_update_wide<<<wg, 256, 0, st>>>(p.d_gram64, p.d_gram_off, p.gram_rows, p.lmax, Acur, A0, ncol, Anew);
        break;
    }
    }
    note_launch();
    return true;
}

void launch_fold_residual(const Plan &p, const double *F, const double *G, int64_t ncol, double *R,
                          cudaStream_t st, int *Ecol, int rlim) {
    const int64_t ncplx = ncol / 2;
    if (rlim < 0 || rlim > p.nrn) rlim = (int)p.nrn;
    if (p.precision == SFB_MIXED && ncplx > 4) {
        // 0x80 bytes: every exponent word starts at -2139062144, below any scale exponent
        if (Ecol) cudaMemsetAsync(Ecol, 0x80, (size_t)2 * (p.lmax + 1) * ncol * sizeof(int), st);
        if (!F && rlim > 0 && rlim <= p.ral) {
            // aliased rings of the Gram refinement: residue buckets (shared memory within limits)
            constexpr int FC = 8;
            int nbk = 1;
            for (int r = 0; r < rlim; ++r) nbk = std::max(nbk, p.h_rings[r].nph);
            const bool mxreg = (p.lmax + 1) * FC <= 256 * FOLD_MXQ;
            const size_t smem = ((size_t)nbk + (mxreg ? 1 : 2) * (size_t)(p.lmax + 1)) * FC * sizeof(float2);
            if (smem <= 200 * 1024) {
                const int rpb = 8;
                dim3 grid((unsigned)((ncplx + FC - 1) / FC), 2, (unsigned)((rlim + rpb - 1) / rpb));
                const double w = 4.0 * M_PI / (double)p.npix;
                if (mxreg) {
                    set_smem(k_fold_alias<FC, true>, smem);
                    k_fold_alias<FC, true><<<grid, 256, smem, st>>>(p.d_rings, (int)p.nrn, rlim, rpb, nbk, p.lmax,
                                                                    w, (const float *)G, ncplx, (float2 *)R, Ecol);
                } else {
                    set_smem(k_fold_alias<FC, false>, smem);
                    k_fold_alias<FC, false><<<grid, 256, smem, st>>>(p.d_rings, (int)p.nrn, rlim, rpb, nbk, p.lmax,
                                                                     w, (const float *)G, ncplx, (float2 *)R, Ecol);
                }
                note_launch();
                return;
            }
        }
        dim3 grid((unsigned)((ncplx + 127) / 128), (unsigned)(2 * (p.lmax + 1)),
                  (unsigned)((rlim + FOLD_RC - 1) / FOLD_RC));
        const double w = 4.0 * M_PI / (double)p.npix;
        k_fold_cols_df<<<grid, 128, 0, st>>>(p.d_rings, (int)p.nrn, rlim, p.lmax, w, (const float2 *)F,
                                             (const float *)G, ncplx, (float2 *)R, Ecol);
        note_launch();
        return;
    }
    if (!F && ncplx > 4) {
        // FP64 Gram refinement, many columns: the aliased-ring term over rings r < rlim
        dim3 grid((unsigned)((ncplx + 127) / 128), (unsigned)(2 * (p.lmax + 1)),
                  (unsigned)((rlim + FOLD_RC - 1) / FOLD_RC));
        const double w = 4.0 * M_PI / (double)p.npix;
        if (rlim > 0)
            k_fold_cols<double><<<grid, 128, 0, st>>>(p.d_rings, (int)p.nrn, rlim, p.lmax, w, nullptr, G, ncplx, R,
                                                      nullptr);
        note_launch();
        return;
    }
    if (ncplx <= 4) {
        const int64_t total = (int64_t)2 * (p.lmax + 1) * rlim * ncplx;
        const unsigned blocks = (unsigned)((total + 255) / 256);
        const double w = 4.0 * M_PI / (double)p.npix;
        if (p.precision == SFB_MIXED)
            k_fold_residual_narrow<float, float2><<<blocks, 256, 0, st>>>(p.d_rings, (int)p.nrn, rlim, p.lmax, w,
                                                                         (const float2 *)F, (const float *)G, ncplx,
                                                                         (float2 *)R);
        else
            k_fold_residual_narrow<double, double><<<blocks, 256, 0, st>>>(p.d_rings, (int)p.nrn, rlim, p.lmax, w, F,
                                                                          G, ncplx, R);
        note_launch();
        return;
    }
    // FP64, many columns, full residual (the mixed transform returned above)
    dim3 grid((unsigned)(p.lmax + 1), (unsigned)p.nrn, 2u);
    const double w = 4.0 * M_PI / (double)p.npix;
    k_fold_residual<double><<<grid, 128, 0, st>>>(p.d_rings, (int)p.nrn, p.lmax, w, F, G, ncplx, R);
    note_launch();
}

// double -> normalised double-float pairs (the mixed transform's map format)
__global__ void k_to_df(const double *in, int64_t n, float2 *out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = in[i];
        const float h = (float)v;
        out[i] = make_float2(h, (float)(v - (double)h));
    }
}

void launch_to_df(const double *in, int64_t n, float2 *out, cudaStream_t st) {
    if (n <= 0) return;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    k_to_df<<<(unsigned)blocks, 256, 0, st>>>(in, n, out);
    note_launch();
}

__global__ void k_to_float(const double *in, int64_t n, float *out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

void launch_to_float(const double *in, int64_t n, float *out, cudaStream_t st) {
    if (n <= 0) return;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    k_to_float<<<(unsigned)blocks, 256, 0, st>>>(in, n, out);
    note_launch();
}

}  // namespace sfb
