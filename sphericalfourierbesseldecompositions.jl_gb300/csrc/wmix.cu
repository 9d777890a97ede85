// Window mixing matrix (reference calc_wmix, src/windows.jl:299-366, with
// calc_wmix_ii :273-296 and calc_gaunts_L :451-465):
//   W[(n l m), (n' l' m')] = (-1)^m sum_L G(l, l', L; -m, m') H_{nl,n'l'}(L, m - m'),
//   H(L, M) = sum_s g_nl(r_s) g_n'l'(r_s) r_s^2 dr W_LM(r_s),
//   G = sqrt((2L+1)(2l+1)(2l'+1) / 4 pi) (l l' L; 0 0 0) (L l l'; M -m m'),
// for m = 0..l (or m = -0..-l with neg_m) and m' = 0..l', W_LM(r_s) the a_lm of
// window shell s to lmax 2 lmax and W_{L,-M} = (-1)^M conj(W_LM).
//
// One CTA per pair of radial modes (P, P'): the shell products g g' r^2 dr go
// to shared memory, one warp per needed (L, |M|) forms H (lanes over the
// shells, coalesced rows of the shell-major window harmonics, which stay in
// L2), then one thread per (m, m') forms its 3j family over L and the sum.
//
// The 3j families come from the three-term recursion in j1 of Schulten and
// Gordon (J. Math. Phys. 16, 1961, 1975): with m1 = -m2 - m3,
//   j A(j+1) f(j+1) + B(j) f(j) + (j+1) A(j) f(j-1) = 0,
//   A(j) = sqrt((j^2 - (j2-j3)^2)((j2+j3+1)^2 - j^2)(j^2 - m1^2)),
//   B(j) = -(2j+1)(j2(j2+1) m1 - j3(j3+1) m1 - j(j+1)(m3 - m2)),
// run forward from j1min while |f| grows (the classically forbidden low end)
// and backward from j1max down to that point (Luscombe and Luban, Phys. Rev. E
// 57, 7274, 1998), scaled to meet, normalised by sum (2j+1) f^2 = 1 with the
// sign of f(j1max) equal to (-1)^(j2 - j3 - m1).
#include "sfb_internal.h"

namespace sfb {

namespace {

constexpr int WMIX_MAXF = 2 * WMIX_LMAX + 1;   // longest 3j family

__device__ __forceinline__ double w3j_A(int j, int j2, int j3, int m1) {
    const double a = (double)j * j - (double)(j2 - j3) * (j2 - j3);
    const double b = (double)(j2 + j3 + 1) * (j2 + j3 + 1) - (double)j * j;
    const double c = (double)j * j - (double)m1 * m1;
    const double v = a * b * c;
    return v > 0.0 ? sqrt(v) : 0.0;
}

__device__ __forceinline__ double w3j_B(int j, int j2, int j3, int m2, int m3, int m1) {
    return -(2.0 * j + 1.0) * ((double)j2 * (j2 + 1) * m1 - (double)j3 * (j3 + 1) * m1 -
                               (double)j * (j + 1) * (m3 - m2));
}

// f[i] = (j1min + i, j2, j3; m1, m2, m3), m1 = -m2 - m3; returns j1min, *nf the count
__device__ int w3j_family(int j2, int j3, int m2, int m3, double *f, int *nf) {
    const int m1 = -m2 - m3;
    const int jmin = max(abs(j2 - j3), abs(m1)), jmax = j2 + j3;
    if (abs(m2) > j2 || abs(m3) > j3 || jmin > jmax) {
        *nf = 0;
        return jmin;
    }
    const int n = jmax - jmin + 1;
    *nf = n;
    if (n == 1) {
        f[0] = 1.0;
    } else {
        int k = 0;
        if (jmin > 0) {
            double prv = 0.0, cur = 1.0;
            f[0] = 1.0;
            while (k + 1 < n) {
                const int j = jmin + k;
                const double nx = -(w3j_B(j, j2, j3, m2, m3, m1) * cur + (j + 1) * w3j_A(j, j2, j3, m1) * prv) /
                                  (j * w3j_A(j + 1, j2, j3, m1));
                if (fabs(nx) <= fabs(cur)) break;
                f[k + 1] = nx;
                prv = cur;
                cur = nx;
                ++k;
            }
        }
        // backward from jmax down to index k (nothing to do when the forward values grew to jmax)
        const double fk = f[k];
        double nxt = 0.0, cur = 1.0;
        if (k < n - 1) f[n - 1] = 1.0;
        for (int i = n - 1; i > k; --i) {
            const int j = jmin + i;
            const double pv = -(w3j_B(j, j2, j3, m2, m3, m1) * cur + j * w3j_A(j + 1, j2, j3, m1) * nxt) /
                              ((j + 1) * w3j_A(j, j2, j3, m1));
            nxt = cur;
            cur = pv;
            if (i - 1 > k) f[i - 1] = pv;
            else {
                // index k: scale the forward part (if any) to meet the backward value
                if (k > 0) {
                    const double sc = pv / fk;
                    for (int q = 0; q < k; ++q) f[q] *= sc;
                }
                f[k] = pv;
            }
        }
    }
    double nrm = 0.0;
    for (int i = 0; i < n; ++i) nrm += (2.0 * (jmin + i) + 1.0) * f[i] * f[i];
    double s = 1.0 / sqrt(nrm);
    const int want = ((j2 - j3 - m1) % 2 + 2) % 2 ? -1 : 1;
    if ((f[n - 1] < 0.0 ? -1 : 1) != want) s = -s;
    for (int i = 0; i < n; ++i) f[i] *= s;
    return jmin;
}

__global__ void __launch_bounds__(256) k_wmix(const int32_t *__restrict__ pair_n, const int32_t *__restrict__ pair_l,
                                              int64_t npairs, const int64_t *__restrict__ noff,
                                              const double *__restrict__ gtab, int64_t nr, double rmin, double dr,
                                              const double *__restrict__ WT, int64_t ldW, int LW, int neg_m,
                                              int64_t nlmsize, double *__restrict__ out) {
    extern __shared__ double sm[];
    const int64_t P = blockIdx.x, Q = blockIdx.y;
    const int l = pair_l[P], n = pair_n[P], lp = pair_l[Q], np = pair_n[Q];
    const int Lmin = abs(l - lp), Lmax = l + lp;
    const int nL = Lmax - Lmin + 1;
    const int Mmax = neg_m ? l + lp : max(l, lp);
    double *gg = sm;                               // [nr]
    double *w000 = gg + nr;                        // [nL]
    double2 *H = reinterpret_cast<double2 *>(w000 + ((nL + 1) & ~1));   // [nL][Mmax + 1]
    const double *g1 = gtab + P * nr, *g2 = gtab + Q * nr;
    for (int64_t s = threadIdx.x; s < nr; s += blockDim.x) {
        const double r = rmin + dr / 2 + s * dr;
        gg[s] = g1[s] * g2[s] * (r * r * dr);
    }
    if (threadIdx.x == 0) {
        int nf = 0;
        double f[WMIX_MAXF];
        const int j0 = w3j_family(l, lp, 0, 0, f, &nf);
        for (int i = 0; i < nL; ++i) {
            const int L = Lmin + i;
            w000[i] = (L >= j0 && L - j0 < nf) ? f[L - j0] : 0.0;
        }
    }
    __syncthreads();
    // H(L, M) for L of the parity l + l' + L even, 0 <= M <= min(L, Mmax): one warp per entry
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int ncols = Mmax + 1;
    for (int e = warp; e < nL * ncols; e += nw) {
        const int iL = e / ncols, M = e - iL * ncols;
        const int L = Lmin + iL;
        double2 h = make_double2(0.0, 0.0);
        if (((l + lp + L) & 1) == 0 && M <= L && L <= LW) {
            const double *w = WT + ((int64_t)L * (L + 1) / 2 + M) * ldW;     // [s][re, im]
            double hr = 0.0, hi = 0.0;
            for (int64_t s = lane; s < nr; s += 32) {
                hr = fma(gg[s], w[2 * s], hr);
                hi = fma(gg[s], w[2 * s + 1], hi);
            }
            for (int off = 16; off > 0; off >>= 1) {
                hr += __shfl_xor_sync(0xffffffffu, hr, off);
                hi += __shfl_xor_sync(0xffffffffu, hi, off);
            }
            h = make_double2(hr, hi);
        }
        if (lane == 0) H[e] = h;
    }
    __syncthreads();
    // one thread per (m, m'): consecutive threads take consecutive m (consecutive output rows)
    const double pref = (2.0 * l + 1.0) * (2.0 * lp + 1.0) / (4.0 * M_PI);
    const int64_t ibase = noff[n - 1] + (int64_t)l * (l + 1) / 2;
    const int64_t jbase = noff[np - 1] + (int64_t)lp * (lp + 1) / 2;
    double f[WMIX_MAXF];
    for (int t = threadIdx.x; t < (l + 1) * (lp + 1); t += blockDim.x) {
        const int mp = t / (l + 1), am = t - mp * (l + 1);
        const int m = neg_m ? -am : am;
        const int M = m - mp;
        int nf = 0;
        const int j0 = w3j_family(l, lp, -m, mp, f, &nf);      // (L l l'; M, -m, m')
        double wr = 0.0, wi = 0.0;
        const int aM = abs(M);
        for (int i = 0; i < nL; ++i) {
            const int L = Lmin + i;
            if (((l + lp + L) & 1) || L < j0 || L - j0 >= nf || aM > L) continue;
            const double gnt = sqrt((2.0 * L + 1.0) * pref) * w000[i] * f[L - j0];
            const double2 h = H[i * ncols + aM];
            wr = fma(gnt, h.x, wr);
            wi = fma(gnt, h.y, wi);
        }
        if (M < 0) {                                // W_{L,-|M|} = (-1)^M conj(W_{L,|M|})
            const double sg = (aM & 1) ? -1.0 : 1.0;
            wr *= sg;
            wi *= -sg;
        }
        const double sm_ = (abs(m) & 1) ? -1.0 : 1.0;   // (-1)^m
        double *o = out + 2 * ((ibase + am) + nlmsize * (jbase + mp));
        o[0] = sm_ * wr;
        o[1] = sm_ * wi;
    }
}

}  // namespace

size_t wmix_smem_bytes(int l, int lp, int64_t nr, int neg_m) {
    const int nL = 2 * min(l, lp) + 1;
    const int Mmax = neg_m ? l + lp : max(l, lp);
    return (size_t)(nr + ((nL + 1) & ~1)) * sizeof(double) + (size_t)nL * (Mmax + 1) * sizeof(double2);
}

void launch_wmix(const Plan &p, const int64_t *noff, const double *gtab, int64_t nr, double rmin, double dr,
                 const double *WT, int64_t ldW, int LW, int neg_m, double *out, size_t smem, cudaStream_t st) {
    set_smem(k_wmix, smem);
    dim3 grid((unsigned)p.npairs, (unsigned)p.npairs);
    k_wmix<<<grid, 256, smem, st>>>(p.d_pair_n, p.d_pair_l, p.npairs, noff, gtab, nr, rmin, dr, WT, ldW, LW, neg_m,
                                    p.nlmsize, out);
    note_launch();
}

}  // namespace sfb
