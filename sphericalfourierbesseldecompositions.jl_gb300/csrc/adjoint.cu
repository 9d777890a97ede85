// Adjoint (vector-Jacobian products) of the transforms, FP64: the transpose
// of map2alm with niter refinement, of the radial projection and of the
// deposit, for gradients of a loss through cat2amln (dL/dw_i) and
// field2anlm (dL/dfield).
//
// With A = analysis (weighted ring DFT, then Legendre analysis) and S =
// synthesis (Legendre synthesis, then inverse ring DFT), map2alm with niter
// refinements is  a = sum_{j=0}^{niter} (I - A S)^j A f.  As real-linear maps
// (re and im parts of a_lm as separate coordinates) A^T = w S E and
// S^T = (1/w) E^-1 A, w = 4 pi / npix, E = 1 for m = 0 and 1/2 for m >= 1
// (the synthesis counts the m >= 1 terms twice), so
//   f_bar = w S sum_{j=0}^{niter} (I - A S)^j (E a_bar),
// evaluated as x <- b + x - A S x (niter times, from x = b = E a_bar) with
// the same synthesis, aliasing fold and analysis kernels as the forward
// refinement.  Reference: the transforms are those of src/cat2anlm.jl:257-357
// (cat2amln, field2anlm_v2) around src/healpix_helpers.jl:50-56 (map2alm).
#include <algorithm>
#include <cmath>

#include "sfb_internal.h"

namespace sfb {

// alm[lm][c] *= 1/2 for m >= 1 (E above); lm = l (l+1)/2 + m
__global__ void k_halve_m(double *alm, int64_t lmsize, int64_t ncol) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= lmsize * ncol) return;
    const int64_t lm = i / ncol;
    int l = (int)((sqrt(8.0 * (double)lm + 1.0) - 1.0) * 0.5);
    while ((int64_t)(l + 1) * (l + 2) / 2 <= lm) ++l;
    while ((int64_t)l * (l + 1) / 2 > lm) --l;
    if (lm - (int64_t)l * (l + 1) / 2 >= 1) alm[i] *= 0.5;
}

__global__ void k_scale(double *x, int64_t n, double s) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= s;
}

// Transpose of the radial projection a_nlm = s sum_b c[pair(n,l)][b] A_b[lm]:
//   Abar[lm][2b + t] = s sum_n c[pair(n,l)][b] abar[noff(n) + lm][t]   (t = re, im)
// for the basis functions b in [b0, b0 + nbc).
__global__ void k_proj_adjoint(const double *__restrict__ abar, const double *__restrict__ coef, int64_t nbasis,
                               const int32_t *__restrict__ pair_index, const int64_t *__restrict__ noff, int lmax,
                               int nmax, int64_t lmsize, int64_t b0, int64_t nbc, double s,
                               double *__restrict__ Abar) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= lmsize * nbc) return;
    const int64_t lm = i / nbc, b = b0 + (i - lm * nbc);
    int l = (int)((sqrt(8.0 * (double)lm + 1.0) - 1.0) * 0.5);
    while ((int64_t)(l + 1) * (l + 2) / 2 <= lm) ++l;
    while ((int64_t)l * (l + 1) / 2 > lm) --l;
    double re = 0.0, im = 0.0;
    for (int n1 = 0; n1 < nmax; ++n1) {
        const int pr = pair_index[(int64_t)n1 * (lmax + 1) + l];
        if (pr < 0) continue;
        const double c = coef[(int64_t)pr * nbasis + b];
        const int64_t o = noff[n1] + lm;
        re = fma(c, abar[2 * o], re);
        im = fma(c, abar[2 * o + 1], im);
    }
    Abar[lm * (2 * nbc) + 2 * (b - b0)] = s * re;
    Abar[lm * (2 * nbc) + 2 * (b - b0) + 1] = s * im;
}

// Transpose of the deposit for the basis functions [b0, b0 + nbc):
//   dw[i] += sum_{b in range} phi_b(r_i) Dbar_b[pix(i)]
// with phi_b the piecewise Legendre basis of the deposit (P_k on the galaxy's
// piece, the constants outside [rmin, rmax]); galaxies are keyed exactly as
// the deposit keys them.
__global__ void k_deposit_adjoint(const double *__restrict__ rtp, int64_t ngal, int64_t nside, int64_t npix,
                                  double rmin, double rmax, double inv_width, int pieces, int deg, int64_t nbasis,
                                  const double *__restrict__ Dbar, int64_t b0, int64_t nbc, double *__restrict__ dw,
                                  int *err) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ngal) return;
    const double r = rtp[3 * i], th = rtp[3 * i + 1], ph = rtp[3 * i + 2];
    if (!(isfinite(r) && isfinite(th) && isfinite(ph))) {
        atomicOr(err, ERR_NONFINITE_INPUT);
        return;
    }
    if (th < 0.0 || th > M_PI) {
        atomicOr(err, ERR_THETA_RANGE);
        return;
    }
    const int64_t pix = ang2pix_ring_fast(nside, th, ph);
    double acc = 0.0;
    if (r < rmin || r > rmax) {
        const int64_t b = nbasis - 2 + (r < rmin ? 0 : 1);
        if (b >= b0 && b < b0 + nbc) acc = Dbar[(b - b0) * npix + pix];
    } else {
        const double u = (r - rmin) * inv_width;
        int slot = (int)u;
        if (slot >= pieces) slot = pieces - 1;
        double x = 2.0 * (u - (double)slot) - 1.0;
        x = fmin(1.0, fmax(-1.0, x));
        const int64_t bs = (int64_t)slot * (deg + 1);
        double p0 = 1.0, p1 = x;
        for (int k = 0; k <= deg; ++k) {
            const double pk = k == 0 ? 1.0 : k == 1 ? x : 0.0;
            double v = pk;
            if (k >= 2) {
                // (k) P_k = (2k - 1) x P_{k-1} - (k - 1) P_{k-2}
                v = ((double)(2 * k - 1) * x * p1 - (double)(k - 1) * p0) / (double)k;
                p0 = p1;
                p1 = v;
            }
            const int64_t b = bs + k;
            if (b >= b0 && b < b0 + nbc) acc = fma(v, Dbar[(b - b0) * npix + pix], acc);
        }
    }
    dw[i] += acc;
}

void launch_halve_m(double *alm, int64_t lmsize, int64_t ncol, cudaStream_t st) {
    const int64_t n = lmsize * ncol;
    if (n <= 0) return;
    k_halve_m<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(alm, lmsize, ncol);
    note_launch();
}

void launch_scale(double *x, int64_t n, double s, cudaStream_t st) {
    if (n <= 0) return;
    k_scale<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(x, n, s);
    note_launch();
}

void launch_proj_adjoint(const Plan &p, const double *abar, const int32_t *pair_index, const int64_t *noff, int64_t b0,
                         int64_t nbc, double s, double *Abar, cudaStream_t st) {
    const int64_t n = p.lmsize * nbc;
    if (n <= 0) return;
    k_proj_adjoint<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(abar, p.d_coef, p.nbasis, pair_index, noff, p.lmax,
                                                                (int)p.nmax, p.lmsize, b0, nbc, s, Abar);
    note_launch();
}

void launch_deposit_adjoint(const Plan &p, const double *rtp, int64_t ngal, const double *Dbar, int64_t b0,
                            int64_t nbc, double *dw, cudaStream_t st) {
    if (ngal <= 0) return;
    k_deposit_adjoint<<<(unsigned)((ngal + 255) / 256), 256, 0, st>>>(
        rtp, ngal, p.nside, p.npix, p.rmin, p.rmax, (double)p.pieces / (p.rmax - p.rmin), p.pieces, p.degree,
        p.nbasis, Dbar, b0, nbc, dw, p.d_err);
    note_launch();
}

}  // namespace sfb
