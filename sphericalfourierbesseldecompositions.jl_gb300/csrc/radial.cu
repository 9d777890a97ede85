// Galaxy deposit, radial basis and radial projection kernels.
//
// cat2amln (reference src/cat2anlm.jl:257-310) forms, for every (n,l),
//   map_nl[p] = sum_{i in p} w_i g_nl(r_i) / (nbar dOmega) - W[p,l,n]
// and keeps row l of map2alm(map_nl).  map2alm is linear, so with
//   g_nl(r) ~= sum_b C[nl][b] phi_b(r)      (piecewise Legendre basis phi_b)
// the galaxy term becomes sum_b C[nl][b] map2alm(D_b) / (nbar dOmega) with
// D_b[p] = sum_{i in p} w_i phi_b(r_i): one transform per basis function
// instead of one per (n,l).  Galaxies below rmin / above rmax use the
// spline's boundary extrapolation (src/Splines.jl:72-77) through two
// constant basis maps.
#include <vector>

#include "sfb_internal.h"

namespace sfb {

__device__ __forceinline__ bool galaxy_ok(double r, double th, double ph, double w, int *err) {
    if (!(isfinite(r) && isfinite(th) && isfinite(ph) && isfinite(w))) {
        atomicOr(err, ERR_NONFINITE_INPUT);
        return false;
    }
    if (th < 0.0 || th > M_PI) {
        atomicOr(err, ERR_THETA_RANGE);
        return false;
    }
    return true;
}

// Spline mode: maps[q][pix] += w * g_{pair0+q}(r) / (nbar dOmega) for a chunk of pairs.
__global__ void k_deposit_spline(const double *__restrict__ rtp, const double *__restrict__ wgt, int64_t ngal,
                                 int64_t nside, int64_t npix, const int64_t *spl_off, const double *sx,
                                 const double *sy, const double *sypp, int64_t pair0, int64_t npair_chunk,
                                 double scale, double *__restrict__ maps, int *err) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ngal) return;
    const double r = rtp[3 * i], th = rtp[3 * i + 1], ph = rtp[3 * i + 2];
    const double w = wgt ? wgt[i] : 1.0;
    if (!galaxy_ok(r, th, ph, w, err)) return;
    const int64_t pix = ang2pix_ring_fast(nside, th, ph);
    for (int64_t q = blockIdx.y; q < npair_chunk; q += gridDim.y) {
        const int64_t pr = pair0 + q;
        const int64_t o = spl_off[pr], N = spl_off[pr + 1] - o;
        const double g = spline_eval_dev(sx + o, sy + o, sypp + o, N, r);
        atomicAdd(maps + q * npix + pix, w * g * scale);
    }
}

void launch_deposit_spline_chunk(const Plan &p, const double *rtp, const double *w, int64_t ngal,
                                 int64_t pair0, int64_t npc, double scale, double *maps, cudaStream_t st) {
    if (ngal <= 0 || npc <= 0) return;
    unsigned gy = (unsigned)(npc < 64 ? npc : 64);
    dim3 grid((unsigned)((ngal + 255) / 256), gy);
    k_deposit_spline<<<grid, 256, 0, st>>>(rtp, w, ngal, p.nside, p.npix, p.d_spl_off, p.d_spl_x, p.d_spl_y,
                                           p.d_spl_ypp, pair0, npc, scale, maps, p.d_err);
                                           note_launch();
}

// maps[q][p] -= dense[p + npix*(l + (lmax+1)*(n-1))] for the chunk's pairs.
__global__ void k_subtract_dense(double *maps, const double *dense, int64_t npix, int lmax, const int32_t *pair_n,
                                 const int32_t *pair_l, int64_t pair0, int64_t npc) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t q = blockIdx.y;
    if (p >= npix || q >= npc) return;
    const int64_t pr = pair0 + q;
    const int64_t off = npix * ((int64_t)pair_l[pr] + (int64_t)(lmax + 1) * (pair_n[pr] - 1));
    maps[q * npix + p] -= dense[off + p];
}

void launch_subtract_dense_chunk(const Plan &p, double *maps, const double *dense, int64_t pair0, int64_t npc,
                                 cudaStream_t st) {
    if (npc <= 0) return;
    dim3 grid((unsigned)((p.npix + 255) / 256), (unsigned)npc);
    k_subtract_dense<<<grid, 256, 0, st>>>(maps, dense, p.npix, p.lmax, p.d_pair_n, p.d_pair_l, pair0, npc);
    note_launch();
}

// maps[q][p] -= mask[p] * W_ln[l + (lmax+1)(n-1)] for the chunk's pairs (separable window).
__global__ void k_subtract_sep(double *maps, const double *mask, const double *w_ln, int64_t npix, int lmax,
                               const int32_t *pair_n, const int32_t *pair_l, int64_t pair0, int64_t npc) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t q = blockIdx.y;
    if (p >= npix || q >= npc) return;
    const int64_t pr = pair0 + q;
    const double wl = w_ln[pair_l[pr] + (int64_t)(lmax + 1) * (pair_n[pr] - 1)];
    maps[q * npix + p] -= mask[p] * wl;
}

void launch_subtract_sep_chunk(const Plan &p, double *maps, const double *mask, const double *w_ln, int64_t pair0,
                               int64_t npc, cudaStream_t st) {
    if (npc <= 0) return;
    dim3 grid((unsigned)((p.npix + 255) / 256), (unsigned)npc);
    k_subtract_sep<<<grid, 256, 0, st>>>(maps, mask, w_ln, p.npix, p.lmax, p.d_pair_n, p.d_pair_l, pair0, npc);
    note_launch();
}

__global__ void k_axpy(double *y, const double *x, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] += x[i];
}

void launch_axpy(double *y, const double *x, int64_t n, cudaStream_t st) {
    if (n <= 0) return;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    k_axpy<<<(unsigned)blocks, 256, 0, st>>>(y, x, n);
    note_launch();
}

// Gather dense window maps of a chunk of pairs: maps[q] = W[:, l, n].
__global__ void k_gather_dense(double *maps, const double *dense, int64_t npix, int lmax, const int32_t *pair_n,
                               const int32_t *pair_l, int64_t pair0, int64_t npc) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t q = blockIdx.y;
    if (p >= npix || q >= npc) return;
    const int64_t pr = pair0 + q;
    const int64_t off = npix * ((int64_t)pair_l[pr] + (int64_t)(lmax + 1) * (pair_n[pr] - 1));
    maps[q * npix + p] = dense[off + p];
}

void launch_gather_dense_chunk(const Plan &p, double *maps, const double *dense, int64_t pair0, int64_t npc,
                               cudaStream_t st) {
    if (npc <= 0) return;
    dim3 grid((unsigned)((p.npix + 255) / 256), (unsigned)npc);
    k_gather_dense<<<grid, 256, 0, st>>>(maps, dense, p.npix, p.lmax, p.d_pair_n, p.d_pair_l, pair0, npc);
    note_launch();
}

// Radial coefficients: C[pair][j*(deg+1)+k] = sum_q PQ[q][k] * g(r_q), with
// r_q the Gauss-Legendre nodes of piece j and PQ[q][k] = w_q (2k+1)/2 P_k(x_q)
// (L2 projection of the spline onto Legendre polynomials on each piece);
// C[pair][nbasis-2] / [nbasis-1] = first / last knot value (extrapolation).
__global__ void k_radial_coeffs(const int64_t *spl_off, const double *sx, const double *sy, const double *sypp,
                                double rmin, double rmax, int pieces, int deg, int64_t nbasis, const double *glx,
                                const double *pq, int Q, double *coef) {
    extern __shared__ double gq[];
    const int64_t pr = blockIdx.x;
    const int j = blockIdx.y;
    const int64_t o = spl_off[pr], N = spl_off[pr + 1] - o;
    const double width = (rmax - rmin) / pieces;
    const double a = rmin + j * width;
    for (int q = threadIdx.x; q < Q; q += blockDim.x) {
        const double r = a + (glx[q] + 1.0) * 0.5 * width;
        gq[q] = spline_eval_dev(sx + o, sy + o, sypp + o, N, r);
    }
    __syncthreads();
    for (int k = threadIdx.x; k <= deg; k += blockDim.x) {
        double acc = 0.0;
        for (int q = 0; q < Q; ++q) acc = fma(pq[(int64_t)q * (deg + 1) + k], gq[q], acc);
        coef[pr * nbasis + (int64_t)j * (deg + 1) + k] = acc;
    }
    if (j == 0 && threadIdx.x == 0) {
        coef[pr * nbasis + nbasis - 2] = sy[o];
        coef[pr * nbasis + nbasis - 1] = sy[o + N - 1];
    }
}

void launch_radial_coeffs(const Plan &p, const double *gl_x, const double *pq, int Q, double *coef,
                          cudaStream_t st) {
    dim3 grid((unsigned)p.npairs, (unsigned)p.pieces);
    k_radial_coeffs<<<grid, 128, Q * sizeof(double), st>>>(p.d_spl_off, p.d_spl_x, p.d_spl_y, p.d_spl_ypp, p.rmin,
                                                          p.rmax, p.pieces, p.degree, p.nbasis, gl_x, pq, Q, coef);
                                                          note_launch();
}

// max over knots of |expansion - y| / max|y| per pair; atomicMax on the bit
// pattern (non-negative doubles order like their bits).
__global__ void k_radial_error(const int64_t *spl_off, const double *sx, const double *sy, const double *ymax,
                               double rmin, double rmax, int pieces, int deg, int64_t nbasis, const double *coef,
                               unsigned long long *err_bits) {
    const int64_t pr = blockIdx.x;
    const int64_t o = spl_off[pr], N = spl_off[pr + 1] - o;
    const double width = (rmax - rmin) / pieces;
    const double *C = coef + pr * nbasis;
    double worst = 0.0;
    // interior knots only: within a few knots of rmin/rmax the reference
    // spline carries its parabolic end-slope error, which no smooth expansion
    // (and no radial resolution below the knot spacing) can follow
    for (int64_t i = 8 + threadIdx.x; i < N - 8; i += blockDim.x) {
        const double r = sx[o + i];
        if (r < rmin || r > rmax) continue;
        int j = (int)((r - rmin) / width);
        if (j >= pieces) j = pieces - 1;
        double x = 2.0 * (r - (rmin + j * width)) / width - 1.0;
        x = fmin(1.0, fmax(-1.0, x));
        const double *Cj = C + (int64_t)j * (deg + 1);
        double p0 = 1.0, p1 = x, v = Cj[0] + (deg >= 1 ? Cj[1] * x : 0.0);
        for (int k = 1; k < deg; ++k) {
            const double p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
            v = fma(Cj[k + 1], p2, v);
            p0 = p1;
            p1 = p2;
        }
        worst = fmax(worst, fabs(v - sy[o + i]));
    }
    worst /= ymax[pr] > 0 ? ymax[pr] : 1.0;
    atomicMax(err_bits, (unsigned long long)__double_as_longlong(worst));
}

void launch_radial_error_impl(const Plan &p, const double *coef, const double *ymax, unsigned long long *err_bits,
                              cudaStream_t st) {
    k_radial_error<<<(unsigned)p.npairs, 128, 0, st>>>(p.d_spl_off, p.d_spl_x, p.d_spl_y, ymax, p.rmin, p.rmax,
                                                       p.pieces, p.degree, p.nbasis, coef, err_bits);
                                                       note_launch();
}

// a_nlm = scale * sum_b C[pair][b] A[lm][b] - window term.
template <typename TA>
__global__ void k_project_poly(const int32_t *out_pair, const int32_t *out_lm, const int32_t *pair_n,
                               const int32_t *pair_l, int64_t nlmsize, int64_t nbasis, const double *coef,
                               const TA *__restrict__ A, int64_t ldA, double scale, int window_kind,
                               const double *w_ln, int lmax, int64_t mask_col, double *out) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nlmsize) return;
    const int pr = out_pair[o];
    const int64_t lm = out_lm[o];
    const double *C = coef + (int64_t)pr * nbasis;
    const TA *Ar = A + lm * ldA;
    double re = 0.0, im = 0.0;
    for (int64_t b = 0; b < nbasis; ++b) {
        const double c = C[b];
        re = fma(c, (double)Ar[2 * b], re);
        im = fma(c, (double)Ar[2 * b + 1], im);
    }
    re *= scale;
    im *= scale;
    if (window_kind == SFB_WINDOW_SEPARABLE) {
        const double wl = w_ln[pair_l[pr] + (int64_t)(lmax + 1) * (pair_n[pr] - 1)];
        re -= wl * (double)Ar[2 * mask_col];
        im -= wl * (double)Ar[2 * mask_col + 1];
    }
    out[2 * o] = re;
    out[2 * o + 1] = im;
}

void launch_project_poly(const Plan &p, const double *A, int64_t ldA, double scale, int window_kind,
                         const double *w_ln, int64_t mask_col, const double *Awin, int64_t ldW, double *out,
                         cudaStream_t st) {
    (void)Awin; (void)ldW;
    if (p.nlmsize <= 0) return;
    // a_lm are held in FP64 in both precision modes
    k_project_poly<double><<<(unsigned)((p.nlmsize + 127) / 128), 128, 0, st>>>(
            p.d_out_pair, p.d_out_lm, p.d_pair_n, p.d_pair_l, p.nlmsize, p.nbasis, p.d_coef, A, ldA, scale,
            window_kind, w_ln, p.lmax, mask_col, out);
        note_launch();
}

// out[o] -= Awin[lm][pair - pair0] for outputs whose pair lies in the chunk.
__global__ void k_sub_window_chunk(const int32_t *out_pair, const int32_t *out_lm, int64_t nlmsize,
                                   const double *Awin, int64_t ldW, int64_t pair0, int64_t npc, double *out) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nlmsize) return;
    const int64_t q = (int64_t)out_pair[o] - pair0;
    if (q < 0 || q >= npc) return;
    const double *a = Awin + (int64_t)out_lm[o] * ldW + 2 * q;
    out[2 * o] -= a[0];
    out[2 * o + 1] -= a[1];
}

void launch_sub_window_chunk(const Plan &p, const double *Awin, int64_t ldW, int64_t pair0, int64_t npc, double *out,
                             cudaStream_t st) {
    if (p.nlmsize <= 0) return;
    k_sub_window_chunk<<<(unsigned)((p.nlmsize + 127) / 128), 128, 0, st>>>(p.d_out_pair, p.d_out_lm, p.nlmsize, Awin,
                                                                           ldW, pair0, npc, out);
                                                                           note_launch();
}

// Spline mode: out[o] = A[lm][pair - pair0] (map already scaled and window-subtracted).
__global__ void k_extract_spline(const int32_t *out_pair, const int32_t *out_lm, int64_t nlmsize, const double *A,
                                 int64_t ldA, int64_t pair0, int64_t npc, double *out) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nlmsize) return;
    const int64_t q = (int64_t)out_pair[o] - pair0;
    if (q < 0 || q >= npc) return;
    const double *a = A + (int64_t)out_lm[o] * ldA + 2 * q;
    out[2 * o] = a[0];
    out[2 * o + 1] = a[1];
}

void launch_extract_spline_chunk(const Plan &p, const double *A, int64_t ldA, int64_t pair0, int64_t npc, double *out,
                                 cudaStream_t st) {
    if (p.nlmsize <= 0) return;
    k_extract_spline<<<(unsigned)((p.nlmsize + 127) / 128), 128, 0, st>>>(p.d_out_pair, p.d_out_lm, p.nlmsize, A, ldA,
                                                                         pair0, npc, out);
                                                                         note_launch();
}

// gtab[pair][s] = g_pair(r_s) * (with_r2dr ? r_s^2 dr : 1), r_s = rmin + (s+1/2) dr.
__global__ void k_gtab(const int64_t *spl_off, const double *sx, const double *sy, const double *sypp,
                       int64_t npairs, int64_t nr, double rmin, double dr, int with_r2dr, double *gtab) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nr) return;
    const double r = rmin + dr / 2 + s * dr;
    for (int64_t pr = blockIdx.y; pr < npairs; pr += gridDim.y) {      // grid y is capped at 65535
        const int64_t o = spl_off[pr], N = spl_off[pr + 1] - o;
        double g = spline_eval_dev(sx + o, sy + o, sypp + o, N, r);
        if (with_r2dr) g *= r * r * dr;
        gtab[pr * nr + s] = g;
    }
}

void launch_gtab(const Plan &p, int64_t nr, double rmin, double dr, int with_r2dr, double *gtab, cudaStream_t st) {
    dim3 grid((unsigned)((nr + 127) / 128), (unsigned)std::min<int64_t>(p.npairs, 65535));
    k_gtab<<<grid, 128, 0, st>>>(p.d_spl_off, p.d_spl_x, p.d_spl_y, p.d_spl_ypp, p.npairs, nr, rmin, dr, with_r2dr,
                                 gtab);
                                 note_launch();
}

// field2anlm radial sum: out[o] = sum_s gtab[pair][s] A[lm][s]  (src/cat2anlm.jl:347-353)
__global__ void k_project_shells(const int32_t *out_pair, const int32_t *out_lm, int64_t nlmsize, const double *gtab,
                                 int64_t nr, const double *__restrict__ A, int64_t ldA, double *out) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nlmsize) return;
    const double *g = gtab + (int64_t)out_pair[o] * nr;
    const double *Ar = A + (int64_t)out_lm[o] * ldA;
    double re = 0.0, im = 0.0;
    for (int64_t s = 0; s < nr; ++s) {
        re = fma(g[s], Ar[2 * s], re);
        im = fma(g[s], Ar[2 * s + 1], im);
    }
    out[2 * o] = re;
    out[2 * o + 1] = im;
}

void launch_project_shells_g(const Plan &p, const double *gtab, int64_t nr, const double *A, int64_t ldA, double *out,
                             cudaStream_t st) {
    if (p.nlmsize <= 0) return;
    k_project_shells<<<(unsigned)((p.nlmsize + 127) / 128), 128, 0, st>>>(p.d_out_pair, p.d_out_lm, p.nlmsize, gtab, nr,
                                                                         A, ldA, out);
                                                                         note_launch();
}

// anlm2field radial sum: A[lm][s] = sum_n gtab[pair(n,l)][s] a[idx(n,l,m)] (src/cat2anlm.jl:403-414)
__global__ void k_shell_alm(const int32_t *pair_index, const int64_t *noff, int nmax, int lmax, const double *gtab,
                            int64_t nr, const double *anlm, double *A, int64_t ldA) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nr) return;
    const int64_t lmsize = (int64_t)(lmax + 1) * (lmax + 2) / 2;
    for (int64_t lm = blockIdx.y; lm < lmsize; lm += gridDim.y) {        // grid y is capped at 65535
        // recover (l, m) from lm = l(l+1)/2 + m
        int l = (int)((sqrt(8.0 * (double)lm + 1.0) - 1.0) / 2.0);
        while ((int64_t)(l + 1) * (l + 2) / 2 <= lm) ++l;
        while ((int64_t)l * (l + 1) / 2 > lm) --l;
        const int m = (int)(lm - (int64_t)l * (l + 1) / 2);
        double re = 0.0, im = 0.0;
        for (int n = 1; n <= nmax; ++n) {
            const int pr = pair_index[(int64_t)(n - 1) * (lmax + 1) + l];
            if (pr < 0) continue;
            const int64_t idx = noff[n - 1] + (int64_t)l * (l + 1) / 2 + m;
            const double g = gtab[(int64_t)pr * nr + s];
            re = fma(g, anlm[2 * idx], re);
            im = fma(g, anlm[2 * idx + 1], im);
        }
        A[lm * ldA + 2 * s] = re;
        A[lm * ldA + 2 * s + 1] = (m == 0) ? 0.0 : im;
    }
}

void launch_shell_alm_g(const Plan &p, const int32_t *pair_index, const int64_t *noff, const double *gtab, int64_t nr,
                        const double *anlm, double *A, int64_t ldA, cudaStream_t st) {
    dim3 grid((unsigned)((nr + 127) / 128), (unsigned)std::min<int64_t>(p.lmsize, 65535));
    k_shell_alm<<<grid, 128, 0, st>>>(pair_index, noff, p.nmax, p.lmax, gtab, nr, anlm, A, ldA);
    note_launch();
}

// W_ln[l + (lmax+1)(n-1)] = sum_s gtab[pair][s] phi[s]  (gtab includes r^2 dr); NaN off-mode.
__global__ void k_win_sep(const int32_t *pair_n, const int32_t *pair_l, int64_t npairs, const double *gtab, int64_t nr,
                          const double *phi, int lmax, double *out) {
    const int64_t pr = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (pr >= npairs) return;
    double acc = 0.0;
    for (int64_t s = 0; s < nr; ++s) acc += gtab[pr * nr + s] * phi[s];
    out[pair_l[pr] + (int64_t)(lmax + 1) * (pair_n[pr] - 1)] = acc;
}

void launch_win_sep_g(const Plan &p, const double *gtab, int64_t nr, const double *phi, double *out, cudaStream_t st) {
    k_win_sep<<<(unsigned)((p.npairs + 127) / 128), 128, 0, st>>>(p.d_pair_n, p.d_pair_l, p.npairs, gtab, nr, phi,
                                                                  p.lmax, out);
                                                                  note_launch();
}

// Dense: W[p + npix(l + (lmax+1)(n-1))] = sum_s win[s + nr p] gtab[pair][s]
__global__ void k_win_dense(const int32_t *pair_n, const int32_t *pair_l, int64_t npairs, const double *gtab, int64_t nr,
                            const double *win, int64_t npix, int lmax, double *out) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const double *wc = win + p * nr;
    for (int64_t pr = blockIdx.y; pr < npairs; pr += gridDim.y) {      // grid y is capped at 65535
        const double *g = gtab + pr * nr;
        double acc = 0.0;
        for (int64_t s = 0; s < nr; ++s) acc += wc[s] * g[s];
        out[p + npix * ((int64_t)pair_l[pr] + (int64_t)(lmax + 1) * (pair_n[pr] - 1))] = acc;
    }
}

void launch_win_dense_g(const Plan &p, const double *gtab, int64_t nr, const double *win, double *out, cudaStream_t st) {
    dim3 grid((unsigned)((p.npix + 127) / 128), (unsigned)std::min<int64_t>(p.npairs, 65535));
    k_win_dense<<<grid, 128, 0, st>>>(p.d_pair_n, p.d_pair_l, p.npairs, gtab, nr, win, p.npix, p.lmax, out);
    note_launch();
}

// amln2clnn (src/SphericalFourierBesselDecompositions.jl:114-150): one warp per
// (l, n1, n2) column of lnn (3 x nlnn, 1-based n), over nbatch coefficient vectors:
// C = [Re(a1_0 a2_0) + 2 sum_{m>=1} Re(a1_m conj(a2_m))] / (2l + 1).
__global__ void k_amln2clnn(const double *__restrict__ a1, const double *__restrict__ a2, int64_t nlmsize,
                            const int64_t *__restrict__ lnn, int64_t nlnn, int64_t nbatch, const int64_t *noff,
                            double *__restrict__ out) {
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wid >= nlnn * nbatch) return;
    const int64_t b = wid / nlnn, i = wid - b * nlnn;
    const int64_t l = lnn[3 * i], n1 = lnn[3 * i + 1], n2 = lnn[3 * i + 2];
    const double *x = a1 + 2 * (b * nlmsize + noff[n1 - 1] + l * (l + 1) / 2);
    const double *y = a2 + 2 * (b * nlmsize + noff[n2 - 1] + l * (l + 1) / 2);
    double c = 0.0;
    for (int64_t m = lane; m <= l; m += 32) {
        const double xr = x[2 * m], xi = x[2 * m + 1], yr = y[2 * m], yi = y[2 * m + 1];
        c += (m == 0) ? (xr * yr - xi * yi) : 2.0 * (xr * yr + xi * yi);
    }
    for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
    if (lane == 0) out[b * nlnn + i] = c / (double)(2 * l + 1);
}

void launch_amln2clnn(const double *a1, const double *a2, int64_t nlmsize, const int64_t *lnn, int64_t nlnn,
                      int64_t nbatch, const int64_t *noff, double *out, cudaStream_t st) {
    const int64_t threads = nlnn * nbatch * 32;
    if (threads <= 0) return;
    k_amln2clnn<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(a1, a2, nlmsize, lnn, nlnn, nbatch, noff, out);
    note_launch();
}

// winweights2galweights (src/cat2anlm.jl:218-238): w_i = weights[bin(r_i), pix(theta_i, phi_i)]
// with bin = nr if r == rmax, else searchsortedlast(rbounds, r) (1-based), over
// the caller's rbounds[0..nr].  Out-of-range bins set ERR_RANGE_R and give NaN.
__global__ void k_winweights(const double *__restrict__ weights, int64_t nr, int64_t npix, int64_t nside,
                             const double *__restrict__ rbounds, double rmax, const double *__restrict__ rtp,
                             int64_t ngal, double *__restrict__ w, int *err) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ngal) return;
    const double r = rtp[3 * i], th = rtp[3 * i + 1], ph = rtp[3 * i + 2];
    if (!(isfinite(r) && isfinite(th) && isfinite(ph))) {
        atomicOr(err, ERR_NONFINITE_INPUT);
        w[i] = NAN;
        return;
    }
    const int64_t pix = ang2pix_ring_fast(nside, th, ph);
    int64_t bin;
    if (r == rmax) {
        bin = nr;
    } else {
        // largest 1-based j with rbounds[j] <= r (0 if none)
        int64_t lo = 0, hi = nr + 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (rbounds[mid] <= r) lo = mid + 1; else hi = mid;
        }
        bin = lo;
    }
    if (bin < 1 || bin > nr) {
        atomicOr(err, ERR_RANGE_R);
        w[i] = NAN;
        return;
    }
    w[i] = weights[(bin - 1) + nr * pix];
}

void launch_winweights(const double *weights, int64_t nr, int64_t nside, const double *rbounds, double rmax,
                       const double *rtp, int64_t ngal, double *w, int *err, cudaStream_t st) {
    if (ngal <= 0) return;
    k_winweights<<<(unsigned)((ngal + 255) / 256), 256, 0, st>>>(weights, nr, 12 * nside * nside, nside, rbounds, rmax,
                                                                 rtp, ngal, w, err);
    note_launch();
}

__global__ void k_add_mean(double *__restrict__ A, int64_t ldA, int64_t ncol, int64_t nmaps,
                           const double *__restrict__ mu, const double *__restrict__ rmu,
                           const double *__restrict__ rset, int64_t ldr, int64_t lmsize, int64_t set_col) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= lmsize * ncol) return;
    const int64_t lm = e / ncol, j = e - lm * ncol;
    if (j < nmaps) {
        double *a = A + lm * ldA + 2 * j;
        const double m = mu[j];
        a[0] = fma(m, rmu[lm * ldr], a[0]);
        a[1] = fma(m, rmu[lm * ldr + 1], a[1]);
    } else {
        double *a = A + lm * ldA + 2 * set_col;
        a[0] = rset[lm * ldr];
        a[1] = rset[lm * ldr + 1];
    }
}

void launch_add_mean(double *A, int64_t ldA, int64_t nmaps, const double *mu, const double *rmu, const double *rset,
                     int64_t ldr, int64_t lmsize, int64_t set_col, cudaStream_t st) {
    const int64_t ncol = nmaps + (set_col >= 0 ? 1 : 0);
    const int64_t n = lmsize * ncol;
    if (n <= 0) return;
    k_add_mean<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(A, ldA, ncol, nmaps, mu, rmu, rset, ldr, lmsize, set_col);
    note_launch();
}

// ---- mixed-precision radial projection ---------------------------------------
// Double-float helpers (FP32 pairs, ~48 significant bits).
struct df2 {
    float hi, lo;
};
__device__ __forceinline__ df2 dfa(df2 a, df2 b) {
    const float s = a.hi + b.hi;
    const float z = s - a.hi;
    const float e = ((a.hi - (s - z)) + (b.hi - z)) + (a.lo + b.lo);
    const float h = s + e;
    return {h, e - (h - s)};
}
__device__ __forceinline__ df2 dfm(df2 a, df2 b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    const float h = p + e;
    return {h, e - (h - p)};
}

// CT[(l * nbasis + b) * nmax + n - 1] = coef[pair(n, l)][b] as hi + lo (0 where (n, l) is not a mode).
__global__ void k_coef_df(const double *__restrict__ coef, const int32_t *__restrict__ pair_index, int lmax, int nmax,
                          int64_t nbasis, float2 *__restrict__ CT) {
    const int64_t total = (int64_t)(lmax + 1) * nbasis * nmax;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int n1 = (int)(i % nmax);
        const int64_t t = i / nmax;
        const int64_t b = t % nbasis;
        const int l = (int)(t / nbasis);
        const int pr = pair_index[(int64_t)n1 * (lmax + 1) + l];
        const double v = pr >= 0 ? coef[(int64_t)pr * nbasis + b] : 0.0;
        const float h = (float)v;
        CT[i] = make_float2(h, (float)(v - (double)h));
    }
}

void launch_coef_df(const Plan &p, const int32_t *pair_index, float2 *CT, cudaStream_t st) {
    k_coef_df<<<1024, 256, 0, st>>>(p.d_coef, pair_index, p.lmax, (int)p.nmax, p.nbasis, CT);
    note_launch();
}

// s[pair] = sum_b coef[pair][b] mu_b (FP64): the mean part of every pair, one
// warp per pair (lanes over b, coalesced rows).
__global__ void k_mean_proj(const double *__restrict__ coef, int64_t npairs, int64_t nbasis,
                            const double *__restrict__ mu, double *__restrict__ s) {
    const int64_t pr = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (pr >= npairs) return;
    double a = 0.0;
    for (int64_t b = lane; b < nbasis; b += 32) a = fma(coef[pr * nbasis + b], mu[b], a);
    for (int off = 16; off > 0; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
    if (lane == 0) s[pr] = a;
}

// Tiles of the projection: block (l, m0, n0, npt) of the plan's tile list
// covers m = m0 .. m0 + 31 (lane = m) and n = n0 + 1 .. n0 + npt (npt <= 8
// accumulators per thread); its PJ_KS warps split the basis range and add
// their partial sums at the end:
//   a_nlm = scale * sum_b coef[n,l][b] dA_b[lm]              (double-float)
//         + scale * s[pair] * C_lm - w_ln(l, n) * M_lm        (FP64)
// with dA the fluctuation a_lm (double-float copy, row lm of width ldA, the
// pairs re, im of basis b side by side), C_lm / M_lm the FP64 a_lm of the
// count map / the mask (ralm [lm][4]); the mean and window terms are skipped
// when ralm is null / window_kind is not separable.  The coefficient rows CT
// (per (l, b) contiguous in n) are read through L1, each load a broadcast to
// the warp.  The products are formed exactly (TwoProd) and summed with
// TwoSum into the high word; the low word gathers the rounding errors and the
// cross terms, unnormalised until the end.
constexpr int PJ_NPT = 8, PJ_KS = 4;

struct pacc {
    float hi, lo;
};

__device__ __forceinline__ void pj_mac(pacc &a, float2 c, float xh, float xl) {
    const float p = c.x * xh;
    const float e = fmaf(c.x, xh, -p);
    const float s = a.hi + p;
    const float z = s - a.hi;
    const float err = (a.hi - (s - z)) + (p - z);
    a.hi = s;
    a.lo = fmaf(c.y, xh, fmaf(c.x, xl, (a.lo + err) + e));
}

template <int KS>
__global__ void __launch_bounds__(32 * KS) k_project_mixed(const float2 *__restrict__ Adf, int64_t ldA,
                                                              int64_t nbasis, const float2 *__restrict__ CT, int nmax,
                                                              int lmax, const int3 *__restrict__ tiles,
                                                              const int64_t *__restrict__ noff,
                                                              const int32_t *__restrict__ pair_index, double scale,
                                                              const double *__restrict__ smean,
                                                              const double *__restrict__ ralm, int window_kind,
                                                              const double *__restrict__ w_ln,
                                                              double *__restrict__ out) {
    __shared__ float4 part[KS - 1][PJ_NPT][32];
    const int3 t = tiles[blockIdx.x];
    const int l = t.x, m0 = t.y, n0 = t.z & 0xffff, npt = t.z >> 16;
    const int lane = threadIdx.x & 31, ks = threadIdx.x >> 5;
    const int m = m0 + lane;
    const bool live = m <= l;
    const int64_t lm = (int64_t)l * (l + 1) / 2 + (live ? m : l);      // lanes past l read a valid row
    const int64_t kper = (nbasis + KS - 1) / KS;
    const int64_t kb0 = ks * kper, kb1 = kb0 + kper < nbasis ? kb0 + kper : nbasis;
    const float4 *arow = reinterpret_cast<const float4 *>(Adf + lm * ldA);
    const float2 *Cl = CT + (int64_t)l * nbasis * nmax + n0;
    pacc re[PJ_NPT], im[PJ_NPT];
#pragma unroll
    for (int j = 0; j < PJ_NPT; ++j) re[j] = im[j] = pacc{0.f, 0.f};
#pragma unroll 2
    for (int64_t b = kb0; b < kb1; ++b) {
        const float4 a = arow[b];                 // re.hi, re.lo, im.hi, im.lo
        const float2 *cb = Cl + b * nmax;
#pragma unroll
        for (int j = 0; j < PJ_NPT; ++j) {
            if (j < npt) {
                const float2 c = __ldg(cb + j);
                pj_mac(re[j], c, a.x, a.y);
                pj_mac(im[j], c, a.z, a.w);
            }
        }
    }
    if (ks > 0) {
#pragma unroll
        for (int j = 0; j < PJ_NPT; ++j) part[ks - 1][j][lane] = make_float4(re[j].hi, re[j].lo, im[j].hi, im[j].lo);
    }
    __syncthreads();
    if (ks > 0 || !live) return;
#pragma unroll
    for (int j = 0; j < PJ_NPT; ++j) {
        const int n1 = n0 + j;
        if (j >= npt) break;
        const int pr = pair_index[(int64_t)n1 * (lmax + 1) + l];
        if (pr < 0) continue;
        // the parts added in double-float (FP32 units), one conversion to FP64
        df2 sr = df2{re[j].hi, re[j].lo}, si = df2{im[j].hi, im[j].lo};
#pragma unroll
        for (int q = 0; q < KS - 1; ++q) {
            const float4 v = part[q][j][lane];
            sr = dfa(sr, df2{v.x, v.y});
            si = dfa(si, df2{v.z, v.w});
        }
        double vr = scale * ((double)sr.hi + (double)sr.lo);
        double vi = scale * ((double)si.hi + (double)si.lo);
        if (ralm) {
            const double mu = scale * smean[pr];
            vr = fma(mu, ralm[4 * lm], vr);
            vi = fma(mu, ralm[4 * lm + 1], vi);
            if (window_kind == SFB_WINDOW_SEPARABLE) {
                const double wl = w_ln[l + (int64_t)(lmax + 1) * n1];
                vr = fma(-wl, ralm[4 * lm + 2], vr);
                vi = fma(-wl, ralm[4 * lm + 3], vi);
            }
        }
        const int64_t o = noff[n1] + lm;
        out[2 * o] = vr;
        out[2 * o + 1] = vi;
    }
}

// Tile list of the projection: (l, m0, n0 | npt << 16) for m0 = 0, 32, .. <= l
// and n0 = 0, 8, .. below the number of radial modes of l (the valid n form a
// prefix), npt = the modes left from n0 (at most 8).
std::vector<int3> project_tiles(const std::vector<int32_t> &pair_index, int lmax, int nmax) {
    std::vector<int3> t;
    for (int l = 0; l <= lmax; ++l) {
        int nl = 0;
        while (nl < nmax && pair_index[(size_t)nl * (lmax + 1) + l] >= 0) ++nl;
        for (int m0 = 0; m0 <= l; m0 += 32)
            for (int n0 = 0; n0 < nl; n0 += PJ_NPT)
                t.push_back(make_int3(l, m0, n0 | (std::min(PJ_NPT, nl - n0) << 16)));
    }
    return t;
}

void launch_project_mixed(const Plan &p, const float2 *Adf, int64_t ldA, const float2 *CT,
                          const int64_t *noff, const int32_t *pair_index, double scale, const double *mu,
                          double *smean, const double *ralm, int window_kind, const double *w_ln, double *out,
                          cudaStream_t st) {
    if (ralm) {
        k_mean_proj<<<(unsigned)((p.npairs + 3) / 4), 128, 0, st>>>(p.d_coef, p.npairs, p.nbasis, mu, smean);
        note_launch();
    }
    if (p.n_proj_tiles <= 0) return;
    k_project_mixed<PJ_KS><<<(unsigned)p.n_proj_tiles, 32 * PJ_KS, 0, st>>>(
        Adf, ldA, p.nbasis, CT, (int)p.nmax, p.lmax, p.d_proj_tiles, noff, pair_index, scale, smean, ralm, window_kind,
        w_ln, out);
    note_launch();
}

// One block per map: nu = <m, ref> / <ref, ref>, then m -= nu ref.
__global__ void __launch_bounds__(512) k_split_mean(double *maps, int64_t npix, const double *__restrict__ ref,
                                                    double *nu) {
    __shared__ double red[2][16];
    double *m = maps + (int64_t)blockIdx.x * npix;
    double d = 0.0, q = 0.0;
    for (int64_t p = threadIdx.x; p < npix; p += blockDim.x) {
        const double r = ref[p];
        d = fma(m[p], r, d);
        q = fma(r, r, q);
    }
    for (int off = 16; off > 0; off >>= 1) {
        d += __shfl_xor_sync(0xffffffffu, d, off);
        q += __shfl_xor_sync(0xffffffffu, q, off);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        red[0][wid] = d;
        red[1][wid] = q;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double dd = 0.0, qq = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            dd += red[0][w];
            qq += red[1][w];
        }
        red[0][0] = qq > 0.0 ? dd / qq : 0.0;
        nu[blockIdx.x] = red[0][0];
    }
    __syncthreads();
    const double v = red[0][0];
    for (int64_t p = threadIdx.x; p < npix; p += blockDim.x) m[p] = fma(-v, ref[p], m[p]);
}

void launch_split_mean(double *maps, int64_t nmaps, int64_t npix, const double *ref, double *nu, cudaStream_t st) {
    if (nmaps <= 0) return;
    k_split_mean<<<(unsigned)nmaps, 512, 0, st>>>(maps, npix, ref, nu);
    note_launch();
}

__global__ void k_fill(double *x, int64_t n, double v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = v;
}

void launch_fill(double *x, int64_t n, double v, cudaStream_t st) {
    if (n <= 0) return;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    k_fill<<<(unsigned)blocks, 256, 0, st>>>(x, n, v);
    note_launch();
}

}  // namespace sfb

namespace sfb {

// w00[s] = Re a_00 of map s of an FP64 a_lm set (row lm = 0, columns 2 s / 2 s + 1)
__global__ void k_extract_a00(const double *alm, int64_t nm, double *w00) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nm) w00[s] = alm[2 * s];
}

void launch_extract_a00(const double *alm, int64_t ldA, int64_t nm, double *w00, cudaStream_t st) {
    (void)ldA;
    k_extract_a00<<<(unsigned)((nm + 127) / 128), 128, 0, st>>>(alm, nm, w00);
    note_launch();
}

// win_lnn radial integrals (reference calc_intr_gg_fn, src/windows.jl:394-422, trapezoidal
// nodes = shell midpoints, weights = dr, f = W00 / sqrt(4 pi)): one warp per column i of lnn,
//   out[i] = sum_s (g_nl(r_s) r_s sqrt(dr) sqrt(f_s)) (g_n'l(r_s) r_s sqrt(dr) sqrt(f_s)).
__global__ void k_win_lnn(const int32_t *__restrict__ pair_index, int lmax, const double *__restrict__ gtab,
                          int64_t nr, double rmin, double dr, const double *__restrict__ w00,
                          const int64_t *__restrict__ lnn, int64_t nlnn, double *__restrict__ out) {
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nlnn) return;
    const int64_t l = lnn[3 * i], n1 = lnn[3 * i + 1], n2 = lnn[3 * i + 2];
    const double *g1 = gtab + (int64_t)pair_index[(n1 - 1) * (lmax + 1) + l] * nr;
    const double *g2 = gtab + (int64_t)pair_index[(n2 - 1) * (lmax + 1) + l] * nr;
    const double sdr = sqrt(dr), inv4pi = 1.0 / sqrt(4.0 * M_PI);
    double acc = 0.0;
    for (int64_t s = lane; s < nr; s += 32) {
        const double r = rmin + dr / 2 + s * dr;                 // the shell midpoints of k_gtab
        const double w = r * sdr * sqrt(w00[s] * inv4pi);
        acc = fma(g1[s] * w, g2[s] * w, acc);
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (lane == 0) out[i] = acc;
}

void launch_win_lnn(const Plan &p, const int32_t *pair_index, const double *gtab, int64_t nr, double rmin, double dr,
                    const double *w00, const int64_t *lnn, int64_t nlnn, double *out, cudaStream_t st) {
    k_win_lnn<<<(unsigned)((nlnn * 32 + 127) / 128), 128, 0, st>>>(pair_index, p.lmax, gtab, nr, rmin, dr, w00, lnn,
                                                                    nlnn, out);
    note_launch();
}

}  // namespace sfb
