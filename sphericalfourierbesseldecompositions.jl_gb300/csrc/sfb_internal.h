// Internal declarations of the GB300 SFB library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/sfb_gpu.h"

namespace sfb {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);

#define SFB_CUDA_TRY(expr)                                                        \
    do {                                                                          \
        cudaError_t e_ = (expr);                                                  \
        if (e_ != cudaSuccess)                                                    \
            return ::sfb::fail(SFB_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define SFB_TRY(expr)                  \
    do {                               \
        int s_ = (expr);               \
        if (s_ != SFB_OK) return s_;   \
    } while (0)

// Device error word bits (set by kernels with atomicOr, read by the host).
enum : int {
    ERR_NONFINITE_INPUT = 1,
    ERR_THETA_RANGE = 2,
    ERR_NONFINITE_OUTPUT = 4,
    ERR_TC_TIMEOUT = 8,        // a bounded mbarrier wait in a tensor-core kernel gave up
    ERR_RANGE_R = 16,          // a radius outside the shells of winweights2galweights
};

// ---------------------------------------------------------------------------
// HEALPix ring geometry of the north half (rings i = 1..2*nside, equator last)
// ---------------------------------------------------------------------------
struct RingGeom {
    int32_t nph;        // pixels on the ring
    int32_t phi0_den;   // phi of first pixel = pi / phi0_den  (0 -> phi0 = 0)
    int64_t start_n;    // first pixel of the north ring
    int64_t start_s;    // first pixel of the mirrored south ring (== start_n on the equator)
    double z;           // cos(theta) of the north ring
    double sth;         // sin(theta)
    double cfold;       // 2 for a north/south pair, 1 for the equator
};

// ---------------------------------------------------------------------------
// Device buffers owned by the plan
// ---------------------------------------------------------------------------
template <typename T>
struct DevBuf {
    T *ptr = nullptr;
    size_t n = 0;  // elements
};

struct Plan {
    int device = 0;
    // modes
    int64_t nside = 0, npix = 0, nrn = 0;  // nrn = 2*nside north rings incl. equator
    int lmax = 0, nmax = 0;
    std::vector<int64_t> lmax_n;
    int64_t npairs = 0, nlmsize = 0, lmsize = 0;
    double rmin = 0, rmax = 0;
    int niter = 3;
    int precision = SFB_FP64;
    int radial_mode = SFB_RADIAL_POLY;
    // radial basis (poly mode)
    int pieces = 1, degree = 0;
    int64_t nbasis = 0;             // pieces*(degree+1) + 2
    double radial_error = 0;
    // host copies
    std::vector<int64_t> h_spl_off;
    std::vector<RingGeom> h_rings;
    // device tables
    RingGeom *d_rings = nullptr;
    double2 *d_twtab = nullptr;     // e^{-2 pi i t / nph} for every north ring (concatenated)
    int64_t *d_twoff = nullptr;     // [nrn] offset of ring r's block in d_twtab
    double2 *d_phase = nullptr;     // [nrn][lmax+1] e^{-i m phi0(r)}
    double2 *d_wphase = nullptr;    // [nrn][lmax+1] (4 pi / npix) e^{-i m phi0(r)}
    float2 *d_twtab32 = nullptr;    // FP32 copies for the mixed-precision ring transform
    float2 *d_wphase32 = nullptr;
    // tensor-core ring DFT: per-ring sliced tables (uint2 = 4 BF16 slices of
    // w cos(pi k/n), k < 2n; equatorial rings share one), ring classes
    // (polar rings one each, then the two equatorial phase classes)
    uint2 *d_dtw = nullptr;
    int64_t *d_dtw_off = nullptr;
    int32_t *d_cls_rings = nullptr;
    int32_t *d_cls_off = nullptr;      // [n_polar + n_eq_cls + 1]
    int n_polar = 0, n_eq_cls = 0, eq_max_rings = 0;
    // B operand image of the tensor-core ring DFT: per class, column block and
    // 32-pixel chunk the four sliced twiddle planes in shared-memory layout
    // (32 KB); offsets in chunks per class, -1 where the class gathers instead
    unsigned char *d_dtimg = nullptr;
    int64_t *d_dtimg_off = nullptr;
    bool dtimg_polar = false;
    // Gram refinement (mixed precision): rings r < ral alias (nph <= 2 lmax);
    // per block z the Gram matrix of the other rings, sliced in the synthesis
    // layout with its gram_rows output rows as rings (null: not used)
    int ral = 0, gram_rows = 0;
    // field2anlm / its VJP hold the whole shell x pixel field on the device up to this many bytes
    // (0: half of the free device memory at the call), else stream it in chunks of shells
    int64_t field_max_bytes = 0;
    // tiles (l, m0, n0) of the mixed-precision projection
    int3 *d_proj_tiles = nullptr;
    int64_t n_proj_tiles = 0;
    void *d_gramts = nullptr;
    int64_t *d_gramts_off = nullptr;
    double *d_gram64 = nullptr;        // the same Gram matrices in FP64, [li][r] at d_gram_off[z] + li R + r
    int64_t *d_gram_off = nullptr;
    double *d_lam = nullptr;        // Legendre table, FP64
    float *d_lam32 = nullptr;       // the same table rounded to FP32 (mixed precision)
    void *d_lamtc = nullptr;        // split-BF16 table in tensor-core operand layout (analysis)
    int64_t *d_lamtc_off = nullptr; // [2*(lmax+1)+1] block offsets (bf16 elements)
    void *d_lamts = nullptr;        // split-BF16 table in tensor-core operand layout (synthesis)
    int64_t *d_lamts_off = nullptr;
    int2 *d_lamtc_live = nullptr;   // live chunk ranges of the analysis table [z][row tile] (one allocation
    int2 *d_lamts_live = nullptr;   // with the synthesis table's [z][ring tile]); see build_live_ranges
    unsigned char *d_dft_dead = nullptr;   // [ring pair][64-m block]: spectra no analysis chunk reads
    // ring DFT: host copies of the classes, and the A-operand image (the sliced planes of the map rows
    // of every live tile, bulk-copied by the DFT) with its per-class chunk offsets for aimg_nmaps maps
    std::vector<int32_t> h_cls_rings, h_cls_off;
    bool dft_aimg = true;
    bool dft_polar_gather = false;
    bool moments_smem = true;       // mixed deposit moments with shared-memory accumulators  // polar classes gather their twiddles (else the twiddle image)
    DevBuf<double> aimg;
    int64_t *d_aimg_off = nullptr;
    std::vector<int64_t> h_aimg_off;
    int64_t aimg_nmaps = -1;
    // second stream for the ring DFT's equatorial launch, forked from and joined to the call's stream
    cudaStream_t dft_side = nullptr;
    cudaEvent_t dft_fork = nullptr, dft_join = nullptr;
    int64_t *d_lam_off = nullptr;   // [2*(lmax+1)] offset of block (m, parity)
    int64_t lam_elems = 0;
    int64_t *d_spl_off = nullptr;
    double *d_spl_x = nullptr, *d_spl_y = nullptr, *d_spl_ypp = nullptr;
    int32_t *d_pair_l = nullptr;    // [npairs]
    int32_t *d_pair_n = nullptr;    // [npairs] 1-based n
    int64_t *d_pair_lmoff = nullptr;// unused placeholder
    int32_t *d_out_pair = nullptr;  // [nlmsize] pair index of each a_nlm
    int32_t *d_out_lm = nullptr;    // [nlmsize] l(l+1)/2+m of each a_nlm
    double *d_coef = nullptr;       // [npairs * nbasis] radial coefficients (poly mode)
    float2 *d_coefT = nullptr;      // [(lmax+1) * nbasis * nmax] the same as double-float, per l and basis
    int *d_err = nullptr;           // device error word
    // workspaces (grow on demand)
    DevBuf<double> maps;            // [nmaps_alloc * npix]
    DevBuf<double> fbuf, gbuf, rbuf;// ring Fourier buffers [2][lmax+1][nrn][2*nmaps]
    DevBuf<double> alm;             // [lmsize][2*nmaps]
    DevBuf<double> almdf;           // double-float copy of alm (float2), mixed precision
    DevBuf<double> scratch;         // galaxy/window/output staging
    DevBuf<double> scratch2;
    DevBuf<double> dep;             // sorted-deposit workspace
    DevBuf<double> ref;             // reference-map a_lm (FP64) and mean coefficients (mixed precision)
    DevBuf<double> rf, rg, rr, ralm;// workspace of the FP64 reference transform on the side stream
    DevBuf<double> almdf2, adf0;    // Gram refinement: second double-float a_lm, the first pass's copy
    DevBuf<double> ecoef;           // Gram refinement: column exponents of both a_lm sets (ints)
    DevBuf<double> erow;            // ring DFT row exponents [2][nrn][nmaps] (int)
    DevBuf<double> maps32;          // FP32 copy of FP64 maps (mixed precision, spline / dense-window paths)
    DevBuf<double> nzr64;           // FP64 many-column transform: first / last ring pair with data (2 ints)
    int64_t device_bytes = 0;
};

int grow(Plan &p, DevBuf<double> &b, size_t n);

// Count of kernels this library has launched (process-wide).
void note_launch();

// Opt a kernel into `bytes` of dynamic shared memory (only above the 48 KB
// default).  A failure is left for the caller's cudaGetLastError check.
template <typename K>
inline void set_smem(K kernel, size_t bytes) {
    if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// ---------------------------------------------------------------------------
// kernels (launch wrappers; all enqueue on `st`)
// ---------------------------------------------------------------------------
void launch_legendre_table(const Plan &p, cudaStream_t st);
// galaxies -> radial-basis x pixel maps (counting sort + register moments); writes every map element
// Sorted deposit of the catalogue into the basis maps.  With ref (mixed
// precision only) the weighted count map C is written to ref[npix], the maps
// hold D_b - mu_b C and mu[nbasis] receives mu_b; ref_ready (if given) is
// recorded on st once C is complete.
// chunk_ready / nchunks: the catalogue arrives in nchunks equal galaxy ranges,
// range c complete when chunk_ready[c] fires (keys wait per range).
// ring_live (mixed precision with a reference map): receives a device array of 4 nside - 1 ints, 1 for the
// rings that hold a galaxy; the basis maps are left unwritten on the other rings (they are zero there),
// and the ring DFT must be given the array (launch_ring_analysis_tc) so that it does not read them.
int deposit_sorted(Plan &p, const double *rtp, const double *w, int64_t ngal, double *maps, double *ref,
                   double *mu, cudaEvent_t ref_ready, cudaStream_t st, const cudaEvent_t *chunk_ready = nullptr,
                   int nchunks = 0, const int **ring_live = nullptr);

// 0-based ring (1 .. 4 nside - 1 minus one) of a RING-scheme pixel
__host__ __device__ __forceinline__ int ring_of_pixel(int64_t nside, int64_t pix) {
    const int64_t npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
    auto cap = [](int64_t q) {
        int64_t i = (int64_t)((1.0f + sqrtf(1.0f + 2.0f * (float)q)) * 0.5f);
        while (i > 1 && 2 * i * (i - 1) > q) --i;
        while (2 * (i + 1) * i <= q) ++i;
        return i;
    };
    if (pix < ncap) return (int)cap(pix) - 1;
    if (pix >= npix - ncap) return (int)(4 * nside - cap(npix - 1 - pix)) - 1;
    return (int)((pix - ncap) / (4 * nside) + nside) - 1;
}
// A[lm][2j + c] += mu[j] * rmu[lm * ldr + c] for j < nmaps; with set_col >= 0
// also A[lm][2 set_col + c] = rset[lm * ldr + c].
void launch_add_mean(double *A, int64_t ldA, int64_t nmaps, const double *mu, const double *rmu, const double *rset,
                     int64_t ldr, int64_t lmsize, int64_t set_col, cudaStream_t st);
// Mixed-precision radial projection (double-float sums; FP64 mean and window
// terms), replacing add_mean + project_poly for the data term.
void launch_coef_df(const Plan &p, const int32_t *pair_index, float2 *CT, cudaStream_t st);
void launch_project_mixed(const Plan &p, const float2 *Adf, int64_t ldA, const float2 *CT,
                          const int64_t *noff, const int32_t *pair_index, double scale, const double *mu,
                          double *smean, const double *ralm, int window_kind, const double *w_ln, double *out,
                          cudaStream_t st);
// maps[j] -= nu[j] ref with nu[j] = <maps[j], ref> / <ref, ref> (FP64, in place).
void launch_split_mean(double *maps, int64_t nmaps, int64_t npix, const double *ref, double *nu, cudaStream_t st);
// nzr (FP64): receives the first / last ring pair holding a non-zero value in any map
// (preset by the caller to a large value / -1).
// Window mixing matrix (wmix.cu): largest lmax it supports, shared memory of one CTA for the
// radial modes (l, l'), and the launch over every pair of radial modes.
constexpr int WMIX_LMAX = 128;
size_t wmix_smem_bytes(int l, int lp, int64_t nr, int neg_m);
void launch_wmix(const Plan &p, const int64_t *noff, const double *gtab, int64_t nr, double rmin, double dr,
                 const double *WT, int64_t ldW, int LW, int neg_m, double *out, size_t smem, cudaStream_t st);
// Exclusive prefix sum of n int32 counters in place; tile_sums holds scan_tile_count(n) ints.
int64_t scan_tile_count(int64_t n);
void launch_exclusive_scan(int32_t *data, int64_t n, int32_t *tile_sums, cudaStream_t st);
void launch_ring_analysis(const Plan &p, const double *maps, int64_t nmaps, double *F, cudaStream_t st,
                          int *nzr = nullptr);
void launch_ring_synthesis(const Plan &p, const double *G, int64_t nmaps, double *maps, cudaStream_t st);
// rlim: rings r < rlim (analysis: the sum; synthesis: the rings formed); -1 = all.
// nzr (many columns): the analysis sums over the ring pairs [nzr[0], nzr[1]] only.
void launch_leg_analysis(const Plan &p, const double *F, int64_t ncol, double *A, bool accumulate,
                         cudaStream_t st, int rlim = -1, const int *nzr = nullptr);
void launch_leg_synthesis(const Plan &p, const double *A, int64_t ncol, double *G, cudaStream_t st, int rlim = -1);
// FP64 Gram refinement step (any column count); false when the plan has no Gram tables
bool launch_gram_update_fp64(const Plan &p, const double *Acur, const double *A0, int64_t ncol, double *Anew,
                             cudaStream_t st);
// rlim: only rings r < rlim (-1: all); F == nullptr (Gram refinement): R = -w n cfold Fold(G)
void launch_fold_residual(const Plan &p, const double *F, const double *G, int64_t ncol, double *R, cudaStream_t st,
                          int *Ecol = nullptr, int rlim = -1);
void launch_radial_coeffs(const Plan &p, const double *gl_x, const double *pq, int Q, double *coef,
                          cudaStream_t st);
void launch_project_poly(const Plan &p, const double *A, int64_t ldA, double scale, int window_kind,
                         const double *w_ln, int64_t mask_col, const double *Awin, int64_t ldW,
                         double *out, cudaStream_t st);
void launch_to_float(const double *in, int64_t n, float *out, cudaStream_t st);
// double -> normalised double-float pairs (maps of the mixed-precision transform)
void launch_to_df(const double *in, int64_t n, float2 *out, cudaStream_t st);
// Mixed-precision ring analysis on the tensor cores (double-float maps -> double-float F).
// nzr[0..1] receives the first and last ring pair holding a non-zero map row.
// ring_live (optional): rings whose entry is 0 hold zeros in maps [0, nlive) and are not read.
int launch_ring_analysis_tc(Plan &p, const float2 *maps, int64_t nmaps, float2 *F, int *erow, int *nzr,
                            cudaStream_t st, const int *ring_live = nullptr, int64_t nlive = 0,
                            bool skip_unread = false);
uint2 dft_slices(double v, int EB);
int64_t dft_image_offsets(const Plan &p, const std::vector<int32_t> &crings, const std::vector<int32_t> &coff,
                          bool with_polar, std::vector<int64_t> &off, int &max_nch);
void launch_build_dft_image(const Plan &p, int max_nch, cudaStream_t st);
// tensor-core (tcgen05) Legendre analysis, mixed precision
int64_t tc_table_offsets(const Plan &p, std::vector<int64_t> &off);
void launch_build_lamtc(const Plan &p, const int *Ea, const int *Es, cudaStream_t st);
// F: double-float (hi, lo) per element.  Ecol: column scales of F; computed here unless scales_ready
// (the fold wrote them).
// rlim: the sum runs over the first rlim rings only (-1: all).
// Eout (optional): atomicMax of each output column's exponent per block z (preset below every exponent).
// nzr (optional, device): F is zero on the ring pairs outside [nzr[0], nzr[1]]; the sum skips them.
void launch_leg_analysis_tc(const Plan &p, const float2 *F, int64_t ncol, double *A, float2 *Adf, int *Ecol,
                            bool accumulate, cudaStream_t st, bool scales_ready = false, int rlim = -1,
                            int *Eout = nullptr, const int *nzr = nullptr);
int64_t tc_synth_table_offsets(const Plan &p, std::vector<int64_t> &off, int64_t nrn = -1);
void launch_build_lamts(const Plan &p, const int *Es, cudaStream_t st);
int build_live_ranges(Plan &p, cudaStream_t st);
// rlim: ring tiles covering the first rlim rings only (-1: all)
// Ein (optional): the column exponents of Adf per block z, as the analysis wrote them
void launch_leg_synthesis_tc(const Plan &p, const float2 *Adf, int64_t ncol, float *G, cudaStream_t st,
                             int rlim = -1, const int *Ein = nullptr);
// Gram refinement step of the mixed transform (alias-free rings):
//   Anew = A + (A0 - M A) per block, A in FP64 (A) and double-float (Adf)
void launch_gram_update(const Plan &p, const double *A, const float2 *Adf, const float2 *A0, int64_t ncol,
                        double *Anew, float2 *Adfnew, cudaStream_t st, const int *Ein = nullptr,
                        int *Eout = nullptr);
int build_gram_tables(Plan &p, cudaStream_t st);
void launch_df_to_fp64(const float2 *a, int64_t n, double *out, cudaStream_t st);
// adjoint (adjoint.cu)
void launch_halve_m(double *alm, int64_t lmsize, int64_t ncol, cudaStream_t st);
void launch_scale(double *x, int64_t n, double s, cudaStream_t st);
void launch_proj_adjoint(const Plan &p, const double *abar, const int32_t *pair_index, const int64_t *noff, int64_t b0,
                         int64_t nbc, double s, double *Abar, cudaStream_t st);
void launch_deposit_adjoint(const Plan &p, const double *rtp, int64_t ngal, const double *Dbar, int64_t b0,
                            int64_t nbc, double *dw, cudaStream_t st);
std::vector<int3> project_tiles(const std::vector<int32_t> &pair_index, int lmax, int nmax);
void launch_transpose(const double *in, int64_t rows, int64_t cols, double *out, cudaStream_t st);
void launch_check_finite(const double *x, int64_t n, int *err, cudaStream_t st);
void launch_ang2pix(int64_t nside, const double *theta, const double *phi, int64_t n, int64_t *pix,
                    cudaStream_t st);

// ---------------------------------------------------------------------------
// shared device helpers
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
// 0-based HEALPix RING pixel of (z = cos theta, phi); the HEALPix paper
// algorithm (Gorski et al. 2005).  Every operation is an explicitly rounded
// IEEE op (no FMA contraction) so the integer result matches a plain FP64
// evaluation of the same expressions, operation by operation.
__device__ __forceinline__ int64_t ang2pix_ring_z(int64_t nside, double z, double phi) {
    const double inv_halfpi = 0.63661977236758134308;  // 2/pi
    const double za = fabs(z);
    double tt = fmod(__dmul_rn(phi, inv_halfpi), 4.0);
    if (tt < 0) tt = __dadd_rn(tt, 4.0);
    if (tt >= 4.0) tt = 0.0;
    const int64_t ns = nside;
    const double dns = (double)ns;
    if (za <= 2.0 / 3.0) {
        const double temp1 = __dmul_rn(dns, __dadd_rn(0.5, tt));
        const double temp2 = __dmul_rn(__dmul_rn(dns, z), 0.75);
        const int64_t jp = (int64_t)floor(__dsub_rn(temp1, temp2));
        const int64_t jm = (int64_t)floor(__dadd_rn(temp1, temp2));
        const int64_t ir = ns + 1 + jp - jm;
        const int64_t kshift = 1 - (ir & 1);
        const int64_t t1 = jp + jm - ns + kshift + 1 + 8 * ns;
        const int64_t ip = (t1 >> 1) % (4 * ns);
        const int64_t pix = 2 * ns * (ns - 1) + (ir - 1) * 4 * ns + ip;
        // rounding at |z| = 2/3 could put ir one ring outside the belt; keep
        // the index inside the map (the oracle applies the same guard)
        return pix < 0 ? 0 : (pix >= 12 * ns * ns ? 12 * ns * ns - 1 : pix);
    }
    const double tp = __dsub_rn(tt, floor(tt));
    const double tmp = __dmul_rn(dns, __dsqrt_rn(__dmul_rn(3.0, __dsub_rn(1.0, za))));
    const int64_t jp = (int64_t)floor(__dmul_rn(tp, tmp));
    const int64_t jm = (int64_t)floor(__dmul_rn(__dsub_rn(1.0, tp), tmp));
    const int64_t ir = jp + jm + 1;
    int64_t ip = (int64_t)floor(__dmul_rn(tt, (double)ir));
    ip = ip % (4 * ir);
    if (z > 0) return 2 * ir * (ir - 1) + ip;
    return 12 * ns * ns - 2 * ir * (ir + 1) + ip;
}

// ang2pix_ring_z(nside, cos(th), ph) with the result taken from an FP32
// evaluation whenever it provably agrees: every quantity that is floored
// (tt, jp/jm arguments, ip argument) must lie farther than `margin` from an
// integer, and |z| farther than 1e-5 from 2/3.  The FP32 errors are bounded
// by about nside * 1.6e-6 (theta and phi rounded to FP32: 6e-8 relative;
// sincosf / products / fmodf: a few ulp; |phi| <= 4 pi), so margin =
// nside * 4e-6 + 1e-6 leaves a factor 2.5; 1 - |z| is formed as
// 2 sin^2(theta/2) (or 2 cos^2) to keep its relative accuracy near the
// poles.  Otherwise the FP64 path runs, so the pixel is bit-identical to
// ang2pix_ring_z.  ang2pix_ring_try returns -1 instead of running it (callers
// that collect those points for a separate FP64 pass).
// ang2pix_ring_try32 is the FP32 evaluation itself, on th32 = (float)th and
// ph32 = (float)ph, for callers that checked nside <= 2^16 and |ph| <= 4 pi.
__device__ __forceinline__ int64_t ang2pix_ring_try32(int64_t nside, float th32, float ph32) {
    {
        const float ns = (float)nside;
        const float margin = ns * 4e-6f + 1e-6f;
        auto far = [margin](float v) {
            const float f = v - floorf(v);
            return f > margin && f < 1.0f - margin;
        };
        float sn, cs;
        sincosf(th32, &sn, &cs);
        const float z = cs, za = fabsf(z);
        // phi in quarter turns, reduced to [0, 4): t - 4 floor(t / 4) rounds exactly as
        // fmodf(t, 4) (+ 4 when negative) does: the subtraction is exact for t >= 0 and a single
        // rounding of t + 4 m otherwise
        const float t4 = ph32 * 0.636619772f;
        const float tt = t4 - 4.0f * floorf(t4 * 0.25f);      // may round to 4: the margin test then falls back
        if (fabsf(za - 0.6666667f) > 1e-5f && far(tt) && tt < 4.0f - margin) {
            if (za < 0.6666667f) {
                const float temp1 = ns * (0.5f + tt), temp2 = ns * z * 0.75f;
                const float a = temp1 - temp2, b = temp1 + temp2;
                if (far(a) && far(b)) {
                    // ring and in-ring indices fit 32 bits for nside <= 2^16
                    const int n32 = (int)nside;
                    const int jp = (int)floorf(a), jm = (int)floorf(b);
                    const int ir = n32 + 1 + jp - jm;
                    const int kshift = 1 - (ir & 1);
                    const int t1 = jp + jm - n32 + kshift + 1 + 8 * n32;
                    const int ip = (int)((unsigned)(t1 >> 1) % (unsigned)(4 * n32));
                    const int64_t pix = 2 * nside * (nside - 1) + (int64_t)(ir - 1) * 4 * nside + ip;
                    if (pix >= 0 && pix < 12 * nside * nside) return pix;
                }
            } else {
                float sh, ch;
                sincosf(0.5f * th32, &sh, &ch);
                const float omz = 2.0f * (z > 0.0f ? sh * sh : ch * ch);      // 1 - |z|
                const float tp = tt - floorf(tt);
                const float tmp = ns * sqrtf(3.0f * omz);
                const float a = tp * tmp, b = (1.0f - tp) * tmp;
                if (far(a) && far(b)) {
                    const int ir = (int)floorf(a) + (int)floorf(b) + 1;
                    const float q = tt * (float)ir;
                    if (far(q)) {
                        const int ip = (int)((unsigned)floorf(q) % (unsigned)(4 * ir));
                        const int64_t ir64 = ir;
                        return z > 0.0f ? 2 * ir64 * (ir64 - 1) + ip : 12 * nside * nside - 2 * ir64 * (ir64 + 1) + ip;
                    }
                }
            }
        }
    }
    return -1;
}

__device__ __forceinline__ int64_t ang2pix_ring_try(int64_t nside, double th, double ph) {
    if (nside <= (int64_t(1) << 16) && fabs(ph) <= 4.0 * M_PI) return ang2pix_ring_try32(nside, (float)th, (float)ph);
    return -1;
}

__device__ __forceinline__ int64_t ang2pix_ring_fast(int64_t nside, double th, double ph) {
    const int64_t pix = ang2pix_ring_try(nside, th, ph);
    return pix >= 0 ? pix : ang2pix_ring_z(nside, cos(th), ph);
}

// Cubic spline with boundary extrapolation on knots x[0..N-1]
// (reference src/Splines.jl:64-101,327-357).
__device__ __forceinline__ double spline_eval_dev(const double *x, const double *y, const double *ypp,
                                                  int64_t N, double r) {
    if (r < x[0]) return y[0];
    if (r > x[N - 1]) return y[N - 1];
    // largest i with x[i] <= r, clamped to the last piece
    int64_t lo = 0, hi = N - 1;
    while (hi - lo > 1) {
        int64_t mid = (lo + hi) >> 1;
        if (r >= x[mid]) lo = mid; else hi = mid;
    }
    const int64_t i = lo;
    const double x0 = x[i];
    const double h = x[i + 1] - x0;
    const double t = (r - x0) / h;
    const double h2 = h * h;
    const double b = h2 * ypp[i] / 2;
    const double a = h2 * (ypp[i + 1] - ypp[i]) / 6;
    const double d = y[i];
    const double c = y[i + 1] - a - b - d;
    return d + t * (c + t * (b + t * a));
}
#endif

}  // namespace sfb
