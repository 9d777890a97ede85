/*
 * sfb_gpu.h - C ABI of the GB300 catalogue -> spherical Fourier-Bessel path.
 *
 * Drop-in for SuperFaB's Cat2Anlm functions.  Every array argument is a
 * plain pointer with Julia's memory layout (column-major, 1-based indices in
 * the reference become 0-based offsets here); no PyTorch or CUDA types appear
 * in the signatures.  Complex outputs are interleaved (re, im) doubles, which
 * is the memory layout of Julia's Vector{ComplexF64}.
 *
 * Every entry point returns an sfb_status; sfb_last_error() gives the text of
 * the last failure on the calling thread.  Nothing is printed.  There is no
 * CPU fallback: without a usable CUDA device every compute call fails with
 * SFB_ECUDA.
 */
#ifndef SFB_GPU_H
#define SFB_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SFB_OK = 0,
    SFB_EINVAL = 1,      /* bad argument (reference: ArgumentError / @assert) */
    SFB_ENOMEM = 2,      /* device allocation failed */
    SFB_ENONFINITE = 3,  /* non-finite input or result (reference src/cat2anlm.jl:308) */
    SFB_ERANGE = 4,      /* theta outside [0, pi] or lmax > 4*nside (reference src/healpix_helpers.jl:51-54) */
    SFB_ETIMEOUT = 5,    /* a bounded device wait gave up */
    SFB_ECUDA = 6,       /* CUDA runtime error (no device, launch failure) */
    SFB_ENOTSUP = 7      /* combination of options not implemented */
} sfb_status;

typedef enum {
    SFB_FP64 = 0,        /* every stage in FP64 */
    SFB_MIXED = 1        /* FP64 binning/tables/window term, FP32 ring FFT, tensor-core contractions */
} sfb_precision;

/* Element type of a shell x pixel field (sfb_field2anlm_typed and its VJP). */
typedef enum {
    SFB_F64 = 0,         /* double (Julia Matrix{Float64}) */
    SFB_F32 = 1          /* float (Julia Matrix{Float32}) */
} sfb_dtype;

typedef enum {
    /* Galaxy radii enter through a piecewise-Legendre expansion of every
     * g_nl spline (projection error below radial_tol); the spherical-harmonic
     * transforms run once per radial basis function. */
    SFB_RADIAL_POLY = 0,
    /* Every galaxy evaluates every g_nl spline, one map per (n,l) as in the
     * reference loop (src/cat2anlm.jl:278-306).  Cost grows as N * #(n,l). */
    SFB_RADIAL_SPLINE = 1
} sfb_radial_mode;

/* Plan description: the contents of an AnlmModes (reference src/modes.jl:92-105)
 * plus the transform options.  All host pointers; copied at plan creation. */
typedef struct {
    int64_t nside;             /* HEALPix resolution of the transform */
    int64_t lmax;              /* AnlmModes.lmax */
    int64_t nmax;              /* AnlmModes.nmax */
    const int64_t *lmax_n;     /* [nmax] AnlmModes.lmax_n */
    double rmin, rmax;         /* AnlmModes.rmin / rmax */
    /* Cubic splines of amodes.basisfunctions.gnl[n,l+1] (Splines.jl Spline1D{3}:
     * fields x, y, ypp) for every pair (n,l), l <= lmax_n[n], in the a_nlm block
     * order (n slowest, then l).  Spline p occupies [spl_offset[p], spl_offset[p+1]). */
    const int64_t *spl_offset; /* [npairs + 1] */
    const double *spl_x;
    const double *spl_y;
    const double *spl_ypp;
    int32_t niter;             /* map2alm refinement iterations (3 in mymap2alm!) */
    int32_t precision;         /* sfb_precision */
    int32_t radial_mode;       /* sfb_radial_mode */
    int32_t radial_pieces;     /* SFB_RADIAL_POLY: number of pieces, 0 = automatic */
    int32_t radial_degree;     /* SFB_RADIAL_POLY: Legendre degree per piece, 0 = automatic */
    double radial_tol;         /* SFB_RADIAL_POLY: max |g - expansion| / max|g|, 0 = 1e-11 */
} sfb_plan_desc;

/* win_rhat_ln argument of cat2amln (reference src/windows.jl:244-270). */
typedef enum {
    SFB_WINDOW_ZERO = 0,       /* all-zero window term */
    SFB_WINDOW_SEPARABLE = 1,  /* SeparableArray(mask[npix], W_ln[lmax+1, nmax]) */
    SFB_WINDOW_DENSE = 2       /* Array W[npix, lmax+1, nmax] (column-major) */
} sfb_window_kind;

typedef struct {
    int32_t kind;              /* sfb_window_kind */
    const double *mask;        /* [npix] RING order (separable) */
    const double *w_ln;        /* [(lmax+1) * nmax], element (l,n) at l + (lmax+1)*(n-1) */
    const double *dense;       /* [npix * (lmax+1) * nmax], element (p,l,n) at p + npix*(l + (lmax+1)*(n-1)) */
} sfb_window;

typedef struct sfb_plan sfb_plan;

typedef struct {
    int64_t npix;
    int64_t nlmsize;           /* getnlmsize(amodes), reference src/modes.jl:183-189 */
    int64_t npairs;            /* number of (n,l) pairs */
    int64_t nbasis;            /* radial basis functions (maps per catalogue SHT) */
    int32_t radial_pieces;
    int32_t radial_degree;
    double radial_error;       /* measured max projection error / max|g| (poly mode) */
    int64_t device_bytes;      /* device memory held by the plan */
} sfb_plan_info;

/* Create a plan on the current CUDA device.
 * Replaces the per-call setup of cat2amln (src/cat2anlm.jl:257-276). */
int sfb_plan_create(const sfb_plan_desc *desc, sfb_plan **plan);
void sfb_plan_destroy(sfb_plan *plan);
int sfb_plan_get_info(const sfb_plan *plan, sfb_plan_info *info);
int sfb_set_precision(sfb_plan *plan, int32_t precision);

/* cat2amln(rθϕ, amodes, nbar, win_rhat_ln, weight) -> a_nlm
 * (reference src/cat2anlm.jl:257-310; alias cat2nlm :312).
 * rtp: [3*ngal] host array, galaxy i at (r, theta, phi) = rtp[3i..3i+2]
 * (a Julia 3xN Matrix{Float64}).  weight: [ngal] or NULL for ones.
 * ngal may be 0 (empty catalogue).  anlm_out: [2*nlmsize] interleaved complex.
 * Inputs are not modified. */
int sfb_cat2amln(sfb_plan *plan, const double *rtp, const double *weight, int64_t ngal,
                 double nbar, const sfb_window *window, double *anlm_out);

/* Batched mocks: nmocks catalogues sharing one plan and one window (the
 * per-mock loop a caller of cat2amln runs over mock catalogues, reference
 * src/cat2anlm.jl:257-310 per mock).  Mock k is galaxies
 * [offsets[k], offsets[k+1]) of rtp (3 x offsets[nmocks], as in sfb_cat2amln)
 * and weight (NULL for ones), with nbar[k].  anlm_out: [nmocks][2*nlmsize].
 * The next mock's catalogue is copied while the current one is transformed;
 * errors of any mock are reported once for the batch. */
int sfb_cat2amln_batched(sfb_plan *plan, const double *rtp, const double *weight, const int64_t *offsets,
                         int64_t nmocks, const double *nbar, const sfb_window *window, double *anlm_out);

/* Same as sfb_cat2amln with every pointer (rtp, weight, window arrays and
 * anlm_out) in device memory, launched on `stream` (cudaStream_t or NULL for
 * the legacy default stream).  Returns after the result is complete. */
int sfb_cat2amln_device(sfb_plan *plan, const double *rtp, const double *weight, int64_t ngal,
                        double nbar, const sfb_window *window, double *anlm_out, void *stream);

/* Adjoints (vector-Jacobian products), FP64, no reference counterpart (the
 * reference's transforms are libsharp calls without derivatives): for a real
 * loss L of the coefficients, abar = dL/dRe(a) + i dL/dIm(a) per coefficient
 * ([2*nlmsize] interleaved, the a_nlm layout).
 *
 * sfb_cat2amln_vjp: dL/dw_i for the galaxy weights of sfb_cat2amln
 * (rtp as there, the plan's radial basis; needs SFB_RADIAL_POLY); the window
 * term does not depend on the weights.  dw_out: [ngal]. */
int sfb_cat2amln_vjp(sfb_plan *plan, const double *rtp, int64_t ngal, double nbar, const double *abar,
                     double *dw_out);

/* dL/df for sfb_field2anlm: df_out [nr * npix], element (ir, p) at ir + nr*p. */
int sfb_field2anlm_vjp(sfb_plan *plan, const double *abar, int64_t nr, double rmin, double rmax, double *df_out);

/* Transpose of sfb_map2alm (niter refinement included): abar [nmaps][lmsize]
 * complex (map2alm's output layout), maps_out [nmaps][npix]. */
int sfb_map2alm_adjoint(sfb_plan *plan, const double *abar, int64_t nmaps, double *maps_out);

/* field2anlm(f_xyz, wmodes, amodes) (reference field2anlm_v2, src/cat2anlm.jl:323-357).
 * f: [nr * npix] host array, element (ir, p) at ir + nr*p (Julia nr x npix matrix).
 * ConfigurationSpaceModes(rmin, rmax, nr, nside) shells (src/windows.jl:98-103).
 * The shell transforms run in the plan's precision (SFB_MIXED: the tensor-core
 * transform of the FP32-rounded shells; the radial sum in FP64). */
int sfb_field2anlm(sfb_plan *plan, const double *f, int64_t nr, double rmin, double rmax,
                   double *anlm_out);

/* field2anlm with the field's element type given (reference field2anlm_v2,
 * src/cat2anlm.jl:323-357, whose field may be any real matrix): f is
 * [nr * npix] elements of `dtype` (sfb_dtype), element (ir, p) at ir + nr*p.
 * An FP32 field is read as it is (no FP64 copy on the host or the device; the
 * mixed-precision transform takes its shells directly).  The field is held on
 * the device when it fits (SFBGPU_FIELD_MAX_BYTES at plan creation, else half
 * of the free device memory); a larger field streams through the device one
 * chunk of shells at a time. */
int sfb_field2anlm_typed(sfb_plan *plan, const void *f, int32_t dtype, int64_t nr, double rmin, double rmax,
                         double *anlm_out);

/* dL/df of sfb_field2anlm_typed written as `dtype` elements (df_out [nr * npix],
 * element (ir, p) at ir + nr*p), with the same shell streaming.  No counterpart
 * in the reference (its transforms have no derivatives). */
int sfb_field2anlm_vjp_typed(sfb_plan *plan, const double *abar, int64_t nr, double rmin, double rmax,
                             void *df_out, int32_t dtype);

/* anlm2field(f_nlm, wmodes, amodes) (reference src/cat2anlm.jl:383-422).
 * anlm: [2*nlmsize] interleaved complex; f_out: [nr * npix], element (ir,p) at ir + nr*p. */
int sfb_anlm2field(sfb_plan *plan, const double *anlm, int64_t nr, double rmin, double rmax,
                   double *f_out);

/* win_rhat_ln for a separable window (reference src/windows.jl:260-270):
 * W_ln[l,n] = dr * sum_r r^2 g_nl(r) phi(r).  phi: [nr]; w_ln_out: [(lmax+1)*nmax],
 * NaN where l > lmax_n[n]. */
int sfb_win_rhat_ln_separable(sfb_plan *plan, const double *phi, int64_t nr, double rmin,
                              double rmax, double *w_ln_out);

/* win_rhat_ln for a dense window (reference src/windows.jl:244-257).
 * win: [nr * npix], element (ir, p) at ir + nr*p; w_out: [npix*(lmax+1)*nmax]. */
int sfb_win_rhat_ln_dense(sfb_plan *plan, const double *win, int64_t nr, double rmin,
                          double rmax, double *w_out);

/* win_lnn(win, wmodes, cmodes) (reference src/windows.jl:382-392 with
 * calc_intr_gg_fn :394-422): for every column i of lnn (ClnnModes.lnn,
 * 3 x nlnn column-major: l, n1, n2 with 1-based n),
 *   out[i] = sum_s r_s^2 dr g_{n1 l}(r_s) g_{n2 l}(r_s) W00_s / sqrt(4 pi),
 * r_s the shell midpoints of ConfigurationSpaceModes(rmin, rmax, nr) and W00_s
 * the a_00 of shell s of the window (map2alm to lmax 2 lmax with the plan's
 * niter, as the reference's calc_Wr_lm(win, 2 lmax, nside)).  win: [nr * npix]
 * at the plan's nside, element (ir, p) at ir + nr*p.  A shell with a negative
 * mean makes the reference's square roots NaN: SFB_ENONFINITE here.  The first
 * call builds the plan's transform at 2 lmax (needs 2 lmax <= 4 nside). */
int sfb_win_lnn(sfb_plan *plan, const double *win, int64_t nr, double rmin, double rmax, const int64_t *lnn,
                int64_t nlnn, double *out);

/* calc_wmix(win, wmodes, amodes; neg_m) (reference src/windows.jl:299-366,
 * calc_wmix_ii :273-296, calc_gaunts_L :451-465): the window mixing matrix
 *   W[(n l m), (n' l' m')] = (-1)^m sum_L G(l, l', L; -m, m')
 *                            sum_s g_nl(r_s) g_n'l'(r_s) r_s^2 dr W_{L, m - m'}(r_s),
 * G the Gaunt coefficient sqrt((2L+1)(2l+1)(2l'+1)/4 pi) (l l' L; 0 0 0)
 * (L l l'; m - m', -m, m'), m = 0..l (m = -0..-l when neg_m), m' = 0..l',
 * W_LM(r_s) the a_lm of window shell s to lmax 2 lmax (map2alm with the
 * plan's niter, the reference's calc_Wr_lm), W_{L,-M} = (-1)^M conj(W_LM).
 * win: [nr * npix] at the plan's nside, element (ir, p) at ir + nr*p.
 * wmix_out: [nlmsize x nlmsize] complex, column-major like Julia's
 * Matrix{ComplexF64}: element (i, j) at 2 (i + nlmsize j).  Supports
 * lmax <= 128 (SFB_ENOTSUP beyond); the output alone is 16 nlmsize^2 bytes. */
int sfb_calc_wmix(sfb_plan *plan, const double *win, int64_t nr, double rmin, double rmax, int32_t neg_m,
                  double *wmix_out);

/* Batched map2alm with the plan's niter (the transform behind mymap2alm!,
 * src/healpix_helpers.jl:50-56).  maps: [nmaps * npix], map b at b*npix.
 * alm_out: [nmaps * 2 * lmsize], lmsize = (lmax+1)(lmax+2)/2, index l(l+1)/2+m. */
int sfb_map2alm(sfb_plan *plan, const double *maps, int64_t nmaps, double *alm_out);

/* amln2clnn(anlm1, anlm2, cmodes) (reference src/SphericalFourierBesselDecompositions.jl:114-150):
 * C[i] = [Re(a1_{n1 l 0} a2_{n2 l 0}) + 2 sum_{m>=1} Re(a1_{n1 l m} conj(a2_{n2 l m}))] / (2l+1)
 * for every column i of lnn (ClnnModes.lnn, 3 x nlnn column-major: l, n1, n2 with
 * 1-based n), for nbatch coefficient vectors stored one after another
 * (anlm: [nbatch * 2 * nlmsize]; anlm2 may be NULL or equal to anlm1 for the
 * auto spectrum).  clnn_out: [nbatch * nlnn], vector b at b * nlnn. */
int sfb_amln2clnn(sfb_plan *plan, const double *anlm1, const double *anlm2, int64_t nbatch,
                  const int64_t *lnn, int64_t nlnn, double *clnn_out);

/* winweights2galweights(weights, wmodes, rθϕ) (reference src/cat2anlm.jl:218-238):
 * w_out[i] = weights[bin, pix] with pix the RING pixel of (theta_i, phi_i) and
 * bin = nr if r_i == rbounds[nr], else the largest j with rbounds[j-1] <= r_i
 * (Julia's searchsortedlast over get_rbounds(wmodes), passed as rbounds[nr+1]).
 * weights: [nr * npix], element (bin, pix) at (bin-1) + nr*pix.  A radius
 * outside the shells returns SFB_ERANGE (the reference's "r out of bounds"). */
int sfb_winweights2galweights(int64_t nside, const double *weights, int64_t nr, const double *rbounds,
                              const double *rtp, int64_t ngal, double *w_out);

/* No counterpart in the reference.  Same arguments, result and errors as
 * sfb_winweights2galweights, but the call allocates no device memory: inputs
 * and outputs are staged through a fixed 16 MiB device array per device, for
 * callers whose device memory belongs to another allocator or that may not
 * allocate mid-pipeline.  Limit: nr*npix + nr + 1 <= 2080736 doubles
 * (e.g. nside 64 with nr <= 42), else SFB_EINVAL.  The first call on a
 * device does its set-up (device address lookup) and should come before any
 * stream capture.  Calls on one device are serialised inside the library.
 * The call is synchronous: its copies and its kernel run on the legacy
 * default stream, so it waits for, and holds up, work on every blocking
 * stream of the process.  The device address found at set-up is kept for the
 * life of the process; after a cudaDeviceReset of that device it is stale,
 * and such a process must not call this entry point again. */
int sfb_winweights2galweights_noalloc(int64_t nside, const double *weights, int64_t nr,
                                      const double *rbounds, const double *rtp, int64_t ngal,
                                      double *w_out);

/* apply_window(rθϕ, win, rmin, rmax, win_r, win_Δr; rng) (reference
 * src/windows.jl:169-216): the galaxies of rtp ([3*ngal], as in sfb_cat2amln)
 * kept by the window, in input order, written to rtp_out ([3*ngal] capacity),
 * their number to *nkept.  Galaxy i is kept when rmin <= r_i <= rmax, its
 * shell ceil((r_i - rmin)/dr) (0 becoming 1) is at most nr, and
 * u_i <= win[shell, pix_i] * (1 / max(win)); win: [nr * npix], element (ir, p)
 * at ir + nr*p (a Julia nr x npix matrix), pix_i the RING pixel.  u_i =
 * uniform[i] when `uniform` is given (the reference's rand(rng) per galaxy:
 * a caller passing the same draws gets the reference's result exactly), else
 * the counter-based stream (splitmix64(seed + (i+1) * 0x9E3779B97F4A7C15) >> 11)
 * * 2^-53.  A NaN window value or a non-finite direction of a galaxy inside
 * the shells returns SFB_ENONFINITE, theta outside [0, pi] SFB_ERANGE. */
int sfb_apply_window(int64_t nside, const double *win, int64_t nr, double rmin, double rmax, double dr,
                     const double *rtp, int64_t ngal, const double *uniform, uint64_t seed, double *rtp_out,
                     int64_t *nkept);

/* The same with win, rtp, uniform and rtp_out in device memory, on `stream`
 * (cudaStream_t or NULL); returns after *nkept (a host pointer) is known.
 * Thins mock catalogues on the device for sfb_cat2amln_device. */
int sfb_apply_window_device(int64_t nside, const double *win, int64_t nr, double rmin, double rmax, double dr,
                            const double *rtp, int64_t ngal, const double *uniform, uint64_t seed,
                            double *rtp_out, int64_t *nkept, void *stream);

/* HEALPix RING pixel (0-based; Healpix.jl ang2pixRing returns this + 1) of
 * n directions, computed on the device with the binning kernel's arithmetic. */
int sfb_ang2pix_ring(int64_t nside, const double *theta, const double *phi, int64_t n,
                     int64_t *pix_out);

/* Stages of one transform call, for sfb_get_stage_times. */
typedef enum {
    SFB_STAGE_DEPOSIT = 0,       /* galaxy binning into the radial-basis x pixel maps */
    SFB_STAGE_RING_FFT = 1,      /* ring Fourier transforms (analysis and synthesis) */
    SFB_STAGE_LEG_ANALYSIS = 2,  /* Legendre contraction, rings -> a_lm */
    SFB_STAGE_LEG_SYNTHESIS = 3, /* Legendre contraction, a_lm -> rings (refinement) */
    SFB_STAGE_FOLD = 4,          /* refinement residual in ring-Fourier space */
    SFB_STAGE_PROJECT = 5,       /* radial projection and window subtraction */
    SFB_STAGE_OTHER = 6,         /* clears, copies, checks */
    SFB_NSTAGES = 7
} sfb_stage;

/* Stage timing with CUDA events recorded on the call's stream (no extra
 * synchronisation).  Enabling resets the accumulators.  Not part of the
 * reference interface: measurement support for this library. */
int sfb_set_profiling(sfb_plan *plan, int32_t enable);
/* Accumulated device milliseconds and kernel launches per stage since
 * profiling was enabled; ms and launches are arrays of SFB_NSTAGES (either may be NULL). */
int sfb_get_stage_times(const sfb_plan *plan, double *ms, int64_t *launches);
/* Number of kernels this library has launched in this process. */
int64_t sfb_launch_count(void);

/* Failure-detection self-test (no counterpart in the reference): launches one
 * CTA whose bounded mbarrier wait has no arrival, so the wait expires after
 * about a second and the kernel records the timeout in its error word.
 * Returns SFB_ETIMEOUT when the bound works; the CUDA context stays usable. */
int sfb_selftest_wait_timeout(void);

/* Text of the last error on this thread (NUL-terminated, truncated to len). */
int sfb_last_error(char *buf, size_t len);

#ifdef __cplusplus
}
#endif

#endif /* SFB_GPU_H */
