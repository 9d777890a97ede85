// Plan management, orchestration and the C ABI (include/sfb_gpu.h).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sfb_internal.h"

namespace sfb {

static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_error(const std::string &msg) { g_last_error = msg; }
int fail(int code, const std::string &msg) {
    set_error(msg);
    return code;
}

int grow(Plan &p, DevBuf<double> &b, size_t n) {
    if (b.n >= n) return SFB_OK;
    if (b.ptr) {
        cudaFree(b.ptr);
        p.device_bytes -= (int64_t)(b.n * sizeof(double));
        b.ptr = nullptr;
        b.n = 0;
    }
    if (n == 0) return SFB_OK;
    cudaError_t e = cudaMalloc(&b.ptr, n * sizeof(double));
    if (e != cudaSuccess) {
        cudaGetLastError();
        b.ptr = nullptr;
        return fail(SFB_ENOMEM, "device allocation of " + std::to_string(n * sizeof(double)) + " bytes failed");
    }
    b.n = n;
    p.device_bytes += (int64_t)(n * sizeof(double));
    return SFB_OK;
}

template <typename T>
static int upload(Plan &p, T **dst, const T *src, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc(dst, n * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(SFB_ENOMEM, "device allocation failed");
    }
    p.device_bytes += (int64_t)(n * sizeof(T));
    if (src) SFB_CUDA_TRY(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return SFB_OK;
}

// launch wrappers implemented in radial.cu
void launch_deposit_spline_chunk(const Plan &p, const double *rtp, const double *w, int64_t ngal, int64_t pair0,
                                 int64_t npc, double scale, double *maps, cudaStream_t st);
void launch_subtract_dense_chunk(const Plan &p, double *maps, const double *dense, int64_t pair0, int64_t npc,
                                 cudaStream_t st);
void launch_gather_dense_chunk(const Plan &p, double *maps, const double *dense, int64_t pair0, int64_t npc,
                               cudaStream_t st);
void launch_radial_error_impl(const Plan &p, const double *coef, const double *ymax, unsigned long long *err_bits,
                              cudaStream_t st);
void launch_sub_window_chunk(const Plan &p, const double *Awin, int64_t ldW, int64_t pair0, int64_t npc, double *out,
                             cudaStream_t st);
void launch_extract_spline_chunk(const Plan &p, const double *A, int64_t ldA, int64_t pair0, int64_t npc, double *out,
                                 cudaStream_t st);
void launch_gtab(const Plan &p, int64_t nr, double rmin, double dr, int with_r2dr, double *gtab, cudaStream_t st);
void launch_project_shells_g(const Plan &p, const double *gtab, int64_t nr, const double *A, int64_t ldA, double *out,
                             cudaStream_t st);
void launch_shell_alm_g(const Plan &p, const int32_t *pair_index, const int64_t *noff, const double *gtab, int64_t nr,
                        const double *anlm, double *A, int64_t ldA, cudaStream_t st);
void launch_win_sep_g(const Plan &p, const double *gtab, int64_t nr, const double *phi, double *out, cudaStream_t st);
void launch_win_dense_g(const Plan &p, const double *gtab, int64_t nr, const double *win, double *out, cudaStream_t st);
void launch_fill(double *x, int64_t n, double v, cudaStream_t st);
void launch_subtract_sep_chunk(const Plan &p, double *maps, const double *mask, const double *w_ln, int64_t pair0,
                               int64_t npc, cudaStream_t st);
void launch_transpose_ld(const double *in, int64_t ldi, int64_t rows, int64_t cols, double *out, int64_t ldo,
                         cudaStream_t st);
void launch_transpose_ld(const float *in, int64_t ldi, int64_t rows, int64_t cols, double *out, int64_t ldo,
                         cudaStream_t st);
void launch_transpose_ld(const float *in, int64_t ldi, int64_t rows, int64_t cols, float *out, int64_t ldo,
                         cudaStream_t st);
void launch_transpose_ld(const double *in, int64_t ldi, int64_t rows, int64_t cols, float *out, int64_t ldo,
                         cudaStream_t st);
void launch_transpose_ld(const float *in, int64_t ldi, int64_t rows, int64_t cols, float2 *out, int64_t ldo,
                         cudaStream_t st);
void launch_axpy(double *y, const double *x, int64_t n, cudaStream_t st);
void launch_winweights(const double *weights, int64_t nr, int64_t nside, const double *rbounds, double rmax,
                       const double *rtp, int64_t ngal, double *w, int *err, cudaStream_t st);
void launch_amln2clnn(const double *a1, const double *a2, int64_t nlmsize, const int64_t *lnn, int64_t nlnn,
                      int64_t nbatch, const int64_t *noff, double *out, cudaStream_t st);
void launch_win_lnn(const Plan &p, const int32_t *pair_index, const double *gtab, int64_t nr, double rmin, double dr,
                    const double *w00, const int64_t *lnn, int64_t nlnn, double *out, cudaStream_t st);
void launch_extract_a00(const double *alm, int64_t ldA, int64_t nm, double *w00, cudaStream_t st);

}  // namespace sfb

struct sfb_plan {
    sfb::Plan p;
    cudaStream_t stream = nullptr;
    // side stream for the FP64 reference-map transform of the mixed path,
    // forked / joined with the call's stream through events
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // host entry: the catalogue copy runs on the side stream in NCOPY chunks
    static constexpr int NCOPY = 4;
    cudaEvent_t ev_copy[NCOPY] = {};
    int32_t *d_pair_index = nullptr;
    int64_t *d_noff = nullptr;
    // FP64 transform at lmax 2 lmax for the window harmonics of win_lnn (the reference's
    // calc_Wr_lm), created on first use
    sfb_plan *aux = nullptr;
    // stage profiling (events on the call's stream)
    bool profile = false;
    struct Rec {
        int stage;
        cudaEvent_t a, b;
        int64_t launches;
    };
    std::vector<cudaEvent_t> pool;
    std::vector<Rec> recs;
    double stage_ms[SFB_NSTAGES] = {};
    int64_t stage_launches[SFB_NSTAGES] = {};
};

namespace {

cudaEvent_t take_event(sfb_plan *h) {
    if (!h->pool.empty()) {
        cudaEvent_t e = h->pool.back();
        h->pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

// RAII scope: records a start event on construction and an end event on
// destruction when profiling is on; launches counted from the global counter.
struct Stage {
    sfb_plan *h;
    int id;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    int64_t l0 = 0;
    Stage(sfb_plan *h_, int id_, cudaStream_t st_) : h(h_), id(id_), st(st_) {
        if (!h->profile) return;
        a = take_event(h);
        l0 = sfb::g_launches.load();
        if (a) cudaEventRecord(a, st);
    }
    ~Stage() {
        if (!h->profile || !a) return;
        cudaEvent_t b = take_event(h);
        if (!b) return;
        cudaEventRecord(b, st);
        h->recs.push_back({id, a, b, sfb::g_launches.load() - l0});
    }
};

// After the stream is synchronised: fold recorded events into the totals.
void collect_stages(sfb_plan *h) {
    for (auto &r : h->recs) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) h->stage_ms[r.stage] += ms;
        else cudaGetLastError();
        h->stage_launches[r.stage] += r.launches;
        h->pool.push_back(r.a);
        h->pool.push_back(r.b);
    }
    h->recs.clear();
}

}  // namespace

using namespace sfb;

namespace {

// Gauss-Legendre nodes/weights on [-1, 1] (Newton iteration on P_Q).
void gauss_legendre(int Q, std::vector<double> &x, std::vector<double> &w) {
    x.resize(Q);
    w.resize(Q);
    for (int i = 0; i < Q; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (Q + 0.5));
        double dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= Q; ++k) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = Q * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= Q; ++k) {
            const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        dp = Q * (z * p1 - p0) / (z * z - 1.0);
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

int64_t lmsize_of(int64_t l) { return l < 0 ? 0 : (l + 1) * (l + 2) / 2; }

// Compute coefficients for (pieces, degree) and return the measured error.
int radial_fit(sfb_plan *h, const double *d_ymax, double *err_out) {
    Plan &p = h->p;
    p.nbasis = (int64_t)p.pieces * (p.degree + 1) + 2;
    const int Q = std::min(2 * (p.degree + 1) + 24, 4096);
    std::vector<double> gx, gw;
    gauss_legendre(Q, gx, gw);
    std::vector<double> pq((size_t)Q * (p.degree + 1));
    for (int q = 0; q < Q; ++q) {
        double p0 = 1.0, p1 = gx[q];
        for (int k = 0; k <= p.degree; ++k) {
            double pk;
            if (k == 0) pk = 1.0;
            else if (k == 1) pk = gx[q];
            else {
                pk = ((2.0 * (k - 1) + 1.0) * gx[q] * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = pk;
            }
            pq[(size_t)q * (p.degree + 1) + k] = gw[q] * (2.0 * k + 1.0) / 2.0 * pk;
        }
    }
    double *d_gx = nullptr, *d_pq = nullptr;
    unsigned long long *d_eb = nullptr;
    SFB_CUDA_TRY(cudaMalloc(&d_gx, Q * sizeof(double)));
    SFB_CUDA_TRY(cudaMalloc(&d_pq, pq.size() * sizeof(double)));
    SFB_CUDA_TRY(cudaMalloc(&d_eb, sizeof(unsigned long long)));
    SFB_CUDA_TRY(cudaMemcpy(d_gx, gx.data(), Q * sizeof(double), cudaMemcpyHostToDevice));
    SFB_CUDA_TRY(cudaMemcpy(d_pq, pq.data(), pq.size() * sizeof(double), cudaMemcpyHostToDevice));
    SFB_CUDA_TRY(cudaMemset(d_eb, 0, sizeof(unsigned long long)));
    if (p.d_coef) {
        cudaFree(p.d_coef);
        p.device_bytes -= p.npairs * 8;  // approximate bookkeeping; recomputed below
    }
    p.d_coef = nullptr;
    SFB_CUDA_TRY(cudaMalloc(&p.d_coef, (size_t)p.npairs * p.nbasis * sizeof(double)));
    launch_radial_coeffs(p, d_gx, d_pq, Q, p.d_coef, h->stream);
    launch_radial_error_impl(p, p.d_coef, d_ymax, d_eb, h->stream);
    unsigned long long eb = 0;
    SFB_CUDA_TRY(cudaStreamSynchronize(h->stream));
    SFB_CUDA_TRY(cudaGetLastError());
    SFB_CUDA_TRY(cudaMemcpy(&eb, d_eb, sizeof(eb), cudaMemcpyDeviceToHost));
    double e;
    std::memcpy(&e, &eb, sizeof(e));
    *err_out = e;
    cudaFree(d_gx);
    cudaFree(d_pq);
    cudaFree(d_eb);
    return SFB_OK;
}

int choose_radial_basis(sfb_plan *h, const sfb_plan_desc *d) {
    Plan &p = h->p;
    const double L = p.rmax - p.rmin;
    // knot counts encode k: nr = 3 + 12*ceil(2 k L) (src/SphericalBesselGNLs.jl:571)
    double kest = 0.0;
    std::vector<double> ymax(p.npairs);
    for (int64_t i = 0; i < p.npairs; ++i) {
        const int64_t N = p.h_spl_off[i + 1] - p.h_spl_off[i];
        kest = std::max(kest, (double)(N - 4) / (24.0 * L));
        double ym = 0;
        for (int64_t k = p.h_spl_off[i]; k < p.h_spl_off[i + 1]; ++k) ym = std::max(ym, std::fabs(d->spl_y[k]));
        ymax[i] = ym;
    }
    double *d_ymax = nullptr;
    SFB_TRY(upload(p, &d_ymax, ymax.data(), ymax.size()));
    const double tol = d->radial_tol > 0 ? d->radial_tol : 1e-9;
    p.pieces = d->radial_pieces > 0 ? d->radial_pieces : std::max(1, (int)std::ceil(kest * L / 16.0));
    const double omega = kest * L / (2.0 * p.pieces);
    const bool fixed_deg = d->radial_degree > 0;
    p.degree = fixed_deg ? d->radial_degree : (int)std::ceil(omega + 12.0);
    double err = 0;
    SFB_TRY(radial_fit(h, d_ymax, &err));
    if (!fixed_deg) {
        // raise the degree while the projection error still improves markedly
        for (int it = 0; it < 12 && err > tol; ++it) {
            const int prev_deg = p.degree;
            const double prev_err = err;
            p.degree += 4;
            SFB_TRY(radial_fit(h, d_ymax, &err));
            if (err > 0.5 * prev_err) {  // floor reached (spline interpolation error)
                if (err > prev_err) {
                    p.degree = prev_deg;
                    SFB_TRY(radial_fit(h, d_ymax, &err));
                }
                break;
            }
        }
    }
    p.radial_error = err;
    cudaFree(d_ymax);
    return SFB_OK;
}

// map2alm with niter refinement on nm maps; result in p.alm [lmsize][2*nm] (FP64).
// In mixed precision the maps are FP32 ([nm][npix] floats); maps_are_fp64 marks
// FP64 maps that are converted first.
// The ring Fourier buffers and the a_lm of one transform: the plan's own, or
// the side stream's set for the FP64 reference transform that overlaps the
// main one.
struct ShtWork {
    DevBuf<double> *f, *g, *r, *alm;
};

// fp64_out: the FP64 a_lm (alm) is wanted besides the double-float copy (almdf, mixed precision); the
// Gram refinement carries only the double-float one and converts at the end when asked.
// ring_live / nlive (mixed precision): rings marked 0 hold zeros in maps [0, nlive), left unwritten by the
// deposit (deposit_sorted's ring_live).
int sht_analysis(sfb_plan *h, const double *maps, int64_t nm, cudaStream_t st, bool maps_are_fp64 = false,
                 int stage_override = -1, const ShtWork *ws = nullptr, bool fp64_out = true,
                 const int *ring_live = nullptr, int64_t nlive = 0) {
    Plan &p = h->p;
    const ShtWork own{&p.fbuf, &p.gbuf, &p.rbuf, &p.alm};
    if (!ws) ws = &own;
    DevBuf<double> &fbuf = *ws->f, &gbuf = *ws->g, &rbuf = *ws->r, &alm = *ws->alm;
    auto stage = [&](int s) { return stage_override >= 0 ? stage_override : s; };
    if (p.precision == SFB_MIXED && maps_are_fp64) {
        SFB_TRY(grow(p, p.maps32, (size_t)(nm * p.npix)));
        {
            Stage s(h, stage(SFB_STAGE_OTHER), st);
            launch_to_df(maps, nm * p.npix, reinterpret_cast<float2 *>(p.maps32.ptr), st);
        }
        maps = p.maps32.ptr;
    }
    const int64_t ncol = 2 * nm;
    const size_t fsz = (size_t)2 * (p.lmax + 1) * p.nrn * ncol;
    SFB_TRY(grow(p, fbuf, fsz));
    SFB_TRY(grow(p, alm, (size_t)p.lmsize * ncol));
    if (p.niter > 0) {
        SFB_TRY(grow(p, gbuf, fsz));
        SFB_TRY(grow(p, rbuf, fsz));
    }
    // the non-zero ring-pair range of the DFT input, in the two ints past both scale arrays
    int *nzr = nullptr;
    if (p.precision == SFB_MIXED) {
        // row scales of the ring DFT, then column scales of the Legendre analysis (ints)
        SFB_TRY(grow(p, p.erow, (size_t)std::max<int64_t>(p.nrn * nm, (p.lmax + 1) * ncol) + 1));
        SFB_TRY(grow(p, p.almdf, (size_t)p.lmsize * ncol));
        nzr = reinterpret_cast<int *>(p.erow.ptr) + 2 * std::max<int64_t>(p.nrn * nm, (p.lmax + 1) * ncol);
        Stage s(h, stage(SFB_STAGE_RING_FFT), st);
        // the Gram refinement and niter = 0 read the spectra only in the first analysis pass (over the
        // span with data and the live chunks); the full refinement passes fold them over every ring
        const bool skip_unread = (nm > 4 && p.d_gramts && p.niter > 0) || p.niter == 0;
        SFB_TRY(launch_ring_analysis_tc(p, reinterpret_cast<const float2 *>(maps), nm,
                                        reinterpret_cast<float2 *>(fbuf.ptr), reinterpret_cast<int *>(p.erow.ptr), nzr,
                                        st, ring_live, nlive, skip_unread));
    } else {
        // many columns: the FFT records the span of ring pairs with data, over which the
        // first analysis pass sums (the spectra are zero elsewhere)
        if (ncol > 8) {
            SFB_TRY(grow(p, p.nzr64, 1));
            nzr = reinterpret_cast<int *>(p.nzr64.ptr);
            SFB_CUDA_TRY(cudaMemsetAsync(nzr, 0x7f, sizeof(int), st));          // first: a large value
            SFB_CUDA_TRY(cudaMemsetAsync(nzr + 1, 0xff, sizeof(int), st));      // last: -1
        }
        Stage s(h, stage(SFB_STAGE_RING_FFT), st);
        launch_ring_analysis(p, maps, nm, fbuf.ptr, st, nzr);
    }
    const bool tc = p.precision == SFB_MIXED;
    float2 *adf = reinterpret_cast<float2 *>(p.almdf.ptr);
    int *ecol = reinterpret_cast<int *>(p.erow.ptr);          // column scales (the row scales are used up)
    auto analysis = [&](const double *src, bool acc) {
        Stage s(h, stage(SFB_STAGE_LEG_ANALYSIS), st);
        // after the first pass the fold has written the column scales of its residual
        // the first pass reads the DFT output, zero outside the non-zero ring range
        if (tc) launch_leg_analysis_tc(p, (const float2 *)src, ncol, alm.ptr, adf, ecol, acc, st, acc, -1, nullptr,
                                       acc ? nullptr : nzr);
        else launch_leg_analysis(p, src, ncol, alm.ptr, acc, st);
    };
    if (tc && ncol / 2 > 4 && p.d_gramts && p.niter > 0) {
        // Gram refinement: a <- a + (a0 - M a) - A_al(Fold(S_al a)) = a0 - D a - A_al(Fold(S_al a)),
        // M the Gram matrix of the alias-free rings (fold = identity there), D = M - I as the
        // tables store it, S_al / A_al the synthesis and analysis over the aliased rings r < ral.
        // Each pass writes the other (A, Adf) buffer; the last one lands in the plan's.
        SFB_TRY(grow(p, p.almdf2, (size_t)p.lmsize * ncol));
        SFB_TRY(grow(p, p.adf0, (size_t)p.lmsize * ncol));
        // column exponents of each (A, Adf) set, written by whichever kernel completes the set
        const int64_t nE = 2 * (p.lmax + 1) * ncol;
        SFB_TRY(grow(p, p.ecoef, (size_t)nE + 1));
        double *Ab[2] = {nullptr, nullptr};          // FP64 a_lm: formed once at the end (fp64_out)
        float2 *Db[2] = {adf, reinterpret_cast<float2 *>(p.almdf2.ptr)};
        int *Eb[2] = {reinterpret_cast<int *>(p.ecoef.ptr), reinterpret_cast<int *>(p.ecoef.ptr) + nE};
        const float2 *a0 = reinterpret_cast<const float2 *>(p.adf0.ptr);
        int cur = p.niter & 1;
        // 0x80 bytes: every exponent word starts below any scale exponent (atomicMax)
        SFB_CUDA_TRY(cudaMemsetAsync(Eb[cur], 0x80, (size_t)nE * sizeof(int), st));
        {
            Stage s(h, stage(SFB_STAGE_LEG_ANALYSIS), st);
            launch_leg_analysis_tc(p, (const float2 *)fbuf.ptr, ncol, Ab[cur], Db[cur], ecol, false, st, false, -1,
                                   Eb[cur], nzr);
        }
        SFB_CUDA_TRY(cudaMemcpyAsync(p.adf0.ptr, Db[cur], (size_t)p.lmsize * ncol * sizeof(float2),
                                     cudaMemcpyDeviceToDevice, st));
        for (int it = 0; it < p.niter; ++it) {
            const int nxt = cur ^ 1;
            SFB_CUDA_TRY(cudaMemsetAsync(Eb[nxt], 0x80, (size_t)nE * sizeof(int), st));
            {
                Stage s(h, stage(SFB_STAGE_LEG_SYNTHESIS), st);
                if (p.ral > 0) launch_leg_synthesis_tc(p, Db[cur], ncol, (float *)gbuf.ptr, st, p.ral, Eb[cur]);
                // the update records the column exponents of its output; the aliased analysis raises
                // them where it adds (its CTAs without live chunks leave the update's values)
                launch_gram_update(p, Ab[cur], Db[cur], a0, ncol, Ab[nxt], Db[nxt], st, Eb[cur], Eb[nxt]);
            }
            if (p.ral > 0) {
                {
                    Stage s(h, stage(SFB_STAGE_FOLD), st);
                    launch_fold_residual(p, nullptr, gbuf.ptr, ncol, rbuf.ptr, st, ecol, p.ral);
                }
                Stage s(h, stage(SFB_STAGE_LEG_ANALYSIS), st);
                launch_leg_analysis_tc(p, (const float2 *)rbuf.ptr, ncol, Ab[nxt], Db[nxt], ecol, true, st, true,
                                       p.ral, Eb[nxt]);
            }
            cur = nxt;
        }
        if (fp64_out) launch_df_to_fp64(Db[cur], p.lmsize * ncol, alm.ptr, st);
        SFB_CUDA_TRY(cudaGetLastError());
        return SFB_OK;
    }
    if (!tc && p.d_gram64 && p.niter > 0) {
        // FP64 Gram refinement: the same identity as above, in FP64 (narrow kernels for 2, 4 or 8
        // columns: reference maps, small map2alm batches; tiled GEMMs for more, the first pass over
        // the ring pairs with data).  alm holds [current | next | first pass].
        const int64_t na = p.lmsize * ncol;
        SFB_TRY(grow(p, alm, (size_t)(3 * na)));
        double *Ab[2] = {alm.ptr, alm.ptr + na};
        double *a0 = alm.ptr + 2 * na;
        int cur = p.niter & 1;
        {
            Stage s(h, stage(SFB_STAGE_LEG_ANALYSIS), st);
            launch_leg_analysis(p, fbuf.ptr, ncol, Ab[cur], false, st, -1, nzr);
        }
        SFB_CUDA_TRY(cudaMemcpyAsync(a0, Ab[cur], (size_t)na * sizeof(double), cudaMemcpyDeviceToDevice, st));
        for (int it = 0; it < p.niter; ++it) {
            const int nxt = cur ^ 1;
            {
                Stage s(h, stage(SFB_STAGE_LEG_SYNTHESIS), st);
                if (p.ral > 0) launch_leg_synthesis(p, Ab[cur], ncol, gbuf.ptr, st, p.ral);
                launch_gram_update_fp64(p, Ab[cur], a0, ncol, Ab[nxt], st);
            }
            if (p.ral > 0) {
                {
                    Stage s(h, stage(SFB_STAGE_FOLD), st);
                    launch_fold_residual(p, nullptr, gbuf.ptr, ncol, rbuf.ptr, st, nullptr, p.ral);
                }
                Stage s(h, stage(SFB_STAGE_LEG_ANALYSIS), st);
                launch_leg_analysis(p, rbuf.ptr, ncol, Ab[nxt], true, st, p.ral);
            }
            cur = nxt;
        }
        SFB_CUDA_TRY(cudaGetLastError());
        return SFB_OK;
    }
    analysis(fbuf.ptr, false);
    for (int it = 0; it < p.niter; ++it) {
        {
            Stage s(h, stage(SFB_STAGE_LEG_SYNTHESIS), st);
            if (tc) launch_leg_synthesis_tc(p, adf, ncol, (float *)gbuf.ptr, st);
            else launch_leg_synthesis(p, alm.ptr, ncol, gbuf.ptr, st);
        }
        {
            Stage s(h, stage(SFB_STAGE_FOLD), st);
            launch_fold_residual(p, fbuf.ptr, gbuf.ptr, ncol, rbuf.ptr, st, tc ? ecol : nullptr);
        }
        analysis(rbuf.ptr, true);
    }
    SFB_CUDA_TRY(cudaGetLastError());
    return SFB_OK;
}

int finish(sfb_plan *h, const double *out_dev, cudaStream_t st) {
    Plan &p = h->p;
    {
        Stage s(h, SFB_STAGE_OTHER, st);
        launch_check_finite(out_dev, 2 * p.nlmsize, p.d_err, st);
    }
    int err = 0;
    SFB_CUDA_TRY(cudaMemcpyAsync(&err, p.d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    SFB_CUDA_TRY(cudaGetLastError());
    collect_stages(h);
    if (err & ERR_NONFINITE_INPUT) return fail(SFB_ENONFINITE, "non-finite galaxy coordinate or weight");
    if (err & ERR_THETA_RANGE) return fail(SFB_ERANGE, "galaxy theta outside [0, pi]");
    if (err & ERR_TC_TIMEOUT) return fail(SFB_ETIMEOUT, "tensor-core kernel: bounded mbarrier wait expired");
    if (err & ERR_NONFINITE_OUTPUT) return fail(SFB_ENONFINITE, "non-finite a_nlm (all(isfinite.(anlm)) failed)");
    return SFB_OK;
}

// FP64 a_lm of nref reference maps (mixed precision's mean terms), into
// ralm[lmsize][2 nref].
int reference_alm(sfb_plan *h, const double *ref, int64_t nref, double *ralm, cudaStream_t st) {
    Plan &p = h->p;
    const int32_t prec = p.precision;
    p.precision = SFB_FP64;
    const ShtWork ws{&p.rf, &p.rg, &p.rr, &p.ralm};
    const int rc = sht_analysis(h, ref, nref, st, false, SFB_STAGE_OTHER, &ws);
    p.precision = prec;
    SFB_TRY(rc);
    SFB_CUDA_TRY(cudaMemcpyAsync(ralm, p.ralm.ptr, (size_t)2 * nref * p.lmsize * sizeof(double),
                                 cudaMemcpyDeviceToDevice, st));
    return SFB_OK;
}

// Transpose of sht_analysis in FP64 (adjoint.cu): abar [lmsize][2 nm] on the device becomes E abar;
// maps_out [nm][npix] FP64 receives w S sum_j (I - A S)^j E abar.
int sht_analysis_adjoint(sfb_plan *h, double *abar, int64_t nm, double *maps_out, cudaStream_t st) {
    Plan &p = h->p;
    const int32_t prec = p.precision;
    p.precision = SFB_FP64;
    struct Restore {
        Plan &p;
        int32_t v;
        ~Restore() { p.precision = v; }
    } restore{p, prec};
    const int64_t ncol = 2 * nm;
    const size_t fsz = (size_t)2 * (p.lmax + 1) * p.nrn * ncol;
    SFB_TRY(grow(p, p.gbuf, fsz));
    SFB_TRY(grow(p, p.alm, (size_t)p.lmsize * ncol));
    launch_halve_m(abar, p.lmsize, ncol, st);
    double *x = p.alm.ptr;
    SFB_CUDA_TRY(cudaMemcpyAsync(x, abar, (size_t)p.lmsize * ncol * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (p.niter > 0) {
        SFB_TRY(grow(p, p.fbuf, fsz));
        SFB_TRY(grow(p, p.rbuf, fsz));
        SFB_CUDA_TRY(cudaMemsetAsync(p.fbuf.ptr, 0, fsz * sizeof(double), st));     // F = 0: the fold gives -A S x
    }
    for (int it = 0; it < p.niter; ++it) {
        launch_leg_synthesis(p, x, ncol, p.gbuf.ptr, st);
        launch_fold_residual(p, p.fbuf.ptr, p.gbuf.ptr, ncol, p.rbuf.ptr, st);
        launch_leg_analysis(p, p.rbuf.ptr, ncol, x, true, st);                     // x - A S x
        launch_axpy(x, abar, p.lmsize * ncol, st);                                   // + b
    }
    launch_leg_synthesis(p, x, ncol, p.gbuf.ptr, st);
    launch_ring_synthesis(p, p.gbuf.ptr, nm, maps_out, st);
    launch_scale(maps_out, nm * p.npix, 4.0 * M_PI / (double)p.npix, st);
    SFB_CUDA_TRY(cudaGetLastError());
    return SFB_OK;
}

int64_t chunk_pairs(const Plan &p) {
    // keep the per-chunk SHT workspace near 2 GB
    const double per_map = 8.0 * (p.npix + 3.0 * 2 * (p.lmax + 1) * p.nrn * 2 + 2.0 * p.lmsize);
    int64_t c = (int64_t)(2.0e9 / per_map);
    c = std::max<int64_t>(1, std::min<int64_t>(c, p.npairs));
    return c;
}

// defer_finish (batched calls): the device error word is neither cleared nor read here and the
// call does not wait for the device; the caller clears it once and checks it at the end.
int cat2amln_dev(sfb_plan *h, const double *rtp, const double *w, int64_t ngal, double nbar, const sfb_window *win,
                 double *out, cudaStream_t st, const cudaEvent_t *chunk_ready = nullptr, int nchunks = 0,
                 bool defer_finish = false) {
    Plan &p = h->p;
    if (ngal < 0) return fail(SFB_EINVAL, "ngal < 0");
    if (!win) return fail(SFB_EINVAL, "window descriptor is NULL");
    if (ngal > 0 && !rtp) return fail(SFB_EINVAL, "rtp is NULL");
    if (!(std::isfinite(nbar) && nbar != 0.0)) return fail(SFB_ENONFINITE, "nbar must be finite and non-zero");
    const int wk = win->kind;
    if (wk != SFB_WINDOW_ZERO && wk != SFB_WINDOW_SEPARABLE && wk != SFB_WINDOW_DENSE)
        return fail(SFB_EINVAL, "unknown window kind");
    if (wk == SFB_WINDOW_SEPARABLE && !(win->mask && win->w_ln)) return fail(SFB_EINVAL, "separable window needs mask and w_ln");
    if (wk == SFB_WINDOW_DENSE && !win->dense) return fail(SFB_EINVAL, "dense window pointer is NULL");
    const double dOmega = 4.0 * M_PI / (double)p.npix;
    const double scale = 1.0 / (nbar * dOmega);
    if (!defer_finish) SFB_CUDA_TRY(cudaMemsetAsync(p.d_err, 0, sizeof(int), st));
    if (p.radial_mode == SFB_RADIAL_POLY) {
        const int64_t nm = p.nbasis + (wk == SFB_WINDOW_SEPARABLE ? 1 : 0);
        // Mixed precision: the data maps are split into mu_b C + fluctuation
        // with C the weighted galaxy count map, the dense window maps into
        // nu W01 + fluctuation with W01 the window's (l=0, n=1) map; only the
        // fluctuations pass through the FP32 transform, C_lm and the mask's
        // (or W01's) a_lm are computed in FP64, so the cancellation between
        // data and window term happens in FP64.
        const bool split = p.precision == SFB_MIXED && wk != SFB_WINDOW_ZERO;
        const double *W01 = wk == SFB_WINDOW_SEPARABLE ? win->mask : win->dense;
        const int64_t cp = wk == SFB_WINDOW_DENSE ? chunk_pairs(p) : 0;
        double *Cmap = nullptr, *ralm = nullptr, *mu = nullptr, *nu = nullptr, *smean = nullptr;
        if (split) {
            // [C][W01][ralm: lmsize x (C, W01) complex][mu][nu][per-pair mean parts]
            SFB_TRY(grow(p, p.ref, (size_t)(2 * p.npix + 4 * p.lmsize + p.nbasis + cp + p.npairs)));
            Cmap = p.ref.ptr;
            ralm = Cmap + 2 * p.npix;
            mu = ralm + 4 * p.lmsize;
            nu = mu + p.nbasis;
            smean = nu + cp;
            SFB_CUDA_TRY(cudaMemcpyAsync(Cmap + p.npix, W01, p.npix * sizeof(double), cudaMemcpyDeviceToDevice, st));
        }
        SFB_TRY(grow(p, p.maps, (size_t)nm * p.npix));
        const int *ring_live = nullptr;          // rings the deposit wrote (mixed precision)
        if (wk == SFB_WINDOW_SEPARABLE) {
            Stage s(h, SFB_STAGE_OTHER, st);
            if (p.precision == SFB_MIXED)
                launch_to_df(win->mask, p.npix, reinterpret_cast<float2 *>(p.maps.ptr) + p.nbasis * p.npix, st);
            else
                SFB_CUDA_TRY(cudaMemcpyAsync(p.maps.ptr + p.nbasis * p.npix, win->mask, p.npix * sizeof(double),
                                             cudaMemcpyDeviceToDevice, st));
        }
        {
            Stage s(h, SFB_STAGE_DEPOSIT, st);
            SFB_TRY(deposit_sorted(p, rtp, w, ngal, p.maps.ptr, Cmap, mu, split ? h->ev_fork : nullptr, st,
                                   chunk_ready, nchunks, &ring_live));
        }
        if (split) {
            // the FP64 transform of (C, W01) runs on the side stream, in its own workspace, beside
            // the rest of the deposit and the main transform; the projection waits for it
            SFB_CUDA_TRY(cudaStreamWaitEvent(h->side, h->ev_fork, 0));
            SFB_TRY(reference_alm(h, Cmap, 2, ralm, h->side));
            SFB_CUDA_TRY(cudaEventRecord(h->ev_join, h->side));
        }
        // the mixed projection reads the double-float a_lm only
        SFB_TRY(sht_analysis(h, p.maps.ptr, nm, st, false, -1, nullptr, p.precision != SFB_MIXED, ring_live,
                             p.nbasis));
        if (split) SFB_CUDA_TRY(cudaStreamWaitEvent(st, h->ev_join, 0));
        {
            Stage s(h, SFB_STAGE_PROJECT, st);
            if (p.precision == SFB_MIXED)
                launch_project_mixed(p, reinterpret_cast<const float2 *>(p.almdf.ptr), 2 * nm, p.d_coefT, h->d_noff,
                                     h->d_pair_index, scale, mu, smean, split ? ralm : nullptr, wk, win->w_ln, out,
                                     st);
            else
                launch_project_poly(p, p.alm.ptr, 2 * nm, scale, wk, win->w_ln, p.nbasis, nullptr, 0, out, st);
        }
        if (wk == SFB_WINDOW_DENSE) {
            SFB_TRY(grow(p, p.maps, (size_t)cp * p.npix));
            for (int64_t p0 = 0; p0 < p.npairs; p0 += cp) {
                const int64_t npc = std::min(cp, p.npairs - p0);
                launch_gather_dense_chunk(p, p.maps.ptr, win->dense, p0, npc, st);
                if (split) launch_split_mean(p.maps.ptr, npc, p.npix, W01, nu, st);
                SFB_TRY(sht_analysis(h, p.maps.ptr, npc, st, true));
                if (split) launch_add_mean(p.alm.ptr, 2 * npc, npc, nu, ralm + 2, nullptr, 4, p.lmsize, -1, st);
                launch_sub_window_chunk(p, p.alm.ptr, 2 * npc, p0, npc, out, st);
            }
        }
    } else {
        // the spline deposit reads the whole catalogue: wait for every chunk of the copy
        for (int c = 0; chunk_ready && c < nchunks; ++c) SFB_CUDA_TRY(cudaStreamWaitEvent(st, chunk_ready[c], 0));
        // reference order: map = sum w g / (nbar dOmega) - W[:, l, n], then map2alm, keep row l
        const int64_t cp = chunk_pairs(p);
        SFB_TRY(grow(p, p.maps, (size_t)cp * p.npix));
        for (int64_t p0 = 0; p0 < p.npairs; p0 += cp) {
            const int64_t npc = std::min(cp, p.npairs - p0);
            SFB_CUDA_TRY(cudaMemsetAsync(p.maps.ptr, 0, (size_t)npc * p.npix * sizeof(double), st));
            { Stage s(h, SFB_STAGE_DEPOSIT, st); launch_deposit_spline_chunk(p, rtp, w, ngal, p0, npc, scale, p.maps.ptr, st); }
            if (wk == SFB_WINDOW_DENSE) launch_subtract_dense_chunk(p, p.maps.ptr, win->dense, p0, npc, st);
            if (wk == SFB_WINDOW_SEPARABLE) launch_subtract_sep_chunk(p, p.maps.ptr, win->mask, win->w_ln, p0, npc, st);
            SFB_TRY(sht_analysis(h, p.maps.ptr, npc, st, true));
            launch_extract_spline_chunk(p, p.alm.ptr, 2 * npc, p0, npc, out, st);
        }
    }
    SFB_CUDA_TRY(cudaGetLastError());
    if (defer_finish) {
        Stage s(h, SFB_STAGE_OTHER, st);
        launch_check_finite(out, 2 * p.nlmsize, p.d_err, st);
        return SFB_OK;
    }
    return finish(h, out, st);
}

int check_plan(const sfb_plan *h) {
    if (!h) return fail(SFB_EINVAL, "plan is NULL");
    return SFB_OK;
}

int set_device_of(const sfb_plan *h) {
    SFB_CUDA_TRY(cudaSetDevice(h->p.device));
    return SFB_OK;
}

}  // namespace

extern "C" {

int sfb_last_error(char *buf, size_t len) {
    if (!buf || len == 0) return SFB_EINVAL;
    std::strncpy(buf, g_last_error.c_str(), len - 1);
    buf[len - 1] = 0;
    return SFB_OK;
}

int sfb_plan_create(const sfb_plan_desc *d, sfb_plan **out) {
    if (!out) return fail(SFB_EINVAL, "output pointer is NULL");
    *out = nullptr;
    if (!d) return fail(SFB_EINVAL, "plan description is NULL");
    if (d->nside < 1) return fail(SFB_EINVAL, "nside must be >= 1");
    if (d->nside > 1024) return fail(SFB_ENOTSUP, "nside > 1024 is not supported");
    if (d->lmax < 0 || d->nmax < 1 || !d->lmax_n) return fail(SFB_EINVAL, "bad lmax/nmax/lmax_n");
    if (d->lmax > 4 * d->nside) return fail(SFB_ERANGE, "alm.lmax > 4*nside is a poor choice");
    if (!(d->rmin < d->rmax)) return fail(SFB_EINVAL, "rmin >= rmax");
    if (!d->spl_offset || !d->spl_x || !d->spl_y || !d->spl_ypp) return fail(SFB_EINVAL, "spline tables missing");
    if (d->niter < 0 || d->niter > 64) return fail(SFB_EINVAL, "niter out of range");
    if (d->precision != SFB_FP64 && d->precision != SFB_MIXED) return fail(SFB_EINVAL, "unknown precision");
    if (d->radial_mode != SFB_RADIAL_POLY && d->radial_mode != SFB_RADIAL_SPLINE)
        return fail(SFB_EINVAL, "unknown radial mode");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SFB_ECUDA, "no CUDA device available");
    }
    sfb_plan *h = new sfb_plan();
    Plan &p = h->p;
    cudaGetDevice(&p.device);
    p.nside = d->nside;
    p.npix = 12 * p.nside * p.nside;
    p.nrn = 2 * p.nside;
    p.lmax = (int)d->lmax;
    p.nmax = (int)d->nmax;
    p.lmax_n.assign(d->lmax_n, d->lmax_n + d->nmax);
    p.rmin = d->rmin;
    p.rmax = d->rmax;
    p.niter = d->niter;
    p.precision = d->precision;
    p.radial_mode = d->radial_mode;
    // SFBGPU_MOMENTS_SMEM=0: the mixed deposit's moments sum in registers (same bits, fewer resident warps)
    if (const char *e = std::getenv("SFBGPU_MOMENTS_SMEM")) p.moments_smem = e[0] != '0';
    p.lmsize = lmsize_of(p.lmax);
    // pairs and output tables
    std::vector<int32_t> pair_n, pair_l, out_pair, out_lm, pair_index((size_t)p.nmax * (p.lmax + 1), -1);
    std::vector<int64_t> noff(p.nmax + 1, 0);
    for (int n = 1; n <= p.nmax; ++n) {
        const int64_t ln = p.lmax_n[n - 1];
        if (ln < 0 || ln > p.lmax) {
            delete h;
            return fail(SFB_EINVAL, "lmax_n out of range");
        }
        noff[n] = noff[n - 1] + lmsize_of(ln);
        for (int l = 0; l <= ln; ++l) {
            pair_index[(size_t)(n - 1) * (p.lmax + 1) + l] = (int32_t)pair_n.size();
            for (int m = 0; m <= l; ++m) {
                out_pair.push_back((int32_t)pair_n.size());
                out_lm.push_back((int32_t)((int64_t)l * (l + 1) / 2 + m));
            }
            pair_n.push_back(n);
            pair_l.push_back(l);
        }
    }
    p.npairs = (int64_t)pair_n.size();
    p.nlmsize = noff[p.nmax];
    p.h_spl_off.assign(d->spl_offset, d->spl_offset + p.npairs + 1);
    if (p.h_spl_off[0] != 0) {
        delete h;
        return fail(SFB_EINVAL, "spl_offset[0] must be 0");
    }
    for (int64_t i = 0; i < p.npairs; ++i) {
        const int64_t a = p.h_spl_off[i], b = p.h_spl_off[i + 1];
        if (b - a < 4 || !(d->spl_x[a] < d->spl_x[b - 1])) {
            delete h;
            return fail(SFB_EINVAL, "spline " + std::to_string(i) + " needs >= 4 increasing knots");
        }
    }
    const int64_t nknots = p.h_spl_off[p.npairs];
    // ring geometry of the north half
    p.h_rings.resize(p.nrn);
    const int64_t ns = p.nside;
    const double fact2 = 4.0 / (double)p.npix, fact1 = (double)(2 * ns) * fact2;
    for (int64_t r = 0; r < p.nrn; ++r) {
        const int64_t i = r + 1;
        RingGeom g;
        if (i < ns) {
            g.nph = (int32_t)(4 * i);
            g.start_n = 2 * i * (i - 1);
            g.start_s = p.npix - 2 * i * (i + 1);
            const double omz = (double)(i * i) * fact2;
            g.z = 1.0 - omz;
            g.sth = std::sqrt(omz * (2.0 - omz));
            g.phi0_den = (int32_t)(4 * i);
        } else {
            g.nph = (int32_t)(4 * ns);
            g.start_n = 2 * ns * (ns - 1) + (i - ns) * 4 * ns;
            const int64_t is = 4 * ns - i;  // mirrored ring
            g.start_s = 2 * ns * (ns - 1) + (is - ns) * 4 * ns;
            g.z = (double)(2 * ns - i) * fact1;
            g.sth = std::sqrt((1.0 - g.z) * (1.0 + g.z));
            g.phi0_den = ((i + ns) & 1) ? 0 : (int32_t)(4 * ns);
        }
        g.cfold = (g.start_s == g.start_n) ? 1.0 : 2.0;
        p.h_rings[r] = g;
    }
    int st = SFB_OK;
    do {
        if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess ||
            cudaStreamCreateWithFlags(&p.dft_side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&p.dft_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&p.dft_join, cudaEventDisableTiming) != cudaSuccess ||
            [&] {
                for (auto &e : h->ev_copy)
                    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return true;
                return false;
            }()) {
            cudaGetLastError();
            st = fail(SFB_ECUDA, "stream creation failed");
            break;
        }
        if ((st = upload(p, &p.d_rings, p.h_rings.data(), p.h_rings.size())) != SFB_OK) break;
        {
            // twiddle and ring-phase tables (FP64; rounded to the kernel precision on load)
            std::vector<int64_t> twoff(p.nrn);
            std::vector<double2> tw;
            for (int64_t r = 0; r < p.nrn; ++r) {
                const int n = p.h_rings[r].nph;
                twoff[r] = (int64_t)tw.size();
                for (int t = 0; t < n; ++t) {
                    // e^{-2 pi i t/n}: reduce t/n to [0, 1) then use the symmetric range for accuracy
                    const double a = 2.0 * M_PI * (double)t / (double)n;
                    tw.push_back(make_double2(std::cos(a), -std::sin(a)));
                }
            }
            std::vector<double2> ph((size_t)p.nrn * (p.lmax + 1));
            for (int64_t r = 0; r < p.nrn; ++r) {
                const int den = p.h_rings[r].phi0_den;
                for (int m = 0; m <= p.lmax; ++m) {
                    // phi0 = pi/den: reduce m mod 2*den exactly before the trig call
                    const double a = den ? M_PI * (double)(m % (2 * den)) / (double)den : 0.0;
                    ph[(size_t)r * (p.lmax + 1) + m] = make_double2(std::cos(a), -std::sin(a));
                }
            }
            const double wq = 4.0 * M_PI / (double)p.npix;
            std::vector<double2> wph(ph.size());
            std::vector<float2> tw32(tw.size()), wph32(ph.size());
            for (size_t i = 0; i < ph.size(); ++i) {
                wph[i] = make_double2(wq * ph[i].x, wq * ph[i].y);
                wph32[i] = make_float2((float)wph[i].x, (float)wph[i].y);
            }
            for (size_t i = 0; i < tw.size(); ++i) tw32[i] = make_float2((float)tw[i].x, (float)tw[i].y);
            if ((st = upload(p, &p.d_twoff, twoff.data(), twoff.size())) != SFB_OK) break;
            if ((st = upload(p, &p.d_twtab, tw.data(), tw.size())) != SFB_OK) break;
            if ((st = upload(p, &p.d_phase, ph.data(), ph.size())) != SFB_OK) break;
            if ((st = upload(p, &p.d_wphase, wph.data(), wph.size())) != SFB_OK) break;
            if ((st = upload(p, &p.d_twtab32, tw32.data(), tw32.size())) != SFB_OK) break;
            if ((st = upload(p, &p.d_wphase32, wph32.data(), wph32.size())) != SFB_OK) break;
            // tensor-core ring DFT tables: cos(pi k / n), k < 2n, sliced on the scale 2^EB = 2 > |cos|; the
            // quadrature weight is applied in the DFT's epilogue, so cos 0 = 1 is one exact slice (a weighted
            // table entry w would lose its tail slices to the dropped product levels for the small values of
            // a ring, the same loss for every pixel at m = 0, which then adds up instead of averaging out)
            const int EB = 1;
            std::vector<int64_t> doff(p.nrn);
            std::vector<uint2> dtw;
            int64_t eq_off = -1;
            for (int64_t r = 0; r < p.nrn; ++r) {
                const int n = p.h_rings[r].nph;
                const bool eq = r >= ns - 1;
                if (eq && eq_off >= 0) {
                    doff[r] = eq_off;
                    continue;
                }
                doff[r] = (int64_t)dtw.size();
                if (eq) eq_off = doff[r];
                for (int k = 0; k < 2 * n; ++k) {
                    // cos(pi k / n) from the reduced angle: k mod 2n in [0, 2n), symmetric about n
                    const int kk = k <= n ? k : 2 * n - k;
                    double c;
                    if (2 * kk == n) c = 0.0;
                    else if (2 * kk < n) c = std::cos(M_PI * (double)kk / (double)n);
                    else c = -std::cos(M_PI * (double)(n - kk) / (double)n);
                    dtw.push_back(dft_slices(c, EB));
                }
            }
            std::vector<int32_t> crings, coff;
            for (int64_t r = 0; r < ns - 1; ++r) {
                coff.push_back((int32_t)crings.size());
                crings.push_back((int32_t)r);
            }
            p.n_polar = (int)(ns - 1 > 0 ? ns - 1 : 0);
            p.n_eq_cls = 0;
            p.eq_max_rings = 0;
            for (int type = 0; type < 2; ++type) {
                const int32_t start = (int32_t)crings.size();
                for (int64_t r = ns - 1; r < p.nrn; ++r)
                    if ((p.h_rings[r].phi0_den != 0 ? 1 : 0) == type) crings.push_back((int32_t)r);
                if ((int32_t)crings.size() > start) {
                    coff.push_back(start);
                    p.eq_max_rings = std::max(p.eq_max_rings, (int)crings.size() - start);
                    ++p.n_eq_cls;
                }
            }
            coff.push_back((int32_t)crings.size());
            if ((st = upload(p, &p.d_dtw, dtw.data(), dtw.size())) != SFB_OK) break;
            if ((st = upload(p, &p.d_dtw_off, doff.data(), doff.size())) != SFB_OK) break;
            if ((st = upload(p, &p.d_cls_rings, crings.data(), crings.size())) != SFB_OK) break;
            if ((st = upload(p, &p.d_cls_off, coff.data(), coff.size())) != SFB_OK) break;
            p.h_cls_rings = crings;
            p.h_cls_off = coff;
            if ((st = upload<int64_t>(p, &p.d_aimg_off, nullptr, coff.size())) != SFB_OK) break;
            // SFBGPU_DFT_AIMG=0: the DFT's producers slice the map rows themselves (no A image)
            if (const char *e = std::getenv("SFBGPU_DFT_AIMG")) p.dft_aimg = e[0] != '0';
            // SFBGPU_DFT_POLAR_GATHER=1: with the A image, the polar classes gather their twiddles from
            // the ring tables instead of the twiddle image (half the DRAM reads, measured slower)
            if (const char *e = std::getenv("SFBGPU_DFT_POLAR_GATHER")) p.dft_polar_gather = e[0] != '0';
            // B operand image: the polar classes too while the whole image stays under
            // SFBGPU_DFT_IMAGE_MAX_BYTES (default 2 GiB; the equatorial classes are always imaged)
            {
                int64_t IMG_BUDGET = 1LL << 31;
                if (const char *e = std::getenv("SFBGPU_DFT_IMAGE_MAX_BYTES")) IMG_BUDGET = std::atoll(e);
                constexpr int64_t CHUNK_BYTES = 32768;
                std::vector<int64_t> ioff;
                int max_nch = 1;
                p.dtimg_polar = true;
                int64_t nimg = dft_image_offsets(p, crings, coff, true, ioff, max_nch);
                if (nimg * CHUNK_BYTES > IMG_BUDGET) {
                    p.dtimg_polar = false;
                    nimg = dft_image_offsets(p, crings, coff, false, ioff, max_nch);
                }
                if ((st = upload(p, &p.d_dtimg_off, ioff.data(), ioff.size())) != SFB_OK) break;
                if ((st = upload<unsigned char>(p, &p.d_dtimg, nullptr, (size_t)(nimg * CHUNK_BYTES))) != SFB_OK)
                    break;
                launch_build_dft_image(p, max_nch, h->stream);
            }
        }
        std::vector<int64_t> lam_off(2 * (p.lmax + 1));
        int64_t off = 0;
        for (int m = 0; m <= p.lmax; ++m)
            for (int par = 0; par < 2; ++par) {
                lam_off[2 * m + par] = off;
                const int64_t nr = (m + par <= p.lmax) ? (p.lmax - m - par) / 2 + 1 : 0;
                off += nr * p.nrn;
            }
        p.lam_elems = off;
        if ((st = upload(p, &p.d_lam_off, lam_off.data(), lam_off.size())) != SFB_OK) break;
        if ((st = upload<double>(p, &p.d_lam, nullptr, (size_t)off)) != SFB_OK) break;
        if ((st = upload(p, &p.d_spl_off, p.h_spl_off.data(), p.h_spl_off.size())) != SFB_OK) break;
        if ((st = upload(p, &p.d_spl_x, d->spl_x, (size_t)nknots)) != SFB_OK) break;
        if ((st = upload(p, &p.d_spl_y, d->spl_y, (size_t)nknots)) != SFB_OK) break;
        if ((st = upload(p, &p.d_spl_ypp, d->spl_ypp, (size_t)nknots)) != SFB_OK) break;
        if ((st = upload(p, &p.d_pair_n, pair_n.data(), pair_n.size())) != SFB_OK) break;
        if ((st = upload(p, &p.d_pair_l, pair_l.data(), pair_l.size())) != SFB_OK) break;
        if ((st = upload(p, &p.d_out_pair, out_pair.data(), out_pair.size())) != SFB_OK) break;
        if ((st = upload(p, &p.d_out_lm, out_lm.data(), out_lm.size())) != SFB_OK) break;
        if ((st = upload(p, &h->d_pair_index, pair_index.data(), pair_index.size())) != SFB_OK) break;
        if ((st = upload(p, &h->d_noff, noff.data(), noff.size())) != SFB_OK) break;
        if ((st = upload<int>(p, &p.d_err, nullptr, 1)) != SFB_OK) break;
        launch_legendre_table(p, h->stream);
        if ((st = upload<float>(p, &p.d_lam32, nullptr, (size_t)off)) != SFB_OK) break;
        launch_to_float(p.d_lam, off, p.d_lam32, h->stream);
        {
            std::vector<int64_t> toff;
            const int64_t tsz = tc_table_offsets(p, toff);
            if ((st = upload(p, &p.d_lamtc_off, toff.data(), toff.size())) != SFB_OK) break;
            if ((st = upload<uint16_t>(p, (uint16_t **)&p.d_lamtc, nullptr, (size_t)tsz)) != SFB_OK) break;
            if (cudaMemsetAsync(p.d_lamtc, 0, (size_t)tsz * 2, h->stream) != cudaSuccess) {
                st = fail(SFB_ECUDA, "table clear failed");
                break;
            }
            // row scales: Ea per (z, li) row over the rings, Es per (z, ring) over the rows
            const int64_t nrow_tot = off / p.nrn, nes = 2 * (p.lmax + 1) * p.nrn;
            if ((st = grow(p, p.scratch, (size_t)((nrow_tot + nes) / 2 + 2))) != SFB_OK) break;
            int *Ea = reinterpret_cast<int *>(p.scratch.ptr), *Es = Ea + nrow_tot;
            launch_build_lamtc(p, Ea, Es, h->stream);
            std::vector<int64_t> soff;
            const int64_t ssz = tc_synth_table_offsets(p, soff);
            if ((st = upload(p, &p.d_lamts_off, soff.data(), soff.size())) != SFB_OK) break;
            if ((st = upload<uint16_t>(p, (uint16_t **)&p.d_lamts, nullptr, (size_t)ssz)) != SFB_OK) break;
            launch_build_lamts(p, Es, h->stream);
            // SFBGPU_LIVE_CHUNKS=0: no live chunk ranges, so the contractions and the ring DFT run
            // over every chunk and spectrum (the skipped products are exactly zero either way)
            const char *lc = std::getenv("SFBGPU_LIVE_CHUNKS");
            if (!(lc && lc[0] == '0') && (st = build_live_ranges(p, h->stream)) != SFB_OK) break;
        }
        {
            // rings that alias (nph <= 2 lmax) form a prefix: the polar rings grow to the equatorial length
            int ral = 0;
            while (ral < p.nrn && p.h_rings[ral].nph <= 2 * p.lmax) ++ral;
            p.ral = ral;
            p.gram_rows = (int)(p.lmax / 2 + 1);
            // worth it while most rings are alias-free; the FP64 build holds a
            // [2 (lmax+1)][nrn][gram_rows] transient, kept under 4 GiB
            const double build_bytes = 8.0 * 2 * (p.lmax + 1) * (double)p.nrn * p.gram_rows;
            // (SFBGPU_GRAM_REFINEMENT=0 keeps the full synthesis / fold / analysis passes)
            if (const char *fe = std::getenv("SFBGPU_FIELD_MAX_BYTES")) p.field_max_bytes = std::atoll(fe);
            const char *ge = std::getenv("SFBGPU_GRAM_REFINEMENT");
            const bool allowed = !ge || std::atoi(ge) != 0;
            if (allowed && p.niter > 0 && 4 * (int64_t)ral <= 3 * p.nrn && build_bytes <= 4.0 * (1LL << 30)) {
                if ((st = build_gram_tables(p, h->stream)) != SFB_OK) break;
            }
        }
        if (cudaGetLastError() != cudaSuccess) {
            st = fail(SFB_ECUDA, "Legendre table kernel failed to launch");
            break;
        }
        if (p.radial_mode == SFB_RADIAL_POLY) {
            if ((st = choose_radial_basis(h, d)) != SFB_OK) break;
            // double-float coefficients per (l, basis, n) for the mixed-precision projection
            const size_t nct = (size_t)(p.lmax + 1) * p.nbasis * p.nmax;
            if ((st = upload<float2>(p, &p.d_coefT, nullptr, nct)) != SFB_OK) break;
            launch_coef_df(p, h->d_pair_index, p.d_coefT, h->stream);
            const std::vector<int3> tiles = project_tiles(pair_index, (int)p.lmax, (int)p.nmax);
            p.n_proj_tiles = (int64_t)tiles.size();
            if ((st = upload(p, &p.d_proj_tiles, tiles.data(), tiles.size())) != SFB_OK) break;
        } else {
            p.nbasis = p.npairs;
        }
        if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
            st = fail(SFB_ECUDA, std::string("plan setup failed: ") + cudaGetErrorString(cudaGetLastError()));
            break;
        }
    } while (0);
    if (st != SFB_OK) {
        sfb_plan_destroy(h);
        return st;
    }
    *out = h;
    return SFB_OK;
}

void sfb_plan_destroy(sfb_plan *h) {
    if (!h) return;
    Plan &p = h->p;
    cudaSetDevice(p.device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    void *ptrs[] = {p.d_rings, p.d_twtab, p.d_twoff, p.d_phase, p.d_wphase, p.d_twtab32, p.d_wphase32, p.d_dtw,
                    p.d_dtw_off, p.d_dtimg, p.d_dtimg_off, p.d_gramts, p.d_gramts_off, p.d_gram64, p.d_gram_off, p.d_cls_rings, p.d_cls_off, p.d_aimg_off, p.aimg.ptr, p.d_lam, p.d_lam32, p.d_lamtc, p.d_lamtc_off, p.d_lamts, p.d_lamts_off, p.d_lamtc_live, p.d_dft_dead, p.d_lam_off, p.d_spl_off, p.d_spl_x, p.d_spl_y, p.d_spl_ypp,
                    p.d_pair_l, p.d_pair_n, p.d_out_pair, p.d_out_lm, p.d_coef, p.d_coefT, p.d_proj_tiles, p.d_err,
                    p.maps.ptr, p.fbuf.ptr, p.gbuf.ptr, p.rbuf.ptr, p.alm.ptr, p.scratch.ptr, p.scratch2.ptr, p.dep.ptr, p.maps32.ptr,
                    p.ref.ptr, p.rf.ptr, p.rg.ptr, p.rr.ptr, p.ralm.ptr, p.almdf2.ptr, p.adf0.ptr, p.ecoef.ptr, p.erow.ptr, p.almdf.ptr, p.nzr64.ptr, h->d_pair_index, h->d_noff};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (h->aux) sfb_plan_destroy(h->aux);
    collect_stages(h);
    for (cudaEvent_t e : h->pool) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (p.dft_side) cudaStreamDestroy(p.dft_side);
    if (p.dft_fork) cudaEventDestroy(p.dft_fork);
    if (p.dft_join) cudaEventDestroy(p.dft_join);
    for (auto e : h->ev_copy)
        if (e) cudaEventDestroy(e);
    delete h;
}

int sfb_plan_get_info(const sfb_plan *h, sfb_plan_info *info) {
    SFB_TRY(check_plan(h));
    if (!info) return fail(SFB_EINVAL, "info is NULL");
    const Plan &p = h->p;
    info->npix = p.npix;
    info->nlmsize = p.nlmsize;
    info->npairs = p.npairs;
    info->nbasis = p.nbasis;
    info->radial_pieces = p.radial_mode == SFB_RADIAL_POLY ? p.pieces : 0;
    info->radial_degree = p.radial_mode == SFB_RADIAL_POLY ? p.degree : 0;
    info->radial_error = p.radial_mode == SFB_RADIAL_POLY ? p.radial_error : 0.0;
    info->device_bytes = p.device_bytes;
    return SFB_OK;
}

int sfb_set_precision(sfb_plan *h, int32_t precision) {
    SFB_TRY(check_plan(h));
    if (precision != SFB_FP64 && precision != SFB_MIXED) return fail(SFB_EINVAL, "unknown precision");
    h->p.precision = precision;
    return SFB_OK;
}

int sfb_set_profiling(sfb_plan *h, int32_t enable) {
    SFB_TRY(check_plan(h));
    cudaStreamSynchronize(h->stream);
    collect_stages(h);
    h->profile = enable != 0;
    for (int i = 0; i < SFB_NSTAGES; ++i) {
        h->stage_ms[i] = 0;
        h->stage_launches[i] = 0;
    }
    return SFB_OK;
}

int sfb_get_stage_times(const sfb_plan *h, double *ms, int64_t *launches) {
    SFB_TRY(check_plan(h));
    for (int i = 0; i < SFB_NSTAGES; ++i) {
        if (ms) ms[i] = h->stage_ms[i];
        if (launches) launches[i] = h->stage_launches[i];
    }
    return SFB_OK;
}

int64_t sfb_launch_count(void) { return sfb::g_launches.load(); }

int sfb_cat2amln_device(sfb_plan *h, const double *rtp, const double *weight, int64_t ngal, double nbar,
                        const sfb_window *window, double *anlm_out, void *stream) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (!anlm_out) return fail(SFB_EINVAL, "output is NULL");
    return cat2amln_dev(h, rtp, weight, ngal, nbar, window, anlm_out, (cudaStream_t)stream);
}

int sfb_cat2amln(sfb_plan *h, const double *rtp, const double *weight, int64_t ngal, double nbar,
                 const sfb_window *window, double *anlm_out) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (!anlm_out || !window) return fail(SFB_EINVAL, "output or window is NULL");
    if (ngal < 0) return fail(SFB_EINVAL, "ngal < 0");
    if (ngal > 0 && !rtp) return fail(SFB_EINVAL, "rtp is NULL");
    Plan &p = h->p;
    cudaStream_t st = h->stream;
    // device staging: [rtp 3N][w N][out 2*nlmsize][window]
    const int64_t wlen = window->kind == SFB_WINDOW_SEPARABLE ? p.npix + (int64_t)(p.lmax + 1) * p.nmax
                       : window->kind == SFB_WINDOW_DENSE ? p.npix * (int64_t)(p.lmax + 1) * p.nmax : 0;
    const size_t need = (size_t)(3 * ngal + (weight ? ngal : 0) + 2 * p.nlmsize + wlen);
    SFB_TRY(grow(p, p.scratch, need));
    double *d_rtp = p.scratch.ptr;
    double *d_w = weight ? d_rtp + 3 * ngal : nullptr;
    double *d_out = d_rtp + 3 * ngal + (weight ? ngal : 0);
    double *d_win = d_out + 2 * p.nlmsize;
    // the catalogue goes up in NCOPY galaxy ranges on the side stream; the binning of range c
    // starts on the call's stream as soon as range c has landed
    const int ncopy = ngal > 0 ? sfb_plan::NCOPY : 0;
    if (ngal > 0) {
        SFB_CUDA_TRY(cudaEventRecord(h->ev_join, st));          // inputs are the caller's: order after prior work
        SFB_CUDA_TRY(cudaStreamWaitEvent(h->side, h->ev_join, 0));
        const int64_t per = (ngal + ncopy - 1) / ncopy;
        for (int c = 0; c < ncopy; ++c) {
            const int64_t g0 = c * per, n = std::min<int64_t>(per, ngal - g0);
            if (n > 0) {
                SFB_CUDA_TRY(cudaMemcpyAsync(d_rtp + 3 * g0, rtp + 3 * g0, 3 * n * sizeof(double),
                                             cudaMemcpyHostToDevice, h->side));
                if (weight)
                    SFB_CUDA_TRY(cudaMemcpyAsync(d_w + g0, weight + g0, n * sizeof(double), cudaMemcpyHostToDevice,
                                                 h->side));
            }
            SFB_CUDA_TRY(cudaEventRecord(h->ev_copy[c], h->side));
        }
    }
    sfb_window dw = *window;
    if (window->kind == SFB_WINDOW_SEPARABLE) {
        if (!window->mask || !window->w_ln) return fail(SFB_EINVAL, "separable window needs mask and w_ln");
        SFB_CUDA_TRY(cudaMemcpyAsync(d_win, window->mask, p.npix * sizeof(double), cudaMemcpyHostToDevice, st));
        SFB_CUDA_TRY(cudaMemcpyAsync(d_win + p.npix, window->w_ln, (size_t)(p.lmax + 1) * p.nmax * sizeof(double),
                                     cudaMemcpyHostToDevice, st));
        dw.mask = d_win;
        dw.w_ln = d_win + p.npix;
    } else if (window->kind == SFB_WINDOW_DENSE) {
        if (!window->dense) return fail(SFB_EINVAL, "dense window pointer is NULL");
        SFB_CUDA_TRY(cudaMemcpyAsync(d_win, window->dense, (size_t)wlen * sizeof(double), cudaMemcpyHostToDevice, st));
        dw.dense = d_win;
    }
    SFB_TRY(cat2amln_dev(h, ngal > 0 ? d_rtp : nullptr, d_w, ngal, nbar, &dw, d_out, st, ncopy ? h->ev_copy : nullptr,
                         ncopy));
    SFB_CUDA_TRY(cudaMemcpyAsync(anlm_out, d_out, 2 * p.nlmsize * sizeof(double), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    return SFB_OK;
}

// Batched catalogues (mock batches): mock k's galaxies go up on a copy stream into one of two
// staging buffers while mock k - 1 is transformed on the plan's stream; results come back
// per mock.  The device error word collects every mock's errors and is read once.
int sfb_cat2amln_batched(sfb_plan *h, const double *rtp, const double *weight, const int64_t *offsets,
                         int64_t nmocks, const double *nbar, const sfb_window *window, double *anlm_out) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (nmocks < 0 || (nmocks > 0 && (!offsets || !nbar || !anlm_out)) || !window)
        return fail(SFB_EINVAL, "bad batched cat2amln arguments");
    if (nmocks == 0) return SFB_OK;
    int64_t nmax_gal = 0;
    for (int64_t k = 0; k < nmocks; ++k) {
        const int64_t n = offsets[k + 1] - offsets[k];
        if (offsets[k] < 0 || n < 0) return fail(SFB_EINVAL, "offsets must be non-decreasing from 0");
        if (!(std::isfinite(nbar[k]) && nbar[k] != 0.0)) return fail(SFB_ENONFINITE, "nbar must be finite and non-zero");
        nmax_gal = std::max(nmax_gal, n);
    }
    if (offsets[nmocks] > 0 && !rtp) return fail(SFB_EINVAL, "rtp is NULL");
    Plan &p = h->p;
    cudaStream_t st = h->stream;
    const int64_t wlen = window->kind == SFB_WINDOW_SEPARABLE ? p.npix + (int64_t)(p.lmax + 1) * p.nmax
                       : window->kind == SFB_WINDOW_DENSE ? p.npix * (int64_t)(p.lmax + 1) * p.nmax : 0;
    // [window][2 x (rtp 3 nmax_gal, w nmax_gal, out 2 nlmsize)]
    const int64_t per_buf = 3 * nmax_gal + (weight ? nmax_gal : 0) + 2 * p.nlmsize;
    SFB_TRY(grow(p, p.scratch, (size_t)(wlen + 2 * per_buf + 1)));
    double *d_win = p.scratch.ptr;
    sfb_window dw = *window;
    if (window->kind == SFB_WINDOW_SEPARABLE) {
        if (!window->mask || !window->w_ln) return fail(SFB_EINVAL, "separable window needs mask and w_ln");
        SFB_CUDA_TRY(cudaMemcpyAsync(d_win, window->mask, p.npix * sizeof(double), cudaMemcpyHostToDevice, st));
        SFB_CUDA_TRY(cudaMemcpyAsync(d_win + p.npix, window->w_ln, (size_t)(p.lmax + 1) * p.nmax * sizeof(double),
                                     cudaMemcpyHostToDevice, st));
        dw.mask = d_win;
        dw.w_ln = d_win + p.npix;
    } else if (window->kind == SFB_WINDOW_DENSE) {
        if (!window->dense) return fail(SFB_EINVAL, "dense window pointer is NULL");
        SFB_CUDA_TRY(cudaMemcpyAsync(d_win, window->dense, (size_t)wlen * sizeof(double), cudaMemcpyHostToDevice, st));
        dw.dense = d_win;
    } else if (window->kind != SFB_WINDOW_ZERO) {
        return fail(SFB_EINVAL, "unknown window kind");
    }
    cudaStream_t cs = nullptr;
    cudaEvent_t ev[2][sfb_plan::NCOPY + 1] = {};   // per buffer: chunk copies landed, buffer free
    auto release = [&] {
        for (auto &b : ev)
            for (auto &e : b)
                if (e) cudaEventDestroy(e);
        if (cs) cudaStreamDestroy(cs);
    };
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return fail(SFB_ECUDA, "stream creation failed");
    }
    for (auto &b : ev)
        for (auto &e : b)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
                cudaGetLastError();
                release();
                return fail(SFB_ECUDA, "event creation failed");
            }
    int rc = SFB_OK;
    if (cudaMemsetAsync(p.d_err, 0, sizeof(int), st) != cudaSuccess) rc = fail(SFB_ECUDA, "error word reset failed");
    // the copy stream starts after the plan stream's earlier work (the window copy included)
    if (rc == SFB_OK && (cudaEventRecord(ev[1][sfb_plan::NCOPY], st) != cudaSuccess ||
                         cudaEventRecord(ev[0][sfb_plan::NCOPY], st) != cudaSuccess))
        rc = fail(SFB_ECUDA, "event record failed");
    auto dbuf = [&](int64_t k) { return d_win + wlen + (k & 1) * per_buf; };
    // copies of mock k into buffer k & 1, once mock k - 2 released it
    auto enqueue_copy = [&](int64_t k) -> int {
        const int b = (int)(k & 1);
        double *d_rtp = dbuf(k);
        double *d_w = weight ? d_rtp + 3 * nmax_gal : nullptr;
        const int64_t g0 = offsets[k], ngal = offsets[k + 1] - offsets[k];
        if (cudaStreamWaitEvent(cs, ev[b][sfb_plan::NCOPY], 0) != cudaSuccess) return fail(SFB_ECUDA, "stream wait failed");
        const int ncopy = sfb_plan::NCOPY;
        const int64_t per = ngal > 0 ? (ngal + ncopy - 1) / ncopy : 0;
        for (int c = 0; c < ncopy; ++c) {
            const int64_t c0 = c * per, n = std::min<int64_t>(per, ngal - c0);
            if (n > 0) {
                if (cudaMemcpyAsync(d_rtp + 3 * c0, rtp + 3 * (g0 + c0), 3 * n * sizeof(double),
                                    cudaMemcpyHostToDevice, cs) != cudaSuccess ||
                    (weight && cudaMemcpyAsync(d_w + c0, weight + g0 + c0, n * sizeof(double), cudaMemcpyHostToDevice,
                                               cs) != cudaSuccess))
                    return fail(SFB_ECUDA, "catalogue copy failed");
            }
            if (cudaEventRecord(ev[b][c], cs) != cudaSuccess) return fail(SFB_ECUDA, "event record failed");
        }
        return SFB_OK;
    };
    if (rc == SFB_OK) rc = enqueue_copy(0);
    for (int64_t k = 0; k < nmocks && rc == SFB_OK; ++k) {
        // the next mock's copy is queued before this mock's result is read back (which blocks the host
        // for pageable output), so it overlaps this mock's transform
        if (k + 1 < nmocks && (rc = enqueue_copy(k + 1)) != SFB_OK) break;
        const int b = (int)(k & 1);
        double *d_rtp = dbuf(k);
        double *d_w = weight ? d_rtp + 3 * nmax_gal : nullptr;
        double *d_out = d_rtp + 3 * nmax_gal + (weight ? nmax_gal : 0);
        const int64_t ngal = offsets[k + 1] - offsets[k];
        rc = cat2amln_dev(h, ngal > 0 ? d_rtp : nullptr, d_w, ngal, nbar[k], &dw, d_out, st, ev[b],
                          sfb_plan::NCOPY, true);
        if (rc != SFB_OK) break;
        if (cudaEventRecord(ev[b][sfb_plan::NCOPY], st) != cudaSuccess ||
            cudaMemcpyAsync(anlm_out + 2 * p.nlmsize * k, d_out, 2 * p.nlmsize * sizeof(double),
                            cudaMemcpyDeviceToHost, st) != cudaSuccess)
            rc = fail(SFB_ECUDA, "result copy failed");
    }
    int err = 0;
    if (rc == SFB_OK && (cudaMemcpyAsync(&err, p.d_err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                         cudaStreamSynchronize(st) != cudaSuccess))
        rc = fail(SFB_ECUDA, std::string("batched cat2amln failed: ") + cudaGetErrorString(cudaGetLastError()));
    cudaStreamSynchronize(cs);
    release();
    SFB_TRY(rc);
    collect_stages(h);
    if (err & ERR_NONFINITE_INPUT) return fail(SFB_ENONFINITE, "non-finite galaxy coordinate or weight");
    if (err & ERR_THETA_RANGE) return fail(SFB_ERANGE, "galaxy theta outside [0, pi]");
    if (err & ERR_TC_TIMEOUT) return fail(SFB_ETIMEOUT, "tensor-core kernel: bounded mbarrier wait expired");
    if (err & ERR_NONFINITE_OUTPUT) return fail(SFB_ENONFINITE, "non-finite a_nlm (all(isfinite.(anlm)) failed)");
    return SFB_OK;
}

int sfb_map2alm_adjoint(sfb_plan *h, const double *abar, int64_t nmaps, double *maps_out) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (nmaps <= 0 || !abar || !maps_out) return fail(SFB_EINVAL, "bad map2alm adjoint arguments");
    Plan &p = h->p;
    cudaStream_t st = h->stream;
    // abar [nmaps][lmsize] complex (map2alm's output layout) -> [lmsize][2 nmaps] on the device
    std::vector<double> A((size_t)p.lmsize * 2 * nmaps);
    for (int64_t b = 0; b < nmaps; ++b)
        for (int64_t lm = 0; lm < p.lmsize; ++lm) {
            A[(size_t)lm * 2 * nmaps + 2 * b] = abar[(b * p.lmsize + lm) * 2];
            A[(size_t)lm * 2 * nmaps + 2 * b + 1] = abar[(b * p.lmsize + lm) * 2 + 1];
        }
    SFB_TRY(grow(p, p.scratch, A.size()));
    SFB_TRY(grow(p, p.maps, (size_t)nmaps * p.npix));
    SFB_CUDA_TRY(cudaMemcpyAsync(p.scratch.ptr, A.data(), A.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    SFB_TRY(sht_analysis_adjoint(h, p.scratch.ptr, nmaps, p.maps.ptr, st));
    SFB_CUDA_TRY(cudaMemcpyAsync(maps_out, p.maps.ptr, (size_t)nmaps * p.npix * sizeof(double), cudaMemcpyDeviceToHost,
                                 st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    return SFB_OK;
}

int sfb_cat2amln_vjp(sfb_plan *h, const double *rtp, int64_t ngal, double nbar, const double *abar, double *dw_out) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (ngal < 0 || (ngal > 0 && (!rtp || !dw_out)) || !abar) return fail(SFB_EINVAL, "bad cat2amln vjp arguments");
    if (!(std::isfinite(nbar) && nbar != 0.0)) return fail(SFB_ENONFINITE, "nbar must be finite and non-zero");
    Plan &p = h->p;
    if (p.radial_mode != SFB_RADIAL_POLY)
        return fail(SFB_ENOTSUP, "the cat2amln adjoint needs the piecewise-polynomial radial basis (SFB_RADIAL_POLY)");
    if (ngal == 0) return SFB_OK;
    cudaStream_t st = h->stream;
    const double scale = 1.0 / (nbar * 4.0 * M_PI / (double)p.npix);
    const int64_t nbc = std::max<int64_t>(1, std::min<int64_t>(p.nbasis, chunk_pairs(p)));
    // [rtp 3N][dw N][abar 2 nlmsize][Abar lmsize x 2 nbc]
    SFB_TRY(grow(p, p.scratch, (size_t)(4 * ngal + 2 * p.nlmsize + p.lmsize * 2 * nbc)));
    SFB_TRY(grow(p, p.maps, (size_t)nbc * p.npix));
    double *d_rtp = p.scratch.ptr, *d_dw = d_rtp + 3 * ngal, *d_ab = d_dw + ngal, *d_A = d_ab + 2 * p.nlmsize;
    SFB_CUDA_TRY(cudaMemcpyAsync(d_rtp, rtp, 3 * ngal * sizeof(double), cudaMemcpyHostToDevice, st));
    SFB_CUDA_TRY(cudaMemcpyAsync(d_ab, abar, 2 * p.nlmsize * sizeof(double), cudaMemcpyHostToDevice, st));
    SFB_CUDA_TRY(cudaMemsetAsync(d_dw, 0, ngal * sizeof(double), st));
    SFB_CUDA_TRY(cudaMemsetAsync(p.d_err, 0, sizeof(int), st));
    for (int64_t b0 = 0; b0 < p.nbasis; b0 += nbc) {
        const int64_t nb = std::min(nbc, p.nbasis - b0);
        launch_proj_adjoint(p, d_ab, h->d_pair_index, h->d_noff, b0, nb, scale, d_A, st);
        SFB_TRY(sht_analysis_adjoint(h, d_A, nb, p.maps.ptr, st));
        launch_deposit_adjoint(p, d_rtp, ngal, p.maps.ptr, b0, nb, d_dw, st);
    }
    int err = 0;
    SFB_CUDA_TRY(cudaMemcpyAsync(&err, p.d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaMemcpyAsync(dw_out, d_dw, ngal * sizeof(double), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    if (err & ERR_NONFINITE_INPUT) return fail(SFB_ENONFINITE, "non-finite galaxy coordinate");
    if (err & ERR_THETA_RANGE) return fail(SFB_ERANGE, "galaxy theta outside [0, pi]");
    return SFB_OK;
}

// Field staging of field2anlm and its VJP: the whole nr x npix field is held on
// the device when it fits the budget (SFBGPU_FIELD_MAX_BYTES at plan creation,
// else half of the free device memory at the call); otherwise the shells go
// through HBM one chunk at a time, copied between the host field and a
// [npix][chunk] staging buffer with strided (2-D) copies.
// Returns whether the whole field stays resident; otherwise lowers *cs (shells per chunk) so that a
// chunk's staging buffer fits the budget too.
static bool field_resident(const Plan &p, int64_t nr, size_t es, int64_t *cs) {
    int64_t budget = p.field_max_bytes;
    if (budget <= 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
            cudaGetLastError();
            fr = 0;
        }
        budget = (int64_t)(fr / 2);
    }
    const int64_t shell = p.npix * (int64_t)es;
    if (nr * shell <= budget) return true;
    *cs = std::max<int64_t>(1, std::min<int64_t>(*cs, budget / shell));
    return false;
}

static int field2anlm_vjp_impl(sfb_plan *h, const double *abar, int64_t nr, double rmin, double rmax, void *df_out,
                               int32_t dtype) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (!abar || !df_out || nr < 1 || !(rmin < rmax)) return fail(SFB_EINVAL, "bad field2anlm vjp arguments");
    if (dtype != SFB_F64 && dtype != SFB_F32) return fail(SFB_EINVAL, "unknown field dtype");
    Plan &p = h->p;
    cudaStream_t st = h->stream;
    const double dr = (rmax - rmin) / (double)nr;
    int64_t cs = std::max<int64_t>(1, std::min<int64_t>(nr, chunk_pairs(p)));
    const size_t es = dtype == SFB_F32 ? sizeof(float) : sizeof(double);
    const bool resident = field_resident(p, nr, es, &cs);
    const int64_t fld = ((resident ? nr : cs) * p.npix * (int64_t)es + 7) / 8;     // field / staging, in doubles
    // [abar 2 nlmsize][gtab npairs x nr][Abar lmsize x 2 cs][field or staging]
    SFB_TRY(grow(p, p.scratch, (size_t)(2 * p.nlmsize + p.npairs * nr + p.lmsize * 2 * cs + fld)));
    double *d_ab = p.scratch.ptr, *d_g = d_ab + 2 * p.nlmsize, *d_A = d_g + p.npairs * nr;
    double *d_f = d_A + p.lmsize * 2 * cs;
    SFB_CUDA_TRY(cudaMemcpyAsync(d_ab, abar, 2 * p.nlmsize * sizeof(double), cudaMemcpyHostToDevice, st));
    launch_gtab(p, nr, rmin, dr, 1, d_g, st);                // g_nl(r_s) r_s^2 dr, the field2anlm weights
    SFB_TRY(grow(p, p.scratch2, (size_t)cs * p.npairs));
    SFB_TRY(grow(p, p.maps, (size_t)cs * p.npix));
    for (int64_t s0 = 0; s0 < nr; s0 += cs) {
        const int64_t nsc = std::min(cs, nr - s0);
        SFB_CUDA_TRY(cudaMemcpy2DAsync(p.scratch2.ptr, nsc * sizeof(double), d_g + s0, nr * sizeof(double),
                                       nsc * sizeof(double), p.npairs, cudaMemcpyDeviceToDevice, st));
        // Abar_s[lm] = sum_n g_nl(r_s) r_s^2 dr abar_nlm (the transpose of the radial sum)
        launch_shell_alm_g(p, h->d_pair_index, h->d_noff, p.scratch2.ptr, nsc, d_ab, d_A, 2 * nsc, st);
        SFB_TRY(sht_analysis_adjoint(h, d_A, nsc, p.maps.ptr, st));
        // shells s0 .. s0+nsc of df: (ir, p) at ir + nr p (resident) or ir - s0 + nsc p (staging)
        const int64_t ld = resident ? nr : nsc, off = resident ? s0 : 0;
        if (dtype == SFB_F32)
            launch_transpose_ld(p.maps.ptr, p.npix, nsc, p.npix, reinterpret_cast<float *>(d_f) + off, ld, st);
        else
            launch_transpose_ld(p.maps.ptr, p.npix, nsc, p.npix, d_f + off, ld, st);
        if (!resident)
            SFB_CUDA_TRY(cudaMemcpy2DAsync(static_cast<char *>(df_out) + s0 * es, nr * es, d_f, nsc * es, nsc * es,
                                           p.npix, cudaMemcpyDeviceToHost, st));
    }
    SFB_CUDA_TRY(cudaGetLastError());
    if (resident)
        SFB_CUDA_TRY(cudaMemcpyAsync(df_out, d_f, (size_t)nr * p.npix * es, cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    return SFB_OK;
}

int sfb_field2anlm_vjp(sfb_plan *h, const double *abar, int64_t nr, double rmin, double rmax, double *df_out) {
    return field2anlm_vjp_impl(h, abar, nr, rmin, rmax, df_out, SFB_F64);
}

int sfb_field2anlm_vjp_typed(sfb_plan *h, const double *abar, int64_t nr, double rmin, double rmax, void *df_out,
                             int32_t dtype) {
    return field2anlm_vjp_impl(h, abar, nr, rmin, rmax, df_out, dtype);
}

static int sfb_map2alm_impl(sfb_plan *h, const double *maps, int64_t nmaps, double *alm_out) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (nmaps <= 0 || !maps || !alm_out) return fail(SFB_EINVAL, "bad map2alm arguments");
    Plan &p = h->p;
    cudaStream_t st = h->stream;
    SFB_TRY(grow(p, p.maps, (size_t)nmaps * p.npix));
    SFB_CUDA_TRY(cudaMemcpyAsync(p.maps.ptr, maps, (size_t)nmaps * p.npix * sizeof(double), cudaMemcpyHostToDevice, st));
    SFB_TRY(sht_analysis(h, p.maps.ptr, nmaps, st));
    std::vector<double> A((size_t)p.lmsize * 2 * nmaps);
    SFB_CUDA_TRY(cudaMemcpyAsync(A.data(), p.alm.ptr, A.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    for (int64_t b = 0; b < nmaps; ++b)
        for (int64_t lm = 0; lm < p.lmsize; ++lm) {
            alm_out[(b * p.lmsize + lm) * 2] = A[(size_t)lm * 2 * nmaps + 2 * b];
            alm_out[(b * p.lmsize + lm) * 2 + 1] = A[(size_t)lm * 2 * nmaps + 2 * b + 1];
        }
    return SFB_OK;
}

static int sfb_field2anlm_impl(sfb_plan *h, const void *f, int32_t dtype, int64_t nr, double rmin, double rmax,
                               double *anlm_out) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (!f || !anlm_out || nr < 1 || !(rmin < rmax)) return fail(SFB_EINVAL, "bad field2anlm arguments");
    if (dtype != SFB_F64 && dtype != SFB_F32) return fail(SFB_EINVAL, "unknown field dtype");
    Plan &p = h->p;
    cudaStream_t st = h->stream;
    const double dr = (rmax - rmin) / (double)nr;
    int64_t cs = std::max<int64_t>(1, std::min<int64_t>(nr, chunk_pairs(p)));
    const size_t es = dtype == SFB_F32 ? sizeof(float) : sizeof(double);
    const bool resident = field_resident(p, nr, es, &cs);
    const int64_t fld = ((resident ? nr : cs) * p.npix * (int64_t)es + 7) / 8;     // field / staging, in doubles
    // [gtab npairs*nr][out 2*nlmsize][acc 2*nlmsize][field or staging]
    SFB_TRY(grow(p, p.scratch, (size_t)(p.npairs * nr + 4 * p.nlmsize + fld)));
    double *d_g = p.scratch.ptr;
    double *d_out = d_g + p.npairs * nr;
    double *d_acc = d_out + 2 * p.nlmsize;
    double *d_f = d_acc + 2 * p.nlmsize;
    if (resident) SFB_CUDA_TRY(cudaMemcpyAsync(d_f, f, (size_t)nr * p.npix * es, cudaMemcpyHostToDevice, st));
    launch_gtab(p, nr, rmin, dr, 1, d_g, st);
    SFB_CUDA_TRY(cudaMemsetAsync(d_acc, 0, 2 * p.nlmsize * sizeof(double), st));
    SFB_TRY(grow(p, p.scratch2, (size_t)cs * p.npairs));
    const bool mixed = p.precision == SFB_MIXED;
    for (int64_t s0 = 0; s0 < nr; s0 += cs) {
        const int64_t nsc = std::min(cs, nr - s0);
        SFB_TRY(grow(p, p.maps, (size_t)nsc * p.npix));
        if (!resident)
            SFB_CUDA_TRY(cudaMemcpy2DAsync(d_f, nsc * es, static_cast<const char *>(f) + s0 * es, nr * es, nsc * es,
                                           p.npix, cudaMemcpyHostToDevice, st));
        const int64_t ld = resident ? nr : nsc, off = resident ? s0 : 0;
        // maps[s][p] = f[s0+s + nr p]: double-float maps (lo = 0) straight from an FP32 field in mixed
        // precision, else FP64
        bool maps64 = true;
        if (dtype == SFB_F32) {
            const float *src = reinterpret_cast<const float *>(d_f) + off;
            if (mixed) {
                launch_transpose_ld(src, ld, p.npix, nsc, reinterpret_cast<float2 *>(p.maps.ptr), p.npix, st);
                maps64 = false;
            } else {
                launch_transpose_ld(src, ld, p.npix, nsc, p.maps.ptr, p.npix, st);
            }
        } else {
            launch_transpose_ld(d_f + off, ld, p.npix, nsc, p.maps.ptr, p.npix, st);
        }
        SFB_TRY(sht_analysis(h, p.maps.ptr, nsc, st, maps64));     // FP64 maps are converted in mixed precision
        // gtab for this chunk: rows pair, cols nsc (copy sub-block)
        SFB_CUDA_TRY(cudaMemcpy2DAsync(p.scratch2.ptr, nsc * sizeof(double), d_g + s0, nr * sizeof(double),
                                       nsc * sizeof(double), p.npairs, cudaMemcpyDeviceToDevice, st));
        launch_project_shells_g(p, p.scratch2.ptr, nsc, p.alm.ptr, 2 * nsc, d_out, st);
        launch_axpy(d_acc, d_out, 2 * p.nlmsize, st);  // d_acc += d_out
    }
    SFB_CUDA_TRY(cudaMemsetAsync(p.d_err, 0, sizeof(int), st));
    SFB_TRY(finish(h, d_acc, st));
    SFB_CUDA_TRY(cudaMemcpyAsync(anlm_out, d_acc, 2 * p.nlmsize * sizeof(double), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    return SFB_OK;
}

static int sfb_anlm2field_impl(sfb_plan *h, const double *anlm, int64_t nr, double rmin, double rmax, double *f_out) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (!anlm || !f_out || nr < 1 || !(rmin < rmax)) return fail(SFB_EINVAL, "bad anlm2field arguments");
    Plan &p = h->p;
    cudaStream_t st = h->stream;
    const double dr = (rmax - rmin) / (double)nr;
    // [anlm 2*nlmsize][gtab npairs*nr][field nr*npix]
    SFB_TRY(grow(p, p.scratch, (size_t)(2 * p.nlmsize + p.npairs * nr + nr * p.npix)));
    double *d_a = p.scratch.ptr;
    double *d_g = d_a + 2 * p.nlmsize;
    double *d_f = d_g + p.npairs * nr;
    SFB_CUDA_TRY(cudaMemcpyAsync(d_a, anlm, 2 * p.nlmsize * sizeof(double), cudaMemcpyHostToDevice, st));
    launch_gtab(p, nr, rmin, dr, 0, d_g, st);
    const int64_t cs = std::max<int64_t>(1, std::min<int64_t>(nr, chunk_pairs(p)));
    SFB_TRY(grow(p, p.scratch2, (size_t)cs * p.npairs));
    const size_t fsz = (size_t)2 * (p.lmax + 1) * p.nrn * 2 * cs;
    SFB_TRY(grow(p, p.gbuf, fsz));
    SFB_TRY(grow(p, p.alm, (size_t)p.lmsize * 2 * cs));
    SFB_TRY(grow(p, p.maps, (size_t)cs * p.npix));
    for (int64_t s0 = 0; s0 < nr; s0 += cs) {
        const int64_t nsc = std::min(cs, nr - s0);
        SFB_CUDA_TRY(cudaMemcpy2DAsync(p.scratch2.ptr, nsc * sizeof(double), d_g + s0, nr * sizeof(double),
                                       nsc * sizeof(double), p.npairs, cudaMemcpyDeviceToDevice, st));
        launch_shell_alm_g(p, h->d_pair_index, h->d_noff, p.scratch2.ptr, nsc, d_a, p.alm.ptr, 2 * nsc, st);
        launch_leg_synthesis(p, p.alm.ptr, 2 * nsc, p.gbuf.ptr, st);
        launch_ring_synthesis(p, p.gbuf.ptr, nsc, p.maps.ptr, st);
        // f[s0+s + nr p] = maps[s][p]
        launch_transpose_ld(p.maps.ptr, p.npix, nsc, p.npix, d_f + s0, nr, st);
    }
    SFB_CUDA_TRY(cudaGetLastError());
    SFB_CUDA_TRY(cudaMemcpyAsync(f_out, d_f, (size_t)nr * p.npix * sizeof(double), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    return SFB_OK;
}

// The plan's auxiliary FP64 transform at lmax 2 lmax (same nside and niter): one radial
// mode, placeholder splines (it only runs map2alm).
static int aux_plan(sfb_plan *h, sfb_plan **out) {
    if (!h->aux) {
        const Plan &p = h->p;
        const int64_t L = 2 * (int64_t)p.lmax;
        // four knots per spline (the plan's minimum), zero values
        std::vector<int64_t> lmax_n{L}, off((size_t)L + 2);
        std::vector<double> x, zero((size_t)(4 * (L + 1)), 0.0);
        for (int64_t l = 0; l <= L + 1; ++l) off[(size_t)l] = 4 * l;
        for (int64_t l = 0; l <= L; ++l)
            for (int k = 0; k < 4; ++k) x.push_back(p.rmin + (p.rmax - p.rmin) * k / 3.0);
        sfb_plan_desc d{};
        d.nside = p.nside;
        d.lmax = L;
        d.nmax = 1;
        d.lmax_n = lmax_n.data();
        d.rmin = p.rmin;
        d.rmax = p.rmax;
        d.spl_offset = off.data();
        d.spl_x = x.data();
        d.spl_y = zero.data();
        d.spl_ypp = zero.data();
        d.niter = p.niter;
        d.precision = SFB_FP64;
        d.radial_mode = SFB_RADIAL_SPLINE;
        SFB_TRY(sfb_plan_create(&d, &h->aux));
    }
    *out = h->aux;
    return SFB_OK;
}

// a_00 of every shell of a window field win [nr * npix] ((ir, p) at ir + nr p, host), from
// map2alm at lmax 2 lmax with the plan's niter (the reference's calc_Wr_lm(win, 2 lmax, nside)[:, 1]);
// w00 [nr] on the device of h.
static int window_a00(sfb_plan *h, const double *win, int64_t nr, double *w00) {
    sfb_plan *ax = nullptr;
    SFB_TRY(aux_plan(h, &ax));
    Plan &q = ax->p;
    cudaStream_t st = ax->stream;
    const int64_t cs = std::max<int64_t>(1, std::min<int64_t>(nr, chunk_pairs(q)));
    SFB_TRY(grow(q, q.scratch, (size_t)(nr * q.npix)));
    SFB_CUDA_TRY(cudaMemcpyAsync(q.scratch.ptr, win, (size_t)nr * q.npix * sizeof(double), cudaMemcpyHostToDevice,
                                 st));
    for (int64_t s0 = 0; s0 < nr; s0 += cs) {
        const int64_t nsc = std::min(cs, nr - s0);
        SFB_TRY(grow(q, q.maps, (size_t)nsc * q.npix));
        launch_transpose_ld(q.scratch.ptr + s0, nr, q.npix, nsc, q.maps.ptr, q.npix, st);
        SFB_TRY(sht_analysis(ax, q.maps.ptr, nsc, st));
        launch_extract_a00(q.alm.ptr, 2 * nsc, nsc, w00 + s0, st);
    }
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    SFB_CUDA_TRY(cudaGetLastError());
    return SFB_OK;
}

int sfb_win_lnn(sfb_plan *h, const double *win, int64_t nr, double rmin, double rmax, const int64_t *lnn,
                int64_t nlnn, double *out) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (!win || !lnn || nlnn < 0 || (nlnn > 0 && !out) || nr < 1 || !(rmin < rmax))
        return fail(SFB_EINVAL, "bad win_lnn arguments");
    if (nlnn == 0) return SFB_OK;
    Plan &p = h->p;
    if (2 * (int64_t)p.lmax > 4 * p.nside)
        return fail(SFB_ERANGE, "win_lnn: window harmonics to 2 lmax need 2 lmax <= 4 nside");
    for (int64_t i = 0; i < nlnn; ++i) {
        const int64_t l = lnn[3 * i], n1 = lnn[3 * i + 1], n2 = lnn[3 * i + 2];
        if (l < 0 || l > p.lmax || n1 < 1 || n2 < 1 || n1 > p.lmax_n.size() || n2 > p.lmax_n.size() ||
            l > p.lmax_n[n1 - 1] || l > p.lmax_n[n2 - 1])
            return fail(SFB_EINVAL, "win_lnn: (l, n, n') outside the modes");
    }
    cudaStream_t st = h->stream;
    // [w00 nr][gtab npairs x nr][lnn 3 nlnn (int64)][out nlnn]
    SFB_TRY(grow(p, p.scratch2, (size_t)(nr + p.npairs * nr + 3 * nlnn + nlnn)));
    double *d_w00 = p.scratch2.ptr, *d_g = d_w00 + nr;
    int64_t *d_lnn = reinterpret_cast<int64_t *>(d_g + p.npairs * nr);
    double *d_out = reinterpret_cast<double *>(d_lnn + 3 * nlnn);
    SFB_TRY(window_a00(h, win, nr, d_w00));
    const double dr = (rmax - rmin) / (double)nr;
    launch_gtab(p, nr, rmin, dr, 0, d_g, st);                  // g_nl(r_s) at the shell midpoints
    SFB_CUDA_TRY(cudaMemcpyAsync(d_lnn, lnn, (size_t)3 * nlnn * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    launch_win_lnn(p, h->d_pair_index, d_g, nr, rmin, dr, d_w00, d_lnn, nlnn, d_out, st);
    SFB_CUDA_TRY(cudaMemcpyAsync(out, d_out, (size_t)nlnn * sizeof(double), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    SFB_CUDA_TRY(cudaGetLastError());
    for (int64_t i = 0; i < nlnn; ++i)
        if (!std::isfinite(out[i]))
            return fail(SFB_ENONFINITE, "win_lnn: non-finite result (a shell with a negative window mean)");
    return SFB_OK;
}

int sfb_calc_wmix(sfb_plan *h, const double *win, int64_t nr, double rmin, double rmax, int32_t neg_m,
                  double *wmix_out) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (!win || !wmix_out || nr < 1 || !(rmin < rmax)) return fail(SFB_EINVAL, "bad calc_wmix arguments");
    Plan &p = h->p;
    if (p.lmax > WMIX_LMAX) return fail(SFB_ENOTSUP, "calc_wmix: lmax above " + std::to_string(WMIX_LMAX));
    if (2 * (int64_t)p.lmax > 4 * p.nside)
        return fail(SFB_ERANGE, "calc_wmix: window harmonics to 2 lmax need 2 lmax <= 4 nside");
    const size_t smem = wmix_smem_bytes((int)p.lmax, (int)p.lmax, nr, neg_m ? 1 : 0);
    if (smem > 200 * 1024) return fail(SFB_ENOTSUP, "calc_wmix: too many shells for one CTA's shared memory");
    const int64_t LW = 2 * (int64_t)p.lmax, lmsW = (LW + 1) * (LW + 2) / 2;
    const size_t outn = (size_t)2 * p.nlmsize * p.nlmsize;
    // [window harmonics lmsW x 2 nr (shell-major rows)][g table npairs x nr][wmix 2 nlmsize^2]
    double *d = nullptr;
    const size_t total = (size_t)lmsW * 2 * nr + (size_t)p.npairs * nr + outn;
    if (cudaMalloc(&d, total * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return fail(SFB_ENOMEM, "calc_wmix: device allocation failed");
    }
    double *WT = d, *d_g = WT + (size_t)lmsW * 2 * nr, *d_out = d_g + (size_t)p.npairs * nr;
    int st = SFB_OK;
    do {
        sfb_plan *ax = nullptr;
        if ((st = aux_plan(h, &ax)) != SFB_OK) break;
        Plan &q = ax->p;
        cudaStream_t as = ax->stream;
        const int64_t cs = std::max<int64_t>(1, std::min<int64_t>(nr, chunk_pairs(q)));
        if ((st = grow(q, q.scratch, (size_t)(nr * q.npix))) != SFB_OK) break;
        if (cudaMemcpyAsync(q.scratch.ptr, win, (size_t)nr * q.npix * sizeof(double), cudaMemcpyHostToDevice, as) !=
            cudaSuccess) {
            st = fail(SFB_ECUDA, "calc_wmix: window copy failed");
            break;
        }
        for (int64_t s0 = 0; s0 < nr && st == SFB_OK; s0 += cs) {
            const int64_t nsc = std::min(cs, nr - s0);
            if ((st = grow(q, q.maps, (size_t)nsc * q.npix)) != SFB_OK) break;
            launch_transpose_ld(q.scratch.ptr + s0, nr, q.npix, nsc, q.maps.ptr, q.npix, as);
            if ((st = sht_analysis(ax, q.maps.ptr, nsc, as)) != SFB_OK) break;
            // rows lm of the chunk's a_lm (2 nsc doubles) into columns 2 s0 .. of WT's rows
            if (cudaMemcpy2DAsync(WT + 2 * s0, 2 * nr * sizeof(double), q.alm.ptr, 2 * nsc * sizeof(double),
                                  2 * nsc * sizeof(double), (size_t)lmsW, cudaMemcpyDeviceToDevice, as) != cudaSuccess) {
                st = fail(SFB_ECUDA, "calc_wmix: harmonics copy failed");
                break;
            }
        }
        if (st != SFB_OK) break;
        if (cudaStreamSynchronize(as) != cudaSuccess) {
            st = fail(SFB_ECUDA, cudaGetErrorString(cudaGetLastError()));
            break;
        }
        cudaStream_t ms = h->stream;
        const double dr = (rmax - rmin) / (double)nr;
        launch_gtab(p, nr, rmin, dr, 0, d_g, ms);
        launch_wmix(p, h->d_noff, d_g, nr, rmin, dr, WT, 2 * nr, (int)LW, neg_m ? 1 : 0, d_out, smem, ms);
        if (cudaMemcpyAsync(wmix_out, d_out, outn * sizeof(double), cudaMemcpyDeviceToHost, ms) != cudaSuccess ||
            cudaStreamSynchronize(ms) != cudaSuccess) {
            st = fail(SFB_ECUDA, cudaGetErrorString(cudaGetLastError()));
            break;
        }
    } while (0);
    cudaFree(d);
    return st;
}

int sfb_win_rhat_ln_separable(sfb_plan *h, const double *phi, int64_t nr, double rmin, double rmax, double *w_ln_out) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (!phi || !w_ln_out || nr < 1 || !(rmin < rmax)) return fail(SFB_EINVAL, "bad win_rhat_ln arguments");
    Plan &p = h->p;
    cudaStream_t st = h->stream;
    const double dr = (rmax - rmin) / (double)nr;
    const int64_t nout = (int64_t)(p.lmax + 1) * p.nmax;
    SFB_TRY(grow(p, p.scratch, (size_t)(nr + p.npairs * nr + nout)));
    double *d_phi = p.scratch.ptr, *d_g = d_phi + nr, *d_o = d_g + p.npairs * nr;
    SFB_CUDA_TRY(cudaMemcpyAsync(d_phi, phi, nr * sizeof(double), cudaMemcpyHostToDevice, st));
    launch_gtab(p, nr, rmin, dr, 1, d_g, st);
    launch_fill(d_o, nout, NAN, st);
    launch_win_sep_g(p, d_g, nr, d_phi, d_o, st);
    SFB_CUDA_TRY(cudaGetLastError());
    SFB_CUDA_TRY(cudaMemcpyAsync(w_ln_out, d_o, nout * sizeof(double), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    return SFB_OK;
}

int sfb_win_rhat_ln_dense(sfb_plan *h, const double *win, int64_t nr, double rmin, double rmax, double *w_out) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (!win || !w_out || nr < 1 || !(rmin < rmax)) return fail(SFB_EINVAL, "bad win_rhat_ln arguments");
    Plan &p = h->p;
    cudaStream_t st = h->stream;
    const double dr = (rmax - rmin) / (double)nr;
    const int64_t nout = p.npix * (int64_t)(p.lmax + 1) * p.nmax;
    SFB_TRY(grow(p, p.scratch, (size_t)(nr * p.npix + p.npairs * nr + nout)));
    double *d_win = p.scratch.ptr, *d_g = d_win + nr * p.npix, *d_o = d_g + p.npairs * nr;
    SFB_CUDA_TRY(cudaMemcpyAsync(d_win, win, (size_t)nr * p.npix * sizeof(double), cudaMemcpyHostToDevice, st));
    launch_gtab(p, nr, rmin, dr, 1, d_g, st);
    launch_fill(d_o, nout, NAN, st);
    launch_win_dense_g(p, d_g, nr, d_win, d_o, st);
    SFB_CUDA_TRY(cudaGetLastError());
    SFB_CUDA_TRY(cudaMemcpyAsync(w_out, d_o, (size_t)nout * sizeof(double), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    return SFB_OK;
}

int sfb_amln2clnn(sfb_plan *h, const double *anlm1, const double *anlm2, int64_t nbatch, const int64_t *lnn,
                  int64_t nlnn, double *clnn_out) {
    SFB_TRY(check_plan(h));
    SFB_TRY(set_device_of(h));
    if (!anlm1 || !lnn || !clnn_out || nbatch < 1 || nlnn < 0) return fail(SFB_EINVAL, "bad amln2clnn arguments");
    Plan &p = h->p;
    for (int64_t i = 0; i < nlnn; ++i) {
        const int64_t l = lnn[3 * i], n1 = lnn[3 * i + 1], n2 = lnn[3 * i + 2];
        if (n1 < 1 || n2 < 1 || n1 > p.nmax || n2 > p.nmax || l < 0 || l > p.lmax_n[n1 - 1] || l > p.lmax_n[n2 - 1])
            return fail(SFB_EINVAL, "lnn entry " + std::to_string(i) + " is not a mode of the plan");
    }
    if (nlnn == 0) return SFB_OK;
    cudaStream_t st = h->stream;
    const int64_t na = 2 * p.nlmsize * nbatch;
    const bool same = anlm2 == nullptr || anlm2 == anlm1;
    // [a1][a2][lnn (as doubles' storage)][out]
    const size_t need = (size_t)(na * (same ? 1 : 2) + 3 * nlnn + nlnn * nbatch);
    SFB_TRY(grow(p, p.scratch, need));
    double *d1 = p.scratch.ptr;
    double *d2 = same ? d1 : d1 + na;
    int64_t *dl = reinterpret_cast<int64_t *>(d2 + na);
    double *dout = reinterpret_cast<double *>(dl + 3 * nlnn);
    SFB_CUDA_TRY(cudaMemcpyAsync(d1, anlm1, na * sizeof(double), cudaMemcpyHostToDevice, st));
    if (!same) SFB_CUDA_TRY(cudaMemcpyAsync(d2, anlm2, na * sizeof(double), cudaMemcpyHostToDevice, st));
    SFB_CUDA_TRY(cudaMemcpyAsync(dl, lnn, 3 * nlnn * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    launch_amln2clnn(d1, d2, p.nlmsize, dl, nlnn, nbatch, h->d_noff, dout, st);
    SFB_CUDA_TRY(cudaGetLastError());
    SFB_CUDA_TRY(cudaMemcpyAsync(clnn_out, dout, nlnn * nbatch * sizeof(double), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    return SFB_OK;
}

int sfb_winweights2galweights(int64_t nside, const double *weights, int64_t nr, const double *rbounds,
                              const double *rtp, int64_t ngal, double *w_out) {
    if (nside < 1 || nr < 1 || !weights || !rbounds || ngal < 0 || (ngal > 0 && (!rtp || !w_out)))
        return fail(SFB_EINVAL, "bad winweights2galweights arguments");
    if (ngal == 0) return SFB_OK;
    const int64_t npix = 12 * nside * nside;
    const size_t bytes = sizeof(double) * (size_t)(nr * npix + nr + 1 + 3 * ngal + ngal) + sizeof(int);
    char *d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(SFB_ENOMEM, "device allocation failed");
    }
    double *dw = reinterpret_cast<double *>(d);
    double *db = dw + nr * npix;
    double *dr = db + nr + 1;
    double *dout = dr + 3 * ngal;
    int *derr = reinterpret_cast<int *>(dout + ngal);
    int st = SFB_OK;
    int herr = 0;
    do {
        if (cudaMemcpy(dw, weights, sizeof(double) * nr * npix, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(db, rbounds, sizeof(double) * (nr + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dr, rtp, sizeof(double) * 3 * ngal, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemset(derr, 0, sizeof(int)) != cudaSuccess) {
            st = fail(SFB_ECUDA, cudaGetErrorString(cudaGetLastError()));
            break;
        }
        launch_winweights(dw, nr, nside, db, rbounds[nr], dr, ngal, dout, derr, 0);
        if (cudaMemcpy(w_out, dout, sizeof(double) * ngal, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
            st = fail(SFB_ECUDA, cudaGetErrorString(cudaGetLastError()));
            break;
        }
        if (herr & ERR_NONFINITE_INPUT) st = fail(SFB_ENONFINITE, "non-finite galaxy coordinate");
        else if (herr & ERR_RANGE_R) st = fail(SFB_ERANGE, "r out of bounds");
    } while (0);
    cudaFree(d);
    return st;
}

int sfb_ang2pix_ring(int64_t nside, const double *theta, const double *phi, int64_t n, int64_t *pix_out) {
    if (nside < 1 || n < 0 || (n > 0 && (!theta || !phi || !pix_out))) return fail(SFB_EINVAL, "bad ang2pix arguments");
    if (n == 0) return SFB_OK;
    double *d = nullptr;
    int64_t *dp = nullptr;
    SFB_CUDA_TRY(cudaMalloc(&d, 2 * n * sizeof(double)));
    if (cudaMalloc(&dp, n * sizeof(int64_t)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d);
        return fail(SFB_ENOMEM, "allocation failed");
    }
    cudaMemcpy(d, theta, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d + n, phi, n * sizeof(double), cudaMemcpyHostToDevice);
    launch_ang2pix(nside, d, d + n, n, dp, 0);
    cudaError_t e = cudaMemcpy(pix_out, dp, n * sizeof(int64_t), cudaMemcpyDeviceToHost);
    cudaFree(d);
    cudaFree(dp);
    if (e != cudaSuccess) return fail(SFB_ECUDA, cudaGetErrorString(e));
    return SFB_OK;
}

int sfb_map2alm(sfb_plan *h, const double *maps, int64_t nmaps, double *alm_out) {
    SFB_TRY(check_plan(h));
    // these transforms run in FP64 whatever the plan's cat2amln precision
    const int saved = h->p.precision;
    h->p.precision = SFB_FP64;
    const int rc = sfb_map2alm_impl(h, maps, nmaps, alm_out);
    h->p.precision = saved;
    return rc;
}

int sfb_field2anlm(sfb_plan *h, const double *f, int64_t nr, double rmin, double rmax, double *anlm_out) {
    SFB_TRY(check_plan(h));
    // the shell maps go through the plan's transform (FP64, or the mixed tensor-core one)
    return sfb_field2anlm_impl(h, f, SFB_F64, nr, rmin, rmax, anlm_out);
}

int sfb_field2anlm_typed(sfb_plan *h, const void *f, int32_t dtype, int64_t nr, double rmin, double rmax,
                         double *anlm_out) {
    SFB_TRY(check_plan(h));
    return sfb_field2anlm_impl(h, f, dtype, nr, rmin, rmax, anlm_out);
}

int sfb_anlm2field(sfb_plan *h, const double *anlm, int64_t nr, double rmin, double rmax, double *f_out) {
    SFB_TRY(check_plan(h));
    // these transforms run in FP64 whatever the plan's cat2amln precision
    const int saved = h->p.precision;
    h->p.precision = SFB_FP64;
    const int rc = sfb_anlm2field_impl(h, anlm, nr, rmin, rmax, f_out);
    h->p.precision = saved;
    return rc;
}

}  // extern "C"
