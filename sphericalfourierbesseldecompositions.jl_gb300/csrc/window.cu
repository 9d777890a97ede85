// apply_window (reference src/windows.jl:169-216): thinning of a catalogue by a
// shell x pixel window.  Galaxy i is kept when rmin <= r_i <= rmax, its shell
// ceil((r_i - rmin) / dr) (0 becoming 1) is at most nr, and
//   u_i <= win[shell, pix] * (1 / max(win)),
// pix the HEALPix RING pixel of (theta_i, phi_i) and u_i uniform on [0, 1):
// the caller's numbers (the reference draws rand(rng) per galaxy) or the
// counter-based stream u_i = (splitmix64(seed + (i + 1) G) >> 11) 2^-53,
// G = 0x9E3779B97F4A7C15 (Steele, Lea, Flood 2014), which any host can
// reproduce.  The kept galaxies are written in input order: keep flags, an
// exclusive scan of them (the deposit's int32 scan), and a scatter.
//
// Kernels: one pass over the window for its maximum (an atomicMax on an
// order-preserving integer image of the doubles), one pass over the galaxies
// for the flags (24 B read, 4 B written per galaxy), the scan, and the scatter
// (flags read, kept galaxies copied).  All HBM-bound.

#include "sfb_internal.h"

#include <string>

namespace sfb {

namespace {

__device__ __forceinline__ uint64_t splitmix64_at(uint64_t seed, uint64_t i) {
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// order-preserving image of a double (NaN excluded by the caller) and its inverse
__device__ __forceinline__ unsigned long long ord_of_double(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ double double_of_ord(unsigned long long o) {
    const unsigned long long b = (o >> 63) ? (o & 0x7fffffffffffffffull) : ~o;
    return __longlong_as_double((long long)b);
}

// mx: order image of max(win) (preset to 0, below every image); err |= ERR_NONFINITE_INPUT
// for a NaN entry
__global__ void k_window_max(const double *__restrict__ win, int64_t n, unsigned long long *mx, int *err) {
    unsigned long long best = 0;
    bool bad = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = win[i];
        if (v != v) bad = true;
        else best = max(best, ord_of_double(v));
    }
    for (int off = 16; off > 0; off >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, off));
    if ((threadIdx.x & 31) == 0 && best) atomicMax(mx, best);
    if (bad) atomicOr(err, ERR_NONFINITE_INPUT);
}

__global__ void k_window_flags(const double *__restrict__ rtp, int64_t ngal, const double *__restrict__ win,
                               int64_t nr, int64_t nside, double rmin, double rmax, double dr,
                               const double *__restrict__ uniform, uint64_t seed,
                               const unsigned long long *__restrict__ mx, int32_t *__restrict__ flags, int *err) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ngal) return;
    const double r = rtp[3 * i], th = rtp[3 * i + 1], ph = rtp[3 * i + 2];
    int32_t keep = 0;
    if (rmin <= r && r <= rmax) {                           // NaN radii fail the test, as in the reference
        int64_t ir = (int64_t)ceil((r - rmin) / dr);
        if (ir == 0) ir = 1;                                // r == rmin
        if (ir <= nr) {
            if (!isfinite(th) || !isfinite(ph)) {
                atomicOr(err, ERR_NONFINITE_INPUT);
            } else if (th < 0.0 || th > M_PI) {
                atomicOr(err, ERR_THETA_RANGE);
            } else {
                const int64_t pix = ang2pix_ring_fast(nside, th, ph);
                const double oow = 1.0 / double_of_ord(*mx);
                const double u = uniform ? uniform[i] : (double)(splitmix64_at(seed, (uint64_t)i) >> 11) * 0x1.0p-53;
                keep = u <= win[(ir - 1) + nr * pix] * oow ? 1 : 0;
            }
        }
    }
    flags[i] = keep;
}

// off: exclusive scan of the flags (off[ngal] = number kept)
__global__ void k_window_scatter(const double *__restrict__ rtp, int64_t ngal, const int32_t *__restrict__ off,
                                 double *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ngal) return;
    const int32_t o = off[i];
    if (off[i + 1] == o) return;
    out[3 * (int64_t)o] = rtp[3 * i];
    out[3 * (int64_t)o + 1] = rtp[3 * i + 1];
    out[3 * (int64_t)o + 2] = rtp[3 * i + 2];
}

int check_args(int64_t nside, const double *win, int64_t nr, double rmin, double rmax, double dr, const double *rtp,
               int64_t ngal, const double *out, const int64_t *nkept) {
    if (nside < 1 || nside > (int64_t(1) << 13) || nr < 1 || !win || ngal < 0 || !nkept || (ngal > 0 && (!rtp || !out)))
        return fail(SFB_EINVAL, "bad apply_window arguments");
    if (!(rmin <= rmax) || !(dr > 0.0) || !std::isfinite(dr)) return fail(SFB_EINVAL, "apply_window: need rmin <= rmax and dr > 0");
    if (ngal >= (int64_t(1) << 31)) return fail(SFB_EINVAL, "apply_window: more than 2^31 - 1 galaxies");
    return SFB_OK;
}

// Device-pointer core: workspace ws holds [flags ngal + 1][tile sums][max: 1 u64][err: 1 int].
int run(int64_t nside, const double *win, int64_t nr, double rmin, double rmax, double dr, const double *rtp,
        int64_t ngal, const double *uniform, uint64_t seed, double *out, int64_t *nkept, char *ws, cudaStream_t st) {
    const int64_t npix = 12 * nside * nside;
    int32_t *flags = reinterpret_cast<int32_t *>(ws);
    int32_t *tsum = flags + ngal + 1;
    const int64_t ntiles = scan_tile_count(ngal + 1);
    unsigned long long *mx = reinterpret_cast<unsigned long long *>(ws + (((ngal + 1 + ntiles) * 4 + 15) / 16) * 16);
    int *err = reinterpret_cast<int *>(mx + 1);
    SFB_CUDA_TRY(cudaMemsetAsync(mx, 0, sizeof(unsigned long long) + sizeof(int), st));
    k_window_max<<<608, 256, 0, st>>>(win, nr * npix, mx, err);
    note_launch();
    k_window_flags<<<(unsigned)((ngal + 255) / 256), 256, 0, st>>>(rtp, ngal, win, nr, nside, rmin, rmax, dr, uniform,
                                                                   seed, mx, flags, err);
    note_launch();
    SFB_CUDA_TRY(cudaMemsetAsync(flags + ngal, 0, sizeof(int32_t), st));
    launch_exclusive_scan(flags, ngal + 1, tsum, st);
    k_window_scatter<<<(unsigned)((ngal + 255) / 256), 256, 0, st>>>(rtp, ngal, flags, out);
    note_launch();
    int32_t h[2] = {0, 0};
    SFB_CUDA_TRY(cudaMemcpyAsync(&h[0], flags + ngal, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaMemcpyAsync(&h[1], err, sizeof(int), cudaMemcpyDeviceToHost, st));
    SFB_CUDA_TRY(cudaStreamSynchronize(st));
    SFB_CUDA_TRY(cudaGetLastError());
    if (h[1] & ERR_NONFINITE_INPUT) return fail(SFB_ENONFINITE, "apply_window: non-finite window value or direction");
    if (h[1] & ERR_THETA_RANGE) return fail(SFB_ERANGE, "apply_window: galaxy theta outside [0, pi]");
    *nkept = h[0];
    return SFB_OK;
}

size_t workspace_bytes(int64_t ngal) {
    const int64_t ntiles = scan_tile_count(ngal + 1);
    return (size_t)(((ngal + 1 + ntiles) * 4 + 15) / 16) * 16 + 16;
}

}  // namespace
}  // namespace sfb

using namespace sfb;

extern "C" int sfb_apply_window(int64_t nside, const double *win, int64_t nr, double rmin, double rmax, double dr,
                                const double *rtp, int64_t ngal, const double *uniform, uint64_t seed,
                                double *rtp_out, int64_t *nkept) {
    SFB_TRY(check_args(nside, win, nr, rmin, rmax, dr, rtp, ngal, rtp_out, nkept));
    *nkept = 0;
    if (ngal == 0) return SFB_OK;
    const int64_t npix = 12 * nside * nside;
    const size_t wb = sizeof(double) * (size_t)(nr * npix), gb = sizeof(double) * 3 * (size_t)ngal;
    const size_t ub = uniform ? sizeof(double) * (size_t)ngal : 0;
    const size_t total = wb + 2 * gb + ub + workspace_bytes(ngal);
    char *d = nullptr;
    if (cudaMalloc(&d, total) != cudaSuccess) {
        cudaGetLastError();
        return fail(SFB_ENOMEM, "device allocation failed");
    }
    double *dwin = reinterpret_cast<double *>(d);
    double *drtp = reinterpret_cast<double *>(d + wb);
    double *dout = reinterpret_cast<double *>(d + wb + gb);
    double *du = uniform ? reinterpret_cast<double *>(d + wb + 2 * gb) : nullptr;
    char *ws = d + wb + 2 * gb + ub;
    int st = SFB_OK;
    do {
        if (cudaMemcpy(dwin, win, wb, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(drtp, rtp, gb, cudaMemcpyHostToDevice) != cudaSuccess ||
            (du && cudaMemcpy(du, uniform, ub, cudaMemcpyHostToDevice) != cudaSuccess)) {
            st = fail(SFB_ECUDA, cudaGetErrorString(cudaGetLastError()));
            break;
        }
        st = run(nside, dwin, nr, rmin, rmax, dr, drtp, ngal, du, seed, dout, nkept, ws, 0);
        if (st != SFB_OK) break;
        if (*nkept > 0 && cudaMemcpy(rtp_out, dout, sizeof(double) * 3 * (size_t)*nkept, cudaMemcpyDeviceToHost) !=
                              cudaSuccess) {
            st = fail(SFB_ECUDA, cudaGetErrorString(cudaGetLastError()));
            break;
        }
    } while (0);
    cudaFree(d);
    if (st != SFB_OK) *nkept = 0;
    return st;
}

extern "C" int sfb_apply_window_device(int64_t nside, const double *win, int64_t nr, double rmin, double rmax,
                                       double dr, const double *rtp, int64_t ngal, const double *uniform,
                                       uint64_t seed, double *rtp_out, int64_t *nkept, void *stream) {
    SFB_TRY(check_args(nside, win, nr, rmin, rmax, dr, rtp, ngal, rtp_out, nkept));
    *nkept = 0;
    if (ngal == 0) return SFB_OK;
    char *ws = nullptr;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMallocAsync(&ws, workspace_bytes(ngal), st) != cudaSuccess) {
        cudaGetLastError();
        return fail(SFB_ENOMEM, "device allocation failed");
    }
    const int rc = run(nside, win, nr, rmin, rmax, dr, rtp, ngal, uniform, seed, rtp_out, nkept, ws, st);
    cudaFreeAsync(ws, st);
    if (rc != SFB_OK) *nkept = 0;
    return rc;
}
